"""Event sharding: assignment policies and the end-of-job gather, with two
gloo ranks on the CPU (the multi-GPU run shards events with no collective in
the solve; each rank here stands in for one GPU's host process)."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "parallel-fast-marching-method_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from fm3dt import shard  # noqa: E402

NRC = 5


def _fake_times(events):
    """Per-event receiver times a rank would produce (depends on the event only)."""
    e = np.asarray(events, dtype=np.float64)[:, None]
    return (300.0 + 7.0 * e + 0.25 * np.arange(NRC)[None, :]).astype(np.float32)


def _fake_rows(events):
    ptr, cols, vals = [0], [], []
    for e in events:
        for j in range(NRC):
            n = 1 + (e + j) % 3
            cols.append(np.arange(n, dtype=np.int32) + 1 + 10 * e)
            vals.append(np.full(n, -(e + 0.5 * j), dtype=np.float32))
            ptr.append(ptr[-1] + n)
    return shard.FrechetRows(np.array(ptr, np.int64), np.concatenate(cols), np.concatenate(vals))


def test_round_robin_and_balanced_cover_every_event_once():
    for n, ws in [(0, 1), (1, 2), (7, 2), (16, 4), (13, 8)]:
        costs = np.random.default_rng(n).uniform(1, 10, n)
        for policy in ("round_robin", "balanced"):
            parts = shard.assign(costs, ws, policy)
            assert len(parts) == ws
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert all(p == sorted(p) for p in parts)


def test_balanced_is_within_one_event_of_the_mean():
    rng = np.random.default_rng(3)
    # a serving-like mix: cubes of edge 64..256, cost ~ nodes
    edges = rng.integers(64, 257, 200)
    costs = [shard.event_cost((e, e, e)) for e in edges]
    parts = shard.assign(costs, 8, "balanced")
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)


def test_equal_costs_balance_like_round_robin_counts():
    parts = shard.assign([1.0] * 10, 4, "balanced")
    assert sorted(len(p) for p in parts) == [2, 2, 3, 3]


def test_merge_detects_duplicates_and_gaps():
    with pytest.raises(ValueError):
        shard.merge_times(3, [([0, 1], _fake_times([0, 1])), ([1, 2], _fake_times([1, 2]))])
    with pytest.raises(ValueError):
        shard.merge_times(3, [([0, 1], _fake_times([0, 1]))])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, total, out_path):
    import torch.distributed as dist
    sys.path[:0] = [ROOT, PKG]
    from fm3dt import shard as sh
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        costs = [sh.event_cost((64 + 8 * (i % 5),) * 3) for i in range(total)]
        mine = sh.rank_events(costs, ws, rank, "balanced")
        # stand-in for this rank's batched solve of its own events
        piece = (mine, _fake_times(mine), _fake_rows(mine))
        got = sh.gather_to_root(piece, dist)
        if rank == 0:
            times = sh.merge_times(total, [(p[0], p[1]) for p in got])
            rows = sh.merge_frechet(total, NRC, [(p[0], p[2]) for p in got])
            np.savez(out_path, times=times, ptr=rows.row_ptr, cols=rows.cols, vals=rows.vals,
                     sizes=np.array([len(p[0]) for p in got]))
        else:
            assert got is None
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_whole_job(tmp_path):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    total, ws = 11, 2
    out = str(tmp_path / "gathered.npz")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, total, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    z = np.load(out)
    assert z["sizes"].sum() == total and np.all(z["sizes"] > 0)
    assert np.array_equal(z["times"], _fake_times(range(total)))
    ref = _fake_rows(list(range(total)))
    assert np.array_equal(z["ptr"], ref.row_ptr)
    assert np.array_equal(z["cols"], ref.cols)
    assert np.array_equal(z["vals"], ref.vals)
