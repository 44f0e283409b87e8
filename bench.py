#!/usr/bin/env python
"""Benchmark of the batched forward traveltime solve on GB300.

Metric: batched eikonal solves/s (whole job, all GPUs) with p50/p99 step
latency, at <= 1e-5 relative receiver-time error against the plain FP64 GPU
path (checked on a subset of events, untimed).

Workload (default): 128 x 128 x 128 (r, theta, phi) propagation grid, 12 x 14
x 14 B-spline velocity nodes with +-3% Gaussian node noise, 256 teleseismic
plane-wave events (distance 30-90 deg, back-azimuth 0-360 deg), 300 surface
receivers, single-precision offset stencils.  Synthetic, seeded inputs (the
reference publishes no benchmark and its boundary-time file is not
available).

One step = one batched solve of all events of this rank (boundary injection +
tile rounds until convergence).  `value` uses boundary frames already
resident in HBM; `e2e` goes through the public C ABI with pinned host
buffers: boundary frames host->device and receiver times device->host inside
every step.  The traveltime fields (2.1 GB per step) are larger than L2, so
no flush is needed between steps.

Multi-GPU (torchrun): events shard across ranks (each rank solves its own
batch of the same size, weak scaling); no data-path collective, a gloo
barrier and a max-reduce of the timings only.

--impl reference: times the CPU oracle (a C restatement of the reference's
serial fast marching, fm3dt_parallel.f90 local_fmm) on all host cores on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "parallel-fast-marching-method_gb300")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "batched eikonal solves/s + p50/p99 latency at <=1e-5 rel err vs plain GPU path"
B_NODE = {"f32": 12, "f64": 24}      # read t + read s + write t per node of a staged tile


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--scale", type=int, default=0, help="override the grid edge (small profiling cases)")
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--prec", choices=["f32", "f64"], default="f32")
    ap.add_argument("--shape", type=int, default=-1, help="tile shape index (-1: autotune)")
    ap.add_argument("--passes", type=int, default=0)
    ap.add_argument("--sweep-shape", type=int, default=-1, help="sweep tile shape index (-1: same as --shape)")
    ap.add_argument("--no-extras", action="store_true", help="skip the CPU baseline, FP64 check and e2e leg")
    ap.add_argument("--duration", type=float, default=30.0, help="config 4: seconds of Poisson arrivals")
    ap.add_argument("--sweep-mode", type=int, default=1,
                    help="with --shape: 1 sweep then rounds, 2 sweep + verifying sweep, 0 no sweep")
    ap.add_argument("--segments", type=int, nargs=2, default=(0, 0),
                    help="streaming sweep height segments (all events, near-tie events); 0 = automatic")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, rank):
        self.ws, self.rank = ws, rank
        self.pg = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=rank, world_size=ws)
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.proc = None
        self.index = index
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sms.append(float(f[0]))
                maxs.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs), "reasons": sorted(reasons),
                "samples": len(sms)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per node of
# each single-precision solver kernel, from ncu captures of smaller cases of
# the same kernels: a first round with every tile staged (96^3, 64 events)
# and a full mid-sweep launch of a main sweep in four height segments (128^3,
# 64 events); the bench scales it to its own launches by the nodes they
# process.
KERNEL_DRAM_BYTES_PER_NODE = {"round_kernel": 4.15, "stream_sweep_kernel": 30.6}

# Warp instructions per node of the same kernels, from ncu's
# smsp__inst_executed.sum summed over every launch of three solves: per node
# swept on the 128^3 grid with sweeps in two height segments (16 events; the
# 128^3 x 256 workload's main sweeps use two),
# and per node staged by the rounds on the 96^3 case (64 events: first
# rounds after certification and tail rounds together).  The kernels are
# bound by instruction issue, so the bench also reports the issue rate they
# reach against the SMs' peak of four warp instructions per cycle.
KERNEL_WARP_INST_PER_NODE = {"round_kernel": 41.6, "stream_sweep_kernel": 20.15}


def _oracle_event(args):
    """One serial fast-marching solve of one event (spawned worker)."""
    cfg, scale, ev_index, nev = args
    import oracle as O
    from fm3dt import synth
    w = synth.config(cfg, scale=scale or None, nev=nev)
    h = w.header
    g = O.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = O.gridder(g, w.velv)
    p = synth.planewave_params(h, *w.events[ev_index])
    fr = O.planewave_frame(g, O.PlaneWave(*p))
    t = time.perf_counter()
    O.fmm(g, veln, fr, 1)
    return time.perf_counter() - t


def cpu_sample(cfg, scale, nev, n_events, cores):
    """Events across `cores` spawned processes; returns (solves/s, wall s)."""
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    jobs = [(cfg, scale, i % nev, nev) for i in range(n_events)]
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_event, jobs[:cores])          # warm the workers (imports, build check)
        t = time.perf_counter()
        pool.map(_oracle_event, jobs)
        wall = time.perf_counter() - t
    return n_events / wall, wall


def run_reference(a):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    cfg, scale = a.config, a.scale
    from fm3dt import synth
    w = synth.config(cfg, scale=scale or None, nev=a.events or None)
    nev = len(w.events)
    cores = os.cpu_count() or 1
    per_step = cores
    for _ in range(a.warmup):
        cpu_sample(cfg, scale, nev, per_step, cores)
    vals, walls = [], []
    for _ in range(a.steps):
        v, wall = cpu_sample(cfg, scale, nev, per_step, cores)
        vals.append(v)
        walls.append(wall)
    total = sum(walls)
    value = a.steps * per_step / total
    n = w.header.nn
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * total / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"config{cfg}: {n[0]}x{n[1]}x{n[2]} grid, plane-wave events, serial fast marching "
                               f"per event, events spread over {cores} host cores", "grid": list(n)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{per_step} events per step x {a.steps} steps, one event per core "
                                   f"(oracle C restatement of local_fmm; the Fortran/MPI reference cannot be "
                                   f"built: no Fortran or MPI toolchain)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(a):
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    import torch
    import fm3dt
    from fm3dt import autotune, shard, synth
    from fm3dt import build as fb

    d = Dist(ws, rank)
    fb.build()
    w = synth.config(a.config, scale=a.scale or None, nev=a.events or None)
    h = w.header
    nev = len(w.events)
    nnr, nnx, nnz = h.nn
    # shard: the job holds ws x nev events; each rank solves its own share of
    # them (weak scaling), with no collective until the final gather
    mine = list(range(nev))
    events = w.events
    if ws > 1:
        wg = synth.config(a.config, scale=a.scale or None, nev=nev * ws)
        costs = [shard.event_cost(h.nn)] * len(wg.events)
        mine = shard.rank_events(costs, ws, rank, "balanced")
        events = wg.events[mine]
    params = np.array([synth.planewave_params(h, *ev) for ev in events])
    frames = synth.planewave_frames(h, params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.ascontiguousarray(w.rec_elev, dtype=np.float64)
    prec = fm3dt.FP32_OFFSET if a.prec == "f32" else fm3dt.FP64

    solver = fm3dt.Solver(h, fom=1, precision=prec, max_events=nev)
    solver.set_velocity(w.velv)
    d_frames = torch.from_numpy(frames).cuda()
    torch.cuda.synchronize()
    fptr = d_frames.data_ptr()
    solver.set_sweep_segments(*a.segments)

    if a.shape >= 0:
        sweep_shape = a.sweep_shape if a.sweep_shape >= 0 else a.shape
        solver.set_tuning(a.shape, a.passes or 64, 0, a.sweep_mode)
        solver.set_sweep_shape(sweep_shape)
        tuned = (a.shape, a.passes or 64, sweep_shape, None)
    else:
        tuned = autotune.autotune(solver, fptr, nev, device=True)
    shape = fm3dt.tile_shapes()[tuned[0]]
    sweep_shape_dims = fm3dt.sweep_shapes()[tuned[2]]

    for _ in range(a.warmup):
        solver.solve_ptr(nev, fptr, True)
    clocks = Clocks(local if ws > 1 else 0) if rank == 0 else None
    d.barrier()
    torch.cuda.synchronize()
    l0 = solver.launch_count
    t0 = time.perf_counter()
    sts = []
    for _ in range(a.steps):
        sts.append(solver.solve_ptr(nev, fptr, True))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    d.barrier()
    launches = solver.launch_count - l0
    tt, tu = solver.round_trace()
    trace_tiles, trace_updates = [int(x) for x in tt], [int(x) for x in tu]
    trace_ms = [round(float(x), 4) for x in solver.round_trace_ms()]
    clk = clocks.stop() if clocks else None
    dev_ms = sum(s["ms"] for s in sts)
    step_s = max(wall, dev_ms / 1000.0)
    step_s = d.max(step_s)
    value = ws * nev * a.steps / step_s
    lat = sorted(s["ms"] for s in sts)
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]
    # The two solver kernels: the rounds (nodes of staged tiles) and the
    # directional sweep.  The solver's sweep interval (start of the sweep to
    # the end of the other events' main sweep) holds only sweep launches:
    # every event's main sweep, on the context stream and, for the near-tie
    # events, beside it on the second stream.  The rounds' interval also holds
    # the near-tie events' extra sweeps, which run beside the first round, so
    # no interval times the round kernel alone.  The roofline line reports
    # the kernel with more work (warp instructions per node from the ncu count
    # x nodes; device time when there is no count) and, for the sweep, the
    # main sweeps' nodes over the sweep interval: a lower bound, since the
    # near-tie events' extra sweeps start in that interval too.
    round_ms = sum(s["round_ms"] for s in sts)
    round_launches = sum(s["round_launches"] for s in sts)
    staged = sum(s["tile_nodes"] for s in sts)
    sweep_ms = sum(s["sweep_ms"] for s in sts)
    sweep_launches = sum(s["sweep_launches"] for s in sts)
    sweep_nodes = sum(s["sweep_nodes"] for s in sts)
    main_nodes = nev * nnr * nnx * nnz * a.steps if a.sweep_mode == 1 else sweep_nodes
    sweep_name = "stream_sweep_kernel" if sweep_shape_dims[0] == "stream" else "sweep_kernel"
    # name: (interval ms, nodes in it, launches, nodes of all launches)
    kernels = {
        "round_kernel": (round_ms, staged, round_launches, staged),
        sweep_name: (sweep_ms, main_nodes, sweep_launches, sweep_nodes),
    }
    # (the single-precision counts also weigh the double-precision kernels:
    # the same octant work per node; the rounds' interval holds sweeps too, so
    # device time cannot tell them apart)
    if all(k in KERNEL_WARP_INST_PER_NODE for k in kernels):
        work = {k: KERNEL_WARP_INST_PER_NODE[k] * v[3] for k, v in kernels.items()}
    else:
        work = {k: v[0] for k, v in kernels.items()}
    top = max(kernels, key=lambda k: work[k])
    k_ms, k_nodes, k_launches, all_nodes = kernels[top]
    achieved = k_nodes * B_NODE[a.prec] / (k_ms / 1000.0) / 1e9 if k_ms > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()
    per_launch = all_nodes * B_NODE[a.prec] / max(1, k_launches)
    # DRAM bytes per node processed, from the ncu capture of the small case
    # (profiles/solver_kernels_small_case.md), times the nodes one launch
    # processes here on average
    traffic = (KERNEL_DRAM_BYTES_PER_NODE[top] * all_nodes / max(1, k_launches)
               if top in KERNEL_DRAM_BYTES_PER_NODE and a.prec == "f32" else None)

    issue = None
    if top in KERNEL_WARP_INST_PER_NODE and a.prec == "f32" and k_ms > 0:
        n_sm = torch.cuda.get_device_properties(0).multi_processor_count
        mhz = clk["sm_mhz"] if clk else 2070.0
        ach = KERNEL_WARP_INST_PER_NODE[top] * k_nodes / (k_ms / 1000.0) / 1e9
        pk = n_sm * 4 * mhz * 1e6 / 1e9
        issue = {"achieved": ach, "peak": pk, "unit": "G warp-instructions/s", "frac": ach / pk,
                 "inst_per_node": KERNEL_WARP_INST_PER_NODE[top], "sm_mhz": mhz}

    extras = {}
    if not a.no_extras:
        # e2e through the public API with pinned host buffers
        h_frames = torch.from_numpy(frames).pin_memory()
        h_out = torch.empty((nev, len(rcr)), dtype=torch.float32).pin_memory()
        solver.solve_ptr(nev, h_frames.data_ptr(), False)
        solver.receiver_times_into(rcr, rcx, rcz, h_out.data_ptr())
        d.barrier()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            solver.solve_ptr(nev, h_frames.data_ptr(), False)
            solver.receiver_times_into(rcr, rcx, rcz, h_out.data_ptr())
        e2e_s = d.max(time.perf_counter() - t0)
        extras["e2e"] = {"value": ws * nev * a.steps / e2e_s, "unit": "solves/s",
                         "h2d_bytes_per_step": int(frames.nbytes + 3 * rcr.nbytes),
                         "d2h_bytes_per_step": int(h_out.numel() * 4)}
        trr32 = h_out.numpy().astype(np.float64).copy()
        # the job's one collective: receiver times of every rank's events to
        # rank 0 (host gather, after the timed region)
        got = shard.gather_to_root((mine, h_out.numpy().copy()), getattr(d, "dist", None))
        if rank == 0:
            extras["gathered_events"] = int(shard.merge_times(ws * nev, got).shape[0])
        # error against the plain FP64 GPU path on a subset of events (untimed)
        k = min(nev, 8)
        with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64, max_events=k) as s64:
            s64.set_velocity(w.velv)
            s64.solve(frames[:k])
            t64 = s64.receiver_times(rcr, rcx, rcz).astype(np.float64)
            # plain single-event FP64 path: solves/s, one event per solve
            s64.solve(frames[:1])
            t = time.perf_counter()
            n1 = 3
            for i in range(n1):
                s64.solve(frames[i:i + 1])
            plain = n1 / (time.perf_counter() - t)
        rel = float(np.max(np.abs(trr32[:k] - t64) / t64))
        ab = float(np.max(np.abs(trr32[:k] - t64)))
        extras["error_vs_plain_fp64"] = {"max_rel": rel, "max_abs_s": ab, "events_checked": k}
        extras["plain_fp64_single_event"] = {"value": plain, "unit": "solves/s"}
        extras["speedup_vs_plain_fp64"] = value / ws / plain

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1000.0 * step_s / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": a.prec, "data": "synthetic",
        "config": {"workload": f"config{a.config}: batched teleseismic plane-wave events, "
                               f"{nnr}x{nnx}x{nnz} (r,theta,phi) grid, {nev} events per GPU, "
                               f"{len(rcr)} receivers, {'FP32 offset' if a.prec == 'f32' else 'FP64'} stencils",
                   "grid": [nnr, nnx, nnz], "events_per_gpu": nev, "receivers": len(rcr),
                   "tile_shape": list(shape), "max_passes": tuned[1],
                   "sweep_tile_shape": list(sweep_shape_dims),
                   "l2": "inputs larger than L2 (traveltime fields %.1f GB per step)" %
                         (nev * nnr * nnx * nnz * (4 if a.prec == 'f32' else 8) / 1e9)},
        "p50_ms": p50, "p99_ms": p99,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": top, "peak_source": peak_kind,
                     "alg_bytes_per_launch": per_launch,
                     "avg_launch_ms": per_launch / (achieved * 1e6) if achieved > 0 else None,
                     "interval_ms": k_ms, "interval_nodes": k_nodes, "issue": issue},
        "solver": {"rounds_per_solve": round_launches / a.steps,
                   "tile_activations": sum(s["tile_updates"] for s in sts) / a.steps,
                   "node_passes_per_solve": sum(s["node_passes"] for s in sts) / a.steps,
                   "staged_nodes_per_solve": staged / a.steps, "device_ms_per_step": dev_ms / a.steps,
                   "round_ms_per_step": round_ms / a.steps, "sweep_ms_per_step": sweep_ms / a.steps,
                   "sweep_launches_per_step": sweep_launches / a.steps,
                   "sweep_nodes_per_solve": sweep_nodes / a.steps,
                   "work_shares": {k: v / max(1e-9, sum(work.values())) for k, v in work.items()},
                   "round_trace_tiles": trace_tiles, "round_trace_updates": trace_updates,
                   "round_trace_ms": trace_ms},
    }
    line.update(extras)
    if clk:
        line["clocks"] = clk
    if rank == 0 and ws == 1 and not a.no_extras:
        cores = os.cpu_count() or 1
        v, wall = cpu_sample(a.config, a.scale, nev, cores, cores)
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": f"{cores} events of this workload, one per core, serial fast "
                                          f"marching (oracle restatement of local_fmm), {wall:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    d.close()
    return 0


def run_serving(a):
    """Serving workload: Poisson arrivals, 70% teleseismic plane waves on
    cubes of edge U{64..256}, 30% point sources (5-30 km deep, 5x refined
    source grid) on 96^3.  Contexts for every grid of the workload are
    created first (untimed); then an open-loop run at the workload's rate
    gives the latencies, and a saturated run (every request queued at once)
    the throughput."""
    import numpy as np
    import fm3dt
    from fm3dt import serve
    from fm3dt import build as fb
    fb.build()
    models = {}
    dur = a.duration
    wl = serve.Workload(rate=50.0, duration=dur, seed=4001)
    reqs = wl.build(models)
    eng = serve.Engine(models=models, budget_bytes=160 << 30, max_batch=16, workers=6, refine=5, extent=4)
    t0 = time.perf_counter()
    with eng.cv:
        for kind, edge in sorted({(r.kind, r.grid) for r in reqs}):
            eng._admit((kind, edge))
    warm_s = time.perf_counter() - t0
    # warm every context once (first launches, refined-grid contexts)
    warm = [serve.Request(-1 - i, r.kind, r.grid, r.params) for i, r in enumerate(
        {(r.kind, r.grid): r for r in reqs}.values())]
    for r in warm:
        eng.submit(r)
    eng.drain(len(warm), timeout=900)
    clocks = Clocks(0)
    lat, wall = serve.run_open_loop(eng, reqs)
    clk = clocks.stop()
    errors = sum(1 for r in reqs if r.error)
    # saturated: the same requests, all queued at once
    sat = [serve.Request(r.rid, r.kind, r.grid, r.params, 0.0) for r in reqs]
    with eng.cv:
        n0 = len(eng.completed)
    t1 = time.perf_counter()
    for r in sat:
        eng.submit(r)
    eng.drain(n0 + len(sat), timeout=1800)
    sat_s = time.perf_counter() - t1
    batches = [r.batch for r in sat]
    eng.close()
    line = {
        "metric": "serving: solves/s (saturated) + p50/p99 latency at 50 req/s Poisson",
        "value": len(sat) / sat_s, "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": 1000.0 * sat_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"config4: Poisson 50 req/s for {dur:.0f} s (the 300 s trace shortened), 70% "
                               f"teleseismic on cubes of edge U{{64..256}}, 30% point sources on 96^3 at 5-30 km "
                               f"with a 5x refined source grid; 100 receivers per grid",
                   "requests": len(reqs), "grids": len({(r.kind, r.grid) for r in reqs}),
                   "l2": "per-request fields 1-67 MB; no flush between requests (a service sees warm L2)"},
        "p50_ms": float(np.percentile(lat, 50) * 1000.0), "p99_ms": float(np.percentile(lat, 99) * 1000.0),
        "open_loop": {"offered_rps": len(reqs) / dur, "achieved_rps": len(reqs) / wall, "errors": errors,
                      "mean_ms": float(lat.mean() * 1000.0)},
        "saturated": {"requests": len(sat), "seconds": sat_s, "mean_batch": float(np.mean(batches)),
                      "max_batch": int(max(batches))},
        "setup_s": warm_s,
        "cpu_baseline": None,
    }
    if clk:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.config == 4:
        return run_serving(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
