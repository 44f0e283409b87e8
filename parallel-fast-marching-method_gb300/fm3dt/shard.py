"""Event sharding across GPUs (one process per GPU).

The reference solves one source at a time on a 2x2x2 spatial decomposition of
MPI ranks (fm3dt_parallel.f90:6371-6451), exchanging ghost slabs every BSP
round.  One GB300 holds a whole propagation grid, so the GPU version shards
the independent sources ("events") instead: every rank holds the full
velocity model (regenerated from the same .vtx nodes), solves its own subset
of events, and the only collective is one host-side gather of the per-event
results at the end (receiver times and Frechet rows, the inputs of subinv).

Policies:

* ``round_robin`` -- event i goes to rank i % world_size (equal-cost events).
* ``balanced`` -- longest-processing-time greedy on a per-event cost (grid
  nodes x expected sweeps), ties to the lowest rank; each rank's list is
  returned in ascending event order so a rank solves its events in input
  order.
"""
from __future__ import annotations

import heapq
from dataclasses import dataclass

import numpy as np


def event_cost(nn, sweeps: float = 1.0) -> float:
    """Relative cost of one event's solve: propagation nodes x expected
    sweeps over them."""
    nnr, nnx, nnz = nn
    return float(nnr) * float(nnx) * float(nnz) * float(sweeps)


def assign(costs, world_size: int, policy: str = "balanced") -> list[list[int]]:
    """Event indices per rank.  Every event goes to exactly one rank."""
    n = len(costs)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    if policy == "round_robin":
        return [list(range(r, n, world_size)) for r in range(world_size)]
    if policy != "balanced":
        raise ValueError(f"unknown policy {policy!r}")
    order = sorted(range(n), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world_size)]
    out: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(x) for x in out]


def rank_events(costs, world_size: int, rank: int, policy: str = "balanced") -> list[int]:
    return assign(costs, world_size, policy)[rank]


@dataclass
class FrechetRows:
    """CSR rows of one rank (row order = its events x receivers)."""
    row_ptr: np.ndarray     # int64 (nrows + 1)
    cols: np.ndarray        # int32, 1-based model-node columns
    vals: np.ndarray        # float32


def merge_times(total_events: int, pieces) -> np.ndarray:
    """Receiver times of the whole job from per-rank pieces
    ``[(event_indices, times[len(event_indices), nrc]), ...]``."""
    nrc = None
    for idx, t in pieces:
        if len(idx):
            nrc = np.asarray(t).shape[1]
            break
    if nrc is None:
        return np.zeros((total_events, 0), dtype=np.float32)
    out = np.full((total_events, nrc), np.nan, dtype=np.float32)
    seen = np.zeros(total_events, dtype=bool)
    for idx, t in pieces:
        idx = np.asarray(idx, dtype=np.int64)
        if np.any(seen[idx]):
            raise ValueError("an event was solved on two ranks")
        seen[idx] = True
        out[idx] = np.asarray(t, dtype=np.float32).reshape(len(idx), nrc)
    if not np.all(seen):
        raise ValueError("events missing from the gathered pieces: %s" % np.flatnonzero(~seen)[:8].tolist())
    return out


def merge_frechet(total_events: int, nrc: int, pieces) -> FrechetRows:
    """Frechet rows of the whole job in (event, receiver) order from per-rank
    pieces ``[(event_indices, FrechetRows), ...]``; each piece holds
    ``len(event_indices) * nrc`` rows in its own event order."""
    rows: list = [None] * (total_events * nrc)
    for idx, fr in pieces:
        ptr = np.asarray(fr.row_ptr, dtype=np.int64)
        if len(ptr) != len(idx) * nrc + 1:
            raise ValueError("piece has %d rows, expected %d" % (len(ptr) - 1, len(idx) * nrc))
        for k, e in enumerate(idx):
            for j in range(nrc):
                q = k * nrc + j
                g = int(e) * nrc + j
                if rows[g] is not None:
                    raise ValueError("an event was solved on two ranks")
                rows[g] = (fr.cols[ptr[q]:ptr[q + 1]], fr.vals[ptr[q]:ptr[q + 1]])
    if any(r is None for r in rows):
        raise ValueError("events missing from the gathered pieces")
    counts = np.array([len(c) for c, _ in rows], dtype=np.int64)
    row_ptr = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    cols = np.concatenate([c for c, _ in rows]).astype(np.int32) if rows else np.zeros(0, np.int32)
    vals = np.concatenate([v for _, v in rows]).astype(np.float32) if rows else np.zeros(0, np.float32)
    return FrechetRows(row_ptr, cols, vals)


def gather_to_root(obj, dist=None, root: int = 0):
    """Host-side gather of one picklable object per rank (the single
    collective of a sharded run).  Returns the list on ``root`` and None on
    the other ranks; without an initialised process group returns ``[obj]``."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return [obj]
    ws = dist.get_world_size()
    out = [None] * ws if dist.get_rank() == root else None
    dist.gather_object(obj, out, dst=root)
    return out
