#!/usr/bin/env python
"""Benchmark of the batched forward traveltime iteration on GB300.

Metric: batched eikonal solves/s (whole job, all GPUs) with p50/p99 step
latency, at <= 1e-5 relative receiver-time error against the plain FP64 GPU
path (checked on 64 events, untimed).

Workload (default): the tomography grid -- 192 x 224 x 224 (r, theta, phi)
propagation nodes, 16 x 20 x 20 B-spline velocity nodes with a +-5%
checkerboard, 500 teleseismic plane-wave events (distance 30-90 deg,
back-azimuth 0-360 deg), 300 surface receivers, single-precision offset
stencils.  Synthetic, seeded inputs (the reference publishes no benchmark and
its boundary-time file is not available).

One step = one forward iteration of all events of this rank: boundary
injection and the solve to convergence, receiver times, and rays with their
Frechet rows (CSR) -- what one tomography iteration needs before the
subspace step (``--step solve`` times the solve alone).  `value` uses
boundary frames, receivers and outputs in HBM (the device-memory entry
points); `e2e` goes through the host entry points with pinned host buffers:
boundary frames and receivers host->device, receiver times and the Frechet
rows device->host inside every step.  The traveltime fields (19 GB per step)
are larger than L2, so no flush is needed between steps.

Multi-GPU (torchrun): events shard across ranks (each rank solves its own
batch of the same size, weak scaling); no data-path collective, a gloo
barrier and a max-reduce of the timings only.

--impl reference: times the CPU oracle (a C restatement of the reference's
serial fast marching, fm3dt_parallel.f90 local_fmm, with srtimes and
parallel_rpaths) on all host cores, one event per core per step, on the same
workload.
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
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--step", choices=["forward", "solve"], default="forward",
                    help="forward: solve + receiver times + rays and Frechet rows; solve: the solve alone")
    ap.add_argument("--scale", type=int, default=0, help="override the grid edge (small profiling cases)")
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--prec", choices=["f32", "f64"], default="f32")
    ap.add_argument("--shape", type=int, default=-1, help="tile shape index (-1: autotune)")
    ap.add_argument("--passes", type=int, default=0)
    ap.add_argument("--sweep-shape", type=int, default=-1, help="sweep tile shape index (-1: same as --shape)")
    ap.add_argument("--no-extras", action="store_true", help="skip the CPU baseline, FP64 checks and e2e leg")
    ap.add_argument("--separate-calls", action="store_true",
                    help="forward step as three calls (solve, receiver times, rays) instead of fm3dt_forward")
    ap.add_argument("--duration", type=float, default=30.0, help="config 4: seconds of Poisson arrivals")
    ap.add_argument("--sweep-mode", type=int, default=1,
                    help="with --shape: 1 sweep then rounds, 2 sweep + verifying sweep, 0 no sweep")
    ap.add_argument("--segments", type=int, nargs=2, default=(0, 0),
                    help="streaming sweep height segments (all events, near-tie events); 0 = automatic")
    ap.add_argument("--schedule", type=float, nargs=4, default=None,
                    metavar=("TIE_SWEEPS", "TIE_RATIO", "RESWEEPS", "RESWEEP_FRAC"),
                    help="with --shape: the solve schedule (negative keeps the default); without --shape the "
                         "autotuner picks it")
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
# and a full mid-sweep launch of a main sweep (the upstream-only form) in four
# height segments (128^3, 64 events: 118.1 MB over 3.87 M nodes); the bench
# scales it to its own launches by the nodes they process.
KERNEL_DRAM_BYTES_PER_NODE = {"round_kernel": 4.15, "stream_sweep_kernel": 30.5}

# Warp instructions per node of the same kernels, from ncu's
# smsp__inst_executed.sum: for the sweep, the same mid-sweep launch of a main
# sweep (58.9 M over 3.87 M nodes; the sweep interval the roofline line times
# holds the main sweeps and the re-sweeps, and the main sweeps are most of
# it), and per node staged by the rounds on the 96^3 case (64 events: first
# rounds after certification and tail rounds together, summed over every
# launch of three solves).  The kernels are bound by instruction issue, so
# the bench also reports the issue rate they reach against the SMs' peak of
# four warp instructions per cycle.
KERNEL_WARP_INST_PER_NODE = {"round_kernel": 41.6, "stream_sweep_kernel": 15.2}


def workload_config(cfg, step, h, nev, nrc, prec):
    """The `config` object of both arms' lines (the same keys and values)."""
    nnr, nnx, nnz = h.nn
    what = ("solve + receiver times + rays and Frechet rows" if step == "forward" else "solve")
    return {"workload": f"config{cfg}: batched teleseismic plane-wave events, {nnr}x{nnx}x{nnz} (r,theta,phi) "
                        f"grid, {h.nv[0]}x{h.nv[1]}x{h.nv[2]} velocity nodes, {nev} events per GPU, {nrc} "
                        f"receivers; one step = {what} of every event",
            "grid": [nnr, nnx, nnz], "velocity_nodes": list(h.nv), "events_per_gpu": nev, "receivers": nrc,
            "step": step, "precision": "FP32 offset" if prec == "f32" else "FP64",
            "l2": "inputs larger than L2 (traveltime fields %.1f GB per step)" %
                  (nev * nnr * nnx * nnz * (4 if prec == "f32" else 8) / 1e9)}


_ORC_CACHE = {}


def _oracle_setup(cfg, scale, nev):
    """Per worker process, once per workload: grid, gridded velocity,
    receivers and boundary frames (not timed)."""
    key = (cfg, scale, nev)
    if key not in _ORC_CACHE:
        import numpy as np
        import oracle as O
        from fm3dt import synth
        w = synth.config(cfg, scale=scale or None, nev=nev)
        h = w.header
        g = O.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
        veln, _ = O.gridder(g, w.velv)
        rcx, rcz = O.latlon_to_rad(w.rec_lat, w.rec_lon)
        rcr = np.asarray(w.rec_elev, dtype=np.float64)
        _ORC_CACHE[key] = (w, g, veln, rcr, rcx, rcz)
    return _ORC_CACHE[key]


def _oracle_event(args):
    """One event on one core (spawned worker): serial fast marching, receiver
    times and rays with Frechet rows (step forward) or the march alone (step
    solve).  Returns the compute seconds; the setup is cached per worker."""
    cfg, scale, ev_index, nev, step = args
    import oracle as O
    from fm3dt import synth
    w, g, veln, rcr, rcx, rcz = _oracle_setup(cfg, scale, nev)
    p = synth.planewave_params(w.header, *w.events[ev_index])
    fr = O.planewave_frame(g, O.PlaneWave(*p))
    t = time.perf_counter()
    ttn, _ = O.fmm(g, veln, fr, 1)
    if step == "forward":
        O.srtimes(g, ttn, rcr, rcx, rcz)
        O.rays(g, ttn, veln, rcr, rcx, rcz)
    return time.perf_counter() - t


def _oracle_warm(args):
    """Warm-up of a worker: imports, the oracle library and the workload's
    setup (not timed)."""
    cfg, scale, nev = args
    _oracle_setup(cfg, scale, nev)
    return 0.0


class CpuPool:
    """`cores` spawned worker processes, one event per core per step.  A
    step's time is the slowest worker's compute time (all run at once)."""

    def __init__(self, cfg, scale, nev, step, cores):
        import multiprocessing as mp
        import oracle
        oracle.build()
        self.cfg, self.scale, self.nev, self.step, self.cores = cfg, scale, nev, step, cores
        self.pool = mp.get_context("spawn").Pool(cores)
        self.pool.map(_oracle_warm, [(cfg, scale, nev)] * cores, chunksize=1)
        self.next = 0

    def sample(self):
        """One step: `cores` events at once; returns (solves/s, step seconds)."""
        jobs = [(self.cfg, self.scale, (self.next + i) % self.nev, self.nev, self.step) for i in range(self.cores)]
        self.next += self.cores
        secs = self.pool.map(_oracle_event, jobs, chunksize=1)
        t = max(secs)
        return self.cores / t, t

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_modes():
    """The reference's two single-event CPU layouts on the 64^3 plane-wave
    event (the plain single-event workload), timed with the oracle: (a) the
    serial march (one rank), (b) the 2 x 2 x 2 decomposed run, its eight
    blocks on eight threads (the reference's mpirun -np 9 compute ranks).
    Seconds per solve, median of three."""
    import numpy as np
    import oracle as O
    from fm3dt import synth
    O.build()
    w = synth.config(0)
    h = w.header
    g = O.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = O.gridder(g, w.velv)
    fr = O.planewave_frame(g, O.PlaneWave(*synth.planewave_params(h, *w.events[0])))

    def med(f):
        ts = []
        for _ in range(3):
            t = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t)
        return statistics.median(ts)

    old = os.environ.get("ORC_DECOMPOSED_THREADS")
    os.environ["ORC_DECOMPOSED_THREADS"] = "8"
    try:
        a = med(lambda: O.fmm(g, veln, fr, 1))
        b = med(lambda: O.fmm_decomposed(g, w.velv, fr, 1, (2, 2, 2)))
    finally:
        if old is None:
            os.environ.pop("ORC_DECOMPOSED_THREADS", None)
        else:
            os.environ["ORC_DECOMPOSED_THREADS"] = old
    return {"workload": "config0: 64x64x64, one plane-wave event", "unit": "s/solve",
            "a_serial_march": a, "b_decomposed_2x2x2_8_threads": b}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_reference(a):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    from fm3dt import synth
    w = synth.config(a.config, scale=a.scale or None, nev=a.events or None)
    nev = len(w.events)
    cores = os.cpu_count() or 1
    pool = CpuPool(a.config, a.scale, nev, a.step, cores)
    for _ in range(a.warmup):
        pool.sample()
    vals, secs = [], []
    for _ in range(a.steps):
        v, t = pool.sample()
        vals.append(v)
        secs.append(t)
    pool.close()
    total = sum(secs)
    value = a.steps * cores / total
    lat = sorted(1000.0 * t for t in secs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * total / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a.config, a.step, w.header, nev, len(w.rec_elev), a.prec),
        "p50_ms": lat[len(lat) // 2], "p99_ms": lat[-1],
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "cpu_model": cpu_model(), "nproc": os.cpu_count(),
                         "sample": f"{cores} events per step (one per core, at once) x {a.steps} steps; per event "
                                   f"the oracle's serial fast marching (C restatement of local_fmm)"
                                   + (", srtimes and parallel_rpaths" if a.step == "forward" else "") +
                                   "; the step's time is its slowest core's compute time (set-up excluded); the "
                                   "Fortran/MPI reference cannot be built: no Fortran or MPI toolchain"},
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
    forward = a.step == "forward"
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
    rcx = np.ascontiguousarray(rcx)
    rcz = np.ascontiguousarray(rcz)
    nrc = len(rcr)
    nrows = nev * nrc
    prec = fm3dt.FP32_OFFSET if a.prec == "f32" else fm3dt.FP64

    solver = fm3dt.Solver(h, fom=1, precision=prec, max_events=nev)
    solver.set_velocity(w.velv)
    d_frames = torch.from_numpy(frames).cuda()
    d_rec = [torch.from_numpy(x).cuda() for x in (rcr, rcx, rcz)]
    rec_ptrs = [x.data_ptr() for x in d_rec]
    d_times = torch.empty((nev, nrc), dtype=torch.float32, device="cuda")
    d_rowptr = torch.empty(nrows + 1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    fptr = d_frames.data_ptr()
    solver.set_sweep_segments(*a.segments)

    if a.shape >= 0:
        sweep_shape = a.sweep_shape if a.sweep_shape >= 0 else a.shape
        solver.set_tuning(a.shape, a.passes or 64, 0, a.sweep_mode)
        solver.set_sweep_shape(sweep_shape)
        if a.schedule:
            solver.set_schedule(int(a.schedule[0]), a.schedule[1], int(a.schedule[2]), a.schedule[3])
        tuned = (a.shape, a.passes or 64, sweep_shape, None, tuple(a.schedule) if a.schedule else None,
                 a.segments[1])
    else:
        # (tuned on the whole batch, up to 512 events: the choice never changes
        # results; the near-tie sweeps' segments only when not given)
        # (each trial the median of three solves: a single one can be slowed by
        # the host, which drives the rounds)
        tuned = autotune.autotune(solver, fptr, min(nev, 512), device=True, repeats=3,
                                  tune_segments=tuple(a.segments) == (0, 0))
    shape = fm3dt.tile_shapes()[tuned[0]]
    sweep_shape_dims = fm3dt.sweep_shapes()[tuned[2]]

    # the Frechet arrays, sized by one untimed forward pass
    cap = 0
    d_cols = d_vals = None
    if forward:
        solver.solve_ptr(nev, fptr, True)
        cap = solver.rays_frechet_device(nrc, *rec_ptrs, d_rowptr.data_ptr(), 1, 1, 0, strict=False)
        cap = int(cap * 1.05) + 1024
        d_cols = torch.empty(cap, dtype=torch.int32, device="cuda")
        d_vals = torch.empty(cap, dtype=torch.float32, device="cuda")

    phase = {"solve": [], "receivers": [], "rays": [], "forward": []}

    fused = forward and not a.separate_calls

    def step_device():
        t0 = time.perf_counter()
        if fused:
            # one call: the solve with the rays of the part that converges
            # first traced inside it, then the receivers and remaining rays
            st, _ = solver.forward_device(nev, fptr, nrc, *rec_ptrs, d_times.data_ptr(), d_rowptr.data_ptr(),
                                          d_cols.data_ptr(), d_vals.data_ptr(), cap)
            phase["forward"].append(1000.0 * (time.perf_counter() - t0))
            return st
        st = solver.solve_ptr(nev, fptr, True)
        t1 = time.perf_counter()
        if forward:
            solver.receiver_times_device(nrc, *rec_ptrs, d_times.data_ptr())
            t2 = time.perf_counter()
            solver.rays_frechet_device(nrc, *rec_ptrs, d_rowptr.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(),
                                       cap)
            t3 = time.perf_counter()
            phase["receivers"].append(1000.0 * (t2 - t1))
            phase["rays"].append(1000.0 * (t3 - t2))
        phase["solve"].append(1000.0 * (t1 - t0))
        return st

    for _ in range(a.warmup):
        step_device()
    for v in phase.values():
        v.clear()
    clocks = Clocks(local if ws > 1 else 0) if rank == 0 else None
    d.barrier()
    torch.cuda.synchronize()
    l0 = solver.launch_count
    t0 = time.perf_counter()
    sts, lat = [], []
    for _ in range(a.steps):
        ts = time.perf_counter()
        sts.append(step_device())
        torch.cuda.synchronize()
        lat.append(1000.0 * (time.perf_counter() - ts))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    d.barrier()
    launches = solver.launch_count - l0
    tt, tu = solver.round_trace()
    trace_tiles, trace_updates = [int(x) for x in tt], [int(x) for x in tu]
    trace_ms = [round(float(x), 4) for x in solver.round_trace_ms()]
    part_ms = [round(float(x), 3) for x in solver.part_ms()]
    tie_run, tie_skip = solver.tie_sweep_items()
    tie_ms = [round(float(x), 3) for x in solver.tie_sweep_ms()]
    clk = clocks.stop() if clocks else None
    dev_ms = sum(s["ms"] for s in sts)
    step_s = wall if forward else max(wall, dev_ms / 1000.0)
    step_s = d.max(step_s)
    value = ws * nev * a.steps / step_s
    lat.sort()
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]
    # The two solver kernels: the rounds (nodes of staged tiles) and the
    # directional sweep.  The solver's sweep interval (start of the sweep to
    # the end of the other events' main sweep, plus the re-sweeps) holds only
    # sweep launches: every event's main sweep, on the context stream and, for
    # the near-tie events, beside it on the second stream, and the re-sweeps.
    # The rounds' interval also holds the near-tie events' extra sweeps, which
    # run beside the first round, so no interval times the round kernel
    # alone.  The roofline line reports the kernel with more work (warp
    # instructions per node from the ncu count x nodes; device time when there
    # is no count) and, for the sweep, the nodes swept inside the sweep
    # interval over its time: a lower bound, since the near-tie events' extra
    # sweeps can start in that interval too.
    round_ms = sum(s["round_ms"] for s in sts)
    round_launches = sum(s["round_launches"] for s in sts)
    staged = sum(s["tile_nodes"] for s in sts)
    sweep_ms = sum(s["sweep_ms"] for s in sts)
    sweep_launches = sum(s["sweep_launches"] for s in sts)
    sweep_nodes = sum(s["sweep_nodes"] for s in sts)
    # nodes swept inside the sweep interval: every event's main sweep and the
    # re-sweeps (the near-tie events' extra sweeps fall in the rounds' interval
    # when the batch is solved in two parts)
    main_nodes = sum(s["interval_nodes"] for s in sts)
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
    # DRAM bytes per node processed, from an ncu capture of a smaller case of
    # the same kernel (KERNEL_DRAM_BYTES_PER_NODE), times the nodes one launch
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
    if forward:
        extras["forward_ms_per_step"] = {k: statistics.median(v) for k, v in phase.items() if v}
        if fused:
            extras["forward_early_ray_events"] = solver.forward_early_events
        extras["frechet_entries_per_step"] = int(d_rowptr[-1].item())
    if not a.no_extras:
        # e2e through the host entry points with pinned host buffers: frames
        # and receivers in, receiver times and Frechet rows out, every step
        h_frames = torch.from_numpy(frames).pin_memory()
        h_out = torch.empty((nev, nrc), dtype=torch.float32).pin_memory()
        h_rowptr = torch.empty(nrows + 1, dtype=torch.int64).pin_memory() if forward else None
        h_cols = torch.empty(max(cap, 1), dtype=torch.int32).pin_memory() if forward else None
        h_vals = torch.empty(max(cap, 1), dtype=torch.float32).pin_memory() if forward else None

        hphase = {"solve": [], "receivers": [], "rays": [], "forward": []}

        def step_host():
            t0_ = time.perf_counter()
            if fused:
                n = solver.forward_into(nev, h_frames.data_ptr(), rcr, rcx, rcz, h_out.data_ptr(),
                                        h_rowptr.data_ptr(), h_cols.data_ptr(), h_vals.data_ptr(), cap)
                hphase["forward"].append(1000.0 * (time.perf_counter() - t0_))
                return n
            solver.solve_ptr(nev, h_frames.data_ptr(), False)
            t1_ = time.perf_counter()
            solver.receiver_times_into(rcr, rcx, rcz, h_out.data_ptr())
            t2_ = time.perf_counter()
            n = 0
            if forward:
                n = solver.rays_frechet_into(rcr, rcx, rcz, h_rowptr.data_ptr(), h_cols.data_ptr(),
                                             h_vals.data_ptr(), cap)
            t3_ = time.perf_counter()
            hphase["solve"].append(1000.0 * (t1_ - t0_))
            hphase["receivers"].append(1000.0 * (t2_ - t1_))
            hphase["rays"].append(1000.0 * (t3_ - t2_))
            return n

        step_host()
        d.barrier()
        t0 = time.perf_counter()
        entries = 0
        for _ in range(a.steps):
            entries = step_host()
        e2e_s = d.max(time.perf_counter() - t0)
        extras["e2e_ms_per_step"] = {k: statistics.median(v[1:]) for k, v in hphase.items() if len(v) > 1}
        if fused:
            # how page-locked frames and rows crossed the host link (measured
            # on the first call: 0 copy engine, 1 kernels through the mapping)
            extras["e2e_host_link"] = dict(zip(("frames", "rows"), solver.host_link()))
        if forward and not fused:
            extras["e2e_ms_per_step"]["rays_parts"] = dict(zip(("trace", "compact", "copy_out", "wall"),
                                                               [round(float(x), 3) for x in solver.rays_ms()]))
        extras["e2e"] = {"value": ws * nev * a.steps / e2e_s, "unit": "solves/s",
                         "h2d_bytes_per_step": int(frames.nbytes + (2 if forward else 1) * 3 * rcr.nbytes),
                         "d2h_bytes_per_step": int(h_out.numel() * 4 +
                                                   ((nrows + 1) * 8 + entries * 8 if forward else 0))}
        trr32 = h_out.numpy().astype(np.float64).copy()
        # the job's one collective: receiver times of every rank's events to
        # rank 0 (host gather, after the timed region)
        got = shard.gather_to_root((mine, h_out.numpy().copy()), getattr(d, "dist", None))
        if rank == 0:
            extras["gathered_events"] = int(shard.merge_times(ws * nev, got).shape[0])
        if rank == 0:
            extras.update(fp64_checks(a, h, w, fptr, frames, rcr, rcx, rcz, rec_ptrs, trr32, solver, d_rowptr,
                                      d_cols, d_vals, cap, forward, value / ws))

    # (tuning details and solver counters sit outside `config`, which both
    # arms print alike)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1000.0 * step_s / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": a.prec, "data": "synthetic",
        "config": workload_config(a.config, a.step, h, nev, nrc, a.prec),
        "tuning": {"tile_shape": list(shape), "max_passes": tuned[1], "sweep_tile_shape": list(sweep_shape_dims),
                   "schedule": dict(zip(("tie_sweeps", "tie_ratio", "resweeps", "resweep_frac"), tuned[4]))
                   if tuned[4] else "default",
                   "tie_segments": tuned[5] if tuned[5] is not None else a.segments[1]},
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
                   "round_trace_ms": trace_ms,
                   "first_round_parts_ms": dict(zip(("tie_sweeps", "tie_round", "certify", "other_round"), part_ms)),
                   "tie_sweep_items": {"run": [int(x) for x in tie_run], "skipped": [int(x) for x in tie_skip],
                                       "ms": tie_ms}},
    }
    line.update(extras)
    if clk:
        line["clocks"] = clk
    if rank == 0 and ws == 1 and not a.no_extras:
        cores = os.cpu_count() or 1
        pool = CpuPool(a.config, a.scale, nev, a.step, cores)
        v, t = pool.sample()
        pool.close()
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                                "cpu_model": cpu_model(), "nproc": os.cpu_count(),
                                "sample": f"{cores} events of this workload at once, one per core: the oracle's "
                                          f"serial fast marching (restatement of local_fmm)"
                                          + (", srtimes and parallel_rpaths" if forward else "") +
                                          f"; {t:.1f} s for the slowest core (set-up excluded)",
                                "modes": cpu_modes()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    d.close()
    return 0


def fp64_checks(a, h, w, fptr, frames, rcr, rcx, rcz, rec_ptrs, trr32, solver, d_rowptr, d_cols, d_vals, cap,
                forward, value_per_gpu):
    """Untimed against the run: the plain FP64 GPU path on the same workload.
    (1) the plain single-event FP64 path, one event per call (>= 10 calls);
    (2) the batched FP64 path on 64 events; (3) the FP32 line's receiver
    times, ray end points and Frechet rows against (2) on those events."""
    import numpy as np
    import torch
    import fm3dt
    nev = len(frames)
    nrc = len(rcr)
    k = min(nev, 64)
    out = {}
    d_t64 = torch.empty((k, nrc), dtype=torch.float32, device="cuda")
    d_rp64 = torch.empty(k * nrc + 1, dtype=torch.int64, device="cuda")
    d_end64 = torch.empty((k * nrc, 3), dtype=torch.float64, device="cuda")
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64, max_events=k) as s64:
        s64.set_velocity(w.velv)
        s64.solve_ptr(k, fptr, True)
        cap64 = s64.rays_frechet_device(nrc, *rec_ptrs, d_rp64.data_ptr(), 1, 1, 0, strict=False) + 1024
        d_c64 = torch.empty(cap64, dtype=torch.int32, device="cuda")
        d_v64 = torch.empty(cap64, dtype=torch.float32, device="cuda")

        def step64():
            s64.solve_ptr(k, fptr, True)
            s64.receiver_times_device(nrc, *rec_ptrs, d_t64.data_ptr())
            if forward:
                s64.rays_frechet_device(nrc, *rec_ptrs, d_rp64.data_ptr(), d_c64.data_ptr(), d_v64.data_ptr(),
                                        cap64, d_end64.data_ptr())

        step64()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(2):
            step64()
        torch.cuda.synchronize()
        out["fp64_batched"] = {"value": 2 * k / (time.perf_counter() - t), "unit": "solves/s", "events": k,
                               "step": a.step}
        t64 = d_t64.cpu().numpy().astype(np.float64)
        rel = float(np.max(np.abs(trr32[:k] - t64) / t64))
        ab = float(np.max(np.abs(trr32[:k] - t64)))
        out["error_vs_plain_fp64"] = {"max_rel": rel, "max_abs_s": ab, "events_checked": k,
                                      "receivers": nrc, "pairs_checked": k * nrc}
        if forward:
            # the FP32 line's rays and rows for the same events
            d_end32 = torch.empty((nev * nrc, 3), dtype=torch.float64, device="cuda")
            solver.rays_frechet_device(nrc, *rec_ptrs, d_rowptr.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(),
                                       cap, d_end32.data_ptr())
            e32 = d_end32[:k * nrc].cpu().numpy()
            e64 = d_end64.cpu().numpy()
            dn = np.array([h.nstep[0], math.radians(h.nstep[1]), math.radians(h.nstep[2])])
            cells = float(np.max(np.abs(e32 - e64) / dn[None, :]))
            rows = _row_differences(d_rowptr, d_cols, d_vals, d_rp64, d_c64, d_v64, k * nrc)
            out["rays_vs_plain_fp64"] = {"endpoint_max_cells": cells, "frechet_row": rows}
    # plain single-event FP64 path: one event per call, solve + receivers (+ rays)
    n1 = 10
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64, max_events=1) as s1:
        s1.set_velocity(w.velv)
        fbytes = frames[0].nbytes

        def one(i):
            s1.solve_ptr(1, fptr + i * fbytes, True)
            s1.receiver_times_device(nrc, *rec_ptrs, d_t64.data_ptr())
            if forward:
                s1.rays_frechet_device(nrc, *rec_ptrs, d_rp64.data_ptr(), d_c64.data_ptr(), d_v64.data_ptr(), cap64)

        one(0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in range(n1):
            one(i % nev)
        torch.cuda.synchronize()
        plain = n1 / (time.perf_counter() - t)
    out["plain_fp64_single_event"] = {"value": plain, "unit": "solves/s", "calls": n1, "step": a.step}
    out["speedup_vs_plain_fp64"] = value_per_gpu / plain
    return out


def _row_differences(rp32, c32, v32, rp64, c64, v64, nrows):
    """Per-row Frechet differences between two CSR matrices (first nrows rows):
    the largest entry difference over the row's largest entry, and the 2-norm
    ratio; their median, 99th percentile and maximum, and the share of rows
    within 1e-4 by both."""
    import numpy as np
    import scipy.sparse as sp
    n32 = int(rp32[nrows].item())
    n64 = int(rp64[nrows].item())
    nmp = int(max(c32[:n32].max().item(), c64[:n64].max().item()))
    A = sp.csr_matrix((v32[:n32].cpu().numpy().astype(np.float64), c32[:n32].cpu().numpy() - 1,
                       rp32[:nrows + 1].cpu().numpy()), shape=(nrows, nmp))
    B = sp.csr_matrix((v64[:n64].cpu().numpy().astype(np.float64), c64[:n64].cpu().numpy() - 1,
                       rp64[:nrows + 1].cpu().numpy()), shape=(nrows, nmp))
    D = (A - B).tocsr()
    bmax = np.asarray(abs(B).max(axis=1).todense()).ravel()
    dmax = np.asarray(abs(D).max(axis=1).todense()).ravel()
    bl2 = np.sqrt(np.asarray(B.multiply(B).sum(axis=1)).ravel())
    dl2 = np.sqrt(np.asarray(D.multiply(D).sum(axis=1)).ravel())
    ok = bmax > 0
    rmax = dmax[ok] / bmax[ok]
    rl2 = dl2[ok] / bl2[ok]
    q = lambda x: {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)), "max": float(x.max())}
    return {"max_entry_rel": q(rmax), "l2_rel": q(rl2), "rows": int(ok.sum()),
            "rows_within_1e-4": float(np.mean((rmax <= 1e-4) & (rl2 <= 1e-4)))}


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
