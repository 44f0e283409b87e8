"""Serving loop: traveltime requests on one GPU with continuous batching.

A request is one event on one grid: a teleseismic plane wave on a cube of
edge n, or a local point source on the point-source grid; the answer is its
receiver times.  The reference has no such mode (it runs one batch job per
model); this is the service the same solver is deployed behind.

Engine design:

* one solver context per grid, created on first use and kept while the
  device-memory budget allows (admission: a context's fields, max_events x
  nodes x bytes, count against the budget; idle contexts are closed least
  recently used first when a new one would not fit);
* continuous batching: a worker takes every queued request of a grid whose
  context is idle, up to the context's max_events, and solves them as one
  batch -- requests that arrive while a batch runs form the next batch;
* several workers run different grids' batches at once, each context on its
  own CUDA stream (the ctypes calls release the interpreter lock);
* results do not depend on the batch a request lands in: the solve of an
  event is independent of the other events of its batch, bit for bit.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    kind: str                     # "tele" or "point"
    grid: int                     # grid key: cube edge (tele) or the point grid's edge
    params: tuple                 # tele: (t0, p, cos az, sin az); point: (height km, colat, lon)
    arrival: float = 0.0          # seconds on the engine's clock
    done: float = 0.0
    times: np.ndarray = None      # receiver times (float32)
    error: str = ""
    batch: int = 0                # events in the batch that solved it


@dataclass
class GridModel:
    header: object
    velv: np.ndarray
    rcr: np.ndarray
    rcx: np.ndarray
    rcz: np.ndarray


def default_model(edge: int, receivers: int = 100, seed: int = 4001) -> GridModel:
    """The serving workload's grids: a cube of the given edge over the
    synthetic 400 km x 10 deg x 10 deg section with +-3% Gaussian node noise
    and surface receivers."""
    import fm3dt
    from . import synth
    h = synth.section_header(edge, edge, edge, 12, 14, 14)
    velv = synth.velocity_model(h, "gauss", seed)
    el, lat, lon = synth.receivers(h, receivers, seed + 7)
    rcx, rcz = fm3dt.latlon_to_rad(lat, lon)
    return GridModel(h, velv, np.ascontiguousarray(el, dtype=np.float64), rcx, rcz)


class _Ctx:
    def __init__(self, key, model: GridModel, max_events, precision):
        import fm3dt
        self.key = key
        self.model = model
        self.max_events = max_events
        self.solver = fm3dt.Solver(model.header, fom=1, precision=precision, max_events=max_events)
        self.solver.set_velocity(model.velv)
        n = model.header.nn
        self.bytes = int(max_events) * n[0] * n[1] * n[2] * (8 if precision == fm3dt.FP64 else 4)
        self.busy = False
        self.last_used = time.monotonic()

    def close(self):
        self.solver.close()


class Engine:
    def __init__(self, models=None, budget_bytes: int = 64 << 30, max_batch: int = 32, precision=None,
                 workers: int = 4, refine: int = 5, extent: int = 4, event_bytes_cap: int = 2 << 30,
                 ctx_factory=None):
        import fm3dt
        self.precision = fm3dt.FP32_OFFSET if precision is None else precision
        # factory(key, model, max_events) -> context (tests substitute a fake)
        self.ctx_factory = ctx_factory or (lambda key, model, me: _Ctx(key, model, me, self.precision))
        self.models = models if models is not None else {}
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)
        self.refine, self.extent = int(refine), int(extent)
        self.event_bytes_cap = int(event_bytes_cap)
        self.ctxs: dict = {}
        self.queues: dict = collections.defaultdict(collections.deque)
        self.cv = threading.Condition()
        self.stop = False
        self.t0 = time.monotonic()
        self.completed: list = []
        self.stats = collections.Counter()
        self.threads = [threading.Thread(target=self._worker, daemon=True) for _ in range(workers)]
        for t in self.threads:
            t.start()

    # -- clock and submission --------------------------------------------
    def now(self) -> float:
        return time.monotonic() - self.t0

    def submit(self, req: Request):
        with self.cv:
            if not req.arrival:
                req.arrival = self.now()
            self.queues[(req.kind, req.grid)].append(req)
            self.cv.notify()

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        for c in self.ctxs.values():
            c.close()
        self.ctxs.clear()

    def drain(self, n_expected: int, timeout: float = 600.0):
        end = time.monotonic() + timeout
        with self.cv:
            while len(self.completed) < n_expected:
                left = end - time.monotonic()
                if left <= 0:
                    raise TimeoutError(f"{len(self.completed)} of {n_expected} requests finished")
                self.cv.wait(min(left, 0.5))

    # -- contexts and admission -------------------------------------------
    def _model(self, key):
        kind, edge = key
        if edge not in self.models:
            self.models[edge] = default_model(edge)
        return self.models[edge]

    def _max_events(self, model) -> int:
        n = model.header.nn
        per = n[0] * n[1] * n[2] * 4
        return max(1, min(self.max_batch, self.event_bytes_cap // per))

    def _admit(self, key):
        """Context of a grid, creating it within the budget (LRU eviction of
        idle contexts).  Called with the lock held; returns None if it cannot
        be admitted now."""
        c = self.ctxs.get(key)
        if c is not None:
            return c
        model = self._model(key)
        me = self._max_events(model)
        n = model.header.nn
        need = me * n[0] * n[1] * n[2] * 4
        used = sum(x.bytes for x in self.ctxs.values())
        while used + need > self.budget:
            idle = [x for x in self.ctxs.values() if not x.busy]
            if not idle:
                return None
            victim = min(idle, key=lambda x: x.last_used)
            del self.ctxs[victim.key]
            victim.close()
            used -= victim.bytes
            self.stats["evicted"] += 1
        c = self.ctx_factory(key, model, me)
        self.ctxs[key] = c
        self.stats["contexts"] += 1
        return c

    # -- workers ------------------------------------------------------------
    def _pick(self):
        """Oldest waiting request whose grid's context is idle; returns its
        context and up to max_events queued requests of that grid."""
        best = None
        for key, q in self.queues.items():
            if not q:
                continue
            c = self.ctxs.get(key)
            if c is not None and c.busy:
                continue
            if best is None or q[0].arrival < self.queues[best][0].arrival:
                best = key
        if best is None:
            return None, None
        c = self._admit(best)
        if c is None:
            return None, None
        q = self.queues[best]
        batch = [q.popleft() for _ in range(min(len(q), c.max_events))]
        c.busy = True
        return c, batch

    def _worker(self):
        while True:
            with self.cv:
                c = batch = None
                while not self.stop:
                    c, batch = self._pick()
                    if c is not None:
                        break
                    self.cv.wait(0.05)
                if self.stop and c is None:
                    return
            try:
                self._solve(c, batch)
            except Exception as e:  # reported per request, the engine keeps serving
                for r in batch:
                    r.error = str(e)
            finally:
                with self.cv:
                    c.busy = False
                    c.last_used = time.monotonic()
                    t = self.now()
                    for r in batch:
                        r.done = t
                        r.batch = len(batch)
                    self.completed.extend(batch)
                    self.stats["batches"] += 1
                    self.cv.notify_all()

    def _solve(self, c: _Ctx, batch):
        m = c.model
        if batch[0].kind == "tele":
            c.solver.solve_planewave(np.array([r.params for r in batch], dtype=np.float64))
        else:
            c.solver.solve_point(np.array([r.params for r in batch], dtype=np.float64), self.refine, self.extent)
        t = c.solver.receiver_times(m.rcr, m.rcx, m.rcz)
        for i, r in enumerate(batch):
            r.times = t[i].copy()


@dataclass
class Workload:
    """Open-loop arrivals: Poisson at ``rate`` per second for ``duration``
    seconds; a fraction ``point_frac`` are local point sources on the
    ``point_edge`` grid at depth U(5, 30) km, the rest teleseismic plane
    waves (distance U(30, 90) deg, back-azimuth U(0, 360)) on cubes of edge
    U{edge_lo..edge_hi}."""
    rate: float = 50.0
    duration: float = 300.0
    point_frac: float = 0.3
    edge_lo: int = 64
    edge_hi: int = 256
    point_edge: int = 96
    seed: int = 4001
    requests: list = field(default_factory=list)

    def build(self, models: dict):
        from . import synth
        import fm3dt
        rng = np.random.default_rng(self.seed)
        t, rid = 0.0, 0
        out = []
        while True:
            t += rng.exponential(1.0 / self.rate)
            if t >= self.duration:
                break
            if rng.uniform() < self.point_frac:
                edge = self.point_edge
                if edge not in models:
                    models[edge] = default_model(edge)
                h = models[edge].header
                fx = rng.uniform(6, h.nn[1] - 7)
                fz = rng.uniform(6, h.nn[2] - 7)
                colat, lon = fm3dt.latlon_to_rad(np.array([h.norig[1] - fx * h.nstep[1]]),
                                                 np.array([h.norig[2] + fz * h.nstep[2]]))
                out.append(Request(rid, "point", edge, (-rng.uniform(5.0, 30.0), colat[0], lon[0]), t))
            else:
                edge = int(rng.integers(self.edge_lo, self.edge_hi + 1))
                if edge not in models:
                    models[edge] = default_model(edge)
                p = synth.planewave_params(models[edge].header, rng.uniform(30, 90), rng.uniform(0, 360))
                out.append(Request(rid, "tele", edge, tuple(p), t))
            rid += 1
        self.requests = out
        return out


def run_open_loop(engine: Engine, requests, speed: float = 1.0):
    """Submits the requests at their arrival times (scaled by 1/speed) and
    waits for all; returns (latencies s, wall s)."""
    t0 = engine.now()
    with engine.cv:
        n0 = len(engine.completed)
    for r in requests:
        target = t0 + r.arrival / speed
        delay = target - engine.now()
        if delay > 0:
            time.sleep(delay)
        r.arrival = engine.now()
        engine.submit(r)
    engine.drain(n0 + len(requests))
    wall = engine.now() - t0
    lat = np.array([r.done - r.arrival for r in requests])
    return lat, wall
