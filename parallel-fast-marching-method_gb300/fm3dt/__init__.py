"""Python binding of libfm3dt_gpu (the C ABI in include/fm3dt_gpu.h).

This is the host-side mirror of the reference program's per-source pipeline
(fm3dt_parallel.f90): grid header in, velocity nodes in, boundary frames (or
synthetic plane waves) in, traveltime fields, receiver times, rays and
Frechet rows out.  Every call goes through the CUDA library; there is no CPU
fallback, and loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "libfm3dt_gpu.so")

FP64 = 0
FP32_OFFSET = 1

OK, EINVAL, ENOMEM, ECUDA, ENOCONV, ERANGE, ESTATE, ENODEV = 0, -1, -2, -3, -4, -5, -6, -7
_ERRNAMES = {EINVAL: "EINVAL", ENOMEM: "ENOMEM", ECUDA: "ECUDA", ENOCONV: "ENOCONV",
             ERANGE: "ERANGE", ESTATE: "ESTATE", ENODEV: "ENODEV"}


class Fm3dtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [
        ("nvr", C.c_int), ("nvx", C.c_int), ("nvz", C.c_int),
        ("gor", C.c_double), ("goxd", C.c_double), ("gozd", C.c_double),
        ("dvr", C.c_double), ("dvxd", C.c_double), ("dvzd", C.c_double),
        ("nnr", C.c_int), ("nnx", C.c_int), ("nnz", C.c_int),
        ("rgor", C.c_double), ("rgoxd", C.c_double), ("rgozd", C.c_double),
        ("dnr", C.c_double), ("dnxd", C.c_double), ("dnzd", C.c_double),
        ("earth", C.c_double),
        ("fom", C.c_int), ("precision", C.c_int), ("max_events", C.c_int),
    ]


class Status(C.Structure):
    _fields_ = [("rounds", C.c_int), ("converged", C.c_int), ("tile_updates", C.c_int64),
                ("node_passes", C.c_int64), ("tile_nodes", C.c_int64), ("ms", C.c_double),
                ("round_ms", C.c_double), ("round_launches", C.c_int), ("sweep_launches", C.c_int),
                ("sweep_ms", C.c_double), ("sweep_nodes", C.c_int64), ("interval_nodes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = [
    "fm3dt_ctx_create", "fm3dt_set_velocity", "fm3dt_solve", "fm3dt_solve_device", "fm3dt_solve_resume",
    "fm3dt_solve_planewave", "fm3dt_solve_point",
    "fm3dt_receiver_times", "fm3dt_rays_frechet", "fm3dt_receiver_times_device", "fm3dt_rays_frechet_device",
    "fm3dt_forward", "fm3dt_forward_device", "fm3dt_forward_early_events", "fm3dt_set_host_link",
    "fm3dt_host_link", "fm3dt_get_times", "fm3dt_get_velocity", "fm3dt_set_times",
    "fm3dt_set_tuning", "fm3dt_set_schedule", "fm3dt_set_sweep_shape", "fm3dt_set_sweep_segments", "fm3dt_round_trace", "fm3dt_round_trace_ms", "fm3dt_part_ms", "fm3dt_rays_ms", "fm3dt_tie_sweep_items", "fm3dt_tie_sweep_ms", "fm3dt_tile_shapes", "fm3dt_tile_shape",
    "fm3dt_launch_count",
    "fm3dt_last_error", "fm3dt_ctx_destroy",
]

_lib = None


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libfm3dt_gpu.so not built ({p}); run __graft_entry__.build()")
    L = C.CDLL(p)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    L.fm3dt_ctx_create.argtypes = [C.POINTER(GridDesc), C.POINTER(vp)]
    L.fm3dt_set_velocity.argtypes = [vp, dp]
    L.fm3dt_solve.argtypes = [vp, C.c_int, dp, C.POINTER(Status)]
    L.fm3dt_solve_planewave.argtypes = [vp, C.c_int, dp, C.POINTER(Status)]
    L.fm3dt_solve_point.argtypes = [vp, C.c_int, dp, C.c_int, C.c_int, C.POINTER(Status)]
    L.fm3dt_solve_device.argtypes = [vp, C.c_int, C.c_void_p, C.POINTER(Status)]
    L.fm3dt_solve_resume.argtypes = [vp, C.POINTER(Status)]
    L.fm3dt_receiver_times.argtypes = [vp, C.c_int, dp, dp, dp, C.POINTER(C.c_float)]
    L.fm3dt_rays_frechet.argtypes = [vp, C.c_int, dp, dp, dp, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_float), C.c_int64, dp]
    L.fm3dt_receiver_times_device.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.fm3dt_rays_frechet_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, C.c_int64,
                                            C.POINTER(C.c_int64), vp]
    L.fm3dt_forward.argtypes = [vp, C.c_int, dp, C.c_int, dp, dp, dp, C.POINTER(C.c_float), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_int64, dp, C.POINTER(Status)]
    L.fm3dt_forward_device.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_int64,
                                       C.POINTER(C.c_int64), vp, C.POINTER(Status)]
    L.fm3dt_forward_early_events.argtypes = [vp]
    L.fm3dt_set_host_link.argtypes = [vp, C.c_int]
    L.fm3dt_host_link.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.fm3dt_get_times.argtypes = [vp, C.c_int, dp]
    L.fm3dt_set_times.argtypes = [vp, C.c_int, C.c_int, dp]
    L.fm3dt_get_velocity.argtypes = [vp, dp]
    L.fm3dt_set_tuning.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.fm3dt_set_sweep_shape.argtypes = [vp, C.c_int]
    L.fm3dt_set_schedule.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_double]
    L.fm3dt_set_sweep_segments.argtypes = [vp, C.c_int, C.c_int]
    L.fm3dt_round_trace.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.fm3dt_round_trace_ms.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.fm3dt_part_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.fm3dt_rays_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.fm3dt_tie_sweep_items.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.fm3dt_tie_sweep_ms.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.fm3dt_tile_shapes.argtypes = [C.POINTER(C.c_int)]
    L.fm3dt_tile_shape.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.fm3dt_launch_count.argtypes = [vp]
    L.fm3dt_launch_count.restype = C.c_int64
    L.fm3dt_last_error.argtypes = [vp]
    L.fm3dt_last_error.restype = C.c_char_p
    L.fm3dt_ctx_destroy.argtypes = [vp]
    L.fm3dt_ctx_destroy.restype = None
    _lib = L
    return L


def ref_pi() -> float:
    """The value of pi the reference uses (its double-precision pi is set from
    a single-precision literal, fm3dt_parallel.f90:61)."""
    return float(np.float32(3.1415926535898))


def latlon_to_rad(lat, lon):
    """Latitude/longitude in degrees -> colatitude/longitude in radians, as
    fm3dt_parallel.f90:6313-6314 converts receivers and sources."""
    pi = ref_pi()
    lat = np.asarray(lat, dtype=np.float64)
    lon = np.asarray(lon, dtype=np.float64)
    return (90.0 - lat) * pi / 180.0, lon * pi / 180.0


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def tile_shapes():
    L = load()
    n = C.c_int(0)
    L.fm3dt_tile_shapes(C.byref(n))
    out = []
    for i in range(n.value):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        L.fm3dt_tile_shape(i, C.byref(a), C.byref(b), C.byref(c))
        out.append((a.value, b.value, c.value))
    return out


STREAM_SWEEPS = (("stream", 4, 8), ("stream", 2, 16))


def sweep_shapes():
    """Shapes fm3dt_set_sweep_shape accepts: the tile shapes (tile sweep),
    then the streaming sweep's column blocks."""
    return [tuple(s) for s in tile_shapes()] + list(STREAM_SWEEPS)


class Solver:
    """One solver context: a grid, a velocity model and up to max_events
    device-resident traveltime fields."""

    def __init__(self, header, fom: int = 1, precision: int = FP64, max_events: int = 1):
        self._L = load()
        h = header
        d = GridDesc()
        d.nvr, d.nvx, d.nvz = h.nv
        d.gor, d.goxd, d.gozd = h.vorig
        d.dvr, d.dvxd, d.dvzd = h.vstep
        d.nnr, d.nnx, d.nnz = h.nn
        d.rgor, d.rgoxd, d.rgozd = h.norig
        d.dnr, d.dnxd, d.dnzd = h.nstep
        d.earth = h.earth
        d.fom = int(fom)
        d.precision = int(precision)
        d.max_events = int(max_events)
        self.desc = d
        self.header = h
        self.nn = tuple(h.nn)
        self.nv = tuple(h.nv)
        self.max_events = int(max_events)
        self.nev = 0
        ctx = C.c_void_p()
        rc = self._L.fm3dt_ctx_create(C.byref(d), C.byref(ctx))
        if rc != OK:
            raise Fm3dtError(rc, self._L.fm3dt_last_error(None).decode())
        self._ctx = ctx

    def _check(self, rc):
        if rc != OK:
            raise Fm3dtError(rc, self._L.fm3dt_last_error(self._ctx).decode())

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.fm3dt_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def nmp(self) -> int:
        nvr, nvx, nvz = self.nv
        return (nvr + 2) * (nvx + 2) * (nvz + 2)

    @property
    def launch_count(self) -> int:
        return int(self._L.fm3dt_launch_count(self._ctx))

    def set_tuning(self, shape: int = 0, max_passes: int = 0, max_rounds: int = 0, sweep: int = -1):
        self._check(self._L.fm3dt_set_tuning(self._ctx, int(shape), int(max_passes), int(max_rounds), int(sweep)))

    def set_schedule(self, tie_sweeps: int = -1, tie_ratio: float = -1.0, resweeps: int = -1,
                     resweep_frac: float = -1.0):
        """Near-tie extra sweeps and band, re-sweeps and their threshold
        (negative: keep); see fm3dt_set_schedule."""
        self._check(self._L.fm3dt_set_schedule(self._ctx, int(tie_sweeps), float(tie_ratio), int(resweeps),
                                               float(resweep_frac)))

    def set_sweep_shape(self, shape: int):
        self._check(self._L.fm3dt_set_sweep_shape(self._ctx, int(shape)))

    def set_sweep_segments(self, segments: int = 0, tie_segments: int = 0):
        self._check(self._L.fm3dt_set_sweep_segments(self._ctx, int(segments), int(tie_segments)))

    def round_trace(self, cap: int = 8192):
        """(tiles, node updates) per round of the last solve."""
        t = np.zeros(cap, dtype=np.int64)
        u = np.zeros(cap, dtype=np.int64)
        n = self._L.fm3dt_round_trace(self._ctx, cap, t.ctypes.data_as(C.POINTER(C.c_int64)),
                                      u.ctypes.data_as(C.POINTER(C.c_int64)))
        if n < 0:
            self._check(n)
        n = min(n, cap)
        return t[:n], u[:n]

    def round_trace_ms(self, cap: int = 8192):
        """Device time (ms) of each round of the last solve."""
        m = np.zeros(cap, dtype=np.float32)
        n = self._L.fm3dt_round_trace_ms(self._ctx, cap, m.ctypes.data_as(C.POINTER(C.c_float)))
        if n < 0:
            self._check(n)
        return m[:min(n, cap)].astype(np.float64)

    def part_ms(self):
        """Device times (ms) of the last solve's first round in two parts:
        near-tie extra sweeps, their first round, the others' certification,
        their first round (zeros for a solve in one part)."""
        m = np.zeros(4, dtype=np.float32)
        self._check(self._L.fm3dt_part_ms(self._ctx, m.ctypes.data_as(C.POINTER(C.c_float))))
        return m.astype(np.float64)

    def tie_sweep_items(self, cap: int = 16):
        """Items run and skipped by each near-tie extra sweep of the last
        solve: (run, skipped) arrays."""
        run = np.zeros(cap, dtype=np.int64)
        skip = np.zeros(cap, dtype=np.int64)
        n = self._L.fm3dt_tie_sweep_items(self._ctx, cap, run.ctypes.data_as(C.POINTER(C.c_int64)),
                                          skip.ctypes.data_as(C.POINTER(C.c_int64)))
        if n < 0:
            self._check(n)
        n = min(n, cap)
        return run[:n], skip[:n]

    def tie_sweep_ms(self, cap: int = 16):
        """Device time (ms) of each near-tie extra sweep of the last solve
        (two-part solves)."""
        m = np.zeros(cap, dtype=np.float32)
        n = self._L.fm3dt_tie_sweep_ms(self._ctx, cap, m.ctypes.data_as(C.POINTER(C.c_float)))
        if n < 0:
            self._check(n)
        return m[:min(n, cap)].astype(np.float64)

    def rays_ms(self):
        """Times (ms) of the last host-buffer ray call: rays and row pointers,
        compaction, copies out (device), and the call's wall time."""
        m = np.zeros(4, dtype=np.float32)
        self._check(self._L.fm3dt_rays_ms(self._ctx, m.ctypes.data_as(C.POINTER(C.c_float))))
        return m.astype(np.float64)

    def set_velocity(self, velv):
        velv = np.ascontiguousarray(velv, dtype=np.float64)
        if velv.size != self.nmp:
            raise ValueError("velv has the wrong size")
        self._check(self._L.fm3dt_set_velocity(self._ctx, _d(velv)))

    def solve(self, frames) -> dict:
        frames = np.ascontiguousarray(frames, dtype=np.float64)
        nnr, nnx, nnz = self.nn
        nev = frames.size // (nnx * nnz)
        if frames.size != nev * nnx * nnz:
            raise ValueError("frames must be nev x nnx x nnz")
        st = Status()
        self._check(self._L.fm3dt_solve(self._ctx, nev, _d(frames), C.byref(st)))
        self.nev = nev
        return st.as_dict()

    def solve_resume(self) -> dict:
        """Continue the rounds from the current fields (fixed-point check or
        warm start)."""
        st = Status()
        self._check(self._L.fm3dt_solve_resume(self._ctx, C.byref(st)))
        return st.as_dict()

    def solve_ptr(self, nev: int, frames_ptr: int, device: bool) -> dict:
        """Solve from frames at a raw address: host memory (e.g. pinned) when
        device is False, device memory when True."""
        st = Status()
        if device:
            self._check(self._L.fm3dt_solve_device(self._ctx, int(nev), C.c_void_p(frames_ptr), C.byref(st)))
        else:
            self._check(self._L.fm3dt_solve(self._ctx, int(nev),
                                            C.cast(C.c_void_p(frames_ptr), C.POINTER(C.c_double)), C.byref(st)))
        self.nev = int(nev)
        return st.as_dict()

    def receiver_times_into(self, rcr, rcx, rcz, out_ptr: int):
        """Receiver times into caller-owned host memory at out_ptr (nev x nrc floats)."""
        self._check(self._L.fm3dt_receiver_times(self._ctx, len(rcr), _d(rcr), _d(rcx), _d(rcz),
                                                 C.cast(C.c_void_p(out_ptr), C.POINTER(C.c_float))))

    def solve_planewave(self, params) -> dict:
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(-1, 4)
        st = Status()
        self._check(self._L.fm3dt_solve_planewave(self._ctx, len(params), _d(params), C.byref(st)))
        self.nev = len(params)
        return st.as_dict()

    def solve_point(self, src, refine: int = 5, extent: int = 3) -> dict:
        """Point sources: src is (nev, 3) of (height km, colatitude rad,
        longitude rad); see fm3dt_solve_point."""
        src = np.ascontiguousarray(src, dtype=np.float64).reshape(-1, 3)
        st = Status()
        self._check(self._L.fm3dt_solve_point(self._ctx, len(src), _d(src), int(refine), int(extent), C.byref(st)))
        self.nev = len(src)
        return st.as_dict()

    def receiver_times(self, rcr, rcx, rcz) -> np.ndarray:
        rcr = np.ascontiguousarray(rcr, dtype=np.float64)
        rcx = np.ascontiguousarray(rcx, dtype=np.float64)
        rcz = np.ascontiguousarray(rcz, dtype=np.float64)
        out = np.zeros((self.nev, len(rcr)), dtype=np.float32)
        self._check(self._L.fm3dt_receiver_times(self._ctx, len(rcr), _d(rcr), _d(rcx), _d(rcz),
                                                 out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def rays_frechet(self, rcr, rcx, rcz, frechet: bool = True, cap: int | None = None):
        rcr = np.ascontiguousarray(rcr, dtype=np.float64)
        rcx = np.ascontiguousarray(rcx, dtype=np.float64)
        rcz = np.ascontiguousarray(rcz, dtype=np.float64)
        nrows = self.nev * len(rcr)
        row_ptr = np.zeros(nrows + 1, dtype=np.int64)
        ends = np.zeros((nrows, 3), dtype=np.float64)
        if not frechet:
            self._check(self._L.fm3dt_rays_frechet(self._ctx, len(rcr), _d(rcr), _d(rcx), _d(rcz),
                                                   row_ptr.ctypes.data_as(C.POINTER(C.c_int64)), None, None,
                                                   0, _d(ends)))
            return None, None, None, ends
        if cap is None:
            cap = max(1, nrows * 1024)
        while True:
            cols = np.zeros(cap, dtype=np.int32)
            vals = np.zeros(cap, dtype=np.float32)
            rc = self._L.fm3dt_rays_frechet(self._ctx, len(rcr), _d(rcr), _d(rcx), _d(rcz),
                                            row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                            cols.ctypes.data_as(C.POINTER(C.c_int32)),
                                            vals.ctypes.data_as(C.POINTER(C.c_float)), cap, _d(ends))
            if rc == ERANGE and row_ptr[-1] > cap:
                cap = int(row_ptr[-1])
                continue
            self._check(rc)
            n = int(row_ptr[-1])
            return row_ptr, cols[:n], vals[:n], ends

    def receiver_times_device(self, nrc: int, rcr_ptr: int, rcx_ptr: int, rcz_ptr: int, out_ptr: int):
        """Receiver times with receivers and output (nev x nrc floats) in
        device memory (raw device addresses)."""
        self._check(self._L.fm3dt_receiver_times_device(self._ctx, int(nrc), C.c_void_p(rcr_ptr),
                                                        C.c_void_p(rcx_ptr), C.c_void_p(rcz_ptr),
                                                        C.c_void_p(out_ptr)))

    def rays_frechet_device(self, nrc: int, rcr_ptr: int, rcx_ptr: int, rcz_ptr: int, row_ptr_ptr: int,
                            cols_ptr: int, vals_ptr: int, cap: int, ends_ptr: int = 0, strict: bool = True) -> int:
        """Rays and Frechet rows with every array in device memory (raw
        device addresses; cols/vals 0 to trace rays only).  Returns the entry
        count; when it exceeds cap, raises ERANGE (strict) or returns it with
        the rows unwritten."""
        total = C.c_int64(0)
        rc = self._L.fm3dt_rays_frechet_device(
            self._ctx, int(nrc), C.c_void_p(rcr_ptr), C.c_void_p(rcx_ptr), C.c_void_p(rcz_ptr),
            C.c_void_p(row_ptr_ptr or None), C.c_void_p(cols_ptr or None), C.c_void_p(vals_ptr or None),
            int(cap), C.byref(total), C.c_void_p(ends_ptr or None))
        if rc == ERANGE and total.value > cap and not strict:
            return int(total.value)       # the caller sizes its arrays and calls again
        self._check(rc)
        return int(total.value)

    def rays_frechet_into(self, rcr, rcx, rcz, row_ptr_ptr: int, cols_ptr: int, vals_ptr: int, cap: int,
                          ends_ptr: int = 0):
        """Rays and Frechet rows into caller-owned host memory (e.g. pinned):
        row_ptr nev*nrc+1 int64, cols int32 and vals float32 of capacity cap.
        Returns the entry count."""
        self._check(self._L.fm3dt_rays_frechet(
            self._ctx, len(rcr), _d(rcr), _d(rcx), _d(rcz), C.cast(C.c_void_p(row_ptr_ptr), C.POINTER(C.c_int64)),
            C.cast(C.c_void_p(cols_ptr), C.POINTER(C.c_int32)), C.cast(C.c_void_p(vals_ptr), C.POINTER(C.c_float)),
            int(cap), C.cast(C.c_void_p(ends_ptr or None), C.POINTER(C.c_double))))
        return int(C.cast(C.c_void_p(row_ptr_ptr + 8 * self.nev * len(rcr)), C.POINTER(C.c_int64))[0])

    def forward(self, frames, rcr, rcx, rcz, rows: bool = True, cap: int | None = None):
        """One forward step (fm3dt_forward): solve the frames, then receiver
        times, rays and Frechet rows in one call.  Returns (status, times
        nev x nrc, (row_ptr, cols, vals) or None, end points nev*nrc x 3)."""
        frames = np.ascontiguousarray(frames, dtype=np.float64)
        nnr, nnx, nnz = self.nn
        nev = frames.size // (nnx * nnz)
        if frames.size != nev * nnx * nnz:
            raise ValueError("frames must be nev x nnx x nnz")
        rcr, rcx, rcz = (np.ascontiguousarray(v, dtype=np.float64) for v in (rcr, rcx, rcz))
        nrc = len(rcr)
        times = np.zeros((nev, nrc), dtype=np.float32)
        ends = np.zeros((nev * nrc, 3), dtype=np.float64)
        row_ptr = np.zeros(nev * nrc + 1, dtype=np.int64)
        if cap is None:
            cap = nev * nrc * 512 + 1024     # (a smaller capacity costs a second solve when exceeded)
        cols = np.zeros(max(cap, 1), dtype=np.int32) if rows else None
        vals = np.zeros(max(cap, 1), dtype=np.float32) if rows else None
        st = Status()
        for _ in range(2):
            rc = self._L.fm3dt_forward(
                self._ctx, nev, _d(frames), nrc, _d(rcr), _d(rcx), _d(rcz),
                times.ctypes.data_as(C.POINTER(C.c_float)), row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                cols.ctypes.data_as(C.POINTER(C.c_int32)) if rows else None,
                vals.ctypes.data_as(C.POINTER(C.c_float)) if rows else None, int(cap if rows else 0), _d(ends),
                C.byref(st))
            if rows and rc == ERANGE and row_ptr[-1] > cap:
                cap = int(row_ptr[-1])            # sized by the first call: solve once more
                cols = np.zeros(cap, dtype=np.int32)
                vals = np.zeros(cap, dtype=np.float32)
                continue
            break
        self._check(rc)
        self.nev = nev
        out = (row_ptr, cols[:row_ptr[-1]], vals[:row_ptr[-1]]) if rows else None
        return st.as_dict(), times, out, ends

    def forward_device(self, nev: int, frames_ptr: int, nrc: int, rcr_ptr: int, rcx_ptr: int, rcz_ptr: int,
                       times_ptr: int, row_ptr_ptr: int, cols_ptr: int, vals_ptr: int, cap: int,
                       ends_ptr: int = 0) -> tuple[dict, int]:
        """One forward step with every array in device memory (raw device
        addresses; cols/vals 0 to trace rays only).  Returns (status, entry
        count)."""
        total = C.c_int64(0)
        st = Status()
        self._check(self._L.fm3dt_forward_device(
            self._ctx, int(nev), C.c_void_p(frames_ptr), int(nrc), C.c_void_p(rcr_ptr), C.c_void_p(rcx_ptr),
            C.c_void_p(rcz_ptr), C.c_void_p(times_ptr), C.c_void_p(row_ptr_ptr or None),
            C.c_void_p(cols_ptr or None), C.c_void_p(vals_ptr or None), int(cap), C.byref(total),
            C.c_void_p(ends_ptr or None), C.byref(st)))
        self.nev = int(nev)
        return st.as_dict(), int(total.value)

    def forward_into(self, nev: int, frames_ptr: int, rcr, rcx, rcz, times_ptr: int, row_ptr_ptr: int,
                     cols_ptr: int, vals_ptr: int, cap: int) -> int:
        """One forward step with caller-owned host memory (e.g. pinned) at
        raw addresses: frames in, times, row pointers, cols and vals out.
        Returns the entry count."""
        st = Status()
        self._check(self._L.fm3dt_forward(
            self._ctx, int(nev), C.cast(C.c_void_p(frames_ptr), C.POINTER(C.c_double)), len(rcr), _d(rcr),
            _d(rcx), _d(rcz), C.cast(C.c_void_p(times_ptr), C.POINTER(C.c_float)),
            C.cast(C.c_void_p(row_ptr_ptr), C.POINTER(C.c_int64)), C.cast(C.c_void_p(cols_ptr), C.POINTER(C.c_int32)),
            C.cast(C.c_void_p(vals_ptr), C.POINTER(C.c_float)), int(cap), None, C.byref(st)))
        self.nev = int(nev)
        return int(C.cast(C.c_void_p(row_ptr_ptr + 8 * self.nev * len(rcr)), C.POINTER(C.c_int64))[0])

    def set_host_link(self, mode: int):
        """How forward calls move page-locked host buffers: 0 measure on the
        next call, 1 copies, 2 kernels through the device mapping."""
        self._check(self._L.fm3dt_set_host_link(self._ctx, int(mode)))

    def host_link(self) -> tuple[int, int]:
        """The current choice for (frames, rows): -1 not measured, 0
        copies, 1 device mapping."""
        f, r = C.c_int(), C.c_int()
        self._check(self._L.fm3dt_host_link(self._ctx, C.byref(f), C.byref(r)))
        return f.value, r.value

    @property
    def forward_early_events(self) -> int:
        """Events whose rays the last forward call traced inside its solve."""
        return int(self._L.fm3dt_forward_early_events(self._ctx))

    def get_times(self, event: int = 0) -> np.ndarray:
        nnr, nnx, nnz = self.nn
        out = np.zeros(nnr * nnx * nnz, dtype=np.float64)
        self._check(self._L.fm3dt_get_times(self._ctx, int(event), _d(out)))
        return out

    def get_velocity(self) -> np.ndarray:
        nnr, nnx, nnz = self.nn
        out = np.zeros((nnr + 3) * (nnx + 3) * (nnz + 3), dtype=np.float64)
        self._check(self._L.fm3dt_get_velocity(self._ctx, _d(out)))
        return out

    def set_times(self, event: int, nev_total: int, ttn):
        ttn = np.ascontiguousarray(ttn, dtype=np.float64)
        self._check(self._L.fm3dt_set_times(self._ctx, int(event), int(nev_total), _d(ttn)))
        self.nev = int(nev_total)
