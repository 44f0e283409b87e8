"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the serial path of fm3dt_parallel.f90 in plain C
(oracle/fm3dt_oracle.c).  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py may import this module, and only as the checker.

Parity status: unpinned by reference outputs (the Fortran/MPI reference cannot
be built or run here and ships no golden vectors); pinned by analytic
known-answer cases in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib = None


class Grid(C.Structure):
    _fields_ = [
        ("nvr", C.c_int), ("nvx", C.c_int), ("nvz", C.c_int),
        ("gor", C.c_double), ("gox", C.c_double), ("goz", C.c_double),
        ("dvr", C.c_double), ("dvx", C.c_double), ("dvz", C.c_double),
        ("nnr", C.c_int), ("nnx", C.c_int), ("nnz", C.c_int),
        ("rgor", C.c_double), ("rgox", C.c_double), ("rgoz", C.c_double),
        ("dnr", C.c_double), ("dnx", C.c_double), ("dnz", C.c_double),
        ("earth", C.c_double),
    ]


class PlaneWave(C.Structure):
    _fields_ = [("t0", C.c_double), ("p", C.c_double),
                ("cos_az", C.c_double), ("sin_az", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, like the reference's
    left-to-right double-precision arithmetic)."""
    src = os.path.join(_HERE, "fm3dt_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
        subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", _LIB_PATH, src, "-lm"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.orc_pi.restype = C.c_double
        L.orc_grid_from_header.argtypes = [C.POINTER(C.c_int), dp, dp, C.POINTER(C.c_int), dp, dp,
                                           C.c_double, C.POINTER(Grid)]
        L.orc_gridder.argtypes = [C.POINTER(Grid), dp, dp, C.POINTER(C.c_int)]
        L.orc_fmm.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, dp, C.POINTER(C.c_longlong)]
        L.orc_fixed_point.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, dp, C.c_int, C.POINTER(C.c_int)]
        L.orc_fmm_decomposed.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, C.c_int, C.c_int, C.c_int, C.c_int, dp,
                                         C.POINTER(C.c_int)]
        ub = C.POINTER(C.c_ubyte)
        L.orc_fixed_point_field.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, ub, dp, C.c_int, C.POINTER(C.c_int)]
        L.orc_point_start.argtypes = [C.POINTER(Grid), dp, dp, C.c_int, C.c_double, C.c_double, C.c_double,
                                      C.c_int, C.c_int, dp, ub]
        L.orc_srtimes.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, dp, dp, C.POINTER(C.c_float)]
        L.orc_rays.argtypes = [C.POINTER(Grid), dp, dp, C.c_int, dp, dp, dp, C.POINTER(C.c_float),
                               dp, C.POINTER(C.c_int)]
        L.orc_sparsify.argtypes = [C.c_int, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int),
                                   C.POINTER(C.c_float)]
        L.orc_planewave_frame.argtypes = [C.POINTER(Grid), C.POINTER(PlaneWave), dp]
        L.orc_planewave_params.argtypes = [C.POINTER(Grid), C.c_double, C.c_double, C.POINTER(PlaneWave)]
        L.orc_latlon_to_rad.argtypes = [C.c_int, dp, dp, dp, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def ref_pi() -> float:
    return lib().orc_pi()


def grid_from_header(nv, vorig, vstep, nn, norig, nstep, earth) -> Grid:
    g = Grid()
    ia = (C.c_int * 3)(*nv)
    ib = (C.c_int * 3)(*nn)
    da = (C.c_double * 3)(*vorig)
    db = (C.c_double * 3)(*vstep)
    dc = (C.c_double * 3)(*norig)
    dd = (C.c_double * 3)(*nstep)
    lib().orc_grid_from_header(ia, da, db, ib, dc, dd, float(earth), C.byref(g))
    return g


def latlon_to_rad(lat, lon):
    lat = np.ascontiguousarray(lat, dtype=np.float64)
    lon = np.ascontiguousarray(lon, dtype=np.float64)
    colat = np.empty_like(lat)
    lonr = np.empty_like(lon)
    lib().orc_latlon_to_rad(len(lat), _d(lat), _d(lon), _d(colat), _d(lonr))
    return colat, lonr


def gridder(g: Grid, velv: np.ndarray):
    velv = np.ascontiguousarray(velv, dtype=np.float64)
    veln = np.zeros((g.nnr + 3) * (g.nnx + 3) * (g.nnz + 3), dtype=np.float64)
    nclamp = C.c_int(0)
    lib().orc_gridder(C.byref(g), _d(velv), _d(veln), C.byref(nclamp))
    return veln, nclamp.value


def fmm(g: Grid, veln: np.ndarray, bottom: np.ndarray, fom: int = 1):
    veln = np.ascontiguousarray(veln, dtype=np.float64)
    bottom = np.ascontiguousarray(bottom, dtype=np.float64)
    ttn = np.zeros(g.nnr * g.nnx * g.nnz, dtype=np.float64)
    pops = C.c_longlong(0)
    rc = lib().orc_fmm(C.byref(g), _d(veln), int(fom), _d(bottom), _d(ttn), C.byref(pops))
    if rc != 0:
        raise RuntimeError(f"orc_fmm failed: {rc}")
    return ttn, pops.value


def fmm_decomposed(g: Grid, velv: np.ndarray, bottom: np.ndarray, fom: int = 1, blocks=(2, 2, 2),
                   max_rounds: int = 100000):
    """The reference's decomposed run (nr x nx x nz emulated ranks, 2x2x2 in
    its mpirun -np 9 layout); velv are the velocity nodes (each block grids
    its own nodes).  Returns (ttn, rounds)."""
    velv = np.ascontiguousarray(velv, dtype=np.float64)
    bottom = np.ascontiguousarray(bottom, dtype=np.float64)
    ttn = np.zeros(g.nnr * g.nnx * g.nnz, dtype=np.float64)
    rounds = C.c_int(0)
    rc = lib().orc_fmm_decomposed(C.byref(g), _d(velv), int(fom), _d(bottom), int(blocks[0]), int(blocks[1]),
                                  int(blocks[2]), int(max_rounds), _d(ttn), C.byref(rounds))
    if rc != 0:
        raise RuntimeError(f"orc_fmm_decomposed failed: {rc}")
    return ttn, rounds.value


def fixed_point(g: Grid, veln: np.ndarray, bottom: np.ndarray, fom: int = 1, max_sweeps: int = 10000):
    """Fixed point of the reference's stencil (order independent)."""
    veln = np.ascontiguousarray(veln, dtype=np.float64)
    bottom = np.ascontiguousarray(bottom, dtype=np.float64)
    ttn = np.zeros(g.nnr * g.nnx * g.nnz, dtype=np.float64)
    sweeps = C.c_int(0)
    rc = lib().orc_fixed_point(C.byref(g), _d(veln), int(fom), _d(bottom), _d(ttn), int(max_sweeps),
                               C.byref(sweeps))
    if rc != 0:
        raise RuntimeError(f"orc_fixed_point failed: {rc}")
    return ttn, sweeps.value


def fixed_point_field(g: Grid, veln: np.ndarray, init: np.ndarray, fixed: np.ndarray, fom: int = 1,
                      max_sweeps: int = 100000):
    """Fixed point from an arbitrary start (init: inf = unset; fixed: keep)."""
    veln = np.ascontiguousarray(veln, dtype=np.float64)
    init = np.ascontiguousarray(init, dtype=np.float64)
    fixed = np.ascontiguousarray(fixed, dtype=np.uint8)
    ttn = np.zeros(g.nnr * g.nnx * g.nnz, dtype=np.float64)
    sweeps = C.c_int(0)
    rc = lib().orc_fixed_point_field(C.byref(g), _d(veln), int(fom), _d(init),
                                     fixed.ctypes.data_as(C.POINTER(C.c_ubyte)), _d(ttn), int(max_sweeps),
                                     C.byref(sweeps))
    if rc != 0:
        raise RuntimeError(f"orc_fixed_point_field failed: {rc}")
    return ttn, sweeps.value


def point_start(g: Grid, velv, veln, src, refine: int = 5, extent: int = 3, fom: int = 1):
    """(init, fixed) of a point-source solve; src = (height km, colat, lon)."""
    velv = np.ascontiguousarray(velv, dtype=np.float64)
    veln = np.ascontiguousarray(veln, dtype=np.float64)
    n = g.nnr * g.nnx * g.nnz
    init = np.zeros(n, dtype=np.float64)
    fixed = np.zeros(n, dtype=np.uint8)
    rc = lib().orc_point_start(C.byref(g), _d(velv), _d(veln), int(fom), float(src[0]), float(src[1]),
                               float(src[2]), int(refine), int(extent), _d(init),
                               fixed.ctypes.data_as(C.POINTER(C.c_ubyte)))
    if rc != 0:
        raise RuntimeError(f"orc_point_start failed: {rc}")
    return init, fixed


def point_solve(g: Grid, velv, veln, src, refine: int = 5, extent: int = 3, fom: int = 1):
    init, fixed = point_start(g, velv, veln, src, refine, extent, fom)
    return fixed_point_field(g, veln, init, fixed, fom)[0]


def srtimes(g: Grid, ttn: np.ndarray, rcr, rcx, rcz):
    ttn = np.ascontiguousarray(ttn, dtype=np.float64)
    rcr = np.ascontiguousarray(rcr, dtype=np.float64)
    rcx = np.ascontiguousarray(rcx, dtype=np.float64)
    rcz = np.ascontiguousarray(rcz, dtype=np.float64)
    out = np.zeros(len(rcr), dtype=np.float32)
    rc = lib().orc_srtimes(C.byref(g), _d(ttn), len(rcr), _d(rcr), _d(rcx), _d(rcz), _f(out))
    if rc != 0:
        raise RuntimeError(f"orc_srtimes: receiver {-rc - 1} outside the grid")
    return out


def nmp(g: Grid) -> int:
    return (g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2)


def rays(g: Grid, ttn, veln, rcr, rcx, rcz, frechet: bool = True):
    ttn = np.ascontiguousarray(ttn, dtype=np.float64)
    veln = np.ascontiguousarray(veln, dtype=np.float64)
    rcr = np.ascontiguousarray(rcr, dtype=np.float64)
    rcx = np.ascontiguousarray(rcx, dtype=np.float64)
    rcz = np.ascontiguousarray(rcz, dtype=np.float64)
    n = len(rcr)
    fdm = np.zeros((n, nmp(g)), dtype=np.float32) if frechet else None
    ends = np.zeros((n, 3), dtype=np.float64)
    steps = np.zeros(n, dtype=np.int32)
    rc = lib().orc_rays(C.byref(g), _d(ttn), _d(veln), n, _d(rcr), _d(rcx), _d(rcz),
                        _f(fdm) if frechet else None, _d(ends),
                        steps.ctypes.data_as(C.POINTER(C.c_int)))
    if rc != 0:
        raise RuntimeError(f"orc_rays failed: {rc}")
    return fdm, ends, steps


def sparsify(row: np.ndarray):
    row = np.ascontiguousarray(row, dtype=np.float32)
    cols = np.zeros(len(row), dtype=np.int32)
    vals = np.zeros(len(row), dtype=np.float32)
    n = lib().orc_sparsify(len(row), _f(row), len(row), cols.ctypes.data_as(C.POINTER(C.c_int)), _f(vals))
    return cols[:n].copy(), vals[:n].copy()


def planewave_params(g: Grid, delta_deg: float, baz_deg: float) -> PlaneWave:
    pw = PlaneWave()
    lib().orc_planewave_params(C.byref(g), float(delta_deg), float(baz_deg), C.byref(pw))
    return pw


def planewave_frame(g: Grid, pw: PlaneWave) -> np.ndarray:
    out = np.zeros(g.nnz * g.nnx, dtype=np.float64)
    lib().orc_planewave_frame(C.byref(g), C.byref(pw), _d(out))
    return out
