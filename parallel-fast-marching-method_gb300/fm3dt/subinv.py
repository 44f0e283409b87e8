"""ctypes binding of libfm3dt_subinv.so (include/fm3dt_subinv.h): one
subspace inversion step of the reference's subinv program, on the host."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

FP32 = 0
FP64 = 1

_LIB = None


class SubinvError(RuntimeError):
    pass


class _Desc(C.Structure):
    _fields_ = [("nvr", C.c_int), ("nvt", C.c_int), ("nvp", C.c_int),
                ("gor", C.c_double), ("got", C.c_double), ("gop", C.c_double),
                ("dnr", C.c_double), ("dnt", C.c_double), ("dnp", C.c_double),
                ("rmtr", C.c_int), ("epsilon", C.c_float), ("subdim", C.c_int), ("asds", C.c_int),
                ("eta", C.c_float), ("invst", C.c_int), ("stdf", C.c_float), ("fracg", C.c_float),
                ("earth", C.c_float), ("precision", C.c_int)]


@dataclass
class Params:
    """subinv.in values with the reference run's defaults."""
    rmtr: int = 1
    epsilon: float = 10.0
    subdim: int = 10
    asds: int = 1
    eta: float = 10.0
    invst: int = 0
    stdf: float = 10.0
    fracg: float = 0.1
    earth: float = 6371.0


def load():
    global _LIB
    if _LIB is None:
        from . import build as fb
        path = fb.build_subinv()
        lib = C.CDLL(path)
        lib.fm3dt_subinv_step.restype = C.c_int
        lib.fm3dt_subinv_step.argtypes = [C.POINTER(_Desc), C.c_int] + [C.c_void_p] * 14 + \
            [C.POINTER(C.c_int), C.c_char_p, C.c_int]
        _LIB = lib
    return _LIB


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def step(grid, p: Params, nsrc, nrc, mo, cm_sd, mc, tstat, dobs, cd_sd, mtimes, rtimes,
         row_ptr, cols, vals, precision=FP32):
    """One inversion step; returns (dm, subdim_used, message).

    grid: (nv, vorig, vstep) of the reference velocity grid (header lines 1-3
    of gridi.vtx).  mo/cm_sd: the two columns of gridi.vtx; mc: the current
    model (plus station terms when p.invst); tstat/dobs/cd_sd: otimes.dat;
    mtimes: rtravel.out; rtimes: rtimes.dat; row_ptr/cols/vals: every row of
    frechet.out."""
    lib = load()
    nv, vo, vs = grid
    d = _Desc(int(nv[0]), int(nv[1]), int(nv[2]), float(vo[0]), float(vo[1]), float(vo[2]),
              float(vs[0]), float(vs[1]), float(vs[2]), int(p.rmtr), float(p.epsilon), int(p.subdim),
              int(p.asds), float(p.eta), int(p.invst), float(p.stdf), float(p.fracg), float(p.earth),
              int(precision))
    f32 = (lambda x: np.ascontiguousarray(x, dtype=np.float32))
    i32 = (lambda x: np.ascontiguousarray(x, dtype=np.int32))
    nsrc, nrc = i32(nsrc), i32(nrc)
    arrs = [f32(mo), f32(cm_sd), f32(mc), i32(tstat), f32(dobs), f32(cd_sd), f32(mtimes), f32(rtimes),
            np.ascontiguousarray(row_ptr, dtype=np.int64), i32(cols), f32(vals)]
    nmpv = (int(nv[0]) + 2) * (int(nv[1]) + 2) * (int(nv[2]) + 2)
    nmp = nmpv + (int(np.sum(nrc)) if p.invst == 1 else 0)
    ntr = int(np.sum(nsrc * nrc))
    if arrs[0].size != nmpv or arrs[1].size != nmpv or arrs[2].size != nmp:
        raise SubinvError("model arrays do not match the grid")
    if any(a.size != ntr for a in arrs[3:8]) or arrs[8].size != ntr + 1:
        raise SubinvError("data arrays do not match the source and receiver counts")
    dm = np.zeros(nmp)
    used = C.c_int(0)
    msg = C.create_string_buffer(2048)
    rc = lib.fm3dt_subinv_step(C.byref(d), len(nsrc), _p(nsrc), _p(nrc), *[_p(a) for a in arrs], _p(dm),
                               C.byref(used), msg, len(msg))
    text = msg.value.decode(errors="replace")
    if rc != 0:
        raise SubinvError(f"fm3dt_subinv_step failed ({rc}): {text}")
    return dm, used.value, text
