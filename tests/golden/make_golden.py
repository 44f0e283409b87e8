"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no golden vectors and cannot be built here (Fortran + MPI),
so these fixtures record the oracle's restatement of fm3dt_parallel.f90 on small
seeded inputs; tests/test_golden.py checks that the oracle still reproduces
them and that the GPU path matches them.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "parallel-fast-marching-method_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

CASES = [
    # name, config, grid edge, event (distance, back-azimuth), fraction of unset boundary values
    ("checker14", 0, 14, (60.0, 45.0), 0.0),
    ("slab16", 2, 16, (50.0, 100.0), 0.0),
    ("gauss15_holes", 1, 15, (75.0, 10.0), 0.1),
]


def make(name, cfg, n, event, holes):
    import oracle as O
    from fm3dt import synth
    w = synth.config(cfg, scale=n, nev=1)
    h = w.header
    g = O.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, ncl = O.gridder(g, w.velv)
    assert ncl == 0
    params = np.array(synth.planewave_params(h, *event))
    frame = O.planewave_frame(g, O.PlaneWave(*params))
    rng = np.random.default_rng(11)
    frame[rng.uniform(size=frame.size) < holes] = 0.0
    fmm, _ = O.fmm(g, veln, frame, 1)
    fmm1, _ = O.fmm(g, veln, frame, 0)
    fp, _ = O.fixed_point(g, veln, frame, 1)
    colat, lonr = O.latlon_to_rad(w.rec_lat, w.rec_lon)
    nrc = min(20, len(colat))
    rec = (w.rec_elev[:nrc], colat[:nrc], lonr[:nrc])
    trr = O.srtimes(g, fmm, *rec)
    trr_fp = O.srtimes(g, fp, *rec)
    fdm, ends, steps = O.rays(g, fmm, veln, *rec)
    cols, vals, ptr = [], [], [0]
    for i in range(nrc):
        c, v = O.sparsify(fdm[i])
        cols.append(c)
        vals.append(v)
        ptr.append(ptr[-1] + len(c))
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        nv=np.array(h.nv), vorig=np.array(h.vorig), vstep=np.array(h.vstep),
        nn=np.array(h.nn), norig=np.array(h.norig), nstep=np.array(h.nstep), earth=np.array(h.earth),
        velv=w.velv, veln=veln, frame=frame, params=params,
        fmm=fmm, fmm_first_order=fmm1, fixed_point=fp,
        rec_elev=rec[0], rec_colat=rec[1], rec_lon=rec[2], trr=trr, trr_fixed_point=trr_fp,
        ray_ends=ends, ray_steps=steps,
        frechet_ptr=np.array(ptr, dtype=np.int64),
        frechet_cols=np.concatenate(cols).astype(np.int32),
        frechet_vals=np.concatenate(vals).astype(np.float32))


def main():
    for case in CASES:
        make(*case)
        print("wrote", case[0])


if __name__ == "__main__":
    main()
