"""Precision study: the single-precision offset-time solve against the
double-precision one on the same events (the double-precision GPU field is
the oracle's fixed point to 1e-9 s, so this is the error against the oracle).

For every source-receiver pair it compares the receiver time, the ray's end
point (in propagation-grid cells) and the Frechet row (largest entry
difference over the row's largest entry, and the difference's 2-norm over
the row's), and reports the maxima and percentiles.  The rays of the two
solves follow slightly different gradients, so where a ray crosses a
velocity cell boundary a little earlier or later its weights move between
neighbouring nodes: row differences are of the size of that shift, not of
the time error.  ``python -m fm3dt.precision [config] [scale] [events]`` prints
the report as one JSON line; the default is the slab workload (256^3, 16
events).
"""
from __future__ import annotations

import json
import math
import sys

import numpy as np


def _dense(row_ptr, cols, vals, i, n):
    out = np.zeros(n, dtype=np.float64)
    a, b = int(row_ptr[i]), int(row_ptr[i + 1])
    out[cols[a:b] - 1] = vals[a:b]
    return out


def _stats(x):
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return {"max": 0.0, "p99": 0.0, "mean": 0.0}
    return {"max": float(x.max()), "p99": float(np.percentile(x, 99)), "mean": float(x.mean())}


def study(cfg: int = 2, scale: int | None = None, nev: int = 16, batch64: int = 4) -> dict:
    import fm3dt
    from fm3dt import synth
    w = synth.config(cfg, scale=scale, nev=nev)
    h = w.header
    params = np.array([synth.planewave_params(h, *ev) for ev in w.events])
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    nrc = len(rcr)
    out = {}
    for prec, bsz in ((fm3dt.FP32_OFFSET, nev), (fm3dt.FP64, batch64)):
        times, ends, rows = [], [], []
        with fm3dt.Solver(h, fom=1, precision=prec, max_events=bsz) as s:
            s.set_velocity(w.velv)
            for e0 in range(0, nev, bsz):
                p = params[e0:e0 + bsz]
                st = s.solve_planewave(p)
                if st["converged"] != 1:
                    raise RuntimeError("solve did not converge")
                times.append(s.receiver_times(rcr, rcx, rcz).astype(np.float64))
                rp, cols, vals, en = s.rays_frechet(rcr, rcx, rcz)
                ends.append(en)
                rows.append((rp, cols, vals))
        out[prec] = (np.concatenate(times), np.concatenate(ends), rows)
    t32, e32, r32 = out[fm3dt.FP32_OFFSET]
    t64, e64, r64 = out[fm3dt.FP64]
    dt = np.abs(t32 - t64)
    rel = dt / np.abs(t64)
    d2r = math.pi / 180.0
    cell = np.array([h.nstep[0], h.nstep[1] * d2r, h.nstep[2] * d2r])
    dcells = np.max(np.abs(e32 - e64) / cell[None, :], axis=1)
    nmp = (h.nv[0] + 2) * (h.nv[1] + 2) * (h.nv[2] + 2)
    frel, frel2 = [], []
    rp32, c32, v32 = r32[0]
    for b, (rp, cols, vals) in enumerate(r64):
        for i in range(len(rp) - 1):
            q = b * batch64 * nrc + i
            a = _dense(rp, cols, vals, i, nmp)
            g = _dense(rp32, c32, v32, q, nmp)
            m = np.max(np.abs(a))
            if m > 0:
                frel.append(np.max(np.abs(g - a)) / m)
                frel2.append(np.linalg.norm(g - a) / np.linalg.norm(a))
    return {
        "workload": f"config{cfg}", "grid": list(h.nn), "events": nev, "receivers": nrc,
        "pairs": int(t64.size),
        "traveltime_abs_s": _stats(dt.ravel()),
        "traveltime_rel": _stats(rel.ravel()),
        "ray_endpoint_cells": _stats(dcells),
        "frechet_row_rel": _stats(frel),
        "frechet_row_rel_l2": _stats(frel2),
        "bars": {"traveltime_rel": 1e-5, "traveltime_abs_s": 1e-3, "ray_endpoint_cells": 1.0},
    }


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    cfg = int(argv[0]) if len(argv) > 0 else 2
    scale = int(argv[1]) if len(argv) > 1 and int(argv[1]) > 0 else None
    nev = int(argv[2]) if len(argv) > 2 else 16
    print(json.dumps(study(cfg, scale, nev)))


if __name__ == "__main__":
    main()
