"""Autotuner of the tile-round solver.

Times a sample batch for every tile shape (r x theta x phi extents, which
also fixes the CTA size: one thread per column) and a few in-tile pass caps,
then keeps the fastest on the solver.  The converged field does not depend on
the choice (the fixed point is unique), so tuning never changes results.
"""
from __future__ import annotations

import time

import numpy as np

from . import tile_shapes

PASS_CAPS = (16, 64)


def autotune(solver, frames_ptr: int, nev: int, device: bool = True, repeats: int = 1):
    """Returns (shape_index, max_passes, ms) and applies the best setting."""
    best = None
    for shape in range(len(tile_shapes())):
        for cap in PASS_CAPS:
            solver.set_tuning(shape, cap)
            solver.solve_ptr(nev, frames_ptr, device)       # warm
            ms = []
            for _ in range(repeats):
                st = solver.solve_ptr(nev, frames_ptr, device)
                ms.append(st["ms"])
            m = float(np.median(ms))
            if best is None or m < best[2]:
                best = (shape, cap, m)
    solver.set_tuning(best[0], best[1])
    return best
