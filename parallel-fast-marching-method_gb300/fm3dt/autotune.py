"""Autotuner of the tile solver.

Tunes, on a sample batch, (1) the shape of the directional sweep (tile or
streaming),
(2) the tile shape and in-tile pass cap of the fast-iterative rounds (the
shape also fixes the CTA size: one thread per column), (3) the solve
schedule -- how many extra sweeps, alternately reversed and forward, the
near-tie events get and how wide the near-tie band is -- and (4) the height
segments of those sweeps (automatic, or a few more, whose smaller items skip
more where nothing changed), keeping the fastest device time.  The schedule depends most on the model: on a smooth one
(Gaussian node noise) two extra sweeps of the events within ~6 degrees of an
axis are best; on a checkerboard, whose fast cells carry head waves across
the sweep direction, five or six of them over a band twice as wide halve the
rounds.  The converged field does not depend on any of these choices (the
fixed point is unique), so tuning never changes results.
"""
from __future__ import annotations

import numpy as np

from . import sweep_shapes, tile_shapes

PASS_CAPS = (16, 64)
# (extra sweeps of the near-tie events, near-tie band)
SCHEDULES = ((2, 0.1), (3, 0.15), (4, 0.15), (5, 0.15), (5, 0.2), (6, 0.2), (8, 0.2), (10, 0.2))
# height segments of the near-tie events' sweeps (0: the solver's time model)
TIE_SEGMENTS = (0, 4, 8)


def _time(solver, frames_ptr, nev, device, repeats):
    solver.solve_ptr(nev, frames_ptr, device)       # warm
    return float(np.median([solver.solve_ptr(nev, frames_ptr, device)["ms"] for _ in range(repeats)]))


def autotune(solver, frames_ptr: int, nev: int, device: bool = True, repeats: int = 1,
             tune_segments: bool = True):
    """Returns (round_shape, max_passes, sweep_shape, ms, schedule,
    tie_segments) and applies it; schedule = (tie_sweeps, tie_ratio,
    resweeps, resweep_frac), negative values being the defaults kept;
    tie_segments None when not tuned (the solver's setting is kept).

    Coordinate descent: the sweep shape, then the round tiles under the
    default schedule, the schedule under those tiles, the segments; then the
    round tiles once more under the chosen schedule (the best tile depends
    on how much work the rounds get), and if they change, the schedule again."""
    nshapes = len(tile_shapes())
    round_shape, cap = 0, PASS_CAPS[0]
    solver.set_tuning(round_shape, cap, 0, 1)
    best_sweep = None
    for sshape in range(len(sweep_shapes())):
        solver.set_sweep_shape(sshape)
        ms = _time(solver, frames_ptr, nev, device, repeats)
        if best_sweep is None or ms < best_sweep[1]:
            best_sweep = (sshape, ms)
    solver.set_sweep_shape(best_sweep[0])

    def tune_tiles():
        best = None
        for shape in range(nshapes):
            for c in PASS_CAPS:
                solver.set_tuning(shape, c, 0, 1)
                ms = _time(solver, frames_ptr, nev, device, repeats)
                if best is None or ms < best[2]:
                    best = (shape, c, ms)
        solver.set_tuning(best[0], best[1], 0, 1)
        return best

    def tune_schedule():
        best_sched = None
        for ts, tr in SCHEDULES:
            solver.set_schedule(ts, tr, -1, -1.0)
            ms = _time(solver, frames_ptr, nev, device, repeats)
            if best_sched is None or ms < best_sched[2]:
                best_sched = (ts, tr, ms)
        solver.set_schedule(best_sched[0], best_sched[1], -1, -1.0)
        return best_sched

    best = tune_tiles()
    best_sched = tune_schedule()
    best_seg = (None, best_sched[2])
    if tune_segments:
        for ts in TIE_SEGMENTS:
            solver.set_sweep_segments(0, ts)
            ms = _time(solver, frames_ptr, nev, device, repeats)
            if best_seg[0] is None or ms < best_seg[1]:
                best_seg = (ts, ms)
        solver.set_sweep_segments(0, best_seg[0])
    again = tune_tiles()
    ms = again[2]
    if again[:2] != best[:2]:
        best = again
        best_sched = tune_schedule()
        ms = best_sched[2]
    else:
        best = again
    return (best[0], best[1], best_sweep[0], ms, (best_sched[0], best_sched[1], -1, -1.0), best_seg[0])
