"""The autotuner's search (no GPU): a stand-in solver whose solve time has a
known optimum, with the best round tile depending on the schedule, as on the
checkerboard models (more extra sweeps leave the rounds less work, where
larger tiles pay)."""
import pytest


class _Timed:
    """Records the settings the tuner applies and returns a solve time."""

    def __init__(self, best_tiles_by_sweeps, best_schedule, best_segments):
        self.shape = self.cap = self.sweep = 0
        self.sched = (2, 0.1)
        self.tie_segments = 0
        self.best_tiles_by_sweeps = best_tiles_by_sweeps
        self.best_schedule = best_schedule
        self.best_segments = best_segments
        self.solves = 0

    def set_tuning(self, shape, cap, max_rounds, sweep):
        self.shape, self.cap = shape, cap

    def set_sweep_shape(self, s):
        self.sweep = s

    def set_schedule(self, ts, tr, resweeps, frac):
        self.sched = (ts, tr)

    def set_sweep_segments(self, seg, tie_seg):
        self.tie_segments = tie_seg

    def solve_ptr(self, nev, ptr, device):
        self.solves += 1
        ms = 100.0
        ms += 0.0 if self.sweep == 7 else 30.0
        good_tiles = self.best_tiles_by_sweeps(self.sched[0])
        ms += 0.0 if (self.shape, self.cap) == good_tiles else 5.0 + self.shape
        ms += 0.0 if self.sched == self.best_schedule else 10.0 + abs(self.sched[0] - self.best_schedule[0])
        ms += 0.0 if self.tie_segments == self.best_segments else 2.0
        return {"ms": ms}


@pytest.mark.parametrize("best_schedule", [(6, 0.2), (2, 0.1)])
def test_autotune_finds_the_tiles_of_the_chosen_schedule(gpu_lib, best_schedule):
    from fm3dt import autotune, sweep_shapes, tile_shapes
    assert len(sweep_shapes()) == 8 and len(tile_shapes()) == 6
    # tile (3, 16) is best under the default schedule's two sweeps, (1, 64)
    # under five or more
    s = _Timed(lambda ts: (1, 64) if ts >= 5 else (3, 16), best_schedule, 4)
    shape, cap, sweep, ms, sched, seg = autotune.autotune(s, 0, 64, repeats=1)
    want_tiles = (1, 64) if best_schedule[0] >= 5 else (3, 16)
    assert (shape, cap) == want_tiles and (s.shape, s.cap) == want_tiles
    assert sweep == 7 and s.sweep == 7
    assert sched == (best_schedule[0], best_schedule[1], -1, -1.0) and s.sched == best_schedule
    assert seg == 4 and s.tie_segments == 4
    assert ms == pytest.approx(100.0)
    # trials: 8 sweep shapes, 12 tile settings, 8 schedules, 3 segments, 12
    # tile settings again (and 8 schedules when the tiles changed); each a
    # warm-up solve and one timed
    changed = best_schedule[0] >= 5
    trials = 8 + 12 + 8 + 3 + 12 + (8 if changed else 0)
    assert s.solves == 2 * trials


def test_autotune_keeps_segments_when_not_tuned(gpu_lib):
    from fm3dt import autotune
    s = _Timed(lambda ts: (2, 16), (3, 0.15), 8)
    s.tie_segments = 8
    *_, seg = autotune.autotune(s, 0, 64, repeats=1, tune_segments=False)
    assert seg is None and s.tie_segments == 8
