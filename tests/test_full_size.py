"""Full-size cases (the workload grids: 128^3, 256^3, 192x224x224), checked
through properties that do not need the oracle at that size:

* the solve is a fixed point: resuming the rounds from it, every tile
  active, changes no bit of the fields (checked on whole fields of two
  events) or of the receiver times (all events);
* an event's result does not depend on its batch (bit for bit);
* single-precision offset times agree with double precision: receiver times
  within 1e-5 relative and 1 ms (the bar of the batched path).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(1, None, 48), (2, None, 8), (3, None, 24)]


@pytest.mark.parametrize("cfg,scale,nev", CASES, ids=["config1-128", "config2-256", "config3-192x224x224"])
def test_full_size_fixed_point_batch_and_precision(gpu_lib, cfg, scale, nev):
    import fm3dt
    from fm3dt import synth
    w = synth.config(cfg, scale=scale, nev=nev)
    h = w.header
    params = np.array([synth.planewave_params(h, *ev) for ev in w.events])
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP32_OFFSET, max_events=nev) as s:
        s.set_velocity(w.velv)
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        t32 = s.receiver_times(w.rec_elev, rcx, rcz)
        f0 = [s.get_times(e) for e in (0, nev - 1)]
        st = s.solve_resume()
        assert st["converged"] == 1 and st["sweep_launches"] == 0
        assert np.array_equal(s.receiver_times(w.rec_elev, rcx, rcz), t32)
        for e, f in zip((0, nev - 1), f0):
            assert np.array_equal(s.get_times(e), f)
        # the last event alone gives the same bits as inside the batch
        s.solve_planewave(params[-1:])
        assert np.array_equal(s.receiver_times(w.rec_elev, rcx, rcz)[0], t32[-1])
    k = 2
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64, max_events=k) as s:
        s.set_velocity(w.velv)
        st = s.solve_planewave(params[:k])
        assert st["converged"] == 1
        t64 = s.receiver_times(w.rec_elev, rcx, rcz).astype(np.float64)
    a = t32[:k].astype(np.float64)
    assert np.max(np.abs(a - t64)) <= 1e-3
    assert np.max(np.abs(a - t64) / t64) <= 1e-5
