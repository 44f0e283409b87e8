"""The allocation-free receiver-time entry point (fm3dt_receiver_times_noalloc).

Callers that fixed their device memory at start-up (serving loops, embedded
Fortran drivers) use this entry point instead of fm3dt_receiver_times; it keeps
its scratch in a fixed array inside the library.  Its results must be the
receiver times of the ordinary entry point bit for bit (both accumulate the
same single-precision sums in the same order), on consecutive calls that
reuse the shared array with different sizes.  This file runs last so that a
failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(s, rcr, rcx, rcz):
    L = s._L
    f = L.fm3dt_receiver_times_noalloc
    dp = C.POINTER(C.c_double)
    f.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, C.POINTER(C.c_float)]
    rcr = np.ascontiguousarray(rcr, dtype=np.float64)
    rcx = np.ascontiguousarray(rcx, dtype=np.float64)
    rcz = np.ascontiguousarray(rcz, dtype=np.float64)
    out = np.full((s.nev, len(rcr)), np.nan, dtype=np.float32)
    rc = f(s._ctx, len(rcr), rcr.ctypes.data_as(dp), rcx.ctypes.data_as(dp), rcz.ctypes.data_as(dp),
           out.ctypes.data_as(C.POINTER(C.c_float)))
    return rc, out


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_receiver_times(gpu_lib, prec):
    import fm3dt
    from fm3dt import synth
    w = synth.config(1, scale=26, nev=4)
    params = np.array([synth.planewave_params(w.header, *ev) for ev in w.events])
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    with fm3dt.Solver(w.header, precision=prec, max_events=4) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        ref = s.receiver_times(w.rec_elev, rcx, rcz)
        # first call: all receivers, all events
        rc, got = _call(s, w.rec_elev, rcx, rcz)
        assert rc == fm3dt.OK, s._L.fm3dt_last_error(s._ctx)
        assert np.array_equal(got, ref)
        # second call in a row: fewer receivers and fewer events, the shared
        # scratch still holds the first call's larger contents
        s.solve_planewave(params[:2])
        ref2 = s.receiver_times(w.rec_elev[:37], rcx[:37], rcz[:37])
        rc, got2 = _call(s, w.rec_elev[:37], rcx[:37], rcz[:37])
        assert rc == fm3dt.OK
        assert got2.shape == (2, 37)
        assert np.array_equal(got2, ref2)


def test_noalloc_limits_and_errors(gpu_lib):
    import fm3dt
    from fm3dt import synth
    w = synth.config(0, scale=16, nev=1)
    params = np.array([synth.planewave_params(w.header, *w.events[0])])
    with fm3dt.Solver(w.header) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        n = 4097
        rc, _ = _call(s, np.zeros(n), np.full(n, 2.0), np.full(n, 2.5))
        assert rc == fm3dt.EINVAL
        assert b"4096" in s._L.fm3dt_last_error(s._ctx)
        # a receiver outside the grid is reported, and the next call is clean
        rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat[:5], w.rec_lon[:5])
        bad_x = rcx.copy()
        bad_x[3] = 0.1
        rc, _ = _call(s, w.rec_elev[:5], bad_x, rcz)
        assert rc == fm3dt.ERANGE
        rc, got = _call(s, w.rec_elev[:5], rcx, rcz)
        assert rc == fm3dt.OK
        assert np.array_equal(got, s.receiver_times(w.rec_elev[:5], rcx, rcz))


def test_noalloc_at_the_limits(gpu_lib):
    """Exactly at both limits (4096 receivers filling the coordinate block,
    64 x 4096 = 262144 times filling the output block) the results equal
    fm3dt_receiver_times bit for bit; one time more is refused."""
    import fm3dt
    from fm3dt import synth
    w = synth.config(0, scale=16, nev=1)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    n = 4096
    rcr_n, rcx_n, rcz_n = (np.resize(np.asarray(a, dtype=np.float64), n) for a in (w.rec_elev, rcx, rcz))
    ev = np.resize(np.asarray(w.events[0], dtype=np.float64), (65, 2)).copy()
    ev[:, 1] += np.arange(65) * 5.0
    params = np.array([synth.planewave_params(w.header, *e) for e in ev])
    with fm3dt.Solver(w.header, max_events=65) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params[:64])
        ref = s.receiver_times(rcr_n, rcx_n, rcz_n)
        rc, got = _call(s, rcr_n, rcx_n, rcz_n)
        assert rc == fm3dt.OK, s._L.fm3dt_last_error(s._ctx)
        assert got.shape == (64, n)
        assert np.array_equal(got, ref)
        s.solve_planewave(params)
        rc, _ = _call(s, rcr_n, rcx_n, rcz_n)
        assert rc == fm3dt.EINVAL
        assert b"262144" in s._L.fm3dt_last_error(s._ctx)
        # fewer receivers for the 65 events fit again
        rc, got = _call(s, rcr_n[:4000], rcx_n[:4000], rcz_n[:4000])
        assert rc == fm3dt.OK
        assert np.array_equal(got, s.receiver_times(rcr_n[:4000], rcx_n[:4000], rcz_n[:4000]))


@pytest.mark.parametrize("bad", [np.nan, np.inf, 1e300])
def test_noalloc_rejects_non_finite_receivers_like_receiver_times(gpu_lib, bad):
    """A NaN, infinite or huge coordinate is outside the grid for both entry
    points (FM3DT_ERANGE), and neither writes its output."""
    import fm3dt
    from fm3dt import synth
    w = synth.config(0, scale=16, nev=1)
    params = np.array([synth.planewave_params(w.header, *w.events[0])])
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat[:6], w.rec_lon[:6])
    with fm3dt.Solver(w.header) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        for which in range(3):
            coords = [np.array(w.rec_elev[:6], dtype=np.float64), rcx.copy(), rcz.copy()]
            coords[which][4] = bad
            rc, got = _call(s, *coords)
            assert rc == fm3dt.ERANGE
            assert b"receiver 5" in s._L.fm3dt_last_error(s._ctx)
            assert np.isnan(got).all()          # untouched
            with pytest.raises(fm3dt.Fm3dtError) as ei:
                s.receiver_times(*coords)
            assert ei.value.code == fm3dt.ERANGE
