"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances (stated per test):
* gridder, plane-wave frames, receiver interpolation: bit-exact (same double
  precision operation order, no FMA contraction in those kernels);
* solver vs the oracle's fixed point of the reference's octant formulas:
  1e-9 s everywhere (any model, any boundary frame, both orders);
* solver, first order: the iterative fixed point equals the fast-marching
  result to 1e-9 s;
* solver, mixed order: receiver times within 1e-5 relative and 1 ms absolute
  (the parity bar of the batched path); field within 5 ms everywhere and within 1e-6 s at 95%
  of nodes (on rough models fast marching keeps a few sticky intermediate
  minima that the fixed point does not: ~2% of nodes of the slab model by up
  to 2.7 ms; smooth models agree to 1e-12 s);
* single-precision offset mode vs double: receiver times within 1e-5 relative
  and 1 ms;
* rays through an identical field: endpoints within 1e-9 rad / 1e-6 km and
  Frechet rows within 1e-5 relative of the row norm.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(cfg, scale, nev=1, events=None):
    from fm3dt import synth
    w = synth.config(cfg, scale=scale, nev=nev)
    if events is not None:
        w.events = np.asarray(events, dtype=np.float64).reshape(-1, 2)
    return w


def _oracle_grid(orc, h):
    return orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)


def _params(w):
    from fm3dt import synth
    return np.array([synth.planewave_params(w.header, *ev) for ev in w.events])


def _oracle_solve(orc, w, params, fom=1):
    g = _oracle_grid(orc, w.header)
    veln, ncl = orc.gridder(g, w.velv)
    assert ncl == 0
    out = []
    for p in params:
        fr = orc.planewave_frame(g, orc.PlaneWave(*p))
        ttn, _ = orc.fmm(g, veln, fr, fom)
        out.append(ttn)
    return g, veln, out


@pytest.mark.parametrize("cfg,scale", [(0, 24), (3, 20), (2, 18)])
def test_gridder_bitwise(gpu_lib, orc, cfg, scale):
    import fm3dt
    w = _setup(cfg, scale)
    g = _oracle_grid(orc, w.header)
    ref, _ = orc.gridder(g, w.velv)
    with fm3dt.Solver(w.header) as s:
        s.set_velocity(w.velv)
        got = s.get_velocity()
    assert np.array_equal(got, ref)


def test_planewave_frame_bitwise(gpu_lib, orc):
    import fm3dt
    w = _setup(1, 20, nev=3)
    params = _params(w)
    g = _oracle_grid(orc, w.header)
    nnr, nnx, nnz = w.header.nn
    with fm3dt.Solver(w.header, max_events=3) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        for e in range(3):
            t = s.get_times(e).reshape(nnr, nnx * nnz)
            ref = orc.planewave_frame(g, orc.PlaneWave(*params[e]))
            assert np.array_equal(t[-1], ref)


@pytest.mark.parametrize("cfg,scale,event", [
    (0, 24, (60.0, 45.0)), (0, 33, (60.0, 45.0)), (1, 28, (35.0, 200.0)),
    (1, 30, (80.0, 300.0)), (2, 26, (50.0, 100.0)), (3, 24, (45.0, 270.0))])
def test_solve_fp64_matches_fast_marching(gpu_lib, orc, cfg, scale, event):
    import fm3dt
    w = _setup(cfg, scale, events=[event])
    params = _params(w)
    g, veln, refs = _oracle_solve(orc, w, params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    with fm3dt.Solver(w.header, fom=1, precision=fm3dt.FP64) as s:
        s.set_velocity(w.velv)
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        got = s.get_times(0)
        trr = s.receiver_times(w.rec_elev, rcx, rcz)[0].astype(np.float64)
    d = np.abs(got - refs[0])
    assert d.max() < 5e-3
    assert np.mean(d > 1e-6) < 0.05
    ref_trr = orc.srtimes(g, refs[0], w.rec_elev, rcx, rcz).astype(np.float64)
    assert np.max(np.abs(trr - ref_trr)) <= 1e-3
    assert np.max(np.abs(trr - ref_trr) / ref_trr) <= 1e-5


@pytest.mark.parametrize("cfg,scale", [(0, 22), (2, 20)])
def test_solve_first_order_equals_fast_marching(gpu_lib, orc, cfg, scale):
    import fm3dt
    w = _setup(cfg, scale)
    params = _params(w)
    _, _, refs = _oracle_solve(orc, w, params, fom=0)
    with fm3dt.Solver(w.header, fom=0) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        got = s.get_times(0)
    assert np.max(np.abs(got - refs[0])) < 1e-9


def test_host_frames_equal_planewave(gpu_lib, orc):
    import fm3dt
    w = _setup(1, 20, nev=2)
    params = _params(w)
    g = _oracle_grid(orc, w.header)
    frames = np.stack([orc.planewave_frame(g, orc.PlaneWave(*p)) for p in params])
    with fm3dt.Solver(w.header, max_events=2) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        a = [s.get_times(e) for e in range(2)]
        s.solve(frames)
        b = [s.get_times(e) for e in range(2)]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("cfg,scale,event,holes,fom", [
    (0, 22, (60.0, 45.0), 0.0, 1), (2, 26, (50.0, 100.0), 0.0, 1), (3, 24, (45.0, 270.0), 0.0, 1),
    (1, 27, (75.0, 10.0), 0.0, 0), (0, 22, (60.0, 45.0), 0.2, 1), (2, 30, (50.0, 100.0), 0.05, 0)])
def test_solve_equals_fixed_point_of_reference_stencil(gpu_lib, orc, cfg, scale, event, holes, fom):
    """Against the oracle's fixed point of the reference's own octant formulas
    (order independent), the GPU field agrees to 1e-9 s everywhere, including
    rough models, first order, and boundary frames with unset values (<= 0,
    "no time", F:6935-6936) where the heap order of fast marching is not
    causal."""
    import fm3dt
    w = _setup(cfg, scale, events=[event])
    params = _params(w)
    g = _oracle_grid(orc, w.header)
    veln, _ = orc.gridder(g, w.velv)
    fr = orc.planewave_frame(g, orc.PlaneWave(*params[0]))
    rng = np.random.default_rng(5)
    fr[rng.uniform(size=fr.size) < holes] = 0.0
    if holes:
        fr[:5] = -1.0
    ref, _ = orc.fixed_point(g, veln, fr, fom)
    with fm3dt.Solver(w.header, fom=fom) as s:
        s.set_velocity(w.velv)
        st = s.solve(fr[None, :])
        assert st["converged"] == 1
        got = s.get_times(0)
    assert np.max(np.abs(got - ref)) < 1e-9


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_equals_alone_bitwise(gpu_lib, prec):
    """Each event's field is identical solved alone and solved in a batch."""
    import fm3dt
    w = _setup(1, 26, nev=5)
    params = _params(w)
    with fm3dt.Solver(w.header, precision=prec, max_events=5) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        batch = [s.get_times(e) for e in range(5)]
        for e in range(5):
            s.solve_planewave(params[e:e + 1])
            assert np.array_equal(s.get_times(0), batch[e])


@pytest.mark.parametrize("prec", [0, 1])
def test_tile_shapes_and_sweep_bitwise(gpu_lib, prec):
    """The fixed point does not depend on the tile shape, the pass cap, the
    directional sweep or the schedule."""
    import fm3dt
    w = _setup(2, 30, nev=3)
    params = _params(w)
    ref = None
    with fm3dt.Solver(w.header, precision=prec, max_events=3) as s:
        s.set_velocity(w.velv)
        for shape in range(len(fm3dt.tile_shapes())):
            for sweep, cap in ((1, 64), (0, 16), (1, 3)):
                s.set_tuning(shape, cap, 0, sweep)
                st = s.solve_planewave(params)
                assert st["converged"] == 1
                assert (st["sweep_launches"] > 0) == bool(sweep)
                out = np.concatenate([s.get_times(e) for e in range(3)])
                if ref is None:
                    ref = out
                else:
                    assert np.array_equal(out, ref), f"shape {shape} sweep {sweep} cap {cap}"
        # every sweep shape, the streaming column blocks with and without
        # their verification sweep included
        for sweep in (1, 2):
            s.set_tuning(3, 16, 0, sweep)
            for sshape in range(len(fm3dt.sweep_shapes())):
                s.set_sweep_shape(sshape)
                st = s.solve_planewave(params)
                assert st["converged"] == 1 and st["sweep_launches"] > 0
                out = np.concatenate([s.get_times(e) for e in range(3)])
                assert np.array_equal(out, ref), f"sweep shape {fm3dt.sweep_shapes()[sshape]}, mode {sweep}"


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("cfg,scale", [(1, 40), (2, 36), (3, 30)])
def test_sweeps_many_azimuths_bitwise(gpu_lib, prec, cfg, scale):
    """The streaming sweep with its extra sweeps of near-tie events and the
    tile sweep give the same field bit for bit, and it is a fixed point, on
    twenty-four azimuths (near-axis ones included) in three models."""
    import fm3dt
    baz = np.concatenate([np.linspace(0.0, 345.0, 20), [0.3, 89.7, 180.4, 271.0]])
    events = np.stack([np.linspace(32.0, 88.0, len(baz)), baz], axis=1)
    w = _setup(cfg, scale, events=events)
    params = _params(w)
    n = len(params)
    with fm3dt.Solver(w.header, precision=prec, max_events=n) as s:
        s.set_velocity(w.velv)
        s.set_tuning(1, 64, 0, 1)
        s.set_sweep_shape(1)                          # tile sweep
        s.solve_planewave(params)
        ref = np.concatenate([s.get_times(e) for e in range(n)])
        s.set_sweep_shape(len(fm3dt.tile_shapes()))   # streaming sweep
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        got = np.concatenate([s.get_times(e) for e in range(n)])
        assert np.array_equal(got, ref)
        st = s.solve_resume()
        assert st["converged"] == 1
        again = np.concatenate([s.get_times(e) for e in range(n)])
    assert np.array_equal(again, ref)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("cfg,scale", [(1, 40), (3, 30)])
def test_two_part_first_round_bitwise(gpu_lib, prec, cfg, scale):
    """A batch with at least 32 events that are not near ties takes the
    two-part schedule: the near-tie events swept and their first round run on
    a second stream, the others swept once, certified, and recomputed only
    where the certification fails.  Batches of 8 certify their singly swept
    events on one stream.  Both give the same fields bit for bit as rounds
    without a sweep (nothing certified), and they are a fixed point."""
    import fm3dt
    baz = np.concatenate([np.linspace(0.0, 352.5, 48), [0.4, 90.3, 179.6, 270.2]])
    events = np.stack([np.linspace(32.0, 88.0, len(baz)), baz], axis=1)
    w = _setup(cfg, scale, events=events)
    params = _params(w)
    n = len(params)
    with fm3dt.Solver(w.header, precision=prec, max_events=n) as s:
        s.set_velocity(w.velv)
        s.set_tuning(1, 16, 0, 0)                     # (8, 8, 32) tiles, rounds only
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        ref = np.concatenate([s.get_times(e) for e in range(n)])
        s.set_tuning(1, 16, 0, 1)                     # streaming sweep first
        small = []
        for e0 in range(0, n, 8):
            st = s.solve_planewave(params[e0:e0 + 8])
            assert st["converged"] == 1
            small += [s.get_times(e) for e in range(len(params[e0:e0 + 8]))]
        assert np.array_equal(np.concatenate(small), ref)
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        # the certification left most of the other events' tiles out of the
        # first round
        tiles0 = s.round_trace()[0][0]
        got = np.concatenate([s.get_times(e) for e in range(n)])
        assert np.array_equal(got, ref)
        st = s.solve_resume()
        assert st["converged"] == 1
        again = np.concatenate([s.get_times(e) for e in range(n)])
    assert np.array_equal(again, ref)
    h = w.header
    tiles_per_event = -(-h.nn[0] // 8) * -(-h.nn[1] // 8) * -(-h.nn[2] // 32)
    assert 0 < tiles0 < n * tiles_per_event // 2


@pytest.mark.parametrize("prec", [0, 1])
def test_tma_staging_bitwise(gpu_lib, prec, monkeypatch):
    """The rounds stage a tile and its halos by one TMA copy when the phi rows
    are a multiple of 16 bytes, else by thread loads; both give the same field
    bit for bit (the copy fills outside the grid with NaN, which the stencil
    never uses)."""
    import fm3dt
    w = _setup(1, 32, nev=3)
    params = _params(w)
    out = {}
    for tma in ("1", "0"):
        monkeypatch.setenv("FM3DT_TMA", tma)
        with fm3dt.Solver(w.header, precision=prec, max_events=3) as s:
            s.set_velocity(w.velv)
            for shape in range(len(fm3dt.tile_shapes())):
                s.set_tuning(shape, 16, 0, 1)
                st = s.solve_planewave(params)
                assert st["converged"] == 1
                out[(tma, shape)] = np.concatenate([s.get_times(e) for e in range(3)])
    for shape in range(len(fm3dt.tile_shapes())):
        assert np.array_equal(out[("1", shape)], out[("0", shape)]), f"shape {shape}"


@pytest.mark.parametrize("prec", [0, 1])
def test_resume_changes_nothing(gpu_lib, prec):
    """A finished solve is a true fixed point: running the rounds again from
    it, every tile active, changes no bit."""
    import fm3dt
    w = _setup(2, 28, nev=2)
    params = _params(w)
    with fm3dt.Solver(w.header, precision=prec, max_events=2) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        a = np.concatenate([s.get_times(e) for e in range(2)])
        st = s.solve_resume()
        assert st["converged"] == 1 and st["sweep_launches"] == 0
        b = np.concatenate([s.get_times(e) for e in range(2)])
    assert np.array_equal(a, b)


def test_fp32_offset_within_tolerance(gpu_lib):
    import fm3dt
    w = _setup(1, 40, nev=4)
    params = _params(w)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    with fm3dt.Solver(w.header, precision=fm3dt.FP64, max_events=4) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        t64 = s.receiver_times(w.rec_elev, rcx, rcz).astype(np.float64)
    with fm3dt.Solver(w.header, precision=fm3dt.FP32_OFFSET, max_events=4) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        t32 = s.receiver_times(w.rec_elev, rcx, rcz).astype(np.float64)
    assert np.max(np.abs(t32 - t64)) <= 1e-3
    assert np.max(np.abs(t32 - t64) / t64) <= 1e-5


def test_receiver_times_bitwise_on_same_field(gpu_lib, orc):
    import fm3dt
    w = _setup(3, 22)
    params = _params(w)
    g, veln, refs = _oracle_solve(orc, w, params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    ref = orc.srtimes(g, refs[0], w.rec_elev, rcx, rcz)
    with fm3dt.Solver(w.header) as s:
        s.set_velocity(w.velv)
        s.set_times(0, 1, refs[0])
        got = s.receiver_times(w.rec_elev, rcx, rcz)[0]
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("cfg,scale", [(0, 24), (2, 22)])
def test_rays_frechet_on_same_field(gpu_lib, orc, cfg, scale):
    import fm3dt
    w = _setup(cfg, scale)
    params = _params(w)
    g, veln, refs = _oracle_solve(orc, w, params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    fdm, ends, steps = orc.rays(g, refs[0], veln, w.rec_elev, rcx, rcz)
    with fm3dt.Solver(w.header) as s:
        s.set_velocity(w.velv)
        s.set_times(0, 1, refs[0])
        row_ptr, cols, vals, gends = s.rays_frechet(w.rec_elev, rcx, rcz)
    assert np.max(np.abs(gends[:, 0] - ends[:, 0])) < 1e-6
    assert np.max(np.abs(gends[:, 1:] - ends[:, 1:])) < 1e-9
    nmp = orc.nmp(g)
    for i in range(len(rcx)):
        dense = np.zeros(nmp, dtype=np.float64)
        c = cols[row_ptr[i]:row_ptr[i + 1]]
        assert np.all(np.diff(c) > 0)
        dense[c - 1] = vals[row_ptr[i]:row_ptr[i + 1]]
        refrow = fdm[i].astype(np.float64)
        refrow[np.abs(fdm[i]) < np.float32(1e-6)] = 0.0
        scale_ = max(np.max(np.abs(refrow)), 1e-30)
        assert np.max(np.abs(dense - refrow)) <= 1e-5 * scale_


def test_errors_are_reported(gpu_lib):
    import fm3dt
    w = _setup(0, 16)
    with fm3dt.Solver(w.header) as s:
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.solve_planewave(_params(w))
        assert ei.value.code == fm3dt.ESTATE
        s.set_velocity(w.velv)
        s.solve_planewave(_params(w))
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.receiver_times(np.array([0.0]), np.array([0.1]), np.array([0.1]))
        assert ei.value.code == fm3dt.ERANGE
        assert s.launch_count > 0


@pytest.mark.parametrize("prec", [0, 1])
def test_device_memory_entry_points_equal_host_ones(gpu_lib, prec):
    """fm3dt_receiver_times_device and fm3dt_rays_frechet_device (receivers
    and outputs in device memory) give the host entry points' results bit for
    bit; a capacity below the entry count is refused with the count given."""
    import torch
    import fm3dt
    w = _setup(3, 24, nev=3)
    params = _params(w)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    nrc = len(rcr)
    with fm3dt.Solver(w.header, precision=prec, max_events=3) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        ref_t = s.receiver_times(rcr, rcx, rcz)
        ref_ptr, ref_cols, ref_vals, ref_ends = s.rays_frechet(rcr, rcx, rcz)
        d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (rcr, rcx, rcz)]
        out = torch.empty((3, nrc), dtype=torch.float32, device="cuda")
        s.receiver_times_device(nrc, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), out.data_ptr())
        assert np.array_equal(out.cpu().numpy(), ref_t)
        nrows = 3 * nrc
        row_ptr = torch.zeros(nrows + 1, dtype=torch.int64, device="cuda")
        cap = int(ref_ptr[-1])
        cols = torch.zeros(cap, dtype=torch.int32, device="cuda")
        vals = torch.zeros(cap, dtype=torch.float32, device="cuda")
        ends = torch.zeros((nrows, 3), dtype=torch.float64, device="cuda")
        total = s.rays_frechet_device(nrc, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), row_ptr.data_ptr(),
                                      cols.data_ptr(), vals.data_ptr(), cap, ends.data_ptr())
        assert total == cap
        assert np.array_equal(row_ptr.cpu().numpy(), ref_ptr)
        assert np.array_equal(cols.cpu().numpy(), ref_cols)
        assert np.array_equal(vals.cpu().numpy(), ref_vals)
        assert np.array_equal(ends.cpu().numpy(), ref_ends)
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.rays_frechet_device(nrc, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), row_ptr.data_ptr(),
                                  cols.data_ptr(), vals.data_ptr(), cap - 1)
        assert ei.value.code == fm3dt.ERANGE
        assert int(row_ptr[-1].item()) == cap
        # a receiver outside the grid is refused by both
        bad = d[1].clone()
        bad[7] = float("nan")
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.receiver_times_device(nrc, d[0].data_ptr(), bad.data_ptr(), d[2].data_ptr(), out.data_ptr())
        assert ei.value.code == fm3dt.ERANGE
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.rays_frechet_device(nrc, d[0].data_ptr(), bad.data_ptr(), d[2].data_ptr(), 0, 0, 0, 0)
        assert ei.value.code == fm3dt.ERANGE
        badh = rcx.copy()
        badh[7] = np.nan
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.rays_frechet(rcr, badh, rcz)
        assert ei.value.code == fm3dt.ERANGE


@pytest.mark.parametrize("prec", [0, 1])
def test_schedule_does_not_change_the_field(gpu_lib, prec):
    """The solve schedule (near-tie extra sweeps and band, re-sweeps and their
    threshold) only changes how fast the fixed point is reached: on a batch
    large enough for the two-part schedule, every schedule gives the same
    fields bit for bit; out-of-range values are refused."""
    import fm3dt
    baz = np.concatenate([np.linspace(0.0, 352.5, 40), [0.4, 90.3, 179.6, 270.2]])
    events = np.stack([np.linspace(32.0, 88.0, len(baz)), baz], axis=1)
    w = _setup(3, 30, events=events)
    params = _params(w)
    n = len(params)
    with fm3dt.Solver(w.header, precision=prec, max_events=n) as s:
        s.set_velocity(w.velv)
        ref = None
        for sched in ((2, 0.1, 4, 0.01), (0, 0.1, 0, 0.01), (5, 0.25, 2, 0.005), (8, 0.2, 6, 0.02),
                      (3, 0.0, 16, 0.0)):
            s.set_schedule(*sched)
            st = s.solve_planewave(params)
            assert st["converged"] == 1
            out = np.concatenate([s.get_times(e) for e in range(n)])
            if ref is None:
                ref = out
            else:
                assert np.array_equal(out, ref), sched
        for bad in ((17, -1.0, -1, -1.0), (-1, 1.5, -1, -1.0), (-1, float("nan"), -1, -1.0)):
            with pytest.raises(fm3dt.Fm3dtError) as ei:
                s.set_schedule(*bad)
            assert ei.value.code == fm3dt.EINVAL


def test_solve_profile_is_reported(gpu_lib):
    """The last solve's profile: a batch in two parts reports its first
    round's parts, and one time and one item count (run + skipped = every item
    of the sweep) per near-tie extra sweep after the first; a host-buffer ray
    call reports its phases.  The chunk activity and the one-launch sweeps
    leave the field as the schedule without extra sweeps gives it."""
    import fm3dt
    baz = np.concatenate([np.linspace(0.0, 352.5, 40), [0.4, 90.3, 179.6, 270.2]])
    events = np.stack([np.linspace(32.0, 88.0, len(baz)), baz], axis=1)
    w = _setup(3, 30, events=events)
    params = _params(w)
    n = len(params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    with fm3dt.Solver(w.header, precision=fm3dt.FP32_OFFSET, max_events=n) as s:
        s.set_velocity(w.velv)
        s.set_schedule(0, 0.1, 0, 0.01)
        assert s.solve_planewave(params)["converged"] == 1
        ref = np.concatenate([s.get_times(e) for e in range(n)])
        s.set_schedule(4, 0.1, -1, -1.0)
        assert s.solve_planewave(params)["converged"] == 1
        assert np.array_equal(np.concatenate([s.get_times(e) for e in range(n)]), ref)
        parts = s.part_ms()
        assert parts.shape == (4,) and parts[0] > 0.0 and parts[2] > 0.0
        ms = s.tie_sweep_ms()
        assert len(ms) == 4 and np.all(ms > 0.0)
        assert sum(ms) <= parts[0] * 1.01 + 0.05
        run, skipped = s.tie_sweep_items()
        assert len(run) == 4 and run[0] == 0 and skipped[0] == 0
        totals = run[1:] + skipped[1:]
        assert np.all(totals == totals[0]) and totals[0] > 0
        assert np.all(run[1:] <= totals)
        rows = s.rays_frechet(rcr, rcx, rcz)
        assert rows[0][-1] > 0
        rm = s.rays_ms()
        assert rm.shape == (4,) and np.all(rm >= 0.0) and rm[0] > 0.0 and rm[3] > 0.0


@pytest.mark.parametrize("nev", [44, 6])
def test_forward_equals_three_calls(gpu_lib, nev):
    """fm3dt_forward (solve, receiver times, rays and rows in one call, the
    rays of the part that converges first traced inside the solve) gives
    bit for bit what fm3dt_solve, fm3dt_receiver_times and fm3dt_rays_frechet
    give called in turn: on a batch solved in two parts (44 events, some
    near ties) and on a small batch solved in one (6 events);
    the device form and the host form into page-locked arrays match."""
    import torch
    import fm3dt
    from fm3dt import synth
    baz = np.concatenate([np.linspace(0.0, 352.5, 40), [0.4, 90.3, 179.6, 270.2]])
    events = np.stack([np.linspace(32.0, 88.0, len(baz)), baz], axis=1)[:nev]
    w = _setup(3, 30, events=events)
    params = _params(w)
    frames = synth.planewave_frames(w.header, params)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    nrc = len(rcr)
    with fm3dt.Solver(w.header, precision=fm3dt.FP32_OFFSET, max_events=nev) as s:
        s.set_velocity(w.velv)
        s.set_schedule(4, 0.1, -1, -1.0)
        assert s.solve(frames)["converged"] == 1
        t_ref = s.receiver_times(rcr, rcx, rcz)
        rp_ref, c_ref, v_ref, e_ref = s.rays_frechet(rcr, rcx, rcz)
        st, times, (rp, c, v), ends = s.forward(frames, rcr, rcx, rcz)
        assert st["converged"] == 1
        # (early rays when the other events converge before the near-tie
        # events' chain ends, which this small grid does not guarantee)
        print(f"\n{nev} events: rays of {s.forward_early_events} traced inside the solve")
        assert 0 <= s.forward_early_events < nev
        if nev < 32:
            assert s.forward_early_events == 0
        assert np.array_equal(times, t_ref)
        assert np.array_equal(rp, rp_ref) and np.array_equal(c, c_ref) and np.array_equal(v, v_ref)
        assert np.array_equal(ends, e_ref.reshape(-1, 3))
        # the device form, into device arrays
        dev = torch.device("cuda")
        d_frames = torch.from_numpy(frames).to(dev)
        d_rec = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (rcr, rcx, rcz)]
        d_times = torch.empty((nev, nrc), dtype=torch.float32, device=dev)
        d_rp = torch.empty(nev * nrc + 1, dtype=torch.int64, device=dev)
        cap = int(rp_ref[-1])
        d_c = torch.empty(cap, dtype=torch.int32, device=dev)
        d_v = torch.empty(cap, dtype=torch.float32, device=dev)
        d_e = torch.empty((nev * nrc, 3), dtype=torch.float64, device=dev)
        st2, total = s.forward_device(nev, d_frames.data_ptr(), nrc, *[x.data_ptr() for x in d_rec],
                                      d_times.data_ptr(), d_rp.data_ptr(), d_c.data_ptr(), d_v.data_ptr(), cap,
                                      d_e.data_ptr())
        assert st2["converged"] == 1 and total == cap
        assert np.array_equal(d_times.cpu().numpy(), t_ref)
        assert np.array_equal(d_rp.cpu().numpy(), rp_ref)
        assert np.array_equal(d_c.cpu().numpy(), c_ref) and np.array_equal(d_v.cpu().numpy(), v_ref)
        assert np.array_equal(d_e.cpu().numpy(), e_ref.reshape(-1, 3))
        # page-locked host arrays: the rows written there by the compaction kernel
        h_fr = torch.from_numpy(frames).pin_memory()
        h_t = torch.zeros((nev, nrc), dtype=torch.float32).pin_memory()
        h_rp = torch.zeros(nev * nrc + 1, dtype=torch.int64).pin_memory()
        h_c = torch.zeros(cap, dtype=torch.int32).pin_memory()
        h_v = torch.zeros(cap, dtype=torch.float32).pin_memory()
        # (measured choice, then each way forced)
        assert s.host_link() == (-1, -1)
        for mode in (0, 2, 1):
            if mode:
                s.set_host_link(mode)
            for h in (h_t, h_rp, h_c, h_v):
                h.zero_()
            n = s.forward_into(nev, h_fr.data_ptr(), rcr, rcx, rcz, h_t.data_ptr(), h_rp.data_ptr(),
                               h_c.data_ptr(), h_v.data_ptr(), cap)
            assert n == cap
            assert np.array_equal(h_t.numpy(), t_ref) and np.array_equal(h_rp.numpy(), rp_ref)
            assert np.array_equal(h_c.numpy(), c_ref) and np.array_equal(h_v.numpy(), v_ref)
            frames_link, rows_link = s.host_link()
            if mode == 0:
                assert frames_link in (0, 1) and rows_link in (-1, 0, 1)
                print(f"\nhost link measured: frames {frames_link}, rows {rows_link}")
            else:
                assert (frames_link, rows_link) == ((1, 1) if mode == 2 else (0, 0))
        # too small a capacity: ERANGE with the required count
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.forward_device(nev, d_frames.data_ptr(), nrc, *[x.data_ptr() for x in d_rec], d_times.data_ptr(),
                             d_rp.data_ptr(), d_c.data_ptr(), d_v.data_ptr(), cap - 1)
        assert ei.value.code == fm3dt.ERANGE
        # a receiver outside the grid: ERANGE, as fm3dt_receiver_times gives it
        bad = rcx.copy()
        bad[nrc // 2] = 10.0
        with pytest.raises(fm3dt.Fm3dtError) as ei:
            s.forward(frames, rcr, bad, rcz)
        assert ei.value.code == fm3dt.ERANGE
        with pytest.raises(fm3dt.Fm3dtError) as ej:
            s.receiver_times(rcr, bad, rcz)
        assert ej.value.code == fm3dt.ERANGE
        assert f"receiver {nrc // 2 + 1} " in str(ei.value) and f"receiver {nrc // 2 + 1} " in str(ej.value)
