"""Point sources (local events; no reference counterpart).

CPU: the oracle's start of a point-source solve -- the fixed box and its
straight-ray times (exact in a homogeneous model).
GPU, through the C ABI: (1) the double-precision field equals the oracle's
fixed point from the same start to 1e-9 s, with and without the refined
source grid, including a source next to the grid's faces; (2) in a
homogeneous model the times converge to distance/velocity: beyond 400 km
within 2% (max) and 0.5% (mean) on a 48^3 grid, and the fixed box holds the
exact times; (3) single-precision receiver times within 1e-5 relative and
1 ms of double precision; (4) rays after a point solve are refused."""
import numpy as np
import pytest


def _grid(orc, n=24, kind="gauss", homogeneous=None):
    from fm3dt import synth
    w = synth.config(1, scale=n, nev=1)
    h = w.header
    velv = np.full_like(w.velv, homogeneous) if homogeneous else w.velv
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = orc.gridder(g, velv)
    return w, h, g, velv, veln


def _src(orc, h, fr, fx, fz, depth):
    """Source at fractional node coordinates (fx, fz) laterally, depth km."""
    colat, lon = orc.latlon_to_rad(np.array([h.norig[1] - fx * h.nstep[1]]), np.array([h.norig[2] + fz * h.nstep[2]]))
    return np.array([-depth, colat[0], lon[0]])


def _chord_times(h, g, src, v):
    nnr, nnx, nnz = h.nn
    ir, ix, iz = np.meshgrid(np.arange(nnr), np.arange(nnx), np.arange(nnz), indexing="ij")
    r = h.earth + (g.rgor - ir * g.dnr)
    th = g.rgox + ix * g.dnx
    ph = g.rgoz + iz * g.dnz
    rs = h.earth + src[0]
    xs = rs * np.sin(src[1]) * np.cos(src[2])
    ys = rs * np.sin(src[1]) * np.sin(src[2])
    zs = rs * np.cos(src[1])
    d = np.sqrt((r * np.sin(th) * np.cos(ph) - xs) ** 2 + (r * np.sin(th) * np.sin(ph) - ys) ** 2 +
                (r * np.cos(th) - zs) ** 2)
    return d / v, d


def test_oracle_start_box_and_exact_times(orc):
    w, h, g, velv, veln = _grid(orc, 20, homogeneous=6.0)
    src = _src(orc, h, 0, 9.4, 10.6, 23.0)
    init, fixed = orc.point_start(g, velv, veln, src, refine=0, extent=2)
    fixed = fixed.reshape(h.nn).astype(bool)
    idx = np.argwhere(fixed)
    assert fixed.sum() == 4 * 4 * 4
    assert np.all(idx.max(0) - idx.min(0) == 3)
    ta, _ = _chord_times(h, g, src, 6.0)
    got = init.reshape(h.nn)[fixed]
    assert np.max(np.abs(got - ta[fixed])) < 1e-12 * np.max(ta[fixed]) + 1e-12
    assert np.all(np.isinf(init.reshape(h.nn)[~fixed]))
    # refined: the outer layer of the box is left free, except on the grid's
    # own faces (a source 23 km deep touches the top face)
    init5, fixed5 = orc.point_start(g, velv, veln, src, refine=5, extent=3)
    assert np.isfinite(init5).sum() == 5 * 6 * 6 and fixed5.sum() == 4 * 4 * 4
    deep = _src(orc, h, 0, 9.4, 10.6, 160.0)
    init5, fixed5 = orc.point_start(g, velv, veln, deep, refine=5, extent=3)
    assert np.isfinite(init5).sum() == 6 * 6 * 6 and fixed5.sum() == 4 * 4 * 4


def test_oracle_rejects_sources_outside(orc):
    w, h, g, velv, veln = _grid(orc, 16)
    with pytest.raises(RuntimeError):
        orc.point_start(g, velv, veln, np.array([-1000.0, 0.5, 2.4]), 0, 2)


CASES = [  # (fractional x, z, depth km, refine, extent)
    (7.4, 8.6, 18.0, 0, 2), (7.4, 8.6, 18.0, 5, 3), (0.3, 22.2, 5.5, 5, 2), (11.9, 3.1, 120.0, 0, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("fx,fz,depth,refine,extent", CASES)
def test_point_field_equals_oracle(gpu_lib, orc, fx, fz, depth, refine, extent):
    import fm3dt
    w, h, g, velv, veln = _grid(orc, 24)
    src = _src(orc, h, 0, fx, fz, depth)
    ref = orc.point_solve(g, velv, veln, src, refine, extent)
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64) as s:
        s.set_velocity(velv)
        st = s.solve_point(src[None, :], refine=refine, extent=extent)
        assert st["converged"] == 1
        got = s.get_times(0)
    assert np.max(np.abs(got - ref)) < 1e-9


@pytest.mark.gpu
def test_point_homogeneous_converges_to_distance_over_velocity(gpu_lib, orc):
    import fm3dt
    w, h, g, velv, veln = _grid(orc, 48, homogeneous=6.0)
    src = _src(orc, h, 0, 23.3, 24.3, 20.3)
    ta, d = _chord_times(h, g, src, 6.0)
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64) as s:
        s.set_velocity(velv)
        s.solve_point(src[None, :], refine=0, extent=4)
        got = s.get_times(0).reshape(h.nn)
    init, fixed = orc.point_start(g, velv, veln, src, 0, 4)
    fixed = fixed.reshape(h.nn).astype(bool)
    assert np.max(np.abs(got[fixed] - ta[fixed])) < 1e-9
    far = d > 400.0
    rel = np.abs(got - ta)[far] / ta[far]
    assert rel.max() < 0.02 and rel.mean() < 0.005


@pytest.mark.gpu
def test_point_fp32_receivers_within_tolerance(gpu_lib, orc):
    import fm3dt
    w, h, g, velv, veln = _grid(orc, 32)
    srcs = np.stack([_src(orc, h, 0, 10.5, 12.5, 12.0), _src(orc, h, 0, 20.2, 9.8, 25.0)])
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    out = {}
    for prec in (fm3dt.FP64, fm3dt.FP32_OFFSET):
        with fm3dt.Solver(h, fom=1, precision=prec, max_events=2) as s:
            s.set_velocity(velv)
            s.solve_point(srcs, refine=5, extent=3)
            out[prec] = s.receiver_times(w.rec_elev, rcx, rcz).astype(np.float64)
            with pytest.raises(fm3dt.Fm3dtError):
                s.rays_frechet(w.rec_elev, rcx, rcz)
    a, b = out[fm3dt.FP64], out[fm3dt.FP32_OFFSET]
    assert np.max(np.abs(a - b)) <= 1e-3
    assert np.max(np.abs(a - b) / a) <= 1e-5
