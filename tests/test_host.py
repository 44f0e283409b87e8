"""Host-side tests (no GPU): the C ABI library builds, loads and exports every
symbol the public header declares; without a GPU it fails loudly instead of
falling back; synthetic workloads satisfy the grid-coverage contract."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "fm3dt_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fm3dt_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gpu_lib):
    import fm3dt
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(gpu_lib, n), n
    assert sorted(fm3dt.EXPORTS) == sorted(set(fm3dt.EXPORTS))
    assert set(fm3dt.EXPORTS) <= set(names)


def test_tile_shapes_query(gpu_lib):
    import fm3dt
    shapes = fm3dt.tile_shapes()
    assert len(shapes) >= 4
    for tr, tx, tz in shapes:
        assert tr >= 2 and tx * tz <= 1024


def test_no_gpu_fails_loudly(gpu_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import fm3dt
    from fm3dt import synth
    w = synth.config(0, scale=16)
    with pytest.raises(fm3dt.Fm3dtError) as ei:
        fm3dt.Solver(w.header)
    assert ei.value.code in (fm3dt.ENODEV, fm3dt.ECUDA)


def test_bad_descriptor_rejected(gpu_lib):
    import fm3dt
    from fm3dt import synth
    h = synth.section_header(2, 10, 10, 5, 5, 5)
    with pytest.raises(fm3dt.Fm3dtError) as ei:
        fm3dt.Solver(h)
    assert ei.value.code == fm3dt.EINVAL


@pytest.mark.parametrize("cfg", [0, 1, 2, 3])
def test_synthetic_grids_cover_the_propagation_grid(orc, cfg):
    """No velocity index is ever clamped by the gridder (the reference reads
    outside velv when the B-spline support does not cover the ghost ring)."""
    from fm3dt import synth
    w = synth.config(cfg, scale=12, nev=2)
    h = w.header
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, ncl = orc.gridder(g, w.velv)
    assert ncl == 0
    assert np.all(veln > 3.0) and np.all(veln < 12.0)


def test_full_size_headers_cover(orc):
    from fm3dt import synth
    for cfg in (1, 3):
        w = synth.config(cfg, nev=1)
        h = w.header
        g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
        # coverage condition evaluated analytically for the ghost ring
        top = g.rgor + 2 * g.dnr
        bot = g.rgor - g.nnr * g.dnr
        assert g.gor >= top and (g.gor - bot) / g.dvr < g.nvr - 1
        assert g.gox <= g.rgox - 2 * g.dnx and (g.rgox + g.nnx * g.dnx - g.gox) / g.dvx < g.nvx - 1
        assert g.goz <= g.rgoz - 2 * g.dnz and (g.rgoz + g.nnz * g.dnz - g.goz) / g.dvz < g.nvz - 1


def test_receivers_inside(orc):
    from fm3dt import synth
    import fm3dt
    w = synth.config(1, scale=20, nev=1)
    h = w.header
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    ttn = np.ones(g.nnr * g.nnx * g.nnz)
    out = orc.srtimes(g, ttn, w.rec_elev, rcx, rcz)
    assert np.allclose(out, 1.0)


def test_latlon_conversion_matches_oracle(orc):
    import fm3dt
    lat = np.array([-35.4463, -31.5, 0.0, 12.25])
    lon = np.array([147.0653, 138.0, -20.0, 0.5])
    a = fm3dt.latlon_to_rad(lat, lon)
    b = orc.latlon_to_rad(lat, lon)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_forward_entry_points_reject_a_null_context(gpu_lib):
    """The one-call forward step and its host-link switch check their
    arguments before any device work (callable without a GPU)."""
    import ctypes as C
    import fm3dt
    L = gpu_lib
    st = fm3dt.Status()
    assert L.fm3dt_forward(None, 1, None, 0, None, None, None, None, None, None, None, 0, None, C.byref(st)) == fm3dt.EINVAL
    assert L.fm3dt_forward_device(None, 1, None, 0, None, None, None, None, None, None, None, 0, None, None,
                                  C.byref(st)) == fm3dt.EINVAL
    assert L.fm3dt_set_host_link(None, 0) == fm3dt.EINVAL
    f, r = C.c_int(), C.c_int()
    assert L.fm3dt_host_link(None, C.byref(f), C.byref(r)) == fm3dt.EINVAL
    assert L.fm3dt_forward_early_events(None) == 0
