"""Parity at the workload sizes, end to end, through the C ABI.

The double-precision CUDA path (field, receiver times, rays, Frechet rows) is
compared with the oracle's serial fast marching -- the reference's local_fmm
with its heap and octant tables (fm3dt_parallel.f90 F:78-155, F:535-1098) --
followed by the oracle's srtimes (F:7040-7248) and parallel_rpaths
(F:7250-7777) on the oracle's own field.  Nothing is shared between the two
sides but the inputs.

Cases: the single plane-wave event at 64^3 (delta 60 deg, back-azimuth 45 deg,
100 receivers), two events of the 128^3 batch (300 receivers), and one event
of the 192 x 224 x 224 tomography grid (300 receivers), all at full size.

Bars, per the parity contract of the batched path:
* receiver times within 1e-5 relative and 1 ms;
* ray end points within one propagation cell (per axis, in cells);
* Frechet rows within 1e-4 relative: the largest entry difference over the
  row's largest entry, and the 2-norm of the difference over the row's 2-norm;
* the field itself within 1e-9 of the largest time (about 1e-6 s): on these
  models fast marching's heap order reaches the same values as the
  order-independent fixed point the GPU solves for, and the two differ only
  by the rounding of their different (equivalent) operation orders, which a
  long path accumulates to a few 1e-8 s on the 192 x 224 x 224 grid.
Measured on a GB300 (double precision): field 1.3e-12 / 2.2e-12 / 4.2e-8 s;
receiver times equal bit for bit; end points within 1e-9 cells; rows within
7e-7 (largest entry) and 5e-7 (2-norm) relative.  Single precision: receiver
times 1.5e-7 relative (0.12 ms), end points 0.12 cells; its rows differ from
the reference's by up to 1.5e-2 (largest entry) -- the rays follow a field
that differs by up to 8e-5 s -- which this test reports and does not bound.
The single-precision offset path is compared on the same cases for receiver
times and ray end points (the bars of the batched path).  Each case prints
its measured maxima for both precisions (run with -s to see them).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rows_dense(row_ptr, cols, vals, nrows, nmp):
    out = np.zeros((nrows, nmp), dtype=np.float64)
    for i in range(nrows):
        c = cols[row_ptr[i]:row_ptr[i + 1]]
        assert np.all(np.diff(c) > 0)
        out[i, c - 1] = vals[row_ptr[i]:row_ptr[i + 1]]
    return out


def _gpu_side(w, params, prec, rcr, rcx, rcz, nmp):
    import fm3dt
    with fm3dt.Solver(w.header, fom=1, precision=prec, max_events=len(params)) as s:
        s.set_velocity(w.velv)
        st = s.solve_planewave(params)
        assert st["converged"] == 1
        fields = [s.get_times(e) for e in range(len(params))]
        times = s.receiver_times(rcr, rcx, rcz).astype(np.float64)
        row_ptr, cols, vals, ends = s.rays_frechet(rcr, rcx, rcz)
    return fields, times, _rows_dense(row_ptr, cols, vals, len(params) * len(rcr), nmp), ends


def _end_to_end(orc, cfg, events, precisions=(0,)):
    """Both sides on the same inputs; returns {precision: measured maxima}."""
    from fm3dt import synth
    import fm3dt
    w = synth.config(cfg, nev=len(events))
    w.events = np.asarray(events, dtype=np.float64).reshape(-1, 2)
    h = w.header
    params = np.array([synth.planewave_params(h, *ev) for ev in w.events])
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, ncl = orc.gridder(g, w.velv)
    assert ncl == 0
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    nrc = len(rcr)
    nmp = orc.nmp(g)
    gpu = {prec: _gpu_side(w, params, prec, rcr, rcx, rcz, nmp) for prec in precisions}
    reports = {prec: {"field_s": 0.0, "recv_rel": 0.0, "recv_abs_s": 0.0, "end_cells": 0.0, "row_max": 0.0,
                      "row_l2": 0.0} for prec in precisions}
    for e, p in enumerate(params):
        frame = orc.planewave_frame(g, orc.PlaneWave(*p))
        ref, _ = orc.fmm(g, veln, frame, 1)
        rt = orc.srtimes(g, ref, rcr, rcx, rcz).astype(np.float64)
        fdm, ends, _ = orc.rays(g, ref, veln, rcr, rcx, rcz)
        refrows = fdm.astype(np.float64)
        refrows[np.abs(fdm) < np.float32(1e-6)] = 0.0          # the reference keeps |f| >= 1e-6 (F:7263)
        rmax = np.max(np.abs(refrows), axis=1)
        rl2 = np.linalg.norm(refrows, axis=1)
        assert np.all(rmax > 0)
        for prec in precisions:
            fields, times, dense, gends = gpu[prec]
            r = reports[prec]
            r["field_s"] = max(r["field_s"], float(np.max(np.abs(fields[e] - ref))))
            r["field_rel"] = max(r.get("field_rel", 0.0), float(np.max(np.abs(fields[e] - ref)) / np.max(ref)))
            gt = times[e]
            r["recv_rel"] = max(r["recv_rel"], float(np.max(np.abs(gt - rt) / rt)))
            r["recv_abs_s"] = max(r["recv_abs_s"], float(np.max(np.abs(gt - rt))))
            ge = gends[e * nrc:(e + 1) * nrc]
            cells = np.maximum(np.abs(ge[:, 0] - ends[:, 0]) / g.dnr,
                               np.maximum(np.abs(ge[:, 1] - ends[:, 1]) / g.dnx,
                                          np.abs(ge[:, 2] - ends[:, 2]) / g.dnz))
            r["end_cells"] = max(r["end_cells"], float(cells.max()))
            d = dense[e * nrc:(e + 1) * nrc] - refrows
            r["row_max"] = max(r["row_max"], float(np.max(np.max(np.abs(d), axis=1) / rmax)))
            r["row_l2"] = max(r["row_l2"], float(np.max(np.linalg.norm(d, axis=1) / rl2)))
    for prec, r in reports.items():
        print(f"\nconfig {cfg} {h.nn} events {len(params)} {'FP64' if prec == 0 else 'FP32 offset'}: " +
              ", ".join(f"{k} {v:.3e}" for k, v in r.items()))
    if 0 in reports:
        r = reports[0]
        assert r["field_rel"] <= 1e-9
        assert r["recv_rel"] <= 1e-5 and r["recv_abs_s"] <= 1e-3
        assert r["end_cells"] <= 1.0
        assert r["row_max"] <= 1e-4 and r["row_l2"] <= 1e-4
    if 1 in reports:
        # single-precision stencils: receiver times and ray end points meet
        # the bars against the reference's double-precision march
        r = reports[1]
        assert r["recv_rel"] <= 1e-5 and r["recv_abs_s"] <= 1e-3
        assert r["end_cells"] <= 1.0
    return reports


def test_single_event_64_cubed_full_size(gpu_lib, orc):
    _end_to_end(orc, 0, [(60.0, 45.0)])


def test_batch_events_128_cubed_full_size(gpu_lib, orc):
    from fm3dt import synth
    w = synth.config(1, nev=256)
    _end_to_end(orc, 1, w.events[:2], precisions=(0, 1))


def test_tomography_grid_event_full_size(gpu_lib, orc):
    from fm3dt import synth
    w = synth.config(3, nev=500)
    _end_to_end(orc, 3, w.events[:1], precisions=(0, 1))


@pytest.mark.parametrize("cfg,nev", [(0, 1), (1, 2)])
def test_against_the_reference_decomposed_run(gpu_lib, orc, cfg, nev):
    """What the reference's own production run (mpirun -np 9: 2 x 2 x 2
    blocks, oracle.fmm_decomposed) would print, against the GPU.  The
    decomposed run is a different discretisation near block faces and edges
    (first-order terms where a second neighbour lies in another block; edge
    nodes re-solved by the face stencils only), so it differs from the
    serial march -- which the GPU equals -- by more than the 1e-5 bar:
    measured 7.3e-2 s / 1.0e-4 relative at receivers on the 64^3 event,
    2.8e-2 to 3.7e-2 s / 5.7e-5 on 128^3 events.  The test states that gap
    and bounds it at twice the measured relative size."""
    import fm3dt
    from fm3dt import synth
    w = synth.config(cfg, nev=nev)
    h = w.header
    params = np.array([synth.planewave_params(h, *ev) for ev in w.events])
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    rcx, rcz = fm3dt.latlon_to_rad(w.rec_lat, w.rec_lon)
    rcr = np.asarray(w.rec_elev, dtype=np.float64)
    with fm3dt.Solver(h, fom=1, precision=fm3dt.FP64, max_events=len(params)) as s:
        s.set_velocity(w.velv)
        s.solve_planewave(params)
        gt = s.receiver_times(rcr, rcx, rcz).astype(np.float64)
    worst_rel = worst_abs = 0.0
    for e, p in enumerate(params):
        frame = orc.planewave_frame(g, orc.PlaneWave(*p))
        dec, rounds = orc.fmm_decomposed(g, w.velv, frame, 1, (2, 2, 2))
        assert rounds <= 8
        rt = orc.srtimes(g, dec, rcr, rcx, rcz).astype(np.float64)
        worst_rel = max(worst_rel, float(np.max(np.abs(gt[e] - rt) / rt)))
        worst_abs = max(worst_abs, float(np.max(np.abs(gt[e] - rt))))
    print(f"\nconfig {cfg} {h.nn}: GPU vs the 2x2x2 run at receivers: {worst_abs:.3e} s, {worst_rel:.2e} relative")
    assert worst_rel <= 2.5e-4 and worst_abs <= 0.15
