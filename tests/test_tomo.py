"""Tomography driver (the reference's sub.sh loop).

CPU: the REAL(4) text round trip between the stages and subinv.in.
GPU: (1) the first model update of the in-process driver against the same
update computed entirely by the oracles (fixed-point fields, receiver times,
rays and Frechet rows from the C oracle; the subspace step from the numpy
oracle): within 1e-4 of max |dm| with double-precision stencils and the
float64 subspace step (the model-update bar), within 2e-3 with the fast
single-precision stencils and the REAL(4) subspace step; (2) the file loop
(fm3dt_run + fm3dt_subinv in a working directory, as sub.sh runs them) and
the in-process loop produce identical models."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))


def test_real4_text_round_trip():
    from fm3dt import files, tomo
    x = np.array([4.9, 5.0472015, 8.123456789, 6.25], dtype=np.float32)
    t = tomo.real4_text(x)
    assert np.array_equal(t.astype(np.float32), x)
    assert t[0] == float(files.format_real4(np.float32(4.9)))


def test_subinv_in_round_trip(tmp_path):
    from fm3dt import files
    p = str(tmp_path / "subinv.in")
    files.write_subinv_in(p, subdim=7, eta=2.5, invst=1)
    d = files.read_subinv_in(p)
    assert d["subdim"] == 7 and d["eta"] == 2.5 and d["invst"] == 1
    assert d["gridi"] == "gridi.vtx" and d["stfile"] == "stationres.dat" and d["fracg"] == 0.1


def _observed(prob, seed=1):
    """Picks of the true model plus N(0, 50 ms), as residuals relative to the
    starting model (otimes.dat values, REAL(4))."""
    import fm3dt
    from fm3dt import tomo
    from fm3dt import subinv as SI
    surv = tomo.Survey(prob.frames, prob.receivers)
    t = tomo.Tomography(prob.header, prob.velv_start, prob.cm_sd, surv, SI.Params(), precision=fm3dt.FP64)
    t_true = t.forward(prob.velv_true)[0].astype(np.float64)
    t_start = t.forward(prob.velv_start)[0].astype(np.float64)
    t.close()
    rng = np.random.default_rng(seed)
    ntr = t_true.size
    dobs = (t_true + rng.normal(0.0, 0.05, ntr) - t_start).astype(np.float32)
    tstat = (rng.uniform(0, 1, ntr) < 0.9).astype(np.int32)
    cd = np.full(ntr, 0.05, np.float32)
    return tstat, dobs, cd


def _oracle_update(orc, prob, params, tstat, dobs, cd):
    import subinv_oracle as SO
    h = prob.header
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = orc.gridder(g, prob.velv_start)
    times, ptr, cols, vals = [], [0], [], []
    for frames, rec in zip(prob.frames, prob.receivers):
        colat, lon = orc.latlon_to_rad(rec[:, 1], rec[:, 2])
        for fr in frames:
            ttn, _ = orc.fixed_point(g, veln, fr, 1)
            times.append(orc.srtimes(g, ttn, rec[:, 0], colat, lon))
            fdm, _, _ = orc.rays(g, ttn, veln, rec[:, 0], colat, lon)
            for row in fdm:
                c, v = orc.sparsify(row)
                cols.append(c)
                vals.append(v)
                ptr.append(ptr[-1] + len(c))
    times = np.concatenate(times).astype(np.float32)
    nsrc = [len(f) for f in prob.frames]
    nrc = [len(r) for r in prob.receivers]
    mo = prob.velv_start.astype(np.float32)
    dm, used = SO.step(h.nv, h.vorig, h.vstep, params, nsrc, nrc, mo, prob.cm_sd, mo, tstat, dobs, cd, times,
                       times, np.array(ptr), np.concatenate(cols), np.concatenate(vals))
    return dm, used


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "fast"])
def test_first_update_matches_oracle(gpu_lib, orc, mode):
    import fm3dt
    from fm3dt import synth, tomo
    from fm3dt import subinv as SI
    prob = synth.tomography_problem(scale=14, arrays=((4, 12), (3, 10)))
    tstat, dobs, cd = _observed(prob)
    params = SI.Params(subdim=6, epsilon=10.0, eta=10.0)
    # the 1e-4 bar holds for the double-precision path; the single-precision
    # form states its error instead: its rays follow a field ~1e-4 s off, so
    # rows move by up to ~1e-2 and the update by ~1e-3 of max|dm|
    prec, sprec, tol = (fm3dt.FP64, SI.FP64, 1e-4) if mode == "fp64" else (fm3dt.FP32_OFFSET, SI.FP32, 2e-3)
    t = tomo.Tomography(prob.header, prob.velv_start, prob.cm_sd, tomo.Survey(prob.frames, prob.receivers),
                        params, precision=prec, subinv_precision=sprec, batch=3)
    hist = t.run(1, tstat, dobs, cd)
    t.close()
    dm = hist.iterations[1].dm
    ref, used = _oracle_update(orc, prob, params, tstat, dobs, cd)
    assert hist.iterations[1].subdim == used
    rel = float(np.max(np.abs(dm - ref)) / np.max(np.abs(ref)))
    assert rel <= tol, rel
    # the update reduces the misfit to the picks
    assert hist.iterations[1].rms_residual < hist.iterations[0].rms_residual


@pytest.mark.gpu
def test_file_loop_equals_in_process_loop(gpu_lib, tmp_path):
    import fm3dt
    from fm3dt import files, synth, tomo
    from fm3dt import subinv as SI
    prob = synth.tomography_problem(scale=14, arrays=((3, 8), (2, 6)), seed=5)
    tstat, dobs, cd = _observed(prob, seed=2)
    d = str(tmp_path)
    files.write_in_file(os.path.join(d, "fm3dt_parallel.in"), files.InFile(gridv="gridc.vtx"))
    files.write_vtx(os.path.join(d, "gridi.vtx"), prob.header, prob.velv_start, second_column=0.3, fmt="%.8f")
    files.write_sources(os.path.join(d, "sources.dat"), [[(0.0, 0.0, 33.0, "P")] * len(f) for f in prob.frames])
    files.write_receivers(os.path.join(d, "receivers.dat"),
                          [[(r[0], r[1], r[2], "st") for r in rec] for rec in prob.receivers])
    files.write_itimes(os.path.join(d, "itimes.out"), np.concatenate(prob.frames))
    files.write_otimes(os.path.join(d, "otimes.dat"), tstat, dobs, cd)
    files.write_subinv_in(os.path.join(d, "subinv.in"), subdim=5)
    tomo.run_workdir(d, iterations=2)
    _, file_model = files.read_vtx(os.path.join(d, "gridc.vtx"))
    # the in-process loop with the values as the files hold them
    ts, ob, un = files.read_otimes(os.path.join(d, "otimes.dat"))
    t = tomo.Tomography(prob.header, prob.velv_start, prob.cm_sd, tomo.Survey(prob.frames, prob.receivers),
                        SI.Params(subdim=5), precision=fm3dt.FP64, subinv_precision=SI.FP32)
    hist = t.run(2, ts, ob.astype(np.float32), un.astype(np.float32))
    t.close()
    assert np.array_equal(file_model, hist.iterations[-1].model)
    got = files.read_rtravel(os.path.join(d, "rtravel.out"))
    assert np.array_equal(got, hist.iterations[-1].times)
