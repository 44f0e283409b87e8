"""The reference program's file contract: the Python readers/writers, the
host driver fm3dt_run's parsing (--check, no GPU) and its REAL(4) records,
and (GPU) a whole driver run in a working directory against the oracle.

GPU tolerances: receiver times within 1e-5 relative and 1 ms of the oracle's
fast-marching times (smooth model; the FP64 solve agrees with fast marching
to ~1e-12 s there); Frechet rows within 1e-4 of each row's largest entry
(the rays run through the GPU's own field)."""
import json
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def driver(gpu_lib):
    from fm3dt import build as fb
    return fb.build_driver()


def _workdir(path, scale=16, arrays=((3, 4), (2, 5)), cfg=0, fsrt=1, cfd=1, seed=5):
    """Writes a complete reference-style working directory; returns what was
    written (header, velv, frames per array, receivers per array)."""
    from fm3dt import files, synth
    w = synth.config(cfg, scale=scale, nev=1)
    h = w.header
    rng = np.random.default_rng(seed)
    src_arrays, rec_arrays, frames = [], [], []
    k = 0
    for nsrc, nrc in arrays:
        ev = np.stack([rng.uniform(30, 90, nsrc), rng.uniform(0, 360, nsrc)], 1)
        params = np.array([synth.planewave_params(h, *e) for e in ev])
        frames.append(synth.planewave_frames(h, params))
        src_arrays.append([(float(rng.uniform(-60, 60)), float(rng.uniform(-180, 180)), float(rng.uniform(0, 600)),
                            "P" if i % 2 == 0 else "PcP") for i in range(nsrc)])
        rec_arrays.append([(float(w.rec_elev[(k + j) % len(w.rec_elev)]), float(w.rec_lat[(k + j) % len(w.rec_lat)]),
                            float(w.rec_lon[(k + j) % len(w.rec_lon)]), f"st{j:02d}") for j in range(nrc)])
        k += nrc
    files.write_in_file(os.path.join(path, "fm3dt_parallel.in"), files.InFile(fsrt=fsrt, cfd=cfd))
    files.write_vtx(os.path.join(path, "gridc.vtx"), h, w.velv, second_column=0.3)
    files.write_sources(os.path.join(path, "sources.dat"), src_arrays)
    files.write_receivers(os.path.join(path, "receivers.dat"), rec_arrays)
    files.write_itimes(os.path.join(path, "itimes.out"), np.concatenate(frames))
    return h, w.velv, frames, rec_arrays


def _run(driver, *args, cwd=None):
    return subprocess.run([driver, *args], capture_output=True, text=True, cwd=cwd, timeout=600)


def test_real4_records(driver):
    from fm3dt import files
    # the reference's own rtimes.dat holds records like this one
    assert files.format_real4(357.198395) == "   357.198395    "
    vals = [357.198395, 1170.25, 0.5, -12.5, 0.0123456789, 1.0e10, 0.0, 999.99999999, 0.1, 3.0e-7]
    r = _run(driver, "--print-real4", *[repr(v) for v in vals])
    assert r.returncode == 0, r.stderr
    got = r.stdout.split("\n")[:-1]
    assert got == [files.format_real4(v) for v in vals]
    for line, v in zip(got, vals):
        assert np.float32(float(line)) == np.float32(v)


def test_python_readers_round_trip(tmp_path):
    from fm3dt import files
    h, velv, frames, recs = _workdir(str(tmp_path))
    f = files.read_in_file(str(tmp_path / "fm3dt_parallel.in"))
    assert (f.sources, f.itimes, f.receivers, f.gridv, f.rtravel, f.frechet) == (
        "sources.dat", "itimes.out", "receivers.dat", "gridc.vtx", "rtravel.out", "frechet.out")
    assert (f.earth, f.fom, f.ltfr, f.cslat, f.cslong, f.fsrt, f.cfd) == (6371.0, 1, 1, 0.4, 0.4, 1, 1)
    h2, v2 = files.read_vtx(str(tmp_path / "gridc.vtx"))
    assert np.array_equal(v2, velv) and h2.nn == tuple(h.nn) and h2.nv == tuple(h.nv)
    src = files.read_sources(str(tmp_path / "sources.dat"))
    assert [len(a) for a in src] == [3, 2] and src[0][1][3] == "PcP"
    rec = files.read_receivers(str(tmp_path / "receivers.dat"))
    assert [[r[:3] for r in a] for a in recs] == rec
    it = files.read_itimes(str(tmp_path / "itimes.out"), h.nn[1], h.nn[2])
    assert np.array_equal(it, np.concatenate(frames))


def test_frechet_records_round_trip(tmp_path):
    from fm3dt import files
    ptr = np.array([0, 3, 3, 5])
    cols = np.array([7, 9, 12, 1, 4], np.int32)
    vals = np.array([-1.5, -2.25, -0.125, -3.0, -4.0], np.float32)
    p = str(tmp_path / "frechet.out")
    files.write_frechet(p, ptr, cols, vals, [1, 2, 3])
    raw = open(p, "rb").read()
    assert len(raw) == 16 * (3 + 5)
    # header record of row 1: length 8, 3 entries, real(1), length 8
    assert raw[:16] == np.array([8, 3], "=i4").tobytes() + np.float32(1).tobytes() + np.array([8], "=i4").tobytes()
    fr = files.read_frechet(p)
    assert np.array_equal(fr.row_ptr, ptr) and np.array_equal(fr.cols, cols) and np.array_equal(fr.vals, vals)
    assert np.array_equal(fr.recid, [1, 2, 3])


def test_driver_check_parses_like_python(driver, tmp_path):
    h, velv, frames, recs = _workdir(str(tmp_path))
    r = _run(driver, "--check", "-C", str(tmp_path))
    assert r.returncode == 0, r.stderr
    j = json.loads(r.stdout)
    assert j["nn"] == list(h.nn) and j["nv"] == list(h.nv)
    assert j["norig"] == list(h.norig) and j["nstep"] == list(h.nstep)
    assert j["vorig"] == list(h.vorig) and j["vstep"] == list(h.vstep)
    assert j["nsrc"] == [3, 2] and j["nrc"] == [4, 5]
    assert j["velv_n"] == velv.size
    assert j["velv_sum"] == pytest.approx(float(np.sum(velv)), rel=1e-13)
    assert j["itimes_sum"] == pytest.approx(float(np.sum(np.concatenate(frames))), rel=1e-13)
    assert (j["earth"], j["fom"], j["fsrt"], j["cfd"], j["first_phase"]) == (6371.0, 1, 1, 1, "P")


def test_driver_parses_reference_layout(driver, tmp_path):
    """Comments after values, a blank record before the velocities, two
    values per velocity record, Fortran 'd' exponents."""
    from fm3dt import files
    h, velv, frames, recs = _workdir(str(tmp_path))
    p = str(tmp_path / "gridc.vtx")
    lines = open(p).read().splitlines()
    lines[6:] = [""] + ["  %sd0  0.30000000" % repr(float(v)) for v in velv]
    open(p, "w").write("\n".join(lines) + "\n")
    r = _run(driver, "--check", "-C", str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout)["velv_sum"] == pytest.approx(float(np.sum(velv)), rel=1e-13)
    assert np.array_equal(files.read_vtx(p)[1], velv)


def test_driver_rejects_inconsistent_inputs(driver, tmp_path):
    from fm3dt import files
    _workdir(str(tmp_path))
    rec = files.read_receivers(str(tmp_path / "receivers.dat"))
    files.write_receivers(str(tmp_path / "receivers.dat"), [[(a, b, c, "x") for a, b, c in rec[0]]])
    r = _run(driver, "--check", "-C", str(tmp_path))
    assert r.returncode == 1 and "inconsistent" in r.stderr
    _workdir(str(tmp_path))
    p = str(tmp_path / "itimes.out")
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-8])
    r = _run(driver, "--check", "-C", str(tmp_path))
    assert r.returncode == 1 and "itimes.out" in r.stderr


@pytest.mark.gpu
def test_driver_run_matches_oracle(driver, orc, tmp_path):
    from fm3dt import files
    h, velv, frames, recs = _workdir(str(tmp_path))
    r = _run(driver, "-C", str(tmp_path), "--batch", "2")
    assert r.returncode == 0, r.stdout + r.stderr
    times = files.read_rtravel(str(tmp_path / "rtravel.out"))
    fr = files.read_frechet(str(tmp_path / "frechet.out"))
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = orc.gridder(g, velv)
    ref_t, ref_rows, recid = [], [], []
    for fr_a, rec_a in zip(frames, recs):
        el = np.array([x[0] for x in rec_a])
        colat, lon = orc.latlon_to_rad(np.array([x[1] for x in rec_a]), np.array([x[2] for x in rec_a]))
        for frame in fr_a:
            ttn, _ = orc.fmm(g, veln, frame, 1)
            ref_t.append(orc.srtimes(g, ttn, el, colat, lon))
            fdm, _, _ = orc.rays(g, ttn, veln, el, colat, lon)
            ref_rows.extend(np.where(np.abs(fdm) >= np.float32(1e-6), fdm, 0.0))
            recid.extend(range(1, len(rec_a) + 1))
    ref_t = np.concatenate(ref_t).astype(np.float64)
    assert times.shape == ref_t.shape
    err = np.abs(times.astype(np.float64) - ref_t)
    assert np.max(err) <= 1e-3 and np.max(err / ref_t) <= 1e-5
    assert len(fr.row_ptr) - 1 == len(ref_rows)
    assert np.array_equal(fr.recid, recid)
    nmp = (h.nv[0] + 2) * (h.nv[1] + 2) * (h.nv[2] + 2)
    for q, ref in enumerate(ref_rows):
        got = np.zeros(nmp)
        c = fr.cols[fr.row_ptr[q]:fr.row_ptr[q + 1]]
        assert np.all(np.diff(c) > 0)
        got[c - 1] = fr.vals[fr.row_ptr[q]:fr.row_ptr[q + 1]]
        assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref))
