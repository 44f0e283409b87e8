"""Subspace inversion (host port of subinv) against the numpy oracle.

Tolerances: FP64 mode within 1e-9 of the oracle (relative to max |dm|; the
two orthonormalise the same span by different methods); FP32 mode (the
reference's REAL(4) arithmetic) within 1e-4 of the oracle, the bar for the
model update (5e-4 with station terms, see below).  The oracle itself is
pinned by a closed form (the one-dimensional subspace is steepest descent
with an exact line search) and by an independent dense restatement of the
Galerkin step."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))


def _problem(nv=(3, 4, 4), arrays=((3, 5), (2, 4)), seed=0, unsorted_rows=0, picked=0.8):
    rng = np.random.default_rng(seed)
    nmpv = (nv[0] + 2) * (nv[1] + 2) * (nv[2] + 2)
    nsrc = np.array([a[0] for a in arrays])
    nrc = np.array([a[1] for a in arrays])
    ntr = int(np.sum(nsrc * nrc))
    ptr, cols, vals = [0], [], []
    for i in range(ntr):
        n = int(rng.integers(4, min(24, nmpv)))
        c = np.sort(rng.choice(nmpv, n, replace=False)) + 1
        if i < unsorted_rows:
            c[[0, -1]] = c[[-1, 0]]
        cols.append(c)
        vals.append(-rng.uniform(0.5, 30.0, n).astype(np.float32))
        ptr.append(ptr[-1] + n)
    mo = (5.8 + 3.0 * rng.uniform(0, 1, nmpv)).astype(np.float32)
    mc = (mo + rng.normal(0, 0.05, nmpv)).astype(np.float32)
    nmps = int(np.sum(nrc))
    mc_full = np.concatenate([mc, rng.normal(0, 0.02, nmps).astype(np.float32)])
    tstat = (rng.uniform(0, 1, ntr) < picked).astype(np.int32)
    mt = rng.uniform(300, 1200, ntr).astype(np.float32)
    rt = (mt - rng.normal(0, 0.3, ntr)).astype(np.float32)
    dobs = rng.normal(0, 0.5, ntr).astype(np.float32)
    cd = rng.uniform(0.03, 0.08, ntr).astype(np.float32)
    cm = np.full(nmpv, 0.3, np.float32)
    grid = (nv, (1.5, -30.0, 135.0), (25.0, 0.239, 0.355))
    return dict(grid=grid, nsrc=nsrc, nrc=nrc, mo=mo, cm_sd=cm, mc=mc, mc_full=mc_full, tstat=tstat, dobs=dobs,
                cd_sd=cd, mtimes=mt, rtimes=rt, row_ptr=np.array(ptr, np.int64),
                cols=np.concatenate(cols).astype(np.int32), vals=np.concatenate(vals))


def _run(pr, params, precision):
    from fm3dt import subinv as S
    mc = pr["mc_full"] if params.invst == 1 else pr["mc"]
    return S.step(pr["grid"], params, pr["nsrc"], pr["nrc"], pr["mo"], pr["cm_sd"], mc, pr["tstat"], pr["dobs"],
                  pr["cd_sd"], pr["mtimes"], pr["rtimes"], pr["row_ptr"], pr["cols"], pr["vals"], precision)


def _oracle(pr, params):
    import subinv_oracle as O
    nv, vo, vs = pr["grid"]
    mc = pr["mc_full"] if params.invst == 1 else pr["mc"]
    return O.step(nv, vo, vs, params, pr["nsrc"], pr["nrc"], pr["mo"], pr["cm_sd"], mc, pr["tstat"], pr["dobs"],
                  pr["cd_sd"], pr["mtimes"], pr["rtimes"], pr["row_ptr"], pr["cols"], pr["vals"])


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


CASES = [  # asds, rmtr, invst, subdim
    (0, 0, 0, 1), (0, 0, 0, 4), (1, 1, 0, 10), (0, 1, 1, 2), (1, 0, 1, 5), (1, 1, 1, 10)]


@pytest.mark.parametrize("asds,rmtr,invst,subdim", CASES)
def test_fp64_matches_oracle(asds, rmtr, invst, subdim):
    from fm3dt import subinv as S
    p = S.Params(asds=asds, rmtr=rmtr, invst=invst, subdim=subdim)
    pr = _problem(seed=subdim + 10 * asds)
    dm, used, _ = _run(pr, p, S.FP64)
    ref, ref_used = _oracle(pr, p)
    assert used == ref_used
    assert _rel(dm, ref) <= 1e-9


@pytest.mark.parametrize("asds,rmtr,invst,subdim", CASES)
def test_fp32_within_update_tolerance(asds, rmtr, invst, subdim):
    """REAL(4) arithmetic against the float64 oracle: within 1e-4 of max |dm|.
    With station terms the reference adds each station term to the model
    time (hundreds of seconds) in REAL(4) before subtracting the reference
    time, which alone costs ~6e-5 s per pick; the bound
    there is 5e-4."""
    from fm3dt import subinv as S
    p = S.Params(asds=asds, rmtr=rmtr, invst=invst, subdim=min(subdim, 4))
    pr = _problem(seed=7 + subdim)
    dm, used, _ = _run(pr, p, S.FP32)
    ref, ref_used = _oracle(pr, p)
    assert used == ref_used
    assert _rel(dm, ref) <= (5e-4 if invst == 1 else 1e-4)


def test_oracle_one_dimensional_subspace_is_steepest_descent():
    """subdim = 1: dm = -a (a^T H a)^-1 a^T gamma, a = Cm gamma / |Cm gamma|."""
    import subinv_oracle as O
    from fm3dt import subinv as S
    p = S.Params(asds=0, rmtr=0, invst=0, subdim=1)
    pr = _problem(seed=3)
    nv, vo, vs = pr["grid"]
    nmpv = (nv[0] + 2) * (nv[1] + 2) * (nv[2] + 2)
    G, Gt, dmod, dob, cd, nmp = O.assemble(pr["nsrc"], pr["nrc"], nmpv, 0, 0, pr["mc"], pr["tstat"], pr["dobs"],
                                           pr["cd_sd"], pr["mtimes"], pr["rtimes"], pr["row_ptr"], pr["cols"],
                                           pr["vals"])
    Gd = G.toarray()
    cm = pr["cm_sd"].astype(np.float64) ** 2
    x = pr["mc"].astype(np.float64) - pr["mo"]
    gamma = Gd.T @ ((dmod - dob) / cd) + p.epsilon * x / cm
    H = Gd.T @ (Gd / cd[:, None]) + np.diag(p.epsilon / cm)
    a = cm * gamma
    a /= np.linalg.norm(a)
    want = -a * (a @ gamma) / (a @ H @ a)
    got, used = O.step(nv, vo, vs, p, pr["nsrc"], pr["nrc"], pr["mo"], pr["cm_sd"], pr["mc"], pr["tstat"],
                       pr["dobs"], pr["cd_sd"], pr["mtimes"], pr["rtimes"], pr["row_ptr"], pr["cols"], pr["vals"])
    assert used == 1 and _rel(got, want) <= 1e-12


def test_oracle_matches_a_dense_galerkin_step():
    """Independent dense restatement: Krylov vectors a1 = Cm gamma,
    a' = Cm G^T Cd^-1 G a + eps a (normalised), SVD basis, then the Galerkin
    step; no smoothing, no station terms."""
    import subinv_oracle as O
    from fm3dt import subinv as S
    p = S.Params(asds=0, rmtr=1, invst=0, subdim=6)
    pr = _problem(seed=9)
    nv, vo, vs = pr["grid"]
    keep = pr["tstat"] == 1
    nmp = pr["mo"].size
    Gd = np.zeros((len(pr["tstat"]), nmp))
    for i in range(len(pr["tstat"])):
        a, b = pr["row_ptr"][i], pr["row_ptr"][i + 1]
        Gd[i, pr["cols"][a:b] - 1] = pr["vals"][a:b]
    Gd = Gd[keep]
    r = (pr["mtimes"].astype(np.float64) - pr["rtimes"])[keep]
    src = np.concatenate([np.repeat(np.arange(ns) + sum(pr["nsrc"][:k]), nr)
                          for k, (ns, nr) in enumerate(zip(pr["nsrc"], pr["nrc"]))])[keep]
    for s_ in np.unique(src):
        r[src == s_] -= r[src == s_].mean()
    cd = pr["cd_sd"][keep].astype(np.float64) ** 2
    cm = pr["cm_sd"].astype(np.float64) ** 2
    x = pr["mc"].astype(np.float64) - pr["mo"]
    gamma = Gd.T @ ((r - pr["dobs"][keep]) / cd) + p.epsilon * x / cm
    H = Gd.T @ (Gd / cd[:, None]) + np.diag(p.epsilon / cm)
    vecs = [cm * gamma / np.linalg.norm(cm * gamma)]
    while len(vecs) < p.subdim:
        a = cm * (Gd.T @ (Gd @ vecs[-1] / cd)) + p.epsilon * vecs[-1]
        vecs.append(a / np.linalg.norm(a))
    U, sv, _ = np.linalg.svd(np.column_stack(vecs), full_matrices=False)
    A = U[:, sv >= 1e-7]
    want = -A @ np.linalg.solve(A.T @ H @ A, A.T @ gamma)
    got, used = O.step(nv, vo, vs, p, pr["nsrc"], pr["nrc"], pr["mo"], pr["cm_sd"], pr["mc"], pr["tstat"],
                       pr["dobs"], pr["cd_sd"], pr["mtimes"], pr["rtimes"], pr["row_ptr"], pr["cols"], pr["vals"])
    assert used == A.shape[1]
    assert _rel(got, want) <= 1e-9


def test_smoothing_transpose_quirk():
    """The reference's D^T uses the theta count as the phi bound (S:698,
    S:931): it is the exact transpose of D when nvt == nvp and not otherwise."""
    import subinv_oracle as O
    D, Dt = O.smoothing((3, 4, 4), 1.5, -30.0, 25.0, 0.239, 0.355, 6371.0)
    assert abs(Dt - D.T).max() == 0.0
    D, Dt = O.smoothing((3, 4, 6), 1.5, -30.0, 25.0, 0.239, 0.355, 6371.0)
    assert abs(Dt - D.T).max() > 0.0


def test_rank_reduction_is_reported():
    """The basis recursion is a power iteration: with many vectors on a small
    model they become dependent and the dimension is reduced."""
    from fm3dt import subinv as S
    p = S.Params(asds=1, rmtr=1, invst=0, subdim=40, epsilon=1.0, eta=0.5, fracg=1.0)
    pr = _problem(nv=(1, 1, 1), arrays=((6, 8),), seed=5)
    dm, used, msg = _run(pr, p, S.FP64)
    ref, ref_used = _oracle(pr, p)
    assert used == ref_used < 40 and ("reduced from 40 to %d" % used) in msg
    assert _rel(dm, ref) <= 1e-6


def test_unsorted_rows_follow_the_reference_transpose():
    """A row whose columns are not ascending loses, in G^T only, everything
    after its first decrease (the reference's transpose loop)."""
    from fm3dt import subinv as S
    p = S.Params(asds=0, rmtr=0, invst=0, subdim=3)
    pr = _problem(seed=11, unsorted_rows=4, picked=1.0)
    dm, used, _ = _run(pr, p, S.FP64)
    ref, _ = _oracle(pr, p)
    assert _rel(dm, ref) <= 1e-9
    srt = dict(pr)
    for i in range(4):
        a, b = pr["row_ptr"][i], pr["row_ptr"][i + 1]
        o = np.argsort(pr["cols"][a:b])
        srt["cols"] = srt["cols"].copy()
        srt["vals"] = srt["vals"].copy()
        srt["cols"][a:b] = pr["cols"][a:b][o]
        srt["vals"][a:b] = pr["vals"][a:b][o]
    dm_sorted, _, _ = _run(srt, p, S.FP64)
    assert _rel(dm, dm_sorted) > 1e-6


def test_errors_are_reported():
    from fm3dt import subinv as S
    pr = _problem(seed=2)
    with pytest.raises(S.SubinvError, match="less than one"):
        _run(pr, S.Params(subdim=0), S.FP32)
    with pytest.raises(S.SubinvError, match="subspace dimension of 1"):
        _run(pr, S.Params(subdim=1, invst=1), S.FP32)
    with pytest.raises(S.SubinvError, match="too large"):
        _run(pr, S.Params(fracg=1e-4), S.FP32)


def test_program_writes_the_reference_files(tmp_path):
    """fm3dt_subinv in a working directory: reads subinv.in and the files it
    names, writes gridc.vtx whose values are mc + dm in REAL(4)."""
    from fm3dt import build as fb, files
    from fm3dt import subinv as S
    fb.build_subinv()
    pr = _problem(seed=4)
    nv, vo, vs = pr["grid"]
    d = str(tmp_path)
    nmpv = pr["mo"].size
    with open(os.path.join(d, "gridi.vtx"), "w") as fh:
        fh.write("%12d%12d%12d\n" % tuple(nv))
        fh.write("%12.6f%12.6f%12.6f\n" % vo)
        fh.write("%12.6f%12.6f%12.6f\n" % vs)
        fh.write("%12d%12d%12d\n" % (31, 110, 140))
        fh.write("%12.6f%12.6f%12.6f\n" % (1.5, -31.5, 138.0))
        fh.write("%12.6f%12.6f%12.6f\n\n" % (10.0, 0.06962, 0.090909))
        for v, c in zip(pr["mo"], pr["cm_sd"]):
            fh.write("  %s  %s\n" % (repr(float(v)), repr(float(c))))
    with open(os.path.join(d, "gridc.vtx"), "w") as fh:
        fh.write("\n" * 6 + "".join(files.format_real4(v) + "\n" for v in pr["mc"]))
    with open(os.path.join(d, "subiter.in"), "w") as fh:
        fh.write("2\n")
    names = ["gridi.vtx", "gridc.vtx", "otimes.dat", "rtimes.dat", "rtravel.out", "1", "frechet.out",
             "sources.dat", "receivers.dat", "subiter.in", "10.0", "4", "1", "10.0", "0", "stationres.dat",
             "10.0", "0.1", "6371.0"]
    with open(os.path.join(d, "subinv.in"), "w") as fh:
        fh.write("c\nc INPUT PARAMETERS\nc\n" + "".join("%-26sc: item\n" % n for n in names))
    files.write_otimes(os.path.join(d, "otimes.dat"), pr["tstat"], pr["dobs"], pr["cd_sd"])
    files.write_rtravel(os.path.join(d, "rtravel.out"), pr["mtimes"])
    files.write_rtravel(os.path.join(d, "rtimes.dat"), pr["rtimes"])
    recid = np.concatenate([np.tile(np.arange(1, nr + 1), ns) for ns, nr in zip(pr["nsrc"], pr["nrc"])])
    files.write_frechet(os.path.join(d, "frechet.out"), pr["row_ptr"], pr["cols"], pr["vals"], recid)
    files.write_sources(os.path.join(d, "sources.dat"),
                        [[(0.0, 0.0, 10.0, "P")] * ns for ns in pr["nsrc"]])
    files.write_receivers(os.path.join(d, "receivers.dat"),
                          [[(0.1, -35.0, 147.0, "x")] * nr for nr in pr["nrc"]])
    r = subprocess.run([fb.SUBINV, "-C", d], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    h, new = files.read_vtx(os.path.join(d, "gridc.vtx"))
    assert h.nv == tuple(nv) and new.size == nmpv
    # the same step through the C ABI, with the values as the files hold them
    mo = np.array([np.float32(repr(float(v))) for v in pr["mo"]])
    otimes = files.read_otimes(os.path.join(d, "otimes.dat"))
    dm, used, _ = S.step(pr["grid"], S.Params(subdim=4), pr["nsrc"], pr["nrc"], mo, pr["cm_sd"],
                         files.read_rtravel(os.path.join(d, "rtravel.out"))[:0].tolist() or
                         np.array([np.float32(float(files.format_real4(v))) for v in pr["mc"]]),
                         otimes[0], otimes[1].astype(np.float32), otimes[2].astype(np.float32),
                         files.read_rtravel(os.path.join(d, "rtravel.out")),
                         files.read_rtravel(os.path.join(d, "rtimes.dat")),
                         pr["row_ptr"], pr["cols"], pr["vals"], S.FP32)
    mc_file = np.array([np.float32(float(files.format_real4(v))) for v in pr["mc"]])
    want = (mc_file + dm.astype(np.float32)).astype(np.float32)
    assert np.array_equal(new.astype(np.float32), want)
