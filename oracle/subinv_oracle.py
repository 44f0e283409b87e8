"""Oracle (test infrastructure only): a float64 numpy restatement of one step
of the reference's subspace inversion, subinv.f90 ("S").

Only the tests import this module; it checks the host implementation in
parallel-fast-marching-method_gb300/subinv/subinv.cpp.  It restates the
algorithm with sparse matrices instead of the reference's loops:

* data assembly: picked rows only (tstat = 1), model times minus
  reference times, station-term column per receiver when invst = 1, each
  source's mean model residual removed when rmtr = 1; the transpose keeps
  each row's leading strictly increasing run of columns;
* gradient gamma = G^T Cd^-1 (dmod - dobs) + eps Cm^-1 (mc - mo)
  [+ eta D~^T D (mc - mo)], with D the scaled second-difference
  operator on the padded velocity grid and D~^T its transpose except that the
  phi+1 neighbour is used when i+2 <= nvt;
* basis: the per-class normalised vectors Cm gamma, then the recursion
  a' = Cm G^T Cd^-1 G a + eps a, normalised per class;
* orthonormal basis from the SVD with singular values >= 1e-7;
* dm = -A (A^T H A)^-1 A^T gamma, H = G^T Cd^-1 G + eps Cm^-1 [+ eta D~^T D]
  (S:832-990).

Parity pin: the reference cannot be compiled here (no Fortran compiler), so
this restatement is checked against analytic properties in the tests (the
full-space limit equals the damped least-squares solution).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

PI = float(np.float32(3.1415926535898))


def assemble(nsrc, nrc, nmpv, invst, rmtr, mc, tstat, dobs, cd_sd, mtimes, rtimes, row_ptr, cols, vals):
    """Picked system: (G forward csr, G transpose csr as the reference builds
    it, dmod, dobs, cd variance)."""
    nsrc = np.asarray(nsrc)
    nrc = np.asarray(nrc)
    src_id, rec_id = [], []
    s0 = r0 = 0
    for ns, nr in zip(nsrc, nrc):
        for j in range(ns):
            for k in range(nr):
                src_id.append(s0 + j)
                rec_id.append(r0 + k)
        s0 += ns
        r0 += nr
    nmp = nmpv + (r0 if invst == 1 else 0)
    fr_rows, fr_cols, fr_vals, t_rows, t_cols, t_vals = [], [], [], [], [], []
    dmod, dob, cd, srcs = [], [], [], []
    for i in range(len(tstat)):
        if tstat[i] != 1:
            continue
        q = len(dmod)
        c = list(np.asarray(cols[row_ptr[i]:row_ptr[i + 1]], dtype=np.int64) - 1)
        v = list(np.asarray(vals[row_ptr[i]:row_ptr[i + 1]], dtype=np.float64))
        dm_i = float(mtimes[i])
        if invst == 1:
            c.append(nmpv + rec_id[i])
            v.append(1.0)
            dm_i += float(mc[nmpv + rec_id[i]])
        for k, (cc, vv) in enumerate(zip(c, v)):
            fr_rows.append(q)
            fr_cols.append(cc)
            fr_vals.append(vv)
        # transpose: leading strictly increasing run
        last = -1
        for cc, vv in zip(c, v):
            if cc <= last:
                break
            t_rows.append(q)
            t_cols.append(cc)
            t_vals.append(vv)
            last = cc
        dmod.append(dm_i - float(rtimes[i]))
        dob.append(float(dobs[i]))
        cd.append(float(cd_sd[i]) ** 2)
        srcs.append(src_id[i])
    dmod = np.array(dmod)
    if rmtr == 1 and len(dmod):
        srcs = np.array(srcs)
        for s in np.unique(srcs):
            m = srcs == s
            dmod[m] -= dmod[m].mean()
    n = len(dmod)
    G = sp.csr_matrix((fr_vals, (fr_rows, fr_cols)), shape=(n, nmp))
    Gt = sp.csr_matrix((t_vals, (t_cols, t_rows)), shape=(nmp, n))
    return G, Gt, dmod, np.array(dob), np.array(cd), nmp


def smoothing(nv, gor, got, dnr, dnt, dnp, earth):
    """(D, D~^T) on the padded grid, r fastest (sparse, float64)."""
    nvr, nvt, nvp = nv[0] + 2, nv[1] + 2, nv[2] + 2
    rdnt = dnt * PI / 180.0
    rdnp = dnp * PI / 180.0
    rgot = (90.0 - got) * PI / 180.0
    idx = lambda i, j, k: (i * nvt + j) * nvr + k   # noqa: E731
    n = nvr * nvt * nvp
    dr, dc, dv, tr, tc, tv = [], [], [], [], [], []
    for i in range(nvp):
        for j in range(nvt):
            thet = np.sin(rgot + j * rdnt)
            for k in range(nvr):
                rad = gor - k * dnr + earth
                st = dnr ** 2 / (rad * rdnt) ** 2
                spp = dnr ** 2 / (rad * thet * rdnp) ** 2
                q = idx(i, j, k)
                # D row q
                if 0 < k < nvr - 1:
                    dr += [q] * 3; dc += [idx(i, j, k - 1), q, idx(i, j, k + 1)]; dv += [1.0, -2.0, 1.0]
                if 0 < j < nvt - 1:
                    dr += [q] * 3; dc += [idx(i, j - 1, k), q, idx(i, j + 1, k)]; dv += [st, -2 * st, st]
                if 0 < i < nvp - 1:
                    dr += [q] * 3; dc += [idx(i - 1, j, k), q, idx(i + 1, j, k)]; dv += [spp, -2 * spp, spp]
                # D~^T row q (1-based tests of the reference)
                k1, j1, i1 = k + 1, j + 1, i + 1
                if k1 != 1 and k1 != nvr:
                    tr.append(q); tc.append(q); tv.append(-2.0)
                if k1 - 2 >= 1:
                    tr.append(q); tc.append(idx(i, j, k - 1)); tv.append(1.0)
                if k1 + 2 <= nvr:
                    tr.append(q); tc.append(idx(i, j, k + 1)); tv.append(1.0)
                if j1 != 1 and j1 != nvt:
                    tr.append(q); tc.append(q); tv.append(-2.0 * st)
                if j1 - 2 >= 1:
                    tr.append(q); tc.append(idx(i, j - 1, k)); tv.append(st)
                if j1 + 2 <= nvt:
                    tr.append(q); tc.append(idx(i, j + 1, k)); tv.append(st)
                if i1 != 1 and i1 != nvp:
                    tr.append(q); tc.append(q); tv.append(-2.0 * spp)
                if i1 - 2 >= 1:
                    tr.append(q); tc.append(idx(i - 1, j, k)); tv.append(spp)
                if i1 + 2 <= nvt and i + 1 < nvp:
                    tr.append(q); tc.append(idx(i + 1, j, k)); tv.append(spp)
    D = sp.csr_matrix((dv, (dr, dc)), shape=(n, n))
    Dt = sp.csr_matrix((tv, (tr, tc)), shape=(n, n))
    return D, Dt


def step(nv, vorig, vstep, params, nsrc, nrc, mo, cm_sd, mc, tstat, dobs, cd_sd, mtimes, rtimes,
         row_ptr, cols, vals):
    """Model perturbation dm (float64) and the subspace dimension used."""
    p = params
    nmpv = (nv[0] + 2) * (nv[1] + 2) * (nv[2] + 2)
    G, Gt, dmod, dob, cd, nmp = assemble(nsrc, nrc, nmpv, p.invst, p.rmtr, mc, tstat, dobs, cd_sd, mtimes,
                                         rtimes, row_ptr, cols, vals)
    mo_full = np.zeros(nmp)
    mo_full[:nmpv] = np.asarray(mo, dtype=np.float64)
    cm = np.ones(nmp)
    cm[:nmpv] = np.asarray(cm_sd, dtype=np.float64) ** 2
    mcv = np.asarray(mc, dtype=np.float64)[:nmp]
    epsv = np.full(nmp, float(p.epsilon))
    epsv[nmpv:] = float(p.stdf)
    gtw = lambda y: Gt @ (y / cd)             # noqa: E731  G^T Cd^-1 y (reference transpose)
    gamma = gtw(dmod - dob) + epsv * (mcv - mo_full) / cm
    if p.asds == 1:
        D, Dt = smoothing(nv, vorig[0], vorig[1], vstep[0], vstep[1], vstep[2], float(p.earth))
        dx = (mcv - mo_full)[:nmpv]
        gamma[:nmpv] += float(p.eta) * (Dt @ (D @ dx))
    classes = [(0, nmpv)] + ([(nmpv, nmp)] if p.invst == 1 else [])
    npc = len(classes)
    sd = int(p.subdim)
    A = np.zeros((nmp, sd))
    for c, (a0, a1) in enumerate(classes):
        A[a0:a1, c] = gamma[a0:a1] * cm[a0:a1]
        A[a0:a1, c] /= np.linalg.norm(A[a0:a1, c])
    if sd > npc:
        nits = is1 = is2 = npc
        done = False
        for _ in range(sd):
            for i in range(1, nits + 1):
                src = is2 - nits + i - 1
                ga = G @ A[:, src] / cd
                gt = Gt @ ga
                for jj, (a0, a1) in enumerate(classes):
                    is1 += 1
                    if is1 > sd:
                        break
                    A[a0:a1, is1 - 1] = gt[a0:a1] * cm[a0:a1] + epsv[a0:a1] * A[a0:a1, src]
                    A[a0:a1, is1 - 1] /= np.linalg.norm(A[a0:a1, is1 - 1])
                if is1 > sd:
                    done = True
                    break
            if done:
                break
            nits *= npc
            is2 += nits
    U, s, _ = np.linalg.svd(A, full_matrices=False)
    A = U[:, s >= 1e-7]
    HA = np.column_stack([Gt @ (G @ A[:, i] / cd) + epsv * A[:, i] / cm for i in range(A.shape[1])])
    if p.asds == 1:
        HA[:nmpv] += float(p.eta) * (Dt @ (D @ A[:nmpv]))
    M = A.T @ HA
    dm = -A @ (np.linalg.inv(M) @ (A.T @ gamma))
    return dm, A.shape[1]
