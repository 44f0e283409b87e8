// subinv.cpp -- the subspace inversion step of subinv.f90 ("S") on the host.
//
// Everything is templated on R, the type of the reference's REAL(KIND=i5)
// variables (float for FM3DT_SUBINV_FP32, double for FM3DT_SUBINV_FP64); the
// grid header stays double (REAL(KIND=i10)) and mixed expressions
// promote exactly where Fortran promotes them.  Sums run in the reference's
// order.  Compiled without floating-point contraction.
#include "../../include/fm3dt_subinv.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace {

constexpr float kPi = 3.1415926535898f;   // S:25, a REAL(4) parameter
constexpr int kMaxSubdim = 50;            // S:77 maxss
constexpr double kWtol = 1.0e-7;          // S:1029 singular values kept when >= wtol
constexpr float kTiny = 1.0e-20f;         // S:1342 pivot floor

struct Fail {
    int code;
    std::string msg;
};

// fn(i) for i in [0, n) on the host's cores.  Each i is computed whole by
// one thread, so results do not depend on the number of threads.
template <typename F>
void parallel_for(int n, F fn)
{
    const int nt = std::max(1, std::min((int)std::thread::hardware_concurrency(), std::min(32, n / 256)));
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) fn(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            const int a = (int)((int64_t)n * t / nt), b = (int)((int64_t)n * (t + 1) / nt);
            for (int i = a; i < b; ++i) fn(i);
        });
    for (auto &x : th) x.join();
}

// fn(t, a, b) on T contiguous chunks [a, b) of [0, n), one thread each.
template <typename F>
void parallel_chunks(int64_t n, int T, F fn)
{
    if (T <= 1) {
        fn(0, (int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] { fn(t, n * t / T, n * (t + 1) / T); });
    for (auto &x : th) x.join();
}

int host_threads(int64_t work, int64_t per_thread)
{
    const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
    return (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(hw, 32), work / per_thread));
}

// Allocator whose resize leaves new elements uninitialised: the entry
// arrays (tens of millions of entries) are written once, in parallel, so
// zero-filling them first would only add a serial pass over the memory.
template <typename T>
struct NoInit : std::allocator<T> {
    template <typename U> struct rebind { using other = NoInit<U>; };
    NoInit() = default;
    template <typename U> NoInit(const NoInit<U> &) {}
    template <typename U> void construct(U *p) { ::new ((void *)p) U; }
    template <typename U, typename... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};
template <typename T> using Big = std::vector<T, NoInit<T>>;

// Picked rows of G and their data plus the transpose.
template <typename R>
struct System {
    int ntr = 0, nmpv = 0, nmp = 0;
    std::vector<int64_t> cnfe{0};          // row starts, ntr+1
    Big<int32_t> fcoln;                    // 1-based model columns
    Big<R> frech;
    std::vector<R> dobs, dmod, cd;         // cd = variance
    std::vector<int64_t> tcnfe;            // column starts, nmp+1
    Big<int32_t> tfcoln;                   // 1-based rows
    Big<R> tfrech;
};

template <typename R>
System<R> assemble(const fm3dt_subinv_desc &d, int nra, const int *nsrc, const int *nrc, int nmpv, int nmp,
                   const std::vector<R> &mc, const int *tstat, const float *dobs, const float *cd_sd,
                   const float *mtimes, const float *rtimes, const int64_t *row_ptr, const int32_t *cols,
                   const float *vals, int ntr_all)
{
    System<R> S;
    S.nmpv = nmpv;
    S.nmp = nmp;
    // source and receiver of every pair
    std::vector<int> idst(ntr_all), idrt(ntr_all);
    int nsum = 0, nmps = 0, q = 0;
    for (int a = 0; a < nra; ++a) {
        for (int j = 0; j < nsrc[a]; ++j)
            for (int k = 0; k < nrc[a]; ++k, ++q) {
                idst[q] = j + 1 + nsum;
                idrt[q] = k + 1 + nmps;
            }
        nsum += nsrc[a];
        nmps += nrc[a];
    }
    // maxf = fracg*ntr*nmp in REAL(4), truncated
    const int64_t maxf = (int64_t)(float)((float)(d.fracg * (float)ntr_all) * (float)nmp);
    std::vector<R> srcm, ntsrc_sum;
    std::vector<int> ntsrc;
    if (d.rmtr == 1) {
        srcm.assign(nsum, R(0));
        ntsrc.assign(nsum, 0);
    }
    // pass 1, in row order: the reference's size check (its running entry
    // count), each picked row's place, the data columns
    std::vector<int> pick;                 // picked rows, in order
    pick.reserve(ntr_all);
    S.cnfe.reserve((size_t)ntr_all + 1);
    int64_t jstep = 0;
    for (int i = 0; i < ntr_all; ++i) {
        R dm_i = (R)mtimes[i];
        const R dref = (R)rtimes[i];
        int64_t nrow = row_ptr[i + 1] - row_ptr[i];
        if (d.invst == 1) {
            dm_i = dm_i + mc[nmpv + idrt[i] - 1];
            nrow += 1;
        }
        if (nrow > 0) {
            if (jstep + nrow > maxf)
                throw Fail{FM3DT_SUBINV_ETOOBIG, "Frechet matrix too large for last input\nparameter in file "
                                                 "subinv.in\nSTOPPING PROGRAM!!!"};
            if (tstat[i] == 1) jstep += nrow;
        }
        if (tstat[i] == 1) {
            const R c = (R)cd_sd[i];
            S.dobs.push_back((R)dobs[i]);
            S.cd.push_back(c * c);
            dm_i = dm_i - dref;
            S.dmod.push_back(dm_i);
            S.cnfe.push_back(jstep);
            pick.push_back(i);
            if (d.rmtr == 1) {
                const int iscn = idst[i] - 1;
                srcm[iscn] = srcm[iscn] + dm_i;
                ntsrc[iscn] += 1;
            }
        }
    }
    // pass 2, rows in parallel: entries (and the station-term entry)
    S.fcoln.resize((size_t)jstep);
    S.frech.resize((size_t)jstep);
    {
        const int np = (int)pick.size();
        std::vector<int> bad(32, 0);
        const int T = host_threads(jstep, 1 << 20);
        parallel_chunks(np, T, [&](int t, int64_t a, int64_t b) {
            for (int64_t r = a; r < b; ++r) {
                const int i = pick[r];
                int64_t o = S.cnfe[r];
                for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k, ++o) {
                    const int32_t c = cols[k];
                    if (c < 1 || c > nmp) bad[t] = bad[t] ? bad[t] : c;
                    S.fcoln[o] = c;
                    S.frech[o] = (R)vals[k];
                }
                if (d.invst == 1) {
                    S.fcoln[o] = nmpv + idrt[i];
                    S.frech[o] = R(1);
                }
            }
        });
        for (int t = 0; t < 32; ++t)
            if (bad[t])
                throw Fail{FM3DT_SUBINV_EINVAL, "Frechet column " + std::to_string(bad[t]) + " outside 1.." +
                                                    std::to_string(nmp)};
    }
    S.ntr = (int)S.dobs.size();
    if (d.rmtr == 1) {
        // each source's picks are contiguous, in source order
        int64_t is = 0;
        for (int s = 0; s < nsum; ++s) {
            const R mean = srcm[s] / (R)ntsrc[s];
            for (int j = 0; j < ntsrc[s]; ++j, ++is) S.dmod[is] = S.dmod[is] - mean;
        }
    }
    // Transpose.  The reference walks columns i = 1..nmp and, in
    // each row, takes the next pending entry when its column equals i; so it
    // keeps each row's leading strictly increasing run of columns (all of a
    // sorted row) and drops the rest.  Entries within a column are by row.
    // Counting sort by column in parallel: each thread counts and then fills
    // a contiguous range of rows, after the earlier ranges' entries of every
    // column, so each column lists its rows in order whatever the threads.
    std::vector<int64_t> take(S.ntr);
    const int T = host_threads((int64_t)S.fcoln.size(), 1 << 20);
    std::vector<std::vector<int64_t>> cnt(T, std::vector<int64_t>(nmp, 0));
    parallel_chunks(S.ntr, T, [&](int t, int64_t a, int64_t b) {
        for (int64_t j = a; j < b; ++j) {
            int64_t k = S.cnfe[j];
            while (k < S.cnfe[j + 1] && (k == S.cnfe[j] || S.fcoln[k] > S.fcoln[k - 1])) ++k;
            take[j] = k;
            for (int64_t q = S.cnfe[j]; q < k; ++q) cnt[t][S.fcoln[q] - 1] += 1;
        }
    });
    S.tcnfe.assign(nmp + 1, 0);
    for (int i = 0; i < nmp; ++i) {
        int64_t c = 0;
        for (int t = 0; t < T; ++t) c += cnt[t][i];
        S.tcnfe[i + 1] = S.tcnfe[i] + c;
    }
    // thread t starts each column after the threads before it
    for (int i = 0; i < nmp; ++i) {
        int64_t o = S.tcnfe[i];
        for (int t = 0; t < T; ++t) {
            const int64_t c = cnt[t][i];
            cnt[t][i] = o;
            o += c;
        }
    }
    S.tfcoln.resize(S.tcnfe[nmp]);
    S.tfrech.resize(S.tcnfe[nmp]);
    parallel_chunks(S.ntr, T, [&](int t, int64_t a, int64_t b) {
        std::vector<int64_t> &fill = cnt[t];
        for (int64_t j = a; j < b; ++j)
            for (int64_t k = S.cnfe[j]; k < take[j]; ++k) {
                const int64_t p = fill[S.fcoln[k] - 1]++;
                S.tfcoln[p] = (int32_t)(j + 1);
                S.tfrech[p] = S.frech[k];
            }
    });
    return S;
}

// y = G x / cd over the picked rows (the ga of S:764-773)
template <typename R>
void g_times(const System<R> &S, const R *x, std::vector<R> &ga)
{
    ga.resize(S.ntr);
    parallel_for(S.ntr, [&](int j) {
        R rsum = 0;
        for (int64_t k = S.cnfe[j]; k < S.cnfe[j + 1]; ++k) rsum = rsum + S.frech[k] * x[S.fcoln[k] - 1];
        ga[j] = rsum / S.cd[j];
    });
}

// (G^T y)_i over the transpose
template <typename R>
R gt_row(const System<R> &S, int i, const std::vector<R> &y)
{
    R rsum = 0;
    for (int64_t k = S.tcnfe[i]; k < S.tcnfe[i + 1]; ++k) rsum = rsum + S.tfrech[k] * y[S.tfcoln[k] - 1];
    return rsum;
}

// (G^T y)_i for every model parameter i, in parallel
template <typename R>
void gt_times(const System<R> &S, const std::vector<R> &y, std::vector<R> &out)
{
    out.resize(S.nmp);
    parallel_for(S.nmp, [&](int i) { out[i] = gt_row(S, i, y); });
}

}  // namespace

namespace {

// Second-derivative smoothing on the padded velocity grid (S:616-703 and
// S:888-942).  dem = D x with x's second differences along r, theta and phi
// scaled by dnr^2/(r dtheta)^2 and dnr^2/(r sin(theta) dphi)^2; ddem_at(q)
// = (D^T dem)_q.  Scale factors are evaluated as the reference does: the
// REAL(4) difference times the REAL(8) dnr**2, over the REAL(4) square.
template <typename R>
struct Smoother {
    int nvr, nvt, nvp;        // padded counts
    double dnr2;
    std::vector<R> thet, rad; // per theta row, per r layer
    R rdnt, rdnp;

    Smoother(const fm3dt_subinv_desc &d)
    {
        nvr = d.nvr + 2;
        nvt = d.nvt + 2;
        nvp = d.nvp + 2;
        rdnt = (R)(d.dnt * (double)kPi / 180.0);
        rdnp = (R)(d.dnp * (double)kPi / 180.0);
        const R rgot = (R)((90.0 - d.got) * (double)kPi / 180.0);
        dnr2 = d.dnr * d.dnr;
        thet.resize(nvt);
        for (int j = 0; j < nvt; ++j) thet[j] = std::sin((R)(rgot + (R)j * rdnt));
        rad.resize(nvr);
        for (int k = 0; k < nvr; ++k) rad[k] = (R)(d.gor - (double)k * d.dnr + (double)d.earth);
    }
    size_t at(int i, int j, int k) const { return ((size_t)i * nvt + j) * nvr + k; }
    R sq_t(int j, int k) const { const R v = rad[k] * rdnt; (void)j; return v * v; }
    R sq_p(int j, int k) const { const R v = rad[k] * thet[j] * rdnp; return v * v; }
    // acc + v * dnr**2 / den, promoted to double like the reference
    R add_scaled(R acc, R v, R den) const { return (R)((double)acc + ((double)v * dnr2) / (double)den); }
    R sub_scaled(R acc, R v, R den) const { return (R)((double)acc - ((double)v * dnr2) / (double)den); }

    // dem from second differences given by diff(is1, is2, is3)
    template <typename Diff>
    void dem_of(std::vector<R> &dem, Diff diff) const
    {
        dem.assign((size_t)nvr * nvt * nvp, R(0));
        for (int i = 0; i < nvp; ++i)
            for (int j = 0; j < nvt; ++j)
                for (int k = 0; k < nvr; ++k) {
                    const size_t is2 = at(i, j, k);
                    if (k != 0 && k != nvr - 1) dem[is2] = dem[is2] + diff(at(i, j, k - 1), is2, at(i, j, k + 1));
                    if (j != 0 && j != nvt - 1)
                        dem[is2] = add_scaled(dem[is2], diff(at(i, j - 1, k), is2, at(i, j + 1, k)), sq_t(j, k));
                    if (i != 0 && i != nvp - 1)
                        dem[is2] = add_scaled(dem[is2], diff(at(i - 1, j, k), is2, at(i + 1, j, k)), sq_p(j, k));
                }
    }
    // (D^T dem) at node (i, j, k).  The phi neighbour i+1 is taken when
    // i+2 <= nvt (1-based), the theta count, as the reference has it
    // (S:698); a neighbour that falls outside the grid reads 0.
    R ddem_at(const std::vector<R> &dem, int i, int j, int k) const
    {
        const size_t is2 = at(i, j, k);
        const int i1 = i + 1, j1 = j + 1, k1 = k + 1;   // 1-based, as in the reference's tests
        R ddem = 0;
        if (k1 != 1 && k1 != nvr) ddem = ddem - R(2) * dem[is2];
        if (k1 - 2 >= 1) ddem = ddem + dem[at(i, j, k - 1)];
        if (k1 + 2 <= nvr) ddem = ddem + dem[at(i, j, k + 1)];
        if (j1 != 1 && j1 != nvt) ddem = sub_scaled(ddem, R(2) * dem[is2], sq_t(j, k));
        if (j1 - 2 >= 1) ddem = add_scaled(ddem, dem[at(i, j - 1, k)], sq_t(j, k));
        if (j1 + 2 <= nvt) ddem = add_scaled(ddem, dem[at(i, j + 1, k)], sq_t(j, k));
        if (i1 != 1 && i1 != nvp) ddem = sub_scaled(ddem, R(2) * dem[is2], sq_p(j, k));
        if (i1 - 2 >= 1) ddem = add_scaled(ddem, dem[at(i - 1, j, k)], sq_p(j, k));
        if (i1 + 2 <= nvt) ddem = add_scaled(ddem, i + 1 < nvp ? dem[at(i + 1, j, k)] : R(0), sq_p(j, k));
        return ddem;
    }
};

// Orthonormal basis of the columns of a (m x n, column-major) with the
// directions whose singular value is below wtol removed (the role of svdcmp,
// S:1013-1276).  One-sided Jacobi rotations orthogonalise the columns; their
// norms are then the singular values and the normalised columns an
// orthonormal basis of the same span.  The subspace step only depends on the
// span, so the basis may differ from the reference's by a rotation.
template <typename R>
int orthonormalise(std::vector<R> &a, int m, int n)
{
    const R tol = sizeof(R) == 4 ? R(1e-6) : R(1e-14);
    auto col = [&](int c) { return a.data() + (size_t)c * m; };
    bool conv = false;
    for (int sweep = 0; sweep < 60 && !conv; ++sweep) {
        conv = true;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                R *x = col(p), *y = col(q);
                double al = 0, be = 0, ga = 0;
                for (int i = 0; i < m; ++i) {
                    al += (double)x[i] * x[i];
                    be += (double)y[i] * y[i];
                    ga += (double)x[i] * y[i];
                }
                // a column far below the cut is dropped anyway; rotating it
                // against rounding noise would never settle
                const double floor2 = 1e-4 * kWtol * kWtol;
                if (al < floor2 || be < floor2) continue;
                if (ga == 0.0 || std::fabs(ga) <= (double)tol * std::sqrt(al * be)) continue;
                conv = false;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < m; ++i) {
                    const double xi = x[i], yi = y[i];
                    x[i] = (R)(c * xi - s * yi);
                    y[i] = (R)(s * xi + c * yi);
                }
            }
    }
    if (!conv) throw Fail{FM3DT_SUBINV_ENOCONV, "No convergence in svdcmp!\nCheck the integrity of your\n"
                                                "input files!!!!!!!!\nTerminating program subinv!"};
    int keep = 0;
    for (int c = 0; c < n; ++c) {
        double nrm = 0;
        for (int i = 0; i < m; ++i) nrm += (double)col(c)[i] * col(c)[i];
        nrm = std::sqrt(nrm);
        if (nrm < kWtol) continue;
        R *dst = col(keep), *src = col(c);
        for (int i = 0; i < m; ++i) dst[i] = (R)(src[i] / nrm);
        ++keep;
    }
    return keep;
}

// Inverse of the n x n column-major matrix by Gaussian elimination with
// scaled partial pivoting (the role of luinv/ludcmp/lubksb).
template <typename R>
void invert(std::vector<R> &m, int n)
{
    std::vector<R> lu(m), inv((size_t)n * n, R(0));
    auto L = [&](int r, int c) -> R & { return lu[(size_t)c * n + r]; };
    std::vector<R> scale(n);
    std::vector<int> perm(n);
    for (int r = 0; r < n; ++r) {
        R big = 0;
        for (int c = 0; c < n; ++c) big = std::max(big, (R)std::fabs(L(r, c)));
        if (big == R(0)) throw Fail{FM3DT_SUBINV_ESINGULAR, "Singular matrix. Try C.G. method"};
        scale[r] = R(1) / big;
        perm[r] = r;
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        R best = -1;
        for (int r = c; r < n; ++r) {
            const R v = scale[r] * (R)std::fabs(L(r, c));
            if (v > best) { best = v; piv = r; }
        }
        if (piv != c) {
            for (int k = 0; k < n; ++k) std::swap(L(piv, k), L(c, k));
            std::swap(scale[piv], scale[c]);
            std::swap(perm[piv], perm[c]);
        }
        if (L(c, c) == R(0)) L(c, c) = (R)kTiny;
        for (int r = c + 1; r < n; ++r) {
            const R f = L(r, c) / L(c, c);
            L(r, c) = f;
            for (int k = c + 1; k < n; ++k) L(r, k) = L(r, k) - f * L(c, k);
        }
    }
    std::vector<R> b(n);
    for (int col = 0; col < n; ++col) {
        for (int r = 0; r < n; ++r) b[r] = perm[r] == col ? R(1) : R(0);
        for (int r = 0; r < n; ++r)
            for (int k = 0; k < r; ++k) b[r] = b[r] - L(r, k) * b[k];
        for (int r = n - 1; r >= 0; --r) {
            for (int k = r + 1; k < n; ++k) b[r] = b[r] - L(r, k) * b[k];
            b[r] = b[r] / L(r, r);
        }
        for (int r = 0; r < n; ++r) inv[(size_t)col * n + r] = b[r];
    }
    m.swap(inv);
}

}  // namespace

namespace {

// The subspace step: dm = -A (A^T H A)^-1 A^T gamma with
// H = G^T Cd^-1 G + epsilon Cm^-1 (+ eta D^T D) and A an orthonormal basis
// of the gradient's Krylov-like sequence.
template <typename R>
void subspace(const fm3dt_subinv_desc &d, const System<R> &S, const std::vector<R> &mo, const std::vector<R> &mc,
              const std::vector<R> &cm, std::vector<double> &dm_out, int &subdim, std::string &note)
{
    const int nmp = S.nmp, nmpv = S.nmpv, ntr = S.ntr;
    const R eps = (R)d.epsilon, eta = (R)d.eta, stdf = (R)d.stdf;
    std::vector<R> dtrav(ntr);
    for (int i = 0; i < ntr; ++i) dtrav[i] = (S.dmod[i] - S.dobs[i]) / S.cd[i];
    // gradient
    std::vector<R> gamma(nmp), gtv;
    gt_times(S, dtrav, gtv);
    R epst = eps;
    for (int i = 0; i < nmp; ++i) {
        const R rsum = gtv[i];
        if (i >= nmpv) epst = stdf;
        gamma[i] = rsum + (epst * (mc[i] - mo[i])) / cm[i];
    }
    Smoother<R> sm(d);
    std::vector<R> dem;
    if (d.asds == 1) {
        sm.dem_of(dem, [&](size_t a, size_t b, size_t c) {
            R r = mc[a] - R(2) * mc[b] + mc[c];
            return r - mo[a] + R(2) * mo[b] - mo[c];
        });
        for (int i = 0; i < sm.nvp; ++i)
            for (int j = 0; j < sm.nvt; ++j)
                for (int k = 0; k < sm.nvr; ++k) {
                    const size_t q = sm.at(i, j, k);
                    gamma[q] = gamma[q] + eta * sm.ddem_at(dem, i, j, k);
                }
    }
    // parameter classes: velocity, then station terms
    const int npc = d.invst == 1 ? 2 : 1;
    const int inds[2] = {0, nmpv}, inde[2] = {nmpv, nmp};
    std::vector<R> a((size_t)nmp * subdim, R(0));
    auto A = [&](int j, int c) -> R & { return a[(size_t)c * nmp + j]; };   // c 0-based column
    auto normalise = [&](int c, int cls) {
        R rsum = 0;
        for (int j = inds[cls]; j < inde[cls]; ++j) rsum = rsum + A(j, c) * A(j, c);
        const R nrm = std::sqrt(rsum);
        if (!(nrm > R(0))) throw Fail{FM3DT_SUBINV_EINVAL, "zero subspace vector (zero gradient)"};
        for (int j = inds[cls]; j < inde[cls]; ++j) A(j, c) = A(j, c) / nrm;
    };
    for (int c = 0; c < npc; ++c)
        for (int j = inds[c]; j < inde[c]; ++j) A(j, c) = gamma[j] * cm[j];
    for (int c = 0; c < npc; ++c) normalise(c, c);
    // remaining vectors, indices as the reference counts them
    std::vector<R> ga;
    if (subdim > npc) {
        int nits = npc, is1 = npc, is2 = npc;
        bool done = false;
        for (int ii = 1; ii <= subdim && !done; ++ii) {
            for (int i = 1; i <= nits && !done; ++i) {
                const int src = is2 - nits + i - 1;      // 0-based source column
                g_times(S, &A(0, src), ga);
                gt_times(S, ga, gtv);
                for (int jj = 0; jj < npc; ++jj) {
                    is1 += 1;
                    if (is1 > subdim) break;
                    const int dst = is1 - 1;
                    for (int j = inds[jj]; j < inde[jj]; ++j) {
                        const R rsum = gtv[j];
                        A(j, dst) = rsum * cm[j] + (j < nmpv ? eps : stdf) * A(j, src);
                    }
                    normalise(dst, jj);
                }
                if (is1 > subdim) done = true;
            }
            if (done) break;
            nits *= npc;
            is2 += nits;
        }
    }
    // orthonormal basis and rank reduction
    const int keep = orthonormalise(a, nmp, subdim);
    if (keep < subdim) {
        note += "Due to redundancy, the subspace dimension\nis being reduced from " + std::to_string(subdim) +
                " to " + std::to_string(keep) + "\nMessage from SVD orthogonalization algorithm\n";
        subdim = keep;
    }
    if (subdim < 1) throw Fail{FM3DT_SUBINV_ESINGULAR, "subspace has no direction left"};
    // projected matrix
    std::vector<R> mati((size_t)subdim * subdim, R(0));
    auto M = [&](int r, int c) -> R & { return mati[(size_t)c * subdim + r]; };
    for (int ii = 0; ii < subdim; ++ii) {
        g_times(S, &A(0, ii), ga);
        gt_times(S, ga, gtv);
        if (d.asds != 1) {
            R ep = eps;
            for (int j = 0; j < nmp; ++j) {
                R rsum = gtv[j];
                if (j >= nmpv) ep = stdf;
                rsum = rsum + (ep * A(j, ii)) / cm[j];
                for (int k = 0; k < subdim; ++k) M(k, ii) = M(k, ii) + rsum * A(j, k);
            }
        } else {
            sm.dem_of(dem, [&](size_t p, size_t q, size_t r) { return A((int)p, ii) - R(2) * A((int)q, ii) + A((int)r, ii); });
            for (int i = 0; i < sm.nvp; ++i)
                for (int j = 0; j < sm.nvt; ++j)
                    for (int k = 0; k < sm.nvr; ++k) {
                        const int q = (int)sm.at(i, j, k);
                        R rsum = gtv[q];
                        const R dd = sm.ddem_at(dem, i, j, k);
                        rsum = rsum + (eps * A(q, ii)) / cm[q] + eta * dd;
                        for (int l = 0; l < subdim; ++l) M(l, ii) = M(l, ii) + rsum * A(q, l);
                    }
            if (d.invst == 1)
                for (int j = nmpv; j < nmp; ++j) {
                    R rsum = gtv[j];
                    rsum = rsum + (stdf * A(j, ii)) / cm[j];
                    for (int k = 0; k < subdim; ++k) M(k, ii) = M(k, ii) + rsum * A(j, k);
                }
        }
    }
    invert(mati, subdim);
    // model perturbation
    std::vector<R> r1(subdim, R(0)), r2(subdim, R(0));
    for (int i = 0; i < subdim; ++i)
        for (int j = 0; j < nmp; ++j) r1[i] = r1[i] + A(j, i) * gamma[j];
    for (int i = 0; i < subdim; ++i)
        for (int j = 0; j < subdim; ++j) r2[i] = r2[i] + M(i, j) * r1[j];
    dm_out.assign(nmp, 0.0);
    for (int i = 0; i < nmp; ++i) {
        R s = 0;
        for (int j = 0; j < subdim; ++j) s = s + A(i, j) * r2[j];
        dm_out[i] = (double)(-s);
    }
}

template <typename R>
int step(const fm3dt_subinv_desc *d, int nra, const int *nsrc, const int *nrc, const float *mo_f,
         const float *cm_sd, const float *mc_f, const int *tstat, const float *dobs, const float *cd_sd,
         const float *mtimes, const float *rtimes, const int64_t *row_ptr, const int32_t *cols,
         const float *vals, double *dm, int *subdim_used, std::string &note)
{
    const int nmpv = (d->nvr + 2) * (d->nvt + 2) * (d->nvp + 2);
    int ntr = 0, nmps = 0;
    for (int a = 0; a < nra; ++a) {
        if (nsrc[a] < 0 || nrc[a] < 0) throw Fail{FM3DT_SUBINV_EINVAL, "negative source or receiver count"};
        ntr += nsrc[a] * nrc[a];
        nmps += nrc[a];
    }
    const int nmp = nmpv + (d->invst == 1 ? nmps : 0);
    std::vector<R> mo(nmp), mc(nmp), cm(nmp);
    // cm = sd**2; station terms start at mo = 0, cm = 1
    for (int i = 0; i < nmpv; ++i) {
        mo[i] = (R)mo_f[i];
        const R c = (R)cm_sd[i];
        cm[i] = c * c;
    }
    for (int i = nmpv; i < nmp; ++i) {
        mo[i] = R(0);
        cm[i] = R(1);
    }
    for (int i = 0; i < nmp; ++i) mc[i] = (R)mc_f[i];
    System<R> S = assemble<R>(*d, nra, nsrc, nrc, nmpv, nmp, mc, tstat, dobs, cd_sd, mtimes, rtimes, row_ptr, cols,
                              vals, ntr);
    int subdim = d->subdim;
    std::vector<double> out;
    subspace<R>(*d, S, mo, mc, cm, out, subdim, note);
    std::copy(out.begin(), out.end(), dm);
    if (subdim_used) *subdim_used = subdim;
    return FM3DT_SUBINV_OK;
}

void put(char *msg, int len, const std::string &s)
{
    if (!msg || len <= 0) return;
    const size_t n = std::min((size_t)len - 1, s.size());
    std::memcpy(msg, s.data(), n);
    msg[n] = '\0';
}

}  // namespace

extern "C" int fm3dt_subinv_step(const fm3dt_subinv_desc *d, int nra, const int *nsrc, const int *nrc,
                                 const float *mo, const float *cm_sd, const float *mc, const int *tstat,
                                 const float *dobs, const float *cd_sd, const float *mtimes, const float *rtimes,
                                 const int64_t *row_ptr, const int32_t *cols, const float *vals, double *dm,
                                 int *subdim_used, char *msg, int msg_len)
{
    std::string note;
    put(msg, msg_len, "");
    if (!d || nra < 0 || (nra > 0 && (!nsrc || !nrc)) || !mo || !cm_sd || !mc || !dm || !row_ptr) {
        put(msg, msg_len, "null or invalid argument");
        return FM3DT_SUBINV_EINVAL;
    }
    if (d->nvr < 1 || d->nvt < 1 || d->nvp < 1) {
        put(msg, msg_len, "bad velocity grid dimensions");
        return FM3DT_SUBINV_EINVAL;
    }
    if (d->subdim < 1) {
        put(msg, msg_len, "Subspace dimension cannot be less than one!!!\nTerminating program!!!");
        return FM3DT_SUBINV_EINVAL;
    }
    if (d->subdim == 1 && d->invst == 1) {
        put(msg, msg_len, "ERROR!!!!!!\nCannot have a subspace dimension of 1\nand invert for velocity AND station "
                          "terms.\nSet subspace dimension to value greater than 1.\nTERMINATING PROGRAM!!!!!");
        return FM3DT_SUBINV_EINVAL;
    }
    if (d->subdim > kMaxSubdim)
        note += "Subspace dimension is larger than " + std::to_string(kMaxSubdim) + "\n";
    try {
        const int rc = d->precision == FM3DT_SUBINV_FP64
                           ? step<double>(d, nra, nsrc, nrc, mo, cm_sd, mc, tstat, dobs, cd_sd, mtimes, rtimes,
                                          row_ptr, cols, vals, dm, subdim_used, note)
                           : step<float>(d, nra, nsrc, nrc, mo, cm_sd, mc, tstat, dobs, cd_sd, mtimes, rtimes,
                                         row_ptr, cols, vals, dm, subdim_used, note);
        put(msg, msg_len, note);
        return rc;
    } catch (const Fail &f) {
        put(msg, msg_len, note + f.msg);
        return f.code;
    } catch (const std::bad_alloc &) {
        put(msg, msg_len, "out of host memory");
        return FM3DT_SUBINV_EINVAL;
    }
}
