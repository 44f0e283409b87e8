// stencil.cuh -- the upwind eikonal node update shared by every solver kernel.
//
// Restates the octant update of fm3dt_parallel.f90 fouds2_all (F:635-1004,
// mixed order) and fouds1_all (F:535-633, first order) in a generic form.
// For each of the eight octants (one direction per axis r, theta, phi) whose
// three neighbours all lie inside the grid (F:710-712), the axes whose
// neighbour is upwind contribute one term of
//     sum_a ((k_a*T - beta_a) / H_a)^2 = s^2,
// with k=1, beta=t1, H=h for a first-order axis and k=3, beta=4*t1-t2, H=2h
// for a second-order axis (F:712-982 enumerate the same cases by hand).  The
// quadratic keeps the reference's root choice and its clamp of a negative
// discriminant to zero (F:991-993); the node takes the minimum over octants
// (F:995-1000).  An axis is second order when its second neighbour is inside
// the grid, upwind and earlier than the first (F:645-707).
//
// Upwind set.  In the reference's fast marching a neighbour is used when it is
// alive, i.e. already final and earlier than the node being computed.  A
// block-parallel iterative solver has no heap order, so "alive" is restated
// as the fixed-point condition t1 < T: each octant adds its neighbours in
// ascending order of t1 and keeps the largest set whose solution T exceeds
// every used t1 (the causal Godunov solve).  At convergence the used set is
// exactly the set of neighbours earlier than the node, which is the set the
// reference's heap has popped when it computes the node.
//
// "Unset" is +infinity here (the reference uses 0.0, which an offset time can
// legitimately equal).  The unknown is solved relative to the earliest used
// neighbour, so every coefficient is a difference of nearby times; this keeps
// single-precision offset times accurate.
#pragma once

#ifndef FM_HD
#ifdef __CUDACC__
#define FM_HD __host__ __device__ __forceinline__
#else
#define FM_HD inline
#endif
#endif

namespace fm3dt {

template <typename R> struct Lim;
template <> struct Lim<double> {
    static FM_HD double inf() { return __builtin_huge_val(); }
};
template <> struct Lim<float> {
    static FM_HD float inf() { return __builtin_huge_valf(); }
};

template <typename R> FM_HD R fm_sqrt(R x);
template <> FM_HD double fm_sqrt<double>(double x) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(x);
#else
    return __builtin_sqrt(x);
#endif
}
template <> FM_HD float fm_sqrt<float>(float x) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}

// Minimum and maximum as the hardware min/max instructions.  They differ from
// a compare-and-select only for NaN and for a +0/-0 pair; in-grid times are
// never NaN and never -0 (offsets from an event's earliest time start at +0,
// and sums of non-negative terms stay +0 or above), so the results are the
// same bits.
template <typename R> FM_HD R fm_min(R a, R b);
template <typename R> FM_HD R fm_max(R a, R b);
#ifdef __CUDA_ARCH__
template <> FM_HD float fm_min<float>(float a, float b) { return fminf(a, b); }
template <> FM_HD double fm_min<double>(double a, double b) { return fmin(a, b); }
template <> FM_HD float fm_max<float>(float a, float b) { return fmaxf(a, b); }
template <> FM_HD double fm_max<double>(double a, double b) { return fmax(a, b); }
#else
template <> FM_HD float fm_min<float>(float a, float b) { return __builtin_fminf(a, b); }
template <> FM_HD double fm_min<double>(double a, double b) { return __builtin_fmin(a, b); }
template <> FM_HD float fm_max<float>(float a, float b) { return __builtin_fmaxf(a, b); }
template <> FM_HD double fm_max<double>(double a, double b) { return __builtin_fmax(a, b); }
#endif

// The two keys of a conditional swap, in order (p: the second is smaller).
// Single precision takes min and max, which do not wait for the comparison;
// double precision keeps the selects, which run on the integer pipe rather
// than the narrow double-precision one.
template <typename R> FM_HD void fm_order_keys(bool p, R &ki, R &kj);
template <> FM_HD void fm_order_keys<float>(bool, float &ki, float &kj)
{
    const float lo = fm_min<float>(ki, kj);
    kj = fm_max<float>(ki, kj);
    ki = lo;
}
template <> FM_HD void fm_order_keys<double>(bool p, double &ki, double &kj)
{
    const double lo = p ? kj : ki;
    kj = p ? ki : kj;
    ki = lo;
}

// Explicit fused multiply-add.  The solver is compiled without automatic
// contraction, so every kernel instantiation (and the host) evaluates the
// stencil with exactly the same roundings; otherwise the compiler may fuse
// differently per instantiation and the iteration map -- hence its fixed
// point -- would differ in the last bits between tile shapes.
template <typename R> FM_HD R fm_fma(R a, R b, R c);
template <> FM_HD double fm_fma<double>(double a, double b, double c) { return __builtin_fma(a, b, c); }
template <> FM_HD float fm_fma<float>(float a, float b, float c) { return __builtin_fmaf(a, b, c); }

// Square root and quotient of the quadratic's root.  Single precision on the
// device uses the hardware approximations (deterministic, <= 2 ulp on a
// time increment of order 0.1-1 s, far below the float spacing of the
// offset times themselves); double precision is IEEE-rounded.
template <typename R> struct Fast;
template <> struct Fast<double> {
    static FM_HD double sqrt(double x) { return fm_sqrt<double>(x); }
    static FM_HD double div(double a, double b) { return a / b; }
};
template <> struct Fast<float> {
    static FM_HD float sqrt(float x) {
#ifdef __CUDA_ARCH__
        float r;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
#else
        return __builtin_sqrtf(x);
#endif
    }
    static FM_HD float div(float a, float b) {
#ifdef __CUDA_ARCH__
        return __fdividef(a, b);
#else
        return a / b;
#endif
    }
};

// Per-node grid spacings: h[a] and 1/h[a]^2 for axes r, theta, phi.
template <typename R> struct Spacing {
    R h[3];
    R w[3];
};

// Neighbour directions: 0 = r-1 (up), 1 = r+1 (down), 2 = x-1, 3 = x+1,
// 4 = z-1, 5 = z+1.
//
// t1[d]: neighbour value (+inf if unset; +inf or NaN when bit d of inb is
//        clear, i.e. outside the grid)
// t2[d]: second neighbour value (+inf if unset; +inf or NaN outside the grid)
// sp:    spacings at the centre node
// s:     slowness at the centre node
// order2: 1 for the mixed-order scheme (fom=1), 0 for first order (fom=0)
// Returns the candidate time (+inf when no neighbour is set).
//
// Each direction is written in first-order form ((T - tau)/g)^2 with
// tau = t1, g = h (first order) or tau = t1 + (t1 - t2)/3, g = 2h/3 (second
// order, the same equation as the reference's (3T - 4 t1 + t2)/(2h) term),
// relative to tmin, the earliest in-grid neighbour.  Every octant sorts its
// three terms by t1 and adds them while t1 < T (the causal solve).
template <typename R>
FM_HD R fm_update(R s, const R t1[6], const R t2[6], unsigned inb, const Spacing<R> &sp, int order2)
{
    const R INF = Lim<R>::inf();
    // (a neighbour outside the grid holds +inf or NaN, which the hardware
    // minimum passes over: no mask needed)
    R tmin = INF;
#pragma unroll
    for (int d = 0; d < 6; ++d) tmin = fm_min(tmin, t1[d]);
    if (!(tmin < INF)) return INF;
    const R s2 = s * s;
    R key[6], e[6], g[6], w[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        const int a = d >> 1;
        const bool o2 = order2 && (t2[d] < t1[d]);
        const R dt = t1[d] - tmin;
        // (an octant is evaluated only when its three neighbours are in the
        // grid, so an outside direction's key is never read)
        key[d] = dt;
        e[d] = o2 ? fm_fma<R>(t1[d] - t2[d], R(1.0 / 3.0), dt) : dt;
        g[d] = o2 ? sp.h[a] * R(2.0 / 3.0) : sp.h[a];
        w[d] = o2 ? sp.w[a] * R(2.25) : sp.w[a];
    }
    R best = INF;
    // Each octant sorts its three terms by key, stably (ties keep the order
    // r, theta, phi).  The lateral pair is sorted once and shared by the two
    // octants that differ only in the radial direction, and the radial term
    // is then inserted in front: two compare-and-swaps per octant instead of
    // three, and the same order as a full three-term network (a stable sort's
    // result is unique).  Both octants of a pair are sorted before either
    // solves, so that their sorts form one straight run of code.  An octant
    // with a neighbour outside the grid is evaluated all the same (from
    // whatever its keys hold) and left out of the minimum by a select rather
    // than branched around.  The minimum over octants does not depend on the
    // order they are visited in.
    // conditional swaps as selects (a branch around four moves costs more)
#define FM_CSWAP(i, j)                                                        \
    {                                                                         \
        const bool p_ = k##j < k##i;                                          \
        fm_order_keys<R>(p_, k##i, k##j);                                     \
        R q_ = p_ ? e##j : e##i; e##j = p_ ? e##i : e##j; e##i = q_;          \
        q_ = p_ ? g##j : g##i; g##j = p_ ? g##i : g##j; g##i = q_;            \
        q_ = p_ ? w##j : w##i; w##j = p_ ? w##i : w##j; w##i = q_;            \
    }
    // the causal two- and three-term solves of a sorted octant, from its
    // one-term solution x
    auto solve = [&](R k1, R k2, R e0, R e1, R e2, R w0, R w1, R w2, R x) -> R {
        if (k1 < x) {
            R a = w0 + w1;
            const R we0 = w0 * e0, we1 = w1 * e1;
            R b = we0 + we1;
            R c = fm_fma<R>(we0, e0, fm_fma<R>(we1, e1, -s2));
            R disc = fm_fma<R>(b, b, -(a * c));
            x = Fast<R>::div(b + Fast<R>::sqrt(fm_max<R>(disc, R(0))), a);
            if (k2 < x) {
                const R we2 = w2 * e2;
                a += w2;
                b += we2;
                c = fm_fma<R>(we2, e2, c);
                disc = fm_fma<R>(b, b, -(a * c));
                x = Fast<R>::div(b + Fast<R>::sqrt(fm_max<R>(disc, R(0))), a);
            }
        }
        return x;
    };
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int dx = 2 + ((q >> 1) & 1), dz = 4 + (q & 1);
        R ka = key[dx], ea = e[dx], ga = g[dx], wa = w[dx];
        R kb = key[dz], eb = e[dz], gb = g[dz], wb = w[dz];
        FM_CSWAP(a, b)
        // terms 0-2: the octant with the upper (r-1) neighbour; 3-5: the
        // lower (r+1) one; om*: the neighbours each needs inside the grid
        const unsigned omu = 1u | (1u << dx) | (1u << dz), omd = 2u | (1u << dx) | (1u << dz);
        R k0 = key[0], e0 = e[0], g0 = g[0], w0 = w[0];
        R k1 = ka, e1 = ea, g1 = ga, w1 = wa;
        R k2 = kb, e2 = eb, g2 = gb, w2 = wb;
        R k3 = key[1], e3 = e[1], g3 = g[1], w3 = w[1];
        R k4 = ka, e4 = ea, g4 = ga, w4 = wa;
        R k5 = kb, e5 = eb, g5 = gb, w5 = wb;
        FM_CSWAP(0, 1)
        FM_CSWAP(3, 4)
        FM_CSWAP(1, 2)
        FM_CSWAP(4, 5)
        // (an octant with no neighbour set has e0 = +inf: its x = +inf leaves
        // best as it is, and no further term passes k < x)
        const R xu = fm_fma<R>(s, g0, e0), xd = fm_fma<R>(s, g3, e3);
        const R vu = solve(k1, k2, e0, e1, e2, w0, w1, w2, xu);
        best = (inb & omu) == omu ? fm_min(best, vu) : best;
        const R vd = solve(k4, k5, e3, e4, e5, w3, w4, w5, xd);
        best = (inb & omd) == omd ? fm_min(best, vd) : best;
    }
#undef FM_CSWAP
    return tmin + best;
}

// The node update of a sweep from an unset field, where every neighbour
// downstream of the sweep (up, r-1, and the lateral directions the sweep runs
// toward) is still unset when the node is computed.  Then only the three
// upstream neighbours -- down (r+1) and the lateral ones the sweep comes
// from, here D, X and Z -- can enter an octant, and each of the eight octants
// is the causal solve of the upstream terms it contains: the octant that
// takes the upstream side on the axes of a subset S of {D, X, Z} and the
// downstream side on the others solves S (its downstream terms are +inf,
// sort last and never pass k < x).  So this returns fm_update's value, bit
// for bit, with +inf at the downstream neighbours: the same keys, the same
// stable order within each subset (key, then axis r, theta, phi), the same
// arithmetic, and an octant counted when its three neighbours lie inside the
// grid.  It evaluates the seven subsets with four quadratic solves instead of
// the eight octants' sixteen: the singletons are one FMA each, the three pairs
// one solve each, and the triple's first two terms are one of the pairs (the
// same order and the same operations, hence the same bits), so only its
// three-term solve is added.
//
// tD/tD2, tX/tX2, tZ/tZ2: upstream first and second neighbour values;
// in*: whether each upstream (u) and downstream (d) neighbour lies inside the
// grid (inD: r+1, inU: r-1).
template <typename R>
FM_HD R fm_update_upstream(R s, R tD, R tD2, R tX, R tX2, R tZ, R tZ2, bool inD, bool inU, bool inXu, bool inXd,
                           bool inZu, bool inZd, const Spacing<R> &sp, int order2)
{
    const R INF = Lim<R>::inf();
    const R tmin = fm_min(fm_min(tD, tX), tZ);
    if (!(tmin < INF)) return INF;
    const R s2 = s * s;
    R k[3], e[3], w[3], x1[3];
    {
        const R t1[3] = {tD, tX, tZ}, t2[3] = {tD2, tX2, tZ2};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const bool o2 = order2 && (t2[a] < t1[a]);
            const R dt = t1[a] - tmin;
            k[a] = dt;
            e[a] = o2 ? fm_fma<R>(t1[a] - t2[a], R(1.0 / 3.0), dt) : dt;
            const R g = o2 ? sp.h[a] * R(2.0 / 3.0) : sp.h[a];
            w[a] = o2 ? sp.w[a] * R(2.25) : sp.w[a];
            x1[a] = fm_fma<R>(s, g, e[a]);        // the one-term solution
        }
    }
    // causal solve of the pair (i, j), i before j in axis order, sorted
    // stably; the two-term step exactly as fm_update's
    auto pair = [&](int i, int j) -> R {
        const bool p = k[j] < k[i];
        const R ks = p ? k[i] : k[j];
        const R ef = p ? e[j] : e[i], es = p ? e[i] : e[j];
        const R wf = p ? w[j] : w[i], ws = p ? w[i] : w[j];
        R x = p ? x1[j] : x1[i];
        if (ks < x) {
            const R a = wf + ws;
            const R wef = wf * ef, wes = ws * es;
            const R b = wef + wes;
            const R c = fm_fma<R>(wef, ef, fm_fma<R>(wes, es, -s2));
            const R disc = fm_fma<R>(b, b, -(a * c));
            x = Fast<R>::div(b + Fast<R>::sqrt(fm_max<R>(disc, R(0))), a);
        }
        return x;
    };
    const R pDX = pair(0, 1), pDZ = pair(0, 2), pXZ = pair(1, 2);
    // the triple, sorted stably by the same comparisons as fm_update's
    // network (the lateral pair first, then D inserted in front); selects,
    // not indexed arrays, so that everything stays in registers.  A/B: the
    // lateral pair in order; F/M/L: first, middle and last of the triple;
    // i*: which term (0 D, 1 X, 2 Z)
    const bool pxz = k[2] < k[1];
    const R kA = pxz ? k[2] : k[1], eA = pxz ? e[2] : e[1], wA = pxz ? w[2] : w[1], xA = pxz ? x1[2] : x1[1];
    const R kB = pxz ? k[1] : k[2], eB = pxz ? e[1] : e[2], wB = pxz ? w[1] : w[2];
    const int iA = pxz ? 2 : 1, iB = pxz ? 1 : 2;
    const bool p1 = kA < k[0];
    const R kF = p1 ? kA : k[0], eF = p1 ? eA : e[0], wF = p1 ? wA : w[0], xF = p1 ? xA : x1[0];
    const R kM0 = p1 ? k[0] : kA, eM0 = p1 ? e[0] : eA, wM0 = p1 ? w[0] : wA;
    const int iM0 = p1 ? 0 : iA;
    const bool p2 = kB < kM0;
    const R kM = p2 ? kB : kM0, eM = p2 ? eB : eM0, wM = p2 ? wB : wM0;
    const R kL = p2 ? kM0 : kB, eL = p2 ? eM0 : eB, wL = p2 ? wM0 : wB;
    const int iL = p2 ? iM0 : iB;
    (void)kF;
    // its first two terms are the pair without L (the same order and the
    // same operations as that pair's solve)
    R xt = iL == 2 ? pDX : (iL == 1 ? pDZ : pXZ);
    if (kM < xF && kL < xt) {
        const R a = (wF + wM) + wL;
        const R wef = wF * eF, wem = wM * eM, wel = wL * eL;
        const R b = (wef + wem) + wel;
        const R c = fm_fma<R>(wel, eL, fm_fma<R>(wef, eF, fm_fma<R>(wem, eM, -s2)));
        const R disc = fm_fma<R>(b, b, -(a * c));
        xt = Fast<R>::div(b + Fast<R>::sqrt(fm_max<R>(disc, R(0))), a);
    }
    // subsets whose octant lies inside the grid (upstream side on the axes in
    // the subset, downstream side on the others)
    const bool rD = inD, rN = inU, xU = inXu, xN = inXd, zU = inZu, zN = inZd;
    R best = INF;
    best = (rD && xN && zN) ? fm_min(best, x1[0]) : best;
    best = (rN && xU && zN) ? fm_min(best, x1[1]) : best;
    best = (rN && xN && zU) ? fm_min(best, x1[2]) : best;
    best = (rD && xU && zN) ? fm_min(best, pDX) : best;
    best = (rD && xN && zU) ? fm_min(best, pDZ) : best;
    best = (rN && xU && zU) ? fm_min(best, pXZ) : best;
    best = (rD && xU && zU) ? fm_min(best, xt) : best;
    return tmin + best;
}

}  // namespace fm3dt
