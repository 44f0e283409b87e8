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

template <typename R> FM_HD R fm_min(R a, R b) { return b < a ? b : a; }

// One upwind term in "first-order form": ((T - tau)/g)^2 with
// tau = t1, g = h (first order) or tau = (4*t1 - t2)/3, g = 2h/3 (second).
// Stored as tau relative to the octant's earliest neighbour (e), the
// neighbour value t1 used for the causality test, and 1/g^2 (w).
template <typename R> struct Term {
    R t1;   // neighbour value used for the upwind test
    R e;    // tau - reference time
    R w;    // 1/g^2
    R g;    // g
};

// solve sum_{i<n} ((x - e_i)^2 * w_i) = s2 for the larger root x
template <typename R>
FM_HD R solve_terms(const Term<R>* t, int n, R s, R s2)
{
    if (n == 1) return t[0].e + s * t[0].g;
    R a = R(0), b = R(0), c = -s2;
    for (int i = 0; i < n; ++i) {
        a += t[i].w;
        b += t[i].w * t[i].e;
        c += t[i].w * t[i].e * t[i].e;
    }
    // a x^2 - 2 b x + c = 0
    R disc = b * b - a * c;
    if (disc < R(0)) disc = R(0);
    return (b + fm_sqrt<R>(disc)) / a;
}

// Neighbour directions: 0 = r-1 (up), 1 = r+1 (down), 2 = x-1, 3 = x+1,
// 4 = z-1, 5 = z+1.
//
// t1[d]: neighbour value (+inf if unset; ignored when bit d of inb is clear)
// t2[d]: second neighbour value (+inf if unset or outside the grid)
// h[a]:  grid spacing of axis a (r, x, z) at the centre node, km
// s:     slowness at the centre node
// order2: 1 for the mixed-order scheme (fom=1), 0 for first order (fom=0)
// Returns the candidate time (+inf when no neighbour is set).
template <typename R>
FM_HD R fm_update(R s, const R t1[6], const R t2[6], unsigned inb, const R h[3], int order2)
{
    const R INF = Lim<R>::inf();
    R tmin = INF;
#pragma unroll
    for (int d = 0; d < 6; ++d)
        if ((inb >> d) & 1u) tmin = fm_min(tmin, t1[d]);
    if (!(tmin < INF)) return INF;
    const R s2 = s * s;
    // per-direction terms relative to tmin
    Term<R> dir[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        const R hh = h[d >> 1];
        const bool o2 = order2 && (t2[d] < t1[d]);
        dir[d].t1 = ((inb >> d) & 1u) ? t1[d] : INF;
        if (o2) {
            dir[d].e = (t1[d] - tmin) + (t1[d] - t2[d]) / R(3);
            dir[d].g = hh * R(2) / R(3);
        } else {
            dir[d].e = t1[d] - tmin;
            dir[d].g = hh;
        }
        dir[d].w = R(1) / (dir[d].g * dir[d].g);
    }
    R best = INF;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        const int dr = (o >> 2) & 1, dx = 2 + ((o >> 1) & 1), dz = 4 + (o & 1);
        const bool inside = ((inb >> dr) & 1u) && ((inb >> dx) & 1u) && ((inb >> dz) & 1u);
        if (!inside) continue;
        Term<R> t[3] = {dir[dr], dir[dx], dir[dz]};
        // ascending t1 (unset neighbours sort last)
        if (t[1].t1 < t[0].t1) { Term<R> q = t[0]; t[0] = t[1]; t[1] = q; }
        if (t[2].t1 < t[1].t1) { Term<R> q = t[1]; t[1] = t[2]; t[2] = q; }
        if (t[1].t1 < t[0].t1) { Term<R> q = t[0]; t[0] = t[1]; t[1] = q; }
        if (!(t[0].t1 < INF)) continue;
        R x = solve_terms<R>(t, 1, s, s2);
        if (t[1].t1 - tmin < x) {
            x = solve_terms<R>(t, 2, s, s2);
            if (t[2].t1 - tmin < x) x = solve_terms<R>(t, 3, s, s2);
        }
        best = fm_min(best, x);
    }
    return tmin + best;
}

}  // namespace fm3dt
