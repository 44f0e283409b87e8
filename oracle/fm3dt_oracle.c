/*
 * fm3dt_oracle.c -- CPU oracle (test infrastructure only) for the forward
 * teleseismic traveltime path of fm3dt_parallel.f90 ("F" below).
 *
 * Parity status: UNPINNED by reference outputs (no Fortran/MPI toolchain, no
 * reference tests or golden vectors, itimes.out missing).  Pinned by analytic
 * known-answer tests instead.  See fm3dt_oracle.h for units and layouts.
 *
 * Every routine restates the serial behaviour of the cited Fortran lines with
 * the reference's operation order (left-to-right, no fused multiply-add), so
 * that double-precision results follow the reference's rounding.  Build with
 * -ffp-contract=off.  The serial routines take the offsets of a single
 * subdomain (roffset = xoffset = zoffset = 1: the (offset-1)*spacing terms are
 * exactly 0.0); orc_fmm_decomposed runs the reference's block split with each
 * block's own offsets, in the reference's operation order.
 */
#include "fm3dt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* F:61 declares pi as REAL(KIND=i10) but initialises it from the default-kind
 * (single precision) literal 3.1415926535898, so the value the reference uses
 * is that literal rounded to float and widened. */
double orc_pi(void) { return (double)3.1415926535898f; }

void orc_grid_from_header(const int nv[3], const double vorig[3], const double vstep[3],
                          const int nn[3], const double norig[3], const double nstep[3],
                          double earth, orc_grid *g)
{
    const double pi = orc_pi();
    g->nvr = nv[0]; g->nvx = nv[1]; g->nvz = nv[2];
    g->gor = vorig[0];
    g->dvr = vstep[0];
    /* F:6110-6117 */
    g->dvx = vstep[1] * pi / 180.0;
    g->dvz = vstep[2] * pi / 180.0;
    g->gox = (90.0 - vorig[1]) * pi / 180.0;
    g->goz = vorig[2] * pi / 180.0;
    g->nnr = nn[0]; g->nnx = nn[1]; g->nnz = nn[2];
    g->rgor = norig[0];
    g->dnr = nstep[0];
    g->dnx = nstep[1] * pi / 180.0;
    g->dnz = nstep[2] * pi / 180.0;
    g->rgox = (90.0 - norig[1]) * pi / 180.0;
    g->rgoz = norig[2] * pi / 180.0;
    g->earth = earth;
}

void orc_latlon_to_rad(int n, const double *lat, const double *lon, double *colat, double *lonr)
{
    const double pi = orc_pi();
    for (int i = 0; i < n; ++i) {
        colat[i] = (90.0 - lat[i]) * pi / 180.0;   /* F:6313 */
        lonr[i] = lon[i] * pi / 180.0;             /* F:6314 */
    }
}

/* ------------------------------------------------------------------------ */
/* B-spline weights (F:7002-7005 and repeated at F:7010-7021, 7671-7682)     */
/* ------------------------------------------------------------------------ */
static void bspline4(double u, double w[4])
{
    const double u2 = u * u, u3 = u * u * u;
    const double om = 1.0 - u;
    w[0] = om * om * om / 6.0;
    w[1] = (4.0 - 6.0 * u2 + 3.0 * u3) / 6.0;
    w[2] = (1.0 + 3.0 * u + 3.0 * u2 - 3.0 * u3) / 6.0;
    w[3] = u3 / 6.0;
}

#define VELV(g, k, j, i) ((size_t)(k) + (size_t)((g)->nvr + 2) * ((size_t)(j) + (size_t)((g)->nvx + 2) * (size_t)(i)))
#define VELN(g, iz, ix, ir) ((size_t)((iz) + 1) + (size_t)((g)->nnz + 3) * ((size_t)((ix) + 1) + (size_t)((g)->nnx + 3) * (size_t)((ir) + 1)))

static int clampi(int v, int lo, int hi, int *hit)
{
    if (v < lo) { *hit = 1; return lo; }
    if (v > hi) { *hit = 1; return hi; }
    return v;
}

/* The gridder of one (sub)domain of rnum x xnum x znum nodes whose first
 * node is global node (roff, xoff, zoff) (F:6989-7038, offsets in the
 * reference's operation order); veln has (znum+3)(xnum+3)(rnum+3) values,
 * indices -1..n+1. */
static int gridder_block(const orc_grid *g, const double *velv, int roff, int xoff, int zoff, int rnum, int xnum,
                         int znum, double *veln, int *nclamped)
{
    int nclamp = 0;
    const size_t VZ3 = (size_t)znum + 3, VX3 = (size_t)xnum + 3;
    for (int i = -1; i <= znum + 1; ++i) {
        /* F:6996-6998 */
        const double zpos = g->rgoz + (double)(zoff - 1) * g->dnz + (double)(i - 1) * g->dnz - g->goz;
        const int zi = (int)floor(zpos / g->dvz) + 1;
        const double distz = zpos - (double)(zi - 1) * g->dvz;
        double wi[4];
        bspline4(distz / g->dvz, wi);
        for (int j = -1; j <= xnum + 1; ++j) {
            const double xpos = g->rgox + (double)(xoff - 1) * g->dnx + (double)(j - 1) * g->dnx - g->gox;
            const int xi = (int)floor(xpos / g->dvx) + 1;
            const double distx = xpos - (double)(xi - 1) * g->dvx;
            double vi[4];
            bspline4(distx / g->dvx, vi);
            for (int k = -1; k <= rnum + 1; ++k) {
                /* F:7015-7016: ri from depth below the velocity origin */
                const int ri = (int)floor((g->gor - g->rgor + (double)(roff - 1) * g->dnr + (double)(k - 1) * g->dnr) /
                                          g->dvr) + 1;
                const double distr = -(g->rgor - (double)(roff - 1) * g->dnr - (double)(k - 1) * g->dnr) +
                                     (g->gor - (double)(ri - 1) * g->dvr);
                double ui[4];
                bspline4(distr / g->dvr, ui);
                double sumi = 0.0;
                for (int i1 = 1; i1 <= 4; ++i1) {
                    double sumj = 0.0;
                    for (int j1 = 1; j1 <= 4; ++j1) {
                        double sumk = 0.0;
                        for (int k1 = 1; k1 <= 4; ++k1) {
                            int hit = 0;
                            const int a = clampi(ri - 2 + k1, 0, g->nvr + 1, &hit);
                            const int b = clampi(xi - 2 + j1, 0, g->nvx + 1, &hit);
                            const int c = clampi(zi - 2 + i1, 0, g->nvz + 1, &hit);
                            nclamp += hit;
                            sumk = sumk + ui[k1 - 1] * velv[VELV(g, a, b, c)];
                        }
                        sumj = sumj + vi[j1 - 1] * sumk;
                    }
                    sumi = sumi + wi[i1 - 1] * sumj;
                }
                veln[(size_t)(i + 1) + VZ3 * ((size_t)(j + 1) + VX3 * (size_t)(k + 1))] = sumi;
            }
        }
    }
    if (nclamped) *nclamped = nclamp;
    return nclamp ? -1 : 0;
}

int orc_gridder(const orc_grid *g, const double *velv, double *veln, int *nclamped)
{
    return gridder_block(g, velv, 1, 1, 1, g->nnr, g->nnx, g->nnz, veln, nclamped);
}

/* ------------------------------------------------------------------------ */
/* Serial fast marching (F:78-155, 535-1098, 6894-6961)                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    const orc_grid *g;
    const double *veln;    /* gridded velocity, indices -1..n+1 of this (sub)domain */
    int VZ3, VX3;          /* its strides: nnz+3, nnx+3 */
    int roff, xoff, zoff;  /* global index of the (sub)domain's first node (F:6159-6168); 1 serially */
    int nnr, nnx, nnz;
    int NZ2, NX2;          /* padded strides: indices 0..n+1 like F:6191 */
    double *ttn;           /* padded (nnz+2)(nnx+2)(nnr+2) */
    int *nsts;             /* padded, same shape */
    int *hr, *hx, *hz;     /* heap btg (F:68-75), 1-based */
    int ntr;
} fmm_state;

#define TI(s, iz, ix, ir) ((size_t)(iz) + (size_t)(s)->NZ2 * ((size_t)(ix) + (size_t)(s)->NX2 * (size_t)(ir)))
#define SV(s, iz, ix, ir) ((s)->veln[(size_t)((iz) + 1) + (size_t)(s)->VZ3 * ((size_t)((ix) + 1) + (size_t)(s)->VX3 * (size_t)((ir) + 1))])

/* The whole grid as one domain (the serial run: offsets 1). */
static void state_serial(fmm_state *s, const orc_grid *g, const double *veln)
{
    memset(s, 0, sizeof *s);
    s->g = g;
    s->veln = veln;
    s->VZ3 = g->nnz + 3;
    s->VX3 = g->nnx + 3;
    s->roff = s->xoff = s->zoff = 1;
    s->nnr = g->nnr; s->nnx = g->nnx; s->nnz = g->nnz;
    s->NZ2 = g->nnz + 2; s->NX2 = g->nnx + 2;
}
#define TT(s, iz, ix, ir) ((s)->ttn[TI(s, iz, ix, ir)])
#define NS(s, iz, ix, ir) ((s)->nsts[TI(s, iz, ix, ir)])

static double sq(double x) { return x * x; }

/* node radius and r*sin(colatitude) at the centre node (F:542-543, 642-643),
 * with the subdomain offsets in the reference's operation order (they add
 * exact zeros in the serial run) */
static void centre_geom(const fmm_state *s, int ix, int ir, double *ri, double *risti)
{
    const orc_grid *g = s->g;
    *ri = g->rgor - (double)(s->roff - 1) * g->dnr - (double)(ir - 1) * g->dnr + g->earth;
    *risti = *ri * sin(g->rgox + (double)(s->xoff - 1) * g->dnx + (double)(ix - 1) * g->dnx);
}

/* fouds1_all: first-order update over the eight octants (F:535-633). */
static void fouds1(fmm_state *s, int iz, int ix, int ir)
{
    const orc_grid *g = s->g;
    const double dnr = g->dnr, dnx = g->dnx, dnz = g->dnz;
    double ri, risti;
    centre_geom(s, ix, ir, &ri, &risti);
    const double slown = 1.0 / SV(s, iz, ix, ir);
    int tsw1 = 0;
    double travm = 0.0;
    for (int i = ir - 1; i <= ir + 1; i += 2)
        for (int j = ix - 1; j <= ix + 1; j += 2)
            for (int k = iz - 1; k <= iz + 1; k += 2) {
                if (i < 1 || i > s->nnr || j < 1 || j > s->nnx || k < 1 || k > s->nnz) continue;
                int swsol = 0;
                double a = 0, b = 0, c = 0, tref = 0;
                if (NS(s, iz, ix, i) == 0) {
                    swsol = 1;
                    if (NS(s, iz, j, ir) == 0 && NS(s, k, ix, ir) == 0) {
                        const double u = dnr, v = ri * dnx, w = risti * dnz;
                        const double em = TT(s, iz, j, ir) - TT(s, iz, ix, i);
                        const double en = TT(s, k, ix, ir) - TT(s, iz, ix, i);
                        const double rd1 = sq(v) * sq(w), rd2 = sq(u) * sq(w), rd3 = sq(u) * sq(v);
                        a = rd1 + rd2 + rd3;
                        b = -2.0 * (em * rd2 + en * rd3);
                        c = sq(em) * rd2 + sq(en) * rd3 - sq(slown) * sq(u) * rd1;
                        tref = TT(s, iz, ix, i);
                    } else if (NS(s, iz, j, ir) == 0) {
                        const double u = dnr, v = ri * dnx;
                        const double em = TT(s, iz, j, ir) - TT(s, iz, ix, i);
                        a = sq(u) + sq(v);
                        b = -2.0 * sq(u) * em;
                        c = sq(u) * (sq(em) - sq(v) * sq(slown));
                        tref = TT(s, iz, ix, i);
                    } else if (NS(s, k, ix, ir) == 0) {
                        const double u = dnr, v = risti * dnz;
                        const double em = TT(s, k, ix, ir) - TT(s, iz, ix, i);
                        a = sq(u) + sq(v);
                        b = -2.0 * sq(u) * em;
                        c = sq(u) * (sq(em) - sq(v) * sq(slown));
                        tref = TT(s, iz, ix, i);
                    } else {
                        a = 1.0; b = 0.0;
                        c = -sq(slown) * sq(dnr);
                        tref = TT(s, iz, ix, i);
                    }
                } else if (NS(s, iz, j, ir) == 0) {
                    swsol = 1;
                    if (NS(s, k, ix, ir) == 0) {
                        const double u = ri * dnx, v = risti * dnz;
                        const double em = TT(s, k, ix, ir) - TT(s, iz, j, ir);
                        a = sq(u) + sq(v);
                        b = -2.0 * sq(u) * em;
                        c = sq(u) * (sq(em) - sq(v) * sq(slown));
                        tref = TT(s, iz, j, ir);
                    } else {
                        a = 1.0; b = 0.0;
                        c = -sq(slown) * sq(ri) * sq(dnx);
                        tref = TT(s, iz, j, ir);
                    }
                } else if (NS(s, k, ix, ir) == 0) {
                    swsol = 1;
                    a = 1.0; b = 0.0;
                    c = -sq(slown * risti * dnz);
                    tref = TT(s, k, ix, ir);
                }
                if (swsol) {
                    double rd1 = sq(b) - 4.0 * a * c;
                    if (rd1 < 0.0) rd1 = 0.0;
                    const double tdsh = (-b + sqrt(rd1)) / (2.0 * a);
                    const double trav = tref + tdsh;
                    if (tsw1) travm = fmin(trav, travm);
                    else { travm = trav; tsw1 = 1; }
                }
            }
    if (TT(s, iz, ix, ir) == 0.0 || TT(s, iz, ix, ir) > travm) TT(s, iz, ix, ir) = travm;
}

/* Upwind switch of one axis direction for fouds2_all (F:645-707): 0 when the
 * second-order one-sided difference applies, -1 otherwise. */
static int sw2(const fmm_state *s, int nb_alive, int nb2_in, int nb2_alive, double tnb, double tnb2)
{
    int sw = -1;
    if (nb2_in && nb2_alive) sw = 0;
    if (nb_alive && sw == 0) {
        sw = -1;
        if (tnb > tnb2) sw = 0;
    } else {
        sw = -1;
    }
    (void)s;
    return sw;
}

/* One octant of fouds2_all (F:710-993): the reference's branch table for
 * the given upwind flags (ai/aj/ak: neighbour used; swi/swj/swk == 0: that
 * axis second order).  Returns 1 and the octant time in *trav when some
 * axis is used. */
/* (ti/ti2, tj/tj2, tk/tk2: the first and second neighbour values of the
 * octant along r, theta and phi; the second ones are read only on branches
 * whose switch proved them in range) */
static int octant2v(const orc_grid *g, double ti, double ti2, double tj, double tj2, double tk, double tk2,
                    int ai, int aj, int ak, int swi, int swj, int swk, double ri, double risti, double slown,
                    double *trav)
{
    const double dnr = g->dnr, dnx = g->dnx, dnz = g->dnz;
        int swsol = 0;
        double a = 0, b = 0, c = 0, u, v, w, em, en, tref = 0, tdiv = 1.0;
        /* neighbour values; second neighbours are only read on the
         * branches whose switch proved them in range */
#define TIv ti
#define TI2 ti2
#define TJv tj
#define TJ2 tj2
#define TKv tk
#define TK2 tk2
        if (swi == 0) {
            swsol = 1;
            if (swj == 0) {
                if (swk == 0) {
                    u = 2.0 * dnr; v = 2.0 * ri * dnx; w = 2.0 * risti * dnz;
                    em = 4.0 * TIv - TI2 - 4.0 * TJv; em = em + TJ2;
                    en = 4.0 * TIv - TI2 - 4.0 * TKv; en = en + TK2;
                    a = sq(v) * sq(w) + sq(u) * sq(w) + sq(u) * sq(v);
                    b = 2.0 * sq(u) * (em * sq(w) + en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(v) * sq(w) * sq(slown));
                    tref = 4.0 * TIv - TI2; tdiv = 3.0;
                } else if (ak) {
                    u = risti * dnz; v = 2.0 * ri * dnx; w = 2.0 * dnr;
                    em = 3.0 * TKv - 4.0 * TJv + TJ2;
                    en = 3.0 * TKv - 4.0 * TIv + TI2;
                    a = sq(v) * sq(w) + 9.0 * sq(u) * sq(w) + 9.0 * sq(u) * sq(v);
                    b = 6.0 * sq(u) * (em * sq(w) + en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(slown) * sq(v) * sq(w));
                    tref = TKv; tdiv = 1.0;
                } else {
                    u = 2.0 * dnr; v = 2.0 * ri * dnx;
                    em = 4.0 * TIv - TI2 - 4.0 * TJv; em = em + TJ2;
                    a = sq(v) + sq(u);
                    b = 2.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(slown) * sq(v));
                    tref = 4.0 * TIv - TI2; tdiv = 3.0;
                }
            } else if (aj) {
                if (swk == 0) {
                    u = ri * dnx; v = 2.0 * dnr; w = 2.0 * risti * dnz;
                    em = 3.0 * TJv - 4.0 * TIv + TI2;
                    en = 3.0 * TJv - 4.0 * TKv + TK2;
                    a = sq(v) * sq(w) + 9.0 * sq(u) * sq(w) + 9.0 * sq(u) * sq(v);
                    b = 6.0 * sq(u) * (em * sq(w) + en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(slown) * sq(v) * sq(w));
                    tref = TJv; tdiv = 1.0;
                } else if (ak) {
                    u = ri * dnx; v = 2.0 * dnr; w = risti * dnz;
                    em = 3.0 * TJv - 4.0 * TIv + TI2;
                    en = TJv - TKv;
                    a = sq(w) * sq(v) + 9.0 * sq(u) * sq(w) + sq(u) * sq(v);
                    b = sq(u) * (6.0 * em * sq(w) + 2.0 * en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(slown) * sq(v) * sq(w));
                    tref = TJv; tdiv = 1.0;
                } else {
                    u = ri * dnx; v = 2.0 * dnr;
                    em = 3.0 * TJv - 4.0 * TIv + TI2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(slown) * sq(v));
                    tref = TJv; tdiv = 1.0;
                }
            } else {
                if (swk == 0) {
                    u = 2.0 * dnr; v = 2.0 * risti * dnz;
                    em = 4.0 * TIv - TI2 - 4.0 * TKv; em = em + TK2;
                    a = sq(u) + sq(v);
                    b = 2.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = 4.0 * TIv - TI2; tdiv = 3.0;
                } else if (ak) {
                    u = risti * dnz; v = 2.0 * dnr;
                    em = 3.0 * TKv - 4.0 * TIv + TI2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TKv; tdiv = 1.0;
                } else {
                    u = 2.0 * dnr;
                    a = 1.0; b = 0.0;
                    c = -sq(u) * sq(slown);
                    tref = 4.0 * TIv - TI2; tdiv = 3.0;
                }
            }
        } else if (ai) {
            swsol = 1;
            if (swj == 0) {
                if (swk == 0) {
                    u = dnr; v = 2.0 * ri * dnx; w = 2.0 * risti * dnz;
                    em = 3.0 * TIv - 4.0 * TJv + TJ2;
                    en = 3.0 * TIv - 4.0 * TKv + TK2;
                    a = sq(v) * sq(w) + 9.0 * sq(u) * sq(w) + 9.0 * sq(u) * sq(v);
                    b = 6.0 * sq(u) * (em * sq(w) + en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(slown) * sq(v) * sq(w));
                    tref = TIv; tdiv = 1.0;
                } else if (ak) {
                    u = dnr; v = 2.0 * ri * dnx; w = risti * dnz;
                    em = 3.0 * TIv - 4.0 * TJv + TJ2;
                    en = TIv - TKv;
                    a = sq(v) * sq(w) + 9.0 * sq(u) * sq(w) + sq(u) * sq(v);
                    b = sq(u) * (6.0 * em * sq(w) + 2.0 * en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(v) * sq(w) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                } else {
                    u = dnr; v = 2.0 * ri * dnx;
                    em = 3.0 * TIv - 4.0 * TJv + TJ2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                }
            } else if (aj) {
                if (swk == 0) {
                    u = dnr; v = ri * dnx; w = 2.0 * risti * dnz;
                    em = TIv - TJv;
                    en = 3.0 * TIv - 4.0 * TKv + TK2;
                    a = sq(v) * sq(w) + sq(u) * sq(w) + 9.0 * sq(u) * sq(v);
                    b = sq(u) * (2.0 * em * sq(w) + 6.0 * en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(v) * sq(w) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                } else if (ak) {
                    u = dnr; v = ri * dnx; w = risti * dnz;
                    em = TJv - TIv;
                    en = TKv - TIv;
                    a = sq(v) * sq(w) + sq(u) * sq(w) + sq(u) * sq(v);
                    b = -2.0 * sq(u) * (em * sq(w) + en * sq(v));
                    c = sq(u) * (sq(em) * sq(w) + sq(en) * sq(v) - sq(slown) * sq(v) * sq(w));
                    tref = TIv; tdiv = 1.0;
                } else {
                    u = dnr; v = ri * dnx;
                    em = TJv - TIv;
                    a = sq(u) + sq(v);
                    b = -2.0 * sq(u) * em;
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                }
            } else {
                if (swk == 0) {
                    u = dnr; v = 2.0 * risti * dnz;
                    em = 3.0 * TIv - 4.0 * TKv + TK2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                } else if (ak) {
                    u = dnr; v = risti * dnz;
                    em = TKv - TIv;
                    a = sq(u) + sq(v);
                    b = -2.0 * sq(u) * em;
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TIv; tdiv = 1.0;
                } else {
                    a = 1.0; b = 0.0;
                    c = -sq(slown) * sq(dnr);
                    tref = TIv; tdiv = 1.0;
                }
            }
        } else {
            if (swj == 0) {
                swsol = 1;
                if (swk == 0) {
                    u = 2.0 * ri * dnx; v = 2.0 * risti * dnz;
                    em = 4.0 * TJv - TJ2 - 4.0 * TKv; em = em + TK2;
                    a = sq(v) + sq(u);
                    b = 2.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(slown) * sq(v));
                    tref = 4.0 * TJv - TJ2; tdiv = 3.0;
                } else if (ak) {
                    u = risti * dnz; v = 2.0 * ri * dnx;
                    em = 3.0 * TKv - 4.0 * TJv + TJ2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(slown) * sq(v));
                    tref = TKv; tdiv = 1.0;
                } else {
                    u = 2.0 * ri * dnx;
                    a = 1.0; b = 0.0;
                    c = -sq(u) * sq(slown);
                    tref = 4.0 * TJv - TJ2; tdiv = 3.0;
                }
            } else if (aj) {
                swsol = 1;
                if (swk == 0) {
                    u = ri * dnx; v = 2.0 * risti * dnz;
                    em = 3.0 * TJv - 4.0 * TKv + TK2;
                    a = sq(v) + 9.0 * sq(u);
                    b = 6.0 * em * sq(u);
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TJv; tdiv = 1.0;
                } else if (ak) {
                    u = ri * dnx; v = risti * dnz;
                    em = TKv - TJv;
                    a = sq(u) + sq(v);
                    b = -2.0 * sq(u) * em;
                    c = sq(u) * (sq(em) - sq(v) * sq(slown));
                    tref = TJv; tdiv = 1.0;
                } else {
                    a = 1.0; b = 0.0;
                    c = -sq(slown) * sq(ri) * sq(dnx);
                    tref = TJv; tdiv = 1.0;
                }
            } else {
                if (swk == 0) {
                    swsol = 1;
                    u = 2.0 * risti * dnz;
                    a = 1.0; b = 0.0;
                    c = -sq(u) * sq(slown);
                    tref = 4.0 * TKv - TK2; tdiv = 3.0;
                } else if (ak) {
                    swsol = 1;
                    a = 1.0; b = 0.0;
                    c = -sq(slown) * sq(risti) * sq(dnz);
                    tref = TKv; tdiv = 1.0;
                }
            }
        }
#undef TIv
#undef TI2
#undef TJv
#undef TJ2
#undef TKv
#undef TK2
        if (swsol) {
        double rd1 = sq(b) - 4.0 * a * c;
        if (rd1 < 0.0) rd1 = 0.0;
        const double tdsh = (-b + sqrt(rd1)) / (2.0 * a);
        *trav = (tref + tdsh) / tdiv;
    }
    return swsol;
}

/* One octant of fouds2_all from the (sub)domain's own field (F:710-993). */
static int octant2(const fmm_state *s, int iz, int ix, int ir, int i, int j, int k, int i2, int j2, int k2,
                   int ai, int aj, int ak, int swi, int swj, int swk, double ri, double risti, double slown,
                   double *trav)
{
    const int i2in = i2 >= 1 && i2 <= s->nnr, j2in = j2 >= 1 && j2 <= s->nnx, k2in = k2 >= 1 && k2 <= s->nnz;
    return octant2v(s->g, TT(s, iz, ix, i), i2in ? TT(s, iz, ix, i2) : 0.0, TT(s, iz, j, ir),
                    j2in ? TT(s, iz, j2, ir) : 0.0, TT(s, k, ix, ir), k2in ? TT(s, k2, ix, ir) : 0.0, ai, aj, ak,
                    swi, swj, swk, ri, risti, slown, trav);
}

/* fouds2_all: mixed-order update over the eight octants (F:635-1004). */
static void fouds2(fmm_state *s, int iz, int ix, int ir)
{
    const orc_grid *g = s->g;
    double ri, risti;
    centre_geom(s, ix, ir, &ri, &risti);
    const double slown = 1.0 / SV(s, iz, ix, ir);
    int tsw1 = 0;
    double travm = 0.0;
    for (int i = ir - 1; i <= ir + 1; i += 2) {
        const int i2 = (i == ir - 1) ? i - 1 : i + 1;
        const int i2in = (i == ir - 1) ? (i2 >= 1) : (i2 <= s->nnr);
        const int swi = sw2(s, NS(s, iz, ix, i) == 0, i2in, i2in && NS(s, iz, ix, i2) == 0,
                            TT(s, iz, ix, i), i2in ? TT(s, iz, ix, i2) : 0.0);
        for (int j = ix - 1; j <= ix + 1; j += 2) {
            const int j2 = (j == ix - 1) ? j - 1 : j + 1;
            const int j2in = (j == ix - 1) ? (j2 >= 1) : (j2 <= s->nnx);
            const int swj = sw2(s, NS(s, iz, j, ir) == 0, j2in, j2in && NS(s, iz, j2, ir) == 0,
                                TT(s, iz, j, ir), j2in ? TT(s, iz, j2, ir) : 0.0);
            for (int k = iz - 1; k <= iz + 1; k += 2) {
                const int k2 = (k == iz - 1) ? k - 1 : k + 1;
                const int k2in = (k == iz - 1) ? (k2 >= 1) : (k2 <= s->nnz);
                const int swk = sw2(s, NS(s, k, ix, ir) == 0, k2in, k2in && NS(s, k2, ix, ir) == 0,
                                    TT(s, k, ix, ir), k2in ? TT(s, k2, ix, ir) : 0.0);
                if (i < 1 || i > s->nnr || j < 1 || j > s->nnx || k < 1 || k > s->nnz) continue;
                const int ai = NS(s, iz, ix, i) == 0, aj = NS(s, iz, j, ir) == 0, ak = NS(s, k, ix, ir) == 0;
                double trav;
                if (octant2(s, iz, ix, ir, i, j, k, i2, j2, k2, ai, aj, ak, swi, swj, swk, ri, risti, slown, &trav)) {
                    if (tsw1) travm = fmin(trav, travm);
                    else { travm = trav; tsw1 = 1; }
                }
            }
        }
    }
    /* F:1001: travm is undefined in the reference when no octant solved;
     * that cannot happen for a neighbour of a popped node. */
    if (TT(s, iz, ix, ir) == 0.0 || TT(s, iz, ix, ir) > travm) TT(s, iz, ix, ir) = travm;
}

/* ------------------------------------------------------------------------ */
/* Fixed point of the reference's stencil (order-independent restatement)    */
/* ------------------------------------------------------------------------ */
/* One octant of fouds1_all (F:547-621) for given upwind flags. */
static int octant1(const fmm_state *s, int iz, int ix, int ir, int i, int j, int k, int ai, int aj, int ak,
                   double ri, double risti, double slown, double *trav)
{
    const orc_grid *g = s->g;
    const double dnr = g->dnr, dnx = g->dnx, dnz = g->dnz;
    double a = 0, b = 0, c = 0, tref = 0;
    int swsol = 0;
    if (ai) {
        swsol = 1;
        if (aj && ak) {
            const double u = dnr, v = ri * dnx, w = risti * dnz;
            const double em = TT(s, iz, j, ir) - TT(s, iz, ix, i);
            const double en = TT(s, k, ix, ir) - TT(s, iz, ix, i);
            const double rd1 = sq(v) * sq(w), rd2 = sq(u) * sq(w), rd3 = sq(u) * sq(v);
            a = rd1 + rd2 + rd3;
            b = -2.0 * (em * rd2 + en * rd3);
            c = sq(em) * rd2 + sq(en) * rd3 - sq(slown) * sq(u) * rd1;
        } else if (aj) {
            const double u = dnr, v = ri * dnx;
            const double em = TT(s, iz, j, ir) - TT(s, iz, ix, i);
            a = sq(u) + sq(v);
            b = -2.0 * sq(u) * em;
            c = sq(u) * (sq(em) - sq(v) * sq(slown));
        } else if (ak) {
            const double u = dnr, v = risti * dnz;
            const double em = TT(s, k, ix, ir) - TT(s, iz, ix, i);
            a = sq(u) + sq(v);
            b = -2.0 * sq(u) * em;
            c = sq(u) * (sq(em) - sq(v) * sq(slown));
        } else {
            a = 1.0; b = 0.0;
            c = -sq(slown) * sq(dnr);
        }
        tref = TT(s, iz, ix, i);
    } else if (aj) {
        swsol = 1;
        if (ak) {
            const double u = ri * dnx, v = risti * dnz;
            const double em = TT(s, k, ix, ir) - TT(s, iz, j, ir);
            a = sq(u) + sq(v);
            b = -2.0 * sq(u) * em;
            c = sq(u) * (sq(em) - sq(v) * sq(slown));
        } else {
            a = 1.0; b = 0.0;
            c = -sq(slown) * sq(ri) * sq(dnx);
        }
        tref = TT(s, iz, j, ir);
    } else if (ak) {
        swsol = 1;
        a = 1.0; b = 0.0;
        c = -sq(slown * risti * dnz);
        tref = TT(s, k, ix, ir);
    }
    if (swsol) {
        double rd1 = sq(b) - 4.0 * a * c;
        if (rd1 < 0.0) rd1 = 0.0;
        *trav = tref + (-b + sqrt(rd1)) / (2.0 * a);
    }
    return swsol;
}

/* Node value at the fixed point's self-consistency condition: in every
 * octant the neighbours are added in ascending time while earlier than the
 * octant's current solution ("alive" of the heap restated as "earlier than
 * the node"), each partial set solved with the reference's own formulas;
 * minimum over octants.  Unset nodes hold +infinity. */
static double fp_update(fmm_state *s, int fom, int iz, int ix, int ir)
{
    const orc_grid *g = s->g;
    double ri, risti;
    centre_geom(s, ix, ir, &ri, &risti);
    const double slown = 1.0 / SV(s, iz, ix, ir);
    double best = INFINITY;
    for (int i = ir - 1; i <= ir + 1; i += 2)
        for (int j = ix - 1; j <= ix + 1; j += 2)
            for (int k = iz - 1; k <= iz + 1; k += 2) {
                if (i < 1 || i > s->nnr || j < 1 || j > s->nnx || k < 1 || k > s->nnz) continue;
                const int i2 = (i == ir - 1) ? i - 1 : i + 1;
                const int j2 = (j == ix - 1) ? j - 1 : j + 1;
                const int k2 = (k == iz - 1) ? k - 1 : k + 1;
                const int i2in = i2 >= 1 && i2 <= s->nnr, j2in = j2 >= 1 && j2 <= s->nnx, k2in = k2 >= 1 && k2 <= s->nnz;
                double val[3] = {TT(s, iz, ix, i), TT(s, iz, j, ir), TT(s, k, ix, ir)};
                int ord[3] = {0, 1, 2};
                /* ascending, ties keep r, theta, phi order */
                if (val[ord[1]] < val[ord[0]]) { int q = ord[0]; ord[0] = ord[1]; ord[1] = q; }
                if (val[ord[2]] < val[ord[1]]) { int q = ord[1]; ord[1] = ord[2]; ord[2] = q; }
                if (val[ord[1]] < val[ord[0]]) { int q = ord[0]; ord[0] = ord[1]; ord[1] = q; }
                int al[3] = {0, 0, 0};
                double cur = INFINITY;
                int have = 0;
                for (int m = 0; m < 3; ++m) {
                    const double v = val[ord[m]];
                    if (!(v < INFINITY)) break;
                    if (have && !(v < cur)) break;
                    al[ord[m]] = 1;
                    double trav = 0.0;
                    int ok;
                    if (fom == 0) {
                        ok = octant1(s, iz, ix, ir, i, j, k, al[0], al[1], al[2], ri, risti, slown, &trav);
                    } else {
                        const int swi = (al[0] && i2in && TT(s, iz, ix, i2) < val[0]) ? 0 : -1;
                        const int swj = (al[1] && j2in && TT(s, iz, j2, ir) < val[1]) ? 0 : -1;
                        const int swk = (al[2] && k2in && TT(s, k2, ix, ir) < val[2]) ? 0 : -1;
                        ok = octant2(s, iz, ix, ir, i, j, k, i2, j2, k2, al[0], al[1], al[2], swi, swj, swk,
                                     ri, risti, slown, &trav);
                    }
                    if (!ok) break;
                    cur = trav;
                    have = 1;
                }
                if (have && cur < best) best = cur;
            }
    return best;
}

static int fixed_point_run(fmm_state *s, unsigned char *fixed, int fom, double *ttn, int max_sweeps,
                           int *sweeps);

int orc_fixed_point(const orc_grid *g, const double *veln, int fom, const double *bottom, double *ttn,
                    int max_sweeps, int *sweeps)
{
    fmm_state s;
    state_serial(&s, g, veln);
    const size_t npad = (size_t)s.NZ2 * (size_t)s.NX2 * (size_t)(g->nnr + 2);
    s.ttn = (double *)malloc(npad * sizeof(double));
    unsigned char *fixed = (unsigned char *)calloc(npad, 1);
    if (!s.ttn || !fixed) { free(s.ttn); free(fixed); return -3; }
    for (size_t q = 0; q < npad; ++q) s.ttn[q] = INFINITY;
    const int rn = g->nnr;
    for (int i = 1; i <= g->nnx; ++i)
        for (int j = 1; j <= g->nnz; ++j) {
            const double v = bottom[(size_t)(j - 1) + (size_t)g->nnz * (size_t)(i - 1)];
            if (v > 0.0) {   /* F:6932-6936 */
                TT(&s, j, i, rn) = v;
                fixed[TI(&s, j, i, rn)] = 1;
            }
        }
    return fixed_point_run(&s, fixed, fom, ttn, max_sweeps, sweeps);
}

int orc_fixed_point_field(const orc_grid *g, const double *veln, int fom, const double *init,
                          const unsigned char *fixed_in, double *ttn, int max_sweeps, int *sweeps)
{
    fmm_state s;
    state_serial(&s, g, veln);
    const size_t npad = (size_t)s.NZ2 * (size_t)s.NX2 * (size_t)(g->nnr + 2);
    s.ttn = (double *)malloc(npad * sizeof(double));
    unsigned char *fixed = (unsigned char *)calloc(npad, 1);
    if (!s.ttn || !fixed) { free(s.ttn); free(fixed); return -3; }
    for (size_t q = 0; q < npad; ++q) s.ttn[q] = INFINITY;
    for (int ir = 1; ir <= g->nnr; ++ir)
        for (int ix = 1; ix <= g->nnx; ++ix)
            for (int iz = 1; iz <= g->nnz; ++iz) {
                const size_t q = (size_t)(iz - 1) + (size_t)g->nnz * ((size_t)(ix - 1) + (size_t)g->nnx * (size_t)(ir - 1));
                TT(&s, iz, ix, ir) = init[q];
                fixed[TI(&s, iz, ix, ir)] = fixed_in[q];
            }
    return fixed_point_run(&s, fixed, fom, ttn, max_sweeps, sweeps);
}

/* Gauss-Seidel sweeps in the eight alternating orders until no value
 * changes; fixed nodes keep their values.  Frees s->ttn and fixed. */
static int fixed_point_run(fmm_state *s_, unsigned char *fixed, int fom, double *ttn, int max_sweeps, int *sweeps)
{
    fmm_state s = *s_;
    const orc_grid *g = s.g;
    int it;
    int converged = 0;
    for (it = 0; it < max_sweeps; ++it) {
        long changed = 0;
        const int o = it % 8;
        const int sr = (o & 4) ? 1 : -1, sx = (o & 2) ? 1 : -1, sz = (o & 1) ? 1 : -1;
        for (int a = 0; a < g->nnr; ++a) {
            const int ir = sr > 0 ? 1 + a : g->nnr - a;
            for (int b = 0; b < g->nnx; ++b) {
                const int ix = sx > 0 ? 1 + b : g->nnx - b;
                for (int c = 0; c < g->nnz; ++c) {
                    const int iz = sz > 0 ? 1 + c : g->nnz - c;
                    if (fixed[TI(&s, iz, ix, ir)]) continue;
                    const double nv = fp_update(&s, fom, iz, ix, ir);
                    const double ov = TT(&s, iz, ix, ir);
                    if (memcmp(&nv, &ov, sizeof nv) != 0) { TT(&s, iz, ix, ir) = nv; changed++; }
                }
            }
        }
        if (!changed) { converged = 1; break; }
    }
    for (int ir = 1; ir <= g->nnr; ++ir)
        for (int ix = 1; ix <= g->nnx; ++ix)
            for (int iz = 1; iz <= g->nnz; ++iz) {
                const double v = TT(&s, iz, ix, ir);
                ttn[(size_t)(iz - 1) + (size_t)g->nnz * ((size_t)(ix - 1) + (size_t)g->nnx * (size_t)(ir - 1))] =
                    v < INFINITY ? v : 0.0;
            }
    if (sweeps) *sweeps = it + 1;
    free(s.ttn);
    free(fixed);
    return converged ? 0 : -4;
}

/* Heap operations (F:1006-1098). Ties keep the reference's order. */
static void addtree(fmm_state *s, int iz, int ix, int ir)
{
    s->ntr++;
    NS(s, iz, ix, ir) = s->ntr;
    s->hr[s->ntr] = ir; s->hx[s->ntr] = ix; s->hz[s->ntr] = iz;
    int tpc = s->ntr, tpp = tpc / 2;
    while (tpp > 0) {
        if (TT(s, iz, ix, ir) < TT(s, s->hz[tpp], s->hx[tpp], s->hr[tpp])) {
            NS(s, iz, ix, ir) = tpp;
            NS(s, s->hz[tpp], s->hx[tpp], s->hr[tpp]) = tpc;
            int t;
            t = s->hr[tpc]; s->hr[tpc] = s->hr[tpp]; s->hr[tpp] = t;
            t = s->hx[tpc]; s->hx[tpc] = s->hx[tpp]; s->hx[tpp] = t;
            t = s->hz[tpc]; s->hz[tpc] = s->hz[tpp]; s->hz[tpp] = t;
            tpc = tpp; tpp = tpc / 2;
        } else {
            tpp = 0;
        }
    }
}

static double hval(const fmm_state *s, int p) { return TT(s, s->hz[p], s->hx[p], s->hr[p]); }

static void hswap_status(fmm_state *s, int tpp, int tpc)
{
    NS(s, s->hz[tpp], s->hx[tpp], s->hr[tpp]) = tpc;
    NS(s, s->hz[tpc], s->hx[tpc], s->hr[tpc]) = tpp;
    int t;
    t = s->hr[tpc]; s->hr[tpc] = s->hr[tpp]; s->hr[tpp] = t;
    t = s->hx[tpc]; s->hx[tpc] = s->hx[tpp]; s->hx[tpp] = t;
    t = s->hz[tpc]; s->hz[tpc] = s->hz[tpp]; s->hz[tpp] = t;
}

static void downtree(fmm_state *s)
{
    if (s->ntr == 1) { s->ntr = 0; return; }
    const int n = s->ntr;
    NS(s, s->hz[n], s->hx[n], s->hr[n]) = 1;
    s->hr[1] = s->hr[n]; s->hx[1] = s->hx[n]; s->hz[1] = s->hz[n];
    s->ntr--;
    int tpp = 1, tpc = 2;
    while (tpc < s->ntr) {
        if (hval(s, tpc) > hval(s, tpc + 1)) tpc++;
        if (hval(s, tpc) < hval(s, tpp)) {
            hswap_status(s, tpp, tpc);
            tpp = tpc; tpc = 2 * tpp;
        } else {
            tpc = s->ntr + 1;
        }
    }
    if (tpc == s->ntr) {
        if (hval(s, tpc) < hval(s, tpp)) hswap_status(s, tpp, tpc);
    }
}

static void updtree(fmm_state *s, int iz, int ix, int ir)
{
    int tpc = NS(s, iz, ix, ir), tpp = tpc / 2;
    while (tpp > 0) {
        if (TT(s, iz, ix, ir) < hval(s, tpp)) {
            NS(s, iz, ix, ir) = tpp;
            NS(s, s->hz[tpp], s->hx[tpp], s->hr[tpp]) = tpc;
            int t;
            t = s->hr[tpc]; s->hr[tpc] = s->hr[tpp]; s->hr[tpp] = t;
            t = s->hx[tpc]; s->hx[tpc] = s->hx[tpp]; s->hx[tpp] = t;
            t = s->hz[tpc]; s->hz[tpc] = s->hz[tpp]; s->hz[tpp] = t;
            tpc = tpp; tpp = tpc / 2;
        } else {
            tpp = 0;
        }
    }
}

static void visit(fmm_state *s, int fom, int iz, int ix, int ir)
{
    const int st = NS(s, iz, ix, ir);
    if (st == -1) {
        if (fom == 0) fouds1(s, iz, ix, ir); else fouds2(s, iz, ix, ir);
        addtree(s, iz, ix, ir);
    } else if (st > 0) {
        if (fom == 0) fouds1(s, iz, ix, ir); else fouds2(s, iz, ix, ir);
        updtree(s, iz, ix, ir);
    }
}

/* local_fmm (F:78-155): pop the earliest node, freeze it, update its
 * far and trial neighbours inside the (sub)domain.  Returns the pops. */
static long long local_fmm(fmm_state *s, int fom)
{
    long long pops = 0;
    while (s->ntr > 0) {
        const int ir = s->hr[1], ix = s->hx[1], iz = s->hz[1];
        NS(s, iz, ix, ir) = 0;
        downtree(s);
        ++pops;
        for (int i = ir - 1; i <= ir + 1; i += 2)
            if (i >= 1 && i <= s->nnr) visit(s, fom, iz, ix, i);
        for (int i = ix - 1; i <= ix + 1; i += 2)
            if (i >= 1 && i <= s->nnx) visit(s, fom, iz, i, ir);
        for (int i = iz - 1; i <= iz + 1; i += 2)
            if (i >= 1 && i <= s->nnz) visit(s, fom, i, ix, ir);
    }
    return pops;
}

int orc_fmm(const orc_grid *g, const double *veln, int fom, const double *bottom,
            double *ttn, long long *npops)
{
    fmm_state s;
    state_serial(&s, g, veln);
    const size_t npad = (size_t)s.NZ2 * (size_t)s.NX2 * (size_t)(g->nnr + 2);
    const size_t nint = (size_t)g->nnz * (size_t)g->nnx * (size_t)g->nnr;
    s.ttn = (double *)calloc(npad, sizeof(double));
    s.nsts = (int *)malloc(npad * sizeof(int));
    s.hr = (int *)malloc((nint + 2) * sizeof(int));
    s.hx = (int *)malloc((nint + 2) * sizeof(int));
    s.hz = (int *)malloc((nint + 2) * sizeof(int));
    if (!s.ttn || !s.nsts || !s.hr || !s.hx || !s.hz) {
        free(s.ttn); free(s.nsts); free(s.hr); free(s.hx); free(s.hz);
        return -3;
    }
    for (size_t q = 0; q < npad; ++q) s.nsts[q] = -1;   /* F:6373-6375 */

    /* start_fmm (F:6908-6960): load the bottom frame, freeze positive
     * values, seed the heap with the single global minimum. */
    const int rn = g->nnr;
    int sw = 0, itmin = 0, jtmin = 0;
    double ttmin = -100.0;
    for (int i = 1; i <= g->nnx; ++i)
        for (int j = 1; j <= g->nnz; ++j) {
            const double rd1 = bottom[(size_t)(j - 1) + (size_t)g->nnz * (size_t)(i - 1)];
            TT(&s, j, i, rn) = rd1;
            if (rd1 > 0.0) {
                if (sw == 0) { ttmin = rd1; itmin = i; jtmin = j; sw = 1; }
                else if (rd1 < ttmin) { ttmin = rd1; itmin = i; jtmin = j; }
                NS(&s, j, i, rn) = 0;
            } else {
                TT(&s, j, i, rn) = 0.0;
            }
        }
    long long pops = 0;
    if (sw) {
        addtree(&s, jtmin, itmin, rn);
        pops = local_fmm(&s, fom);
    }
    for (int ir = 1; ir <= g->nnr; ++ir)
        for (int ix = 1; ix <= g->nnx; ++ix)
            for (int iz = 1; iz <= g->nnz; ++iz)
                ttn[(size_t)(iz - 1) + (size_t)g->nnz * ((size_t)(ix - 1) + (size_t)g->nnx * (size_t)(ir - 1))] = TT(&s, iz, ix, ir);
    if (npops) *npops = pops;
    free(s.ttn); free(s.nsts); free(s.hr); free(s.hx); free(s.hz);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* The decomposed run: nr x nx x nz subdomain ranks (F:6127-6168, 6371-6451)  */
/* ------------------------------------------------------------------------ */
/* Each block is one of the reference's compute ranks, emulated in turn
 * inside every bulk-synchronous round: it marches its own nodes with
 * local_fmm (stencils see only its own nodes), and before each march takes
 * its neighbours' two boundary layers as ghosts (boundary_communication,
 * F:6691-6795), re-solves the boundary nodes a ghost can lower with the face
 * stencils in ghost order and reopens its heap (order_overlap, F:157-416).
 * The rounds stop when no node of any block moved by more than 1e-5 s
 * (error_calculate, F:6963-6987; the single-precision literal of F:6403).
 *
 * Faces in the reference's order (send_direction(1..6)): left (x-1), right
 * (x+1), in (z-1), out (z+1), up (r-1), down (r+1). */
enum { FC_LEFT, FC_RIGHT, FC_IN, FC_OUT, FC_UP, FC_DOWN };

typedef struct {
    fmm_state s;
    double *vel;          /* this block's gridded velocity (its own gridder call) */
    double *prev;         /* ttn_previous_step */
    double *ghost[6][2];  /* ghost layers 1 and 2 of each face, one plane each */
    int nb[6];            /* neighbour block, or -1 (no neighbour: MPI_PROC_NULL) */
    int sw_fmm, dir_send, send_dir[6];
} dec_block;

/* node of the face plane with plane coordinates (a, b): left/right (iz, ir),
 * in/out (ix, ir), up/down (iz, ix) */
static int face_plane_n(const fmm_state *s, int f)
{
    return f <= FC_RIGHT ? s->nnz * s->nnr : (f <= FC_OUT ? s->nnx * s->nnr : s->nnz * s->nnx);
}

static int face_pidx(const fmm_state *s, int f, int iz, int ix, int ir)
{
    if (f <= FC_RIGHT) return (iz - 1) + s->nnz * (ir - 1);
    if (f <= FC_OUT) return (ix - 1) + s->nnx * (ir - 1);
    return (iz - 1) + s->nnz * (ix - 1);
}

/* ghost layer next to the face: 2 for left/in/up, 1 for right/out/down */
static int face_adj(int f) { return (f == FC_LEFT || f == FC_IN || f == FC_UP) ? 2 : 1; }

/* fouds2_left ... fouds2_down (F:1100-2825): a boundary node re-solved with
 * its ghost neighbour across face f always taken (second order when the
 * ghost layer next to the face is later than the one behind it), the two
 * in-plane axes taken by value ("earlier than the node, or the node unset",
 * second order when the second neighbour is set and earlier), over the four
 * octants whose in-plane neighbours lie in the block.  The branch table is
 * fouds2_all's (F:712-982) with the ghost axis always used.  The value is
 * kept when it does not exceed the old one (or the node was unset), and the
 * node goes into, or moves up in, the heap. */
static void fouds2_face(dec_block *B, int f, int iz, int ix, int ir, double old_value)
{
    fmm_state *s = &B->s;
    const orc_grid *g = s->g;
    double ri, risti;
    centre_geom(s, ix, ir, &ri, &risti);
    const double slown = 1.0 / SV(s, iz, ix, ir);
    const int ga = f >= FC_UP ? 0 : (f <= FC_RIGHT ? 1 : 2);     /* ghost axis: r, theta, phi */
    const int p = face_pidx(s, f, iz, ix, ir);
    const int adj = face_adj(f);
    const double gt = B->ghost[f][adj - 1][p], gt2 = B->ghost[f][2 - adj][p];
    const int gsw = gt > gt2 ? 0 : -1;
    const double tc = TT(s, iz, ix, ir);
    const int n[3] = {s->nnr, s->nnx, s->nnz};
    const int c[3] = {ir, ix, iz};
    /* the two in-plane axes */
    int ax[2], m = 0;
    for (int a = 0; a < 3; ++a)
        if (a != ga) ax[m++] = a;
    int tsw1 = 0;
    double travm = 0.0;
    for (int d0 = -1; d0 <= 1; d0 += 2)
        for (int d1 = -1; d1 <= 1; d1 += 2) {
            double t[3], t2[3];
            int used[3], sw[3], inr = 1;
            t[ga] = gt; t2[ga] = gt2; used[ga] = 1; sw[ga] = gsw;
            for (int q = 0; q < 2; ++q) {
                const int a = ax[q], d = q == 0 ? d0 : d1;
                int pn[3] = {ir, ix, iz}, pn2[3] = {ir, ix, iz};
                pn[a] = c[a] + d;
                pn2[a] = c[a] + 2 * d;
                const double tn = TT(s, pn[2], pn[1], pn[0]);   /* padded: 0 outside the block */
                const int n2in = pn2[a] >= 1 && pn2[a] <= n[a];
                const double tn2 = n2in ? TT(s, pn2[2], pn2[1], pn2[0]) : 0.0;
                int w = (n2in && tn2 != 0.0) ? 0 : -1;
                const int u = (tn < tc || tc == 0.0) && tn != 0.0;
                if (u && w == 0) w = tn > tn2 ? 0 : -1;
                else w = -1;
                t[a] = tn; t2[a] = tn2; used[a] = u; sw[a] = w;
                if (pn[a] < 1 || pn[a] > n[a]) inr = 0;
            }
            if (!inr) continue;
            double trav;
            if (octant2v(g, t[0], t2[0], t[1], t2[1], t[2], t2[2], used[0], used[1], used[2], sw[0], sw[1], sw[2],
                         ri, risti, slown, &trav)) {
                if (tsw1) travm = fmin(trav, travm);
                else { travm = trav; tsw1 = 1; }
            }
        }
    if (!tsw1) return;
    if (old_value >= travm || old_value == 0.0) {
        TT(s, iz, ix, ir) = travm;
        if (NS(s, iz, ix, ir) <= 0) addtree(s, iz, ix, ir);
        else updtree(s, iz, ix, ir);
    }
}

/* order_overlap (F:157-416) */
static void order_overlap(dec_block *B)
{
    fmm_state *s = &B->s;
    const int nmax = s->nnr * s->nnx * s->nnz + 1;
    int *ha = (int *)malloc(sizeof(int) * (size_t)(nmax + 1));
    int *hb = (int *)malloc(sizeof(int) * (size_t)(nmax + 1));
    double *hk = (double *)malloc(sizeof(double) * (size_t)(nmax + 1));
    for (int f = 0; f < 6; ++f) {
        if (B->send_dir[f] != 1) continue;
        const int adj = face_adj(f);
        const double *G = B->ghost[f][adj - 1];
        /* the face's boundary nodes that a ghost can lower (or that are
         * unset), in a heap keyed by the ghost value next to them, built by
         * insertion in the reference's loop order */
        int temp = 0;
        const int outer = f >= FC_UP ? s->nnx : s->nnr;
        const int inner = (f == FC_IN || f == FC_OUT) ? s->nnx : s->nnz;
        for (int i = 1; i <= outer; ++i)
            for (int j = 1; j <= inner; ++j) {
                int iz, ix, ir;
                switch (f) {
                    case FC_LEFT:  iz = j; ix = 1;      ir = i; break;
                    case FC_RIGHT: iz = j; ix = s->nnx; ir = i; break;
                    case FC_IN:    iz = 1;      ix = j; ir = i; break;
                    case FC_OUT:   iz = s->nnz; ix = j; ir = i; break;
                    case FC_UP:    iz = j; ix = i; ir = 1; break;
                    default:       iz = j; ix = i; ir = s->nnr; break;
                }
                const double gv = G[face_pidx(s, f, iz, ix, ir)];
                const double tv = TT(s, iz, ix, ir);
                if (!(gv < tv || tv == 0.0)) continue;
                ++temp;
                ha[temp] = j; hb[temp] = i; hk[temp] = gv;
                int tpc = temp, tpp = tpc / 2;
                while (tpp > 0) {
                    if (gv < hk[tpp]) {
                        int x = ha[tpc]; ha[tpc] = ha[tpp]; ha[tpp] = x;
                        x = hb[tpc]; hb[tpc] = hb[tpp]; hb[tpp] = x;
                        double y = hk[tpc]; hk[tpc] = hk[tpp]; hk[tpp] = y;
                        tpc = tpp; tpp = tpc / 2;
                    } else {
                        tpp = 0;
                    }
                }
            }
        /* in ghost order: re-solve, then pop (downtree_left ... downtree_down,
         * F:5747-6009) */
        while (temp > 0) {
            const int j = ha[1], i = hb[1];
            int iz, ix, ir;
            switch (f) {
                case FC_LEFT:  iz = j; ix = 1;      ir = i; break;
                case FC_RIGHT: iz = j; ix = s->nnx; ir = i; break;
                case FC_IN:    iz = 1;      ix = j; ir = i; break;
                case FC_OUT:   iz = s->nnz; ix = j; ir = i; break;
                case FC_UP:    iz = j; ix = i; ir = 1; break;
                default:       iz = j; ix = i; ir = s->nnr; break;
            }
            fouds2_face(B, f, iz, ix, ir, TT(s, iz, ix, ir));
            if (temp == 1) { temp = 0; break; }
            ha[1] = ha[temp]; hb[1] = hb[temp]; hk[1] = hk[temp];
            --temp;
            int tpp = 1, tpc = 2;
            while (tpc < temp) {
                if (hk[tpc] > hk[tpc + 1]) ++tpc;
                if (hk[tpc] < hk[tpp]) {
                    int x = ha[tpc]; ha[tpc] = ha[tpp]; ha[tpp] = x;
                    x = hb[tpc]; hb[tpc] = hb[tpp]; hb[tpp] = x;
                    double y = hk[tpc]; hk[tpc] = hk[tpp]; hk[tpp] = y;
                    tpp = tpc; tpc = 2 * tpp;
                } else {
                    tpc = temp + 1;
                }
            }
            if (tpc == temp && hk[tpc] < hk[tpp]) {
                int x = ha[tpc]; ha[tpc] = ha[tpp]; ha[tpp] = x;
                x = hb[tpc]; hb[tpc] = hb[tpp]; hb[tpp] = x;
                double y = hk[tpc]; hk[tpc] = hk[tpp]; hk[tpp] = y;
            }
        }
    }
    free(ha); free(hb); free(hk);
    /* reopen (F:387-415): nodes between the heap's earliest and latest value
     * go back into the heap, earlier ones are frozen, later ones far */
    if (s->ntr >= 1) {
        B->sw_fmm = 1;
        const double mini = hval(s, 1);
        double maxi = 0.0;
        for (int q = 1; q <= s->ntr; ++q)
            if (hval(s, q) > maxi) maxi = hval(s, q);
        for (int ir = 1; ir <= s->nnr; ++ir)
            for (int ix = 1; ix <= s->nnx; ++ix)
                for (int iz = 1; iz <= s->nnz; ++iz) {
                    if (NS(s, iz, ix, ir) > 0) continue;
                    const double v = TT(s, iz, ix, ir);
                    if (v > 0.0) {
                        if (v <= mini) NS(s, iz, ix, ir) = 0;
                        else if (v >= maxi) NS(s, iz, ix, ir) = -1;
                        else addtree(s, iz, ix, ir);
                    } else {
                        NS(s, iz, ix, ir) = -1;
                    }
                }
    }
}

/* one axis of the block split (F:6127-6168): sizes n/np (+1 for the first
 * n mod np ranks), offsets contiguous from 1 */
static void split_axis(int n, int np, int rank, int *num, int *off)
{
    int o = 1;
    for (int r = 0; r <= rank; ++r) {
        const int sz = n / np + ((n % np) && r < n % np ? 1 : 0);
        if (r == rank) { *num = sz; *off = o; }
        o += sz;
    }
}

/* threads for the blocks of a round: one per block unless
 * ORC_DECOMPOSED_THREADS says otherwise (1 = the blocks in turn) */
static int dec_threads(int nb)
{
    const char *e = getenv("ORC_DECOMPOSED_THREADS");
    const int t = e ? atoi(e) : nb;
    return t >= 1 ? t : 1;
}

int orc_fmm_decomposed(const orc_grid *g, const double *velv, int fom, const double *bottom, int nr, int nx,
                       int nz, int max_rounds, double *ttn, int *rounds_out)
{
    const int nb = nr * nx * nz;
    if (nr < 1 || nx < 1 || nz < 1 || g->nnr / nr < 2 || g->nnx / nx < 2 || g->nnz / nz < 2) return -2;
    dec_block *B = (dec_block *)calloc((size_t)nb, sizeof(dec_block));
    if (!B) return -3;
    int rc = 0;
    for (int br = 0; br < nr; ++br)
        for (int bx = 0; bx < nx; ++bx)
            for (int bz = 0; bz < nz; ++bz) {
                dec_block *b = &B[(br * nx + bx) * nz + bz];
                fmm_state *s = &b->s;
                int rnum, xnum, znum, roff, xoff, zoff;
                split_axis(g->nnr, nr, br, &rnum, &roff);
                split_axis(g->nnx, nx, bx, &xnum, &xoff);
                split_axis(g->nnz, nz, bz, &znum, &zoff);
                memset(s, 0, sizeof *s);
                s->g = g;
                s->roff = roff; s->xoff = xoff; s->zoff = zoff;
                s->nnr = rnum; s->nnx = xnum; s->nnz = znum;
                s->NZ2 = znum + 2; s->NX2 = xnum + 2;
                s->VZ3 = znum + 3; s->VX3 = xnum + 3;
                const size_t npad = (size_t)s->NZ2 * (size_t)s->NX2 * (size_t)(rnum + 2);
                const size_t nint = (size_t)znum * (size_t)xnum * (size_t)rnum;
                b->vel = (double *)malloc(sizeof(double) * (size_t)(znum + 3) * (size_t)(xnum + 3) * (size_t)(rnum + 3));
                s->ttn = (double *)calloc(npad, sizeof(double));
                s->nsts = (int *)malloc(npad * sizeof(int));
                s->hr = (int *)malloc((nint + 2) * sizeof(int));
                s->hx = (int *)malloc((nint + 2) * sizeof(int));
                s->hz = (int *)malloc((nint + 2) * sizeof(int));
                b->prev = (double *)calloc(nint, sizeof(double));
                for (int f = 0; f < 6; ++f)
                    for (int l = 0; l < 2; ++l) b->ghost[f][l] = (double *)calloc((size_t)face_plane_n(s, f), sizeof(double));
                if (!b->vel || !s->ttn || !s->nsts || !s->hr || !s->hx || !s->hz || !b->prev) { rc = -3; continue; }
                for (int f = 0; f < 6; ++f)
                    if (!b->ghost[f][0] || !b->ghost[f][1]) rc = -3;
                s->veln = b->vel;
                int ncl = 0;
                gridder_block(g, velv, roff, xoff, zoff, rnum, xnum, znum, b->vel, &ncl);
                for (size_t q = 0; q < npad; ++q) s->nsts[q] = -1;
                b->nb[FC_LEFT] = bx > 0 ? (br * nx + bx - 1) * nz + bz : -1;
                b->nb[FC_RIGHT] = bx < nx - 1 ? (br * nx + bx + 1) * nz + bz : -1;
                b->nb[FC_IN] = bz > 0 ? (br * nx + bx) * nz + bz - 1 : -1;
                b->nb[FC_OUT] = bz < nz - 1 ? (br * nx + bx) * nz + bz + 1 : -1;
                b->nb[FC_UP] = br > 0 ? ((br - 1) * nx + bx) * nz + bz : -1;
                b->nb[FC_DOWN] = br < nr - 1 ? ((br + 1) * nx + bx) * nz + bz : -1;
            }
    if (rc) goto done;
    {
        /* start_fmm (F:6894-6961) on the bottom blocks: load their part of
         * the frame, freeze positive values; the block (or blocks) holding
         * the earliest time seed their heap with it and march */
        double gmin = INFINITY;
        double bmin[4096];
        int bi[4096], bj[4096];
        if (nx * nz > 4096) { rc = -2; goto done; }
        for (int q = 0; q < nx * nz; ++q) {
            dec_block *b = &B[(nr - 1) * nx * nz + q];
            fmm_state *s = &b->s;
            const int rn = s->nnr;
            int sw = 0;
            double ttmin = -100.0;
            for (int i = 1; i <= s->nnx; ++i)
                for (int j = 1; j <= s->nnz; ++j) {
                    const int xg = s->xoff + i - 1, zg = s->zoff + j - 1;
                    const double rd1 = bottom[(size_t)(zg - 1) + (size_t)g->nnz * (size_t)(xg - 1)];
                    TT(s, j, i, rn) = rd1;
                    if (rd1 > 0.0) {
                        if (sw == 0) { ttmin = rd1; bi[q] = i; bj[q] = j; sw = 1; }
                        else if (rd1 < ttmin) { ttmin = rd1; bi[q] = i; bj[q] = j; }
                        NS(s, j, i, rn) = 0;
                    } else {
                        TT(s, j, i, rn) = 0.0;
                    }
                }
            bmin[q] = ttmin;
            if (ttmin != -100.0 && ttmin < gmin) gmin = ttmin;
        }
        for (int q = 0; q < nx * nz; ++q) {
            if (bmin[q] == -100.0 || bmin[q] > gmin) continue;   /* F:6945-6955 */
            dec_block *b = &B[(nr - 1) * nx * nz + q];
            addtree(&b->s, bj[q], bi[q], b->s.nnr);
            local_fmm(&b->s, fom);
            b->sw_fmm = 1;
        }
    }
    {
        const double tol = (double)0.00001f;      /* F:6403, a default-kind literal */
        double err = 0.0;
        int rounds = 0;
        for (;;) {
            /* error_calculate (F:6963-6987): the largest change of any node */
            err = 0.0;
            for (int q = 0; q < nb; ++q) {
                fmm_state *s = &B[q].s;
                size_t k = 0;
                for (int ir = 1; ir <= s->nnr; ++ir)
                    for (int ix = 1; ix <= s->nnx; ++ix)
                        for (int iz = 1; iz <= s->nnz; ++iz, ++k) {
                            const double d = fabs(TT(s, iz, ix, ir) - B[q].prev[k]);
                            if (d > err) err = d;
                        }
            }
            if (!(err > tol)) break;
            if (rounds >= max_rounds) { rc = -4; break; }
            ++rounds;
            for (int q = 0; q < nb; ++q) {
                fmm_state *s = &B[q].s;
                size_t k = 0;
                for (int ir = 1; ir <= s->nnr; ++ir)
                    for (int ix = 1; ix <= s->nnx; ++ix)
                        for (int iz = 1; iz <= s->nnz; ++iz, ++k) B[q].prev[k] = TT(s, iz, ix, ir);
                B[q].dir_send = B[q].sw_fmm;
                B[q].sw_fmm = 0;
            }
            for (int q = 0; q < nb; ++q)
                for (int f = 0; f < 6; ++f)
                    if (B[q].nb[f] >= 0) B[q].send_dir[f] = B[B[q].nb[f]].dir_send;
            /* boundary_communication: the neighbour's two layers next to the
             * face, layer 1 the farther one for left/in/up */
            for (int q = 0; q < nb; ++q) {
                fmm_state *s = &B[q].s;
                for (int f = 0; f < 6; ++f) {
                    if (B[q].send_dir[f] != 1) continue;
                    const fmm_state *o = &B[B[q].nb[f]].s;
                    for (int l = 1; l <= 2; ++l) {
                        double *G = B[q].ghost[f][l - 1];
                        switch (f) {
                            case FC_LEFT:   /* left's x = n-1, n */
                            case FC_RIGHT: { /* right's x = 1, 2 */
                                const int xs = f == FC_LEFT ? o->nnx - 2 + l : l;
                                for (int ir = 1; ir <= s->nnr; ++ir)
                                    for (int iz = 1; iz <= s->nnz; ++iz)
                                        G[face_pidx(s, f, iz, 0, ir)] = TT(o, iz, xs, ir);
                                break;
                            }
                            case FC_IN:
                            case FC_OUT: {
                                const int zs = f == FC_IN ? o->nnz - 2 + l : l;
                                for (int ir = 1; ir <= s->nnr; ++ir)
                                    for (int ix = 1; ix <= s->nnx; ++ix)
                                        G[face_pidx(s, f, 0, ix, ir)] = TT(o, zs, ix, ir);
                                break;
                            }
                            default: {
                                const int rs = f == FC_UP ? o->nnr - 2 + l : l;
                                for (int ix = 1; ix <= s->nnx; ++ix)
                                    for (int iz = 1; iz <= s->nnz; ++iz)
                                        G[face_pidx(s, f, iz, ix, 0)] = TT(o, iz, ix, rs);
                                break;
                            }
                        }
                    }
                }
            }
            /* the ranks' work of a round is independent given the ghosts:
             * one thread per block (the reference's one process per rank) */
#pragma omp parallel for schedule(dynamic, 1) num_threads(dec_threads(nb))
            for (int q = 0; q < nb; ++q) {
                order_overlap(&B[q]);
                local_fmm(&B[q].s, fom);
            }
        }
        if (rounds_out) *rounds_out = rounds;
        /* the blocks' nodes into the global field */
        for (int q = 0; q < nb; ++q) {
            fmm_state *s = &B[q].s;
            for (int ir = 1; ir <= s->nnr; ++ir)
                for (int ix = 1; ix <= s->nnx; ++ix)
                    for (int iz = 1; iz <= s->nnz; ++iz) {
                        const size_t gz = (size_t)(s->zoff + iz - 2), gx = (size_t)(s->xoff + ix - 2),
                                     gr = (size_t)(s->roff + ir - 2);
                        ttn[gz + (size_t)g->nnz * (gx + (size_t)g->nnx * gr)] = TT(s, iz, ix, ir);
                    }
        }
    }
done:
    for (int q = 0; q < nb; ++q) {
        free(B[q].vel); free(B[q].prev);
        free(B[q].s.ttn); free(B[q].s.nsts); free(B[q].s.hr); free(B[q].s.hx); free(B[q].s.hz);
        for (int f = 0; f < 6; ++f) { free(B[q].ghost[f][0]); free(B[q].ghost[f][1]); }
    }
    free(B);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Receiver traveltimes (F:7066-7106)                                        */
/* ------------------------------------------------------------------------ */
#define TD(g, iz, ix, ir) ttn[(size_t)((iz) - 1) + (size_t)(g)->nnz * ((size_t)((ix) - 1) + (size_t)(g)->nnx * (size_t)((ir) - 1))]

int orc_srtimes(const orc_grid *g, const double *ttn, int nrc, const double *rcr,
                const double *rcx, const double *rcz, float *trr)
{
    for (int i = 0; i < nrc; ++i) {
        int irr = (int)floor((g->rgor - rcr[i]) / g->dnr) + 1;
        int irx = (int)floor((rcx[i] - g->rgox) / g->dnx) + 1;
        int irz = (int)floor((rcz[i] - g->rgoz) / g->dnz) + 1;
        if (irx == g->nnx) irx = irx - 1;   /* F:7069-7070 on the last subdomain */
        if (irz == g->nnz) irz = irz - 1;
        if (irr < 1 || irr >= g->nnr || irx < 1 || irx >= g->nnx || irz < 1 || irz >= g->nnz)
            return -(1 + i);
        const double drx = (rcx[i] - g->rgox) - (double)(irx - 1) * g->dnx;
        const double drz = (rcz[i] - g->rgoz) - (double)(irz - 1) * g->dnz;
        const double drr = (g->rgor - rcr[i]) - (double)(irr - 1) * g->dnr;
        float acc = 0.0f;
        for (int j = 1; j <= 2; ++j)
            for (int k = 1; k <= 2; ++k)
                for (int l = 1; l <= 2; ++l) {
                    double produ = (1.0 - fabs(((double)(l - 1) * g->dnz - drz) / g->dnz)) *
                                   (1.0 - fabs(((double)(k - 1) * g->dnx - drx) / g->dnx));
                    produ = produ * (1.0 - fabs(((double)(j - 1) * g->dnr - drr) / g->dnr));
                    acc = (float)((double)acc + TD(g, irz - 1 + l, irx - 1 + k, irr - 1 + j) * produ);
                }
        trr[i] = acc;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Rays and Frechet derivatives (F:7250-7777)                                */
/* ------------------------------------------------------------------------ */

/* trilinear velocity at a point whose propagation cell is (ipz,ipx,ipr) and
 * offsets drr,drx,drz; loop nesting order of F:7632-7641 (r, x, z) or
 * F:7689-7698 (same order). */
static double trilin_vel(const orc_grid *g, const double *veln, int ipz, int ipx, int ipr,
                         double drr, double drx, double drz)
{
    double vel = 0.0;
    for (int k = 1; k <= 2; ++k)
        for (int l = 1; l <= 2; ++l)
            for (int m = 1; m <= 2; ++m) {
                double produ = (1.0 - fabs(((double)(m - 1) * g->dnz - drz) / g->dnz));
                produ = produ * (1.0 - fabs(((double)(l - 1) * g->dnx - drx) / g->dnx));
                produ = produ * (1.0 - fabs(((double)(k - 1) * g->dnr - drr) / g->dnr));
                if (ipz - 1 + m <= g->nnz + 1 && ipx - 1 + l <= g->nnx + 1 && ipr - 1 + k <= g->nnr + 1)
                    vel = vel + veln[VELN(g, ipz - 1 + m, ipx - 1 + l, ipr - 1 + k)] * produ;
            }
    return vel;
}

#define FDM(ivz, ivx, ivr) ((size_t)(ivr) + (size_t)(g->nvr + 2) * ((size_t)(ivx) + (size_t)(g->nvx + 2) * (size_t)(ivz)))

int orc_rays(const orc_grid *g, const double *ttn, const double *veln, int nrc,
             const double *rcr, const double *rcx, const double *rcz,
             float *fdm_all, double *endpoints, int *nsteps)
{
    const int maxrp = 100000;             /* F:7262 */
    const double dpl = g->dnr;            /* F:7290 */
    const size_t nmp = (size_t)(g->nvr + 2) * (size_t)(g->nvx + 2) * (size_t)(g->nvz + 2);
    int rc = 0;
    for (int iray = 0; iray < nrc; ++iray) {
        float *fdm = fdm_all ? fdm_all + nmp * (size_t)iray : NULL;
        if (fdm) memset(fdm, 0, nmp * sizeof(float));
        double r0 = rcr[iray], x0 = rcx[iray], z0 = rcz[iray];
        int ipr = (int)floor((g->rgor - r0) / g->dnr) + 1;
        int ipx = (int)floor((x0 - g->rgox) / g->dnx) + 1;
        int ipz = (int)floor((z0 - g->rgoz) / g->dnz) + 1;
        /* F:7320-7333: first-round clamp on the last subdomain of each axis */
        if (ipr == g->nnr) ipr--;
        if (ipx == g->nnx) ipx--;
        if (ipz == g->nnz) ipz--;
        if (endpoints) { endpoints[3 * iray] = r0; endpoints[3 * iray + 1] = x0; endpoints[3 * iray + 2] = z0; }
        if (nsteps) nsteps[iray] = 0;
        if (ipr < 1 || ipr >= g->nnr || ipx < 1 || ipx >= g->nnx || ipz < 1 || ipz >= g->nnz)
            continue;
        double rgr = r0, rgx = x0, rgz = z0;
        int steps = 0;
        for (int jstep = 1; jstep <= maxrp; ++jstep) {
            ++steps;
            /* F:7348-7378: cell-averaged gradient */
            double dtr = 0.0;
            int temp = 0;
            if (TD(g, ipz, ipx, ipr + 1) < TD(g, ipz, ipx, ipr)) { dtr = dtr + TD(g, ipz, ipx, ipr + 1) - TD(g, ipz, ipx, ipr); temp++; }
            if (TD(g, ipz + 1, ipx, ipr + 1) < TD(g, ipz + 1, ipx, ipr)) { dtr = dtr + TD(g, ipz + 1, ipx, ipr + 1) - TD(g, ipz + 1, ipx, ipr); temp++; }
            if (TD(g, ipz + 1, ipx + 1, ipr + 1) < TD(g, ipz + 1, ipx + 1, ipr)) { dtr = dtr + TD(g, ipz + 1, ipx + 1, ipr + 1) - TD(g, ipz + 1, ipx + 1, ipr); temp++; }
            if (TD(g, ipz, ipx + 1, ipr + 1) < TD(g, ipz, ipx + 1, ipr)) { dtr = dtr + TD(g, ipz, ipx + 1, ipr + 1) - TD(g, ipz, ipx + 1, ipr); temp++; }
            if (temp != 0) dtr = dtr / ((double)temp * g->dnr);
            const double rcell = g->earth + g->rgor - (double)(ipr - 1) * g->dnr;
            double dtx = TD(g, ipz, ipx + 1, ipr) - TD(g, ipz, ipx, ipr);
            dtx = dtx + TD(g, ipz + 1, ipx + 1, ipr) - TD(g, ipz + 1, ipx, ipr);
            dtx = dtx + TD(g, ipz + 1, ipx + 1, ipr + 1) - TD(g, ipz + 1, ipx, ipr + 1);
            dtx = dtx + TD(g, ipz, ipx + 1, ipr + 1) - TD(g, ipz, ipx, ipr + 1);
            dtx = dtx / (4.0 * rcell * g->dnx);
            const double sx = sin(rgx);
            double dtz = TD(g, ipz + 1, ipx, ipr) - TD(g, ipz, ipx, ipr);
            dtz = dtz + TD(g, ipz + 1, ipx + 1, ipr + 1) - TD(g, ipz, ipx + 1, ipr + 1);
            dtz = dtz + TD(g, ipz + 1, ipx + 1, ipr) - TD(g, ipz, ipx + 1, ipr);
            dtz = dtz + TD(g, ipz + 1, ipx, ipr + 1) - TD(g, ipz, ipx, ipr + 1);
            dtz = dtz / (4.0 * rcell * sx * g->dnz);
            const double crad = g->earth + rgr;
            double rd1 = sqrt(dtr * dtr + dtx * dtx + dtz * dtz);
            double nr = rgr + dpl * dtr / rd1;
            double nx = rgx - dpl * dtx / (crad * rd1);
            double nz = rgz - dpl * dtz / (crad * sx * rd1);
            const int ipro = ipr, ipxo = ipx, ipzo = ipz;
            ipr = (int)floor((g->rgor - nr) / g->dnr) + 1;
            ipx = (int)floor((nx - g->rgox) / g->dnx) + 1;
            ipz = (int)floor((nz - g->rgoz) / g->dnz) + 1;
            const int swr = (ipr < 1 || ipr >= g->nnr);
            const int swx = (ipx < 1 || ipx >= g->nnx);
            const int swz = (ipz < 1 || ipz >= g->nnz);
            int stop = 0;
            if (swr || swx || swz) {
                /* F:7474-7541: clip to the first outer face crossed */
                int sw = 0;
                double atio = 0.0;
                if (swr) {
                    double ri;
                    if (ipr < 1) { ri = g->rgor; ipr = 1; }
                    else { ri = g->rgor - (double)(g->nnr - 1) * g->dnr; ipr = g->nnr - 1; }
                    atio = (ri - rgr) / (nr - rgr);
                    sw = 1;
                }
                if (swx) {
                    double xi;
                    if (ipx < 1) { xi = g->rgox; ipx = 1; }
                    else { xi = g->rgox + (double)(g->nnx - 1) * g->dnx; ipx = g->nnx - 1; }
                    const double r1 = (xi - rgx) / (nx - rgx);
                    if (sw == 1) { if (r1 < atio) { atio = r1; sw = 2; } }
                    else { atio = r1; sw = 2; }
                }
                if (swz) {
                    double zi;
                    if (ipz < 1) { zi = g->rgoz; ipz = 1; }
                    else { zi = g->rgoz + (double)(g->nnz - 1) * g->dnz; ipz = g->nnz - 1; }
                    const double r1 = (zi - rgz) / (nz - rgz);
                    if (sw != 0) { if (r1 < atio) { atio = r1; sw = 3; } }
                    else { atio = r1; sw = 3; }
                }
                if (sw == 1) { ipx = ipxo; ipz = ipzo; }
                else if (sw == 2) { ipr = ipro; ipz = ipzo; }
                else if (sw == 3) { ipr = ipro; ipx = ipxo; }
                nz = rgz + atio * (nz - rgz);
                nx = rgx + atio * (nx - rgx);
                nr = rgr + atio * (nr - rgr);
                stop = 1;
            }
            if (fdm) {
                /* F:7543-7733: split at velocity-cell crossings, trapezoid
                 * integration of -B/v^2 ds into the single-precision fdm */
                const int ivr = (int)floor((g->gor - nr) / g->dvr) + 1;
                const int ivx = (int)floor((nx - g->gox) / g->dvx) + 1;
                const int ivz = (int)floor((nz - g->goz) / g->dvz) + 1;
                const int ivro = (int)floor((g->gor - rgr) / g->dvr) + 1;
                const int ivxo = (int)floor((rgx - g->gox) / g->dvx) + 1;
                const int ivzo = (int)floor((rgz - g->goz) / g->dvz) + 1;
                double vrat[4];
                int chp[4];
                int nhp = 0;
                if (ivr != ivro) {
                    const double ri = (ivr > ivro) ? g->gor - (double)(ivr - 1) * g->dvr : g->gor - (double)ivr * g->dvr;
                    vrat[nhp] = (ri - rgr) / (nr - rgr);
                    chp[nhp] = 1;
                    nhp++;
                }
                if (ivx != ivxo) {
                    const double xi = (ivx > ivxo) ? g->gox + (double)(ivx - 1) * g->dvx : g->gox + (double)ivx * g->dvx;
                    const double r1 = (xi - rgx) / (nx - rgx);
                    nhp++;
                    if (nhp == 1) { vrat[0] = r1; chp[0] = 2; }
                    else if (r1 >= vrat[nhp - 2]) { vrat[nhp - 1] = r1; chp[nhp - 1] = 2; }
                    else { vrat[nhp - 1] = vrat[nhp - 2]; chp[nhp - 1] = chp[nhp - 2]; vrat[nhp - 2] = r1; chp[nhp - 2] = 2; }
                }
                if (ivz != ivzo) {
                    const double zi = (ivz > ivzo) ? g->goz + (double)(ivz - 1) * g->dvz : g->goz + (double)ivz * g->dvz;
                    const double r1 = (zi - rgz) / (nz - rgz);
                    nhp++;
                    /* 1-based positions as in F:7590-7624 */
                    const int n = nhp;
                    if (n == 1) { vrat[0] = r1; chp[0] = 3; }
                    else if (n == 2) {
                        if (r1 >= vrat[0]) { vrat[1] = r1; chp[1] = 3; }
                        else { vrat[1] = vrat[0]; chp[1] = chp[0]; vrat[0] = r1; chp[0] = 3; }
                    } else {
                        if (r1 >= vrat[1]) { vrat[2] = r1; chp[2] = 3; }
                        else if (r1 >= vrat[0]) { vrat[2] = vrat[1]; chp[2] = chp[1]; vrat[1] = r1; chp[1] = 3; }
                        else { vrat[2] = vrat[1]; chp[2] = chp[1]; vrat[1] = vrat[0]; chp[1] = chp[0]; vrat[0] = r1; chp[0] = 3; }
                    }
                }
                vrat[nhp] = 1.0;
                chp[nhp] = 0;
                nhp++;
                /* velocity and B-spline weights at the segment start */
                double drr = (g->rgor - rgr) - (double)(ipro - 1) * g->dnr;
                double drx = (rgx - g->rgox) - (double)(ipxo - 1) * g->dnx;
                double drz = (rgz - g->rgoz) - (double)(ipzo - 1) * g->dnz;
                double vel = trilin_vel(g, veln, ipzo, ipxo, ipro, drr, drx, drz);
                double ui[4], vi[4], wi[4], uio[4], vio[4], wio[4];
                drr = (g->gor - rgr) - (double)(ivro - 1) * g->dvr;
                drx = (rgx - g->gox) - (double)(ivxo - 1) * g->dvx;
                drz = (rgz - g->goz) - (double)(ivzo - 1) * g->dvz;
                bspline4(drr / g->dvr, ui);
                bspline4(drx / g->dvx, vi);
                bspline4(drz / g->dvz, wi);
                int ivrt = ivro, ivxt = ivxo, ivzt = ivzo;
                for (int k = 0; k < nhp; ++k) {
                    const double velo = vel;
                    memcpy(uio, ui, sizeof ui); memcpy(vio, vi, sizeof vi); memcpy(wio, wi, sizeof wi);
                    if (k > 0) {
                        if (chp[k - 1] == 1) ivrt = ivr;
                        else if (chp[k - 1] == 2) ivxt = ivx;
                        else if (chp[k - 1] == 3) ivzt = ivz;
                    }
                    const double rigz = rgz + vrat[k] * (nz - rgz);
                    const double rigx = rgx + vrat[k] * (nx - rgx);
                    const double rigr = rgr + vrat[k] * (nr - rgr);
                    const int iprt = (int)floor((g->rgor - rigr) / g->dnr) + 1;
                    const int ipxt = (int)floor((rigx - g->rgox) / g->dnx) + 1;
                    const int ipzt = (int)floor((rigz - g->rgoz) / g->dnz) + 1;
                    drr = (g->rgor - rigr) - (double)(iprt - 1) * g->dnr;
                    drx = (rigx - g->rgox) - (double)(ipxt - 1) * g->dnx;
                    drz = (rigz - g->rgoz) - (double)(ipzt - 1) * g->dnz;
                    vel = trilin_vel(g, veln, ipzt, ipxt, iprt, drr, drx, drz);
                    drr = (g->gor - rigr) - (double)(ivrt - 1) * g->dvr;
                    drx = (rigx - g->gox) - (double)(ivxt - 1) * g->dvx;
                    drz = (rigz - g->goz) - (double)(ivzt - 1) * g->dvz;
                    bspline4(drr / g->dvr, ui);
                    bspline4(drx / g->dvx, vi);
                    bspline4(drz / g->dvz, wi);
                    const double dinc = (k == 0) ? vrat[k] * dpl : (vrat[k] - vrat[k - 1]) * dpl;
                    if (ivzt - 1 < 0 || ivzt + 2 > g->nvz + 1 || ivxt - 1 < 0 || ivxt + 2 > g->nvx + 1 ||
                        ivrt - 1 < 0 || ivrt + 2 > g->nvr + 1) {
                        rc = -2;
                        continue;
                    }
                    for (int n = 1; n <= 4; ++n)
                        for (int m = 1; m <= 4; ++m)
                            for (int l = 1; l <= 4; ++l) {
                                double a1 = ui[n - 1] * vi[m - 1] * wi[l - 1] / (vel * vel);
                                double a2 = uio[n - 1] * vio[m - 1] * wio[l - 1] / (velo * velo);
                                a1 = -(a1 + a2) * dinc / 2.0;
                                const size_t q = FDM(ivzt - 2 + l, ivxt - 2 + m, ivrt - 2 + n);
                                fdm[q] = (float)(a1 + (double)fdm[q]);
                            }
                }
            }
            rgr = nr; rgx = nx; rgz = nz;
            if (stop) break;
        }
        if (endpoints) { endpoints[3 * iray] = rgr; endpoints[3 * iray + 1] = rgx; endpoints[3 * iray + 2] = rgz; }
        if (nsteps) nsteps[iray] = steps;
    }
    return rc;
}

int orc_sparsify(int nmp, const float *row, int cap, int *cols, float *vals)
{
    const float ftol = 1.0e-6f;   /* F:7263, REAL(KIND=i5) */
    int n = 0;
    for (int q = 0; q < nmp; ++q) {
        if (fabsf(row[q]) >= ftol) {
            if (n < cap) { cols[n] = q + 1; vals[n] = row[q]; }
            n++;
        }
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* Synthetic plane-wave boundary frames (test inputs; not in the reference)  */
/* ------------------------------------------------------------------------ */
void orc_planewave_params(const orc_grid *g, double delta_deg, double baz_deg, orc_planewave *pw)
{
    const double d2r = M_PI / 180.0;
    const double rb = g->earth + (g->rgor - (double)(g->nnr - 1) * g->dnr);
    /* synthetic distance law, seconds with delta in degrees */
    pw->t0 = 150.0 + 10.0 * delta_deg - 0.025 * delta_deg * delta_deg;
    pw->p = (10.0 - 0.05 * delta_deg) / (rb * d2r);
    const double az = (baz_deg + 180.0) * d2r;
    pw->cos_az = cos(az);
    pw->sin_az = sin(az);
}

void orc_planewave_frame(const orc_grid *g, const orc_planewave *pw, double *frame)
{
    const double rb = g->earth + (g->rgor - (double)(g->nnr - 1) * g->dnr);
    const double thc = g->rgox + (double)(g->nnx - 1) * g->dnx * 0.5;
    const double phc = g->rgoz + (double)(g->nnz - 1) * g->dnz * 0.5;
    const double rbs = rb * sin(thc);
    for (int ix = 1; ix <= g->nnx; ++ix) {
        const double th = g->rgox + (double)(ix - 1) * g->dnx;
        const double dn = rb * (thc - th);
        for (int iz = 1; iz <= g->nnz; ++iz) {
            const double ph = g->rgoz + (double)(iz - 1) * g->dnz;
            const double de = rbs * (ph - phc);
            const double d = dn * pw->cos_az + de * pw->sin_az;
            frame[(size_t)(iz - 1) + (size_t)g->nnz * (size_t)(ix - 1)] = pw->t0 + pw->p * d;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Point sources (no reference counterpart; restates the GPU library's      */
/* start of a local-event solve, csrc/point.cu and fm3dt_solve_point)       */
/* ------------------------------------------------------------------------ */
static double node_slow(const orc_grid *g, const double *veln, int ir, int ix, int iz)
{
    /* 0-based node (ir, ix, iz) -> padded veln with 1-based indices */
    return 1.0 / veln[VELN(g, iz + 1, ix + 1, ir + 1)];
}

static void to_cart(double r, double th, double ph, double *x, double *y, double *z)
{
    const double st = sin(th);
    *x = r * st * cos(ph);
    *y = r * st * sin(ph);
    *z = r * cos(th);
}

/* straight-ray times on box nodes b (0-based, inclusive) of a field */
static void point_analytic(const orc_grid *g, const double *veln, double h, double th, double ph, const int b[6],
                           double *field)
{
    const double fr = (g->rgor - h) / g->dnr, fx = (th - g->rgox) / g->dnx, fz = (ph - g->rgoz) / g->dnz;
    int ir = (int)floor(fr), ix = (int)floor(fx), iz = (int)floor(fz);
    if (ir < 0) ir = 0;
    if (ir > g->nnr - 2) ir = g->nnr - 2;
    if (ix < 0) ix = 0;
    if (ix > g->nnx - 2) ix = g->nnx - 2;
    if (iz < 0) iz = 0;
    if (iz > g->nnz - 2) iz = g->nnz - 2;
    const double ar = fr - ir, ax = fx - ix, az = fz - iz;
    double ss = 0.0;
    for (int c = 0; c < 8; ++c) {
        const int dr = (c >> 2) & 1, dx = (c >> 1) & 1, dz = c & 1;
        const double w = (dr ? ar : 1.0 - ar) * (dx ? ax : 1.0 - ax) * (dz ? az : 1.0 - az);
        ss = ss + w * node_slow(g, veln, ir + dr, ix + dx, iz + dz);
    }
    double xs, ys, zs;
    to_cart(g->earth + h, th, ph, &xs, &ys, &zs);
    for (int kr = b[0]; kr <= b[1]; ++kr)
        for (int kx = b[2]; kx <= b[3]; ++kx)
            for (int kz = b[4]; kz <= b[5]; ++kz) {
                double xn, yn, zn;
                to_cart(g->earth + (g->rgor - (double)kr * g->dnr), g->rgox + (double)kx * g->dnx,
                        g->rgoz + (double)kz * g->dnz, &xn, &yn, &zn);
                const double d = sqrt((xn - xs) * (xn - xs) + (yn - ys) * (yn - ys) + (zn - zs) * (zn - zs));
                field[((size_t)kr * g->nnx + kx) * g->nnz + kz] = d * (0.5 * (ss + node_slow(g, veln, kr, kx, kz)));
            }
}

int orc_point_start(const orc_grid *g, const double *velv, const double *veln, int fom, double h, double th,
                    double ph, int refine, int extent, double *init, unsigned char *fixed)
{
    const int n[3] = {g->nnr, g->nnx, g->nnz};
    const double f[3] = {(g->rgor - h) / g->dnr, (th - g->rgox) / g->dnx, (ph - g->rgoz) / g->dnz};
    int box[6], fix[6];
    for (int a = 0; a < 3; ++a) {
        if (!(f[a] >= 0.0 && f[a] < (double)(n[a] - 1))) return -5;
        const int c = (int)floor(f[a]);
        const int lo = c - extent + 1 > 0 ? c - extent + 1 : 0;
        const int hi = c + extent < n[a] - 1 ? c + extent : n[a] - 1;
        box[2 * a] = lo;
        box[2 * a + 1] = hi;
        fix[2 * a] = (refine && lo > 0) ? lo + 1 : lo;
        fix[2 * a + 1] = (refine && hi < n[a] - 1) ? hi - 1 : hi;
    }
    const size_t N = (size_t)g->nnr * g->nnx * g->nnz;
    for (size_t q = 0; q < N; ++q) { init[q] = INFINITY; fixed[q] = 0; }
    if (!refine) {
        point_analytic(g, veln, h, th, ph, box, init);
    } else {
        orc_grid fg = *g;
        fg.nnr = (box[1] - box[0]) * refine + 1;
        fg.nnx = (box[3] - box[2]) * refine + 1;
        fg.nnz = (box[5] - box[4]) * refine + 1;
        fg.rgor = g->rgor - (double)box[0] * g->dnr;
        fg.rgox = g->rgox + (double)box[2] * g->dnx;
        fg.rgoz = g->rgoz + (double)box[4] * g->dnz;
        fg.dnr = g->dnr / refine;
        fg.dnx = g->dnx / refine;
        fg.dnz = g->dnz / refine;
        const size_t Nf = (size_t)fg.nnr * fg.nnx * fg.nnz;
        const size_t npf = (size_t)(fg.nnr + 3) * (fg.nnx + 3) * (fg.nnz + 3);
        double *vf = (double *)malloc(npf * sizeof(double));
        double *tf = (double *)malloc(Nf * sizeof(double));
        double *of = (double *)malloc(Nf * sizeof(double));
        unsigned char *xf = (unsigned char *)calloc(Nf, 1);
        if (!vf || !tf || !of || !xf) { free(vf); free(tf); free(of); free(xf); return -3; }
        orc_gridder(&fg, velv, vf, NULL);
        const int nf[3] = {fg.nnr, fg.nnx, fg.nnz};
        const double ff[3] = {(fg.rgor - h) / fg.dnr, (th - fg.rgox) / fg.dnx, (ph - fg.rgoz) / fg.dnz};
        int fb[6];
        for (int a = 0; a < 3; ++a) {
            int c = (int)floor(ff[a]);
            if (c < 0) c = 0;
            if (c > nf[a] - 2) c = nf[a] - 2;
            fb[2 * a] = c - 1 > 0 ? c - 1 : 0;
            fb[2 * a + 1] = c + 2 < nf[a] - 1 ? c + 2 : nf[a] - 1;
        }
        for (size_t q = 0; q < Nf; ++q) tf[q] = INFINITY;
        point_analytic(&fg, vf, h, th, ph, fb, tf);
        for (int kr = fb[0]; kr <= fb[1]; ++kr)
            for (int kx = fb[2]; kx <= fb[3]; ++kx)
                for (int kz = fb[4]; kz <= fb[5]; ++kz) xf[((size_t)kr * fg.nnx + kx) * fg.nnz + kz] = 1;
        const int rc = orc_fixed_point_field(&fg, vf, fom, tf, xf, of, 100000, NULL);
        if (rc == 0)
            for (int kr = box[0]; kr <= box[1]; ++kr)
                for (int kx = box[2]; kx <= box[3]; ++kx)
                    for (int kz = box[4]; kz <= box[5]; ++kz) {
                        const size_t q = ((size_t)((kr - box[0]) * refine) * fg.nnx + (size_t)((kx - box[2]) * refine)) *
                                             fg.nnz + (size_t)((kz - box[4]) * refine);
                        init[((size_t)kr * g->nnx + kx) * g->nnz + kz] = of[q];
                    }
        free(vf); free(tf); free(of); free(xf);
        if (rc != 0) return rc;
    }
    for (int kr = fix[0]; kr <= fix[1]; ++kr)
        for (int kx = fix[2]; kx <= fix[3]; ++kx)
            for (int kz = fix[4]; kz <= fix[5]; ++kz) fixed[((size_t)kr * g->nnx + kx) * g->nnz + kz] = 1;
    return 0;
}
