/*
 * fm3dt_subinv.h -- C ABI of the subspace inversion step (host code).
 *
 * Replaces one run of the reference's subinv program (subinv.f90, "S"
 * below): it assembles the picked traveltime residuals and Frechet rows
 * (S:335-432), builds the transpose of the Frechet matrix, and
 * computes the model perturbation with the n-dimensional subspace method
 * (S:547-1002): gradient, optional second-derivative smoothing, Krylov-like
 * basis, orthonormalisation with rank reduction, projected
 * Hessian and its inverse.  Host-side, by design: the system is
 * at most a few thousand unknowns and a few tens of basis vectors.
 *
 * Precision: FM3DT_SUBINV_FP32 follows the reference's REAL(4) arithmetic
 * (and its REAL(8) grid-header promotions) in the reference's summation
 * order; FM3DT_SUBINV_FP64 computes everything in double.
 *
 * Inputs are the contents of the files the reference reads, already parsed
 * (all REAL(4) file values passed as float):
 *   gridi.vtx  -> mo, cm_sd   (columns 1 and 2 of the velocity records)
 *   gridc.vtx  -> mc          (current model; nmpv values, then the nmps
 *                              station terms of stationres.dat if invst)
 *   otimes.dat -> tstat, dobs, cd_sd   (one row per source-receiver pair)
 *   rtravel.out-> mtimes,  rtimes.dat -> rtimes
 *   frechet.out-> row_ptr/cols/vals, one CSR row per source-receiver pair
 *                (every pair, picked or not, in file order)
 *   sources.dat / receivers.dat -> nra, nsrc[], nrc[]
 */
#ifndef FM3DT_SUBINV_H
#define FM3DT_SUBINV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FM3DT_SUBINV_FP32 = 0,      /* the reference's REAL(4) arithmetic */
    FM3DT_SUBINV_FP64 = 1
};

enum {
    FM3DT_SUBINV_OK = 0,
    FM3DT_SUBINV_EINVAL = -1,   /* bad argument or inconsistent sizes */
    FM3DT_SUBINV_ESINGULAR = -2,/* projected matrix singular */
    FM3DT_SUBINV_ENOCONV = -3,  /* orthonormalisation did not converge */
    FM3DT_SUBINV_ETOOBIG = -4   /* Frechet entries exceed fracg*ntr*nmp */
};

/* subinv.in parameters and the velocity grid header
 * (gridi.vtx lines 1-3: node counts, origin km/deg/deg, spacing km/deg/deg). */
typedef struct {
    int nvr, nvt, nvp;
    double gor, got, gop;
    double dnr, dnt, dnp;
    int rmtr;                   /* remove each source's mean model residual */
    float epsilon;              /* damping */
    int subdim;                 /* subspace dimension, 1..50 */
    int asds;                   /* second-derivative smoothing on/off */
    float eta;                  /* smoothing weight */
    int invst;                  /* invert for station terms */
    float stdf;                 /* station-term damping */
    float fracg;                /* fraction of ntr*nmp allowed as Frechet entries */
    float earth;                /* Earth radius km */
    int precision;              /* FM3DT_SUBINV_FP32 or FM3DT_SUBINV_FP64 */
} fm3dt_subinv_desc;

/* One inversion step.  nmpv = (nvr+2)(nvt+2)(nvp+2); nmp = nmpv, plus the
 * total receiver count when invst = 1.  ntr = sum over arrays of
 * nsrc[a]*nrc[a].  dm receives the model perturbation (nmp doubles; the new
 * model the reference writes is mc + dm in REAL(4)).  subdim_used receives
 * the subspace dimension after rank reduction.  msg (nullable)
 * receives the reference's informational or error text. */
int fm3dt_subinv_step(const fm3dt_subinv_desc *d, int nra, const int *nsrc, const int *nrc,
                      const float *mo, const float *cm_sd, const float *mc,
                      const int *tstat, const float *dobs, const float *cd_sd,
                      const float *mtimes, const float *rtimes,
                      const int64_t *row_ptr, const int32_t *cols, const float *vals,
                      double *dm, int *subdim_used, char *msg, int msg_len);

#ifdef __cplusplus
}
#endif
#endif
