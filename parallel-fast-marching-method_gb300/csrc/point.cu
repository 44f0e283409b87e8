// point.cu -- start of a point-source solve (local events).
//
// The reference has no point sources: its sources are teleseismic boundary
// frames (start_fmm, F:6894-6961).  Local events start from a box of nodes
// around the source whose times are fixed before the rounds run:
//   * straight-ray times: distance from the source (Cartesian chord) times
//     the mean of the slowness at the source (trilinear in the cell) and at
//     the node, in double precision;
//   * or, on a k-times refined grid over the box, the same start within two
//     fine cells of the source, solved to its fixed point, then sampled at the
//     coarse nodes (every k-th fine node).
// Compiled without FMA contraction: the oracle restates these formulas.
#include <cmath>

#include "internal.h"

namespace fm3dt {

namespace {

__device__ __forceinline__ double slow_at(const Geom &g, const double *veln, int ir, int ix, int iz)
{
    // padded veln, indices -1..n+1 (1-based nodes at +1)
    const size_t q = (size_t)(iz + 2) + (size_t)(g.nnz + 3) * ((size_t)(ix + 2) + (size_t)(g.nnx + 3) * (size_t)(ir + 2));
    return 1.0 / veln[q];
}

__device__ __forceinline__ void cart(double r, double th, double ph, double &x, double &y, double &z)
{
    const double st = sin(th);
    x = r * st * cos(ph);
    y = r * st * sin(ph);
    z = r * cos(th);
}

}  // namespace

// One block per event: straight-ray times at the nodes of the event's box.
template <typename R>
__global__ void point_analytic_kernel(Geom g, const double *__restrict__ veln, const PointSource *__restrict__ src,
                                      const int *__restrict__ box, R *__restrict__ T)
{
    const int e = blockIdx.x;
    const PointSource p = src[e];
    const size_t N = (size_t)g.nnr * g.nnx * g.nnz;
    // source cell and its trilinear slowness
    const double fr = (g.rgor - p.h) / g.dnr, fx = (p.th - g.rgox) / g.dnx, fz = (p.ph - g.rgoz) / g.dnz;
    const int ir = min(max((int)floor(fr), 0), g.nnr - 2);
    const int ix = min(max((int)floor(fx), 0), g.nnx - 2);
    const int iz = min(max((int)floor(fz), 0), g.nnz - 2);
    const double ar = fr - ir, ax = fx - ix, az = fz - iz;
    double ss = 0.0;
    for (int c = 0; c < 8; ++c) {
        const int dr = (c >> 2) & 1, dx = (c >> 1) & 1, dz = c & 1;
        const double w = (dr ? ar : 1.0 - ar) * (dx ? ax : 1.0 - ax) * (dz ? az : 1.0 - az);
        ss = ss + w * slow_at(g, veln, ir + dr, ix + dx, iz + dz);
    }
    double xs, ys, zs;
    cart(g.earth + p.h, p.th, p.ph, xs, ys, zs);
    const int *b = box + 6 * e;
    const int nr = b[1] - b[0] + 1, nx = b[3] - b[2] + 1, nz = b[5] - b[4] + 1;
    for (int q = threadIdx.x; q < nr * nx * nz; q += blockDim.x) {
        const int kz = b[4] + q % nz, kx = b[2] + (q / nz) % nx, kr = b[0] + q / (nz * nx);
        double xn, yn, zn;
        cart(g.earth + (g.rgor - (double)kr * g.dnr), g.rgox + (double)kx * g.dnx, g.rgoz + (double)kz * g.dnz, xn,
             yn, zn);
        const double d = sqrt((xn - xs) * (xn - xs) + (yn - ys) * (yn - ys) + (zn - zs) * (zn - zs));
        const double t = d * (0.5 * (ss + slow_at(g, veln, kr, kx, kz)));
        T[(size_t)e * N + ((size_t)kr * g.nnx + kx) * g.nnz + kz] = (R)t;
    }
}

// Coarse nodes of a box from a refined grid whose node (0,0,0) is the box's
// corner and whose spacing is 1/refine of the coarse one.
template <typename R>
__global__ void point_sample_kernel(const R *__restrict__ Tf, int nnx_f, int nnz_f, int refine, int r0, int r1,
                                    int x0, int x1, int z0, int z1, int nnx, int nnz, R *__restrict__ T)
{
    const int nr = r1 - r0 + 1, nx = x1 - x0 + 1, nz = z1 - z0 + 1;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nr * nx * nz; q += gridDim.x * blockDim.x) {
        const int kz = q % nz, kx = (q / nz) % nx, kr = q / (nz * nx);
        const size_t f = ((size_t)(kr * refine) * nnx_f + (size_t)(kx * refine)) * nnz_f + (size_t)(kz * refine);
        T[((size_t)(r0 + kr) * nnx + (x0 + kx)) * nnz + (z0 + kz)] = Tf[f];
    }
}

void launch_point_analytic(const Geom &g, int prec, const double *veln, int nev, const PointSource *src,
                           const int *box, void *T, cudaStream_t st)
{
    if (prec == FM3DT_FP64)
        point_analytic_kernel<double><<<nev, 256, 0, st>>>(g, veln, src, box, (double *)T);
    else
        point_analytic_kernel<float><<<nev, 256, 0, st>>>(g, veln, src, box, (float *)T);
}

void launch_point_sample(int prec, const void *Tf, int nnx_f, int nnz_f, int refine, const int box[6], int nnx,
                         int nnz, void *T_event, cudaStream_t st)
{
    const int n = (box[1] - box[0] + 1) * (box[3] - box[2] + 1) * (box[5] - box[4] + 1);
    const int blocks = (n + 255) / 256;
    if (prec == FM3DT_FP64)
        point_sample_kernel<double><<<blocks, 256, 0, st>>>((const double *)Tf, nnx_f, nnz_f, refine, box[0], box[1],
                                                            box[2], box[3], box[4], box[5], nnx, nnz,
                                                            (double *)T_event);
    else
        point_sample_kernel<float><<<blocks, 256, 0, st>>>((const float *)Tf, nnx_f, nnz_f, refine, box[0], box[1],
                                                           box[2], box[3], box[4], box[5], nnx, nnz, (float *)T_event);
}

// One block per event: the tiles that overlap its box start active, every
// node recomputed.
__global__ void initial_tiles_box_kernel(int tiles_per_event, int ntx, int ntz, int tr, int tx, int tz,
                                         const int *__restrict__ box, int *list, int *count, int *flag)
{
    const int e = blockIdx.x;
    const int *b = box + 6 * e;
    const int a0 = b[0] / tr, a1 = b[1] / tr, c0 = b[2] / tx, c1 = b[3] / tx, d0 = b[4] / tz, d1 = b[5] / tz;
    const int na = a1 - a0 + 1, nc = c1 - c0 + 1, nd = d1 - d0 + 1;
    for (int q = threadIdx.x; q < na * nc * nd; q += blockDim.x) {
        const int d = d0 + q % nd, c = c0 + (q / nd) % nc, a = a0 + q / (nd * nc);
        const int w = e * tiles_per_event + (a * ntx + c) * ntz + d;
        flag[w] = kFull | kQueued;
        list[atomicAdd(count, 1)] = w;
    }
}

void launch_initial_tiles_box(int nev, int tiles_per_event, int ntx, int ntz, int tr, int tx, int tz,
                              const int *box, int *list, int *count, int *flag, cudaStream_t st)
{
    cudaMemsetAsync(count, 0, sizeof(int), st);
    initial_tiles_box_kernel<<<nev, 128, 0, st>>>(tiles_per_event, ntx, ntz, tr, tx, tz, box, list, count, flag);
}

}  // namespace fm3dt
