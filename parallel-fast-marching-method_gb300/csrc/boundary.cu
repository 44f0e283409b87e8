// boundary.cu -- kernel (c): teleseismic boundary-time injection
// (fm3dt_parallel.f90 start_fmm, F:6894-6961), plus field initialisation and
// conversion helpers.
//
// Frames are double precision end to end.  In the single-precision offset
// mode each event's times are stored relative to its earliest positive
// boundary time (the node start_fmm seeds the heap with, F:6926-6941), so a
// few hundred seconds of absolute time do not consume the float mantissa.
// Compiled without FMA contraction (plane-wave frames match the oracle's
// double-precision formula bit for bit).
#include <cfloat>

#include "internal.h"

namespace fm3dt {

__global__ void planewave_kernel(Geom g, PlaneWaveGeom pg, int nev, const double *__restrict__ params,
                                 double *__restrict__ frames)
{
    const long long nb = (long long)g.nnx * g.nnz;
    const long long total = nb * nev;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(q / nb);
        const long long f = q - (long long)e * nb;
        const int iz = (int)(f % g.nnz);
        const int ix = (int)(f / g.nnz);
        const double t0 = params[4 * e], p = params[4 * e + 1];
        const double ca = params[4 * e + 2], sa = params[4 * e + 3];
        const double th = g.rgox + (double)ix * g.dnx;
        const double dn = pg.rb * (pg.thc - th);
        const double ph = g.rgoz + (double)iz * g.dnz;
        const double de = pg.rbs * (ph - pg.phc);
        const double d = dn * ca + de * sa;
        frames[q] = t0 + p * d;
    }
}

// One block per event: earliest positive boundary time, then the bottom layer
// (fixed nodes and their values) of the event's field.
template <typename R>
__global__ void finalize_kernel(Geom g, const double *__restrict__ frames, R *__restrict__ T,
                                uint8_t *__restrict__ frozen, double *__restrict__ base, int offset_mode)
{
    const int e = blockIdx.x;
    const long long nb = (long long)g.nnx * g.nnz;
    const size_t N = (size_t)nb * g.nnr;
    const double *fr = frames + (size_t)e * nb;
    __shared__ double red[32];
    double m = DBL_MAX;
    for (long long q = threadIdx.x; q < nb; q += blockDim.x) {
        const double v = fr[q];
        if (v > 0.0 && v < m) m = v;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x + 31) / 32) ? red[threadIdx.x] : DBL_MAX;
        for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) red[0] = m;
    }
    __syncthreads();
    const double b = (offset_mode && red[0] < DBL_MAX) ? red[0] : 0.0;
    if (threadIdx.x == 0) base[e] = b;
    R *bottom = T + (size_t)e * N + (size_t)(g.nnr - 1) * (size_t)nb;
    uint8_t *fz = frozen + (size_t)e * nb;
    for (long long q = threadIdx.x; q < nb; q += blockDim.x) {
        const double v = fr[q];
        const bool fix = v > 0.0;                       // F:6932-6936
        fz[q] = fix ? 1 : 0;
        bottom[q] = fix ? (R)(v - b) : (R)INFINITY;
    }
}

// One block per event: the dominant lateral propagation direction of the
// boundary frame (sign of its summed theta and phi differences over pairs of
// fixed nodes), which orders the solver's sweep.  bit 0: times grow with
// theta (sweep +theta), bit 1: times grow with phi; bits 2 and 3: theta /
// phi is a near tie (sweep it both ways).
__global__ void directions_kernel(Geom g, const double *__restrict__ frames, int *__restrict__ dir, double tie_ratio)
{
    const int e = blockIdx.x;
    const long long nb = (long long)g.nnx * g.nnz;
    const double *fr = frames + (size_t)e * nb;
    double sx = 0.0, sz = 0.0;
    for (long long q = threadIdx.x; q < nb; q += blockDim.x) {
        const int iz = (int)(q % g.nnz), ix = (int)(q / g.nnz);
        const double v = fr[q];
        if (!(v > 0.0)) continue;
        if (ix + 1 < g.nnx && fr[q + g.nnz] > 0.0) sx += fr[q + g.nnz] - v;
        if (iz + 1 < g.nnz && fr[q + 1] > 0.0) sz += fr[q + 1] - v;
    }
    __shared__ double rx[32], rz[32];
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if ((threadIdx.x & 31) == 0) { rx[threadIdx.x >> 5] = sx; rz[threadIdx.x >> 5] = sz; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ax = 0.0, az = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) { ax += rx[w]; az += rz[w]; }
        // bits 2 / 3: the wave's theta / phi component is below tie_ratio
        // times the other (0.1: within ~6 degrees of an axis), so its theta /
        // phi direction is ambiguous under heterogeneity and sweeps with that
        // direction reversed are worth their cost
        const double mx = fabs(ax), mz = fabs(az);
        dir[e] = (ax >= 0.0 ? 1 : 0) | (az >= 0.0 ? 2 : 0) | (mx < tie_ratio * mz ? 4 : 0) | (mz < tie_ratio * mx ? 8 : 0);
    }
}

template <typename R>
__global__ void fill_inf_kernel(R *__restrict__ T, size_t n)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        T[q] = (R)INFINITY;
}

__global__ void initial_tiles_kernel(int nev, const int *events, int tiles_per_event, int first, int cnt,
                                     int *list, int *count, int *flag)
{
    const int total = nev * cnt;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        const int k = q / cnt, j = q - k * cnt;
        const int e = events ? events[k] : k;
        const int w = e * tiles_per_event + first + j;
        list[q] = w;
        flag[w] = kFull | kQueued;   // new to the solve: recompute every node
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = total;
}

template <typename R>
__global__ void to_absolute_kernel(const R *__restrict__ T, size_t n, double base, double *__restrict__ out)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const R v = T[q];
        out[q] = isinf((double)v) ? 0.0 : (double)v + base;
    }
}

template <typename R>
__global__ void from_absolute_kernel(const double *__restrict__ in, size_t n, double base, R *__restrict__ T)
{
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const double v = in[q];
        T[q] = v > 0.0 ? (R)(v - base) : (R)INFINITY;
    }
}

static int blocks_for(long long n, int block)
{
    long long b = (n + block - 1) / block;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)(b < 1 ? 1 : b);
}

void launch_planewave_frames(const Geom &g, const PlaneWaveGeom &pg, int nev, const double *params,
                             double *frames, cudaStream_t st)
{
    const long long n = (long long)nev * g.nnx * g.nnz;
    planewave_kernel<<<blocks_for(n, 256), 256, 0, st>>>(g, pg, nev, params, frames);
}

void launch_finalize_frames(const Geom &g, int nev, int prec, const double *frames, void *T, uint8_t *frozen,
                            double *base, cudaStream_t st)
{
    if (prec == FM3DT_FP64)
        finalize_kernel<double><<<nev, 512, 0, st>>>(g, frames, (double *)T, frozen, base, 0);
    else
        finalize_kernel<float><<<nev, 512, 0, st>>>(g, frames, (float *)T, frozen, base, 1);
}

void launch_sweep_directions(const Geom &g, int nev, const double *frames, int *dir, double tie_ratio,
                             cudaStream_t st)
{
    directions_kernel<<<nev, 256, 0, st>>>(g, frames, dir, tie_ratio);
}

void launch_fill_inf(void *T, size_t n, int prec, cudaStream_t st)
{
    if (prec == FM3DT_FP64)
        fill_inf_kernel<double><<<blocks_for((long long)n, 256), 256, 0, st>>>((double *)T, n);
    else
        fill_inf_kernel<float><<<blocks_for((long long)n, 256), 256, 0, st>>>((float *)T, n);
}

void launch_initial_tiles(int nev, const int *events, int tiles_per_event, int first_tile, int count_per_event,
                          int *list, int *count, int *flag, cudaStream_t st)
{
    const long long n = (long long)nev * count_per_event;
    if (n <= 0) return;
    initial_tiles_kernel<<<blocks_for(n, 256), 256, 0, st>>>(nev, events, tiles_per_event, first_tile,
                                                           count_per_event, list, count, flag);
}

// n doubles copied by a kernel between device memory and the device mapping
// of page-locked host memory (either side): many loads and stores in flight
// over the host link, which on some hosts moves data faster than one
// copy-engine transfer.  16-byte elements when both ends allow it.
__global__ void link_copy_kernel(const double2 *__restrict__ src2, double2 *__restrict__ dst2, size_t n2,
                                 const double *__restrict__ src, double *__restrict__ dst, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (src2) {
        for (size_t i = t; i < n2; i += stride) dst2[i] = __ldcs(src2 + i);
    } else {
        for (size_t i = t; i < n; i += stride) dst[i] = __ldcs(src + i);
    }
}

// `bytes` bytes, both ends 16-byte aligned: 16-byte elements, then the
// remaining bytes by the first threads of block 0.
__global__ void link_copy_bytes_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n16,
                                       const unsigned char *__restrict__ src_tail,
                                       unsigned char *__restrict__ dst_tail, int ntail)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = __ldcs(src + i);
    if (blockIdx.x == 0 && (int)threadIdx.x < ntail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

void launch_link_copy_bytes(const void *src, void *dst, size_t bytes, cudaStream_t st)
{
    if (bytes == 0) return;
    const size_t n16 = bytes / 16;
    const int ntail = (int)(bytes % 16);
    link_copy_bytes_kernel<<<152 * 8, 256, 0, st>>>((const uint4 *)src, (uint4 *)dst, n16,
                                                    (const unsigned char *)src + 16 * n16,
                                                    (unsigned char *)dst + 16 * n16, ntail);
}

void launch_link_copy(const double *src, double *dst, size_t n, cudaStream_t st)
{
    if (n == 0) return;
    const bool vec = ((uintptr_t)src % 16 == 0) && ((uintptr_t)dst % 16 == 0) && (n % 2 == 0);
    const int grid = 152 * 8;
    if (vec)
        link_copy_kernel<<<grid, 256, 0, st>>>((const double2 *)src, (double2 *)dst, n / 2, nullptr, nullptr, 0);
    else
        link_copy_kernel<<<grid, 256, 0, st>>>(nullptr, nullptr, 0, src, dst, n);
}

void launch_to_absolute(const Geom &g, int prec, const void *T, size_t offset, double base, double *out,
                        cudaStream_t st)
{
    const size_t n = (size_t)g.nnr * g.nnx * g.nnz;
    if (prec == FM3DT_FP64)
        to_absolute_kernel<double><<<blocks_for((long long)n, 256), 256, 0, st>>>((const double *)T + offset, n,
                                                                                0.0, out);
    else
        to_absolute_kernel<float><<<blocks_for((long long)n, 256), 256, 0, st>>>((const float *)T + offset, n,
                                                                               base, out);
}

void launch_from_absolute(const Geom &g, int prec, const double *in, double base, void *T, size_t offset,
                          cudaStream_t st)
{
    const size_t n = (size_t)g.nnr * g.nnx * g.nnz;
    if (prec == FM3DT_FP64)
        from_absolute_kernel<double><<<blocks_for((long long)n, 256), 256, 0, st>>>(in, n, 0.0,
                                                                                  (double *)T + offset);
    else
        from_absolute_kernel<float><<<blocks_for((long long)n, 256), 256, 0, st>>>(in, n, base,
                                                                                 (float *)T + offset);
}

}  // namespace fm3dt
