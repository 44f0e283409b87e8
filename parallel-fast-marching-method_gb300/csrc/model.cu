// model.cu -- kernel (a): cubic B-spline gridder of the velocity nodes onto
// the propagation grid (fm3dt_parallel.f90 gridder, F:6989-7038), and the
// slowness field the solver reads.
//
// Compiled without FMA contraction so that every double-precision value is
// rounded exactly like the reference's left-to-right Fortran arithmetic.
#include "internal.h"

namespace fm3dt {

__device__ __forceinline__ void bspline4(double u, double w[4])
{
    // F:7002-7005
    const double u2 = u * u, u3 = u * u * u;
    const double om = 1.0 - u;
    w[0] = om * om * om / 6.0;
    w[1] = (4.0 - 6.0 * u2 + 3.0 * u3) / 6.0;
    w[2] = (1.0 + 3.0 * u + 3.0 * u2 - 3.0 * u3) / 6.0;
    w[3] = u3 / 6.0;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// One thread per padded propagation node (indices -1..n+1 on every axis).
// Velocity indices that would fall outside 0..nv+1 are clamped (the
// reference reads outside its array there; inputs that cover the grid, as
// the .vtx convention intends, never clamp).
__global__ void gridder_kernel(Geom g, const double *__restrict__ velv, double *__restrict__ veln)
{
    const int PZ = g.nnz + 3, PX = g.nnx + 3, PR = g.nnr + 3;
    const long long total = (long long)PZ * PX * PR;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int qz = (int)(q % PZ);
        const int qx = (int)((q / PZ) % PX);
        const int qr = (int)(q / ((long long)PZ * PX));
        const int i = qz - 1, j = qx - 1, k = qr - 1;   // reference indices
        const double zpos = g.rgoz + (double)(i - 1) * g.dnz - g.goz;
        const int zi = (int)floor(zpos / g.dvz) + 1;
        const double distz = zpos - (double)(zi - 1) * g.dvz;
        const double xpos = g.rgox + (double)(j - 1) * g.dnx - g.gox;
        const int xi = (int)floor(xpos / g.dvx) + 1;
        const double distx = xpos - (double)(xi - 1) * g.dvx;
        const int ri = (int)floor((g.gor - g.rgor + (double)(k - 1) * g.dnr) / g.dvr) + 1;
        const double distr = -(g.rgor - (double)(k - 1) * g.dnr) + (g.gor - (double)(ri - 1) * g.dvr);
        double wi[4], vi[4], ui[4];
        bspline4(distz / g.dvz, wi);
        bspline4(distx / g.dvx, vi);
        bspline4(distr / g.dvr, ui);
        const int NVR = g.nvr + 2, NVX = g.nvx + 2;
        double sumi = 0.0;
        for (int i1 = 0; i1 < 4; ++i1) {
            const int c = clampi(zi - 1 + i1, 0, g.nvz + 1);
            double sumj = 0.0;
            for (int j1 = 0; j1 < 4; ++j1) {
                const int b = clampi(xi - 1 + j1, 0, g.nvx + 1);
                const double *col = velv + (size_t)NVR * ((size_t)b + (size_t)NVX * (size_t)c);
                double sumk = 0.0;
                for (int k1 = 0; k1 < 4; ++k1) {
                    const int a = clampi(ri - 1 + k1, 0, g.nvr + 1);
                    sumk = sumk + ui[k1] * __ldg(col + a);
                }
                sumj = sumj + vi[j1] * sumk;
            }
            sumi = sumi + wi[i1] * sumj;
        }
        veln[q] = sumi;
    }
}

// slowness = 1/velocity at the interior nodes (F:642), stored in the solver's
// precision, phi fastest.
template <typename R>
__global__ void slowness_kernel(Geom g, const double *__restrict__ veln, R *__restrict__ s)
{
    const long long total = (long long)g.nnz * g.nnx * g.nnr;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(q % g.nnz);
        const int ix = (int)((q / g.nnz) % g.nnx);
        const int ir = (int)(q / ((long long)g.nnz * g.nnx));
        const size_t p = (size_t)(iz + 2) + (size_t)(g.nnz + 3) * ((size_t)(ix + 2) + (size_t)(g.nnx + 3) * (size_t)(ir + 2));
        s[q] = (R)(1.0 / veln[p]);
    }
}

static int grid_for(long long n, int block)
{
    long long b = (n + block - 1) / block;
    if (b > 152LL * 64) b = 152LL * 64;
    return (int)(b < 1 ? 1 : b);
}

void launch_gridder(const Geom &g, const double *velv, double *veln, cudaStream_t st)
{
    const long long n = (long long)(g.nnz + 3) * (g.nnx + 3) * (g.nnr + 3);
    gridder_kernel<<<grid_for(n, 256), 256, 0, st>>>(g, velv, veln);
}

void launch_slowness(const Geom &g, const double *veln, void *s, int prec, cudaStream_t st)
{
    const long long n = (long long)g.nnz * g.nnx * g.nnr;
    if (prec == FM3DT_FP64)
        slowness_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(g, veln, (double *)s);
    else
        slowness_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(g, veln, (float *)s);
}

}  // namespace fm3dt
