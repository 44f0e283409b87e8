// receivers.cu -- receiver traveltimes (fm3dt_parallel.f90 srtimes,
// F:7040-7248): trilinear interpolation of the traveltime field inside the
// receiver's cell, accumulated in single precision exactly like the REAL(4)
// trr of the reference (each partial sum rounded to float, F:7098-7106).
// The cell and its offsets are located on the host (F:7066-7097).
// Compiled without FMA contraction.
#include "internal.h"

namespace fm3dt {

template <typename R>
__global__ void receivers_kernel(Geom g, const R *__restrict__ T, const double *__restrict__ base, int nev, int nrc,
                                 const RecCell *__restrict__ cells, float *__restrict__ out)
{
    const size_t NB = (size_t)g.nnx * g.nnz;
    const size_t N = NB * g.nnr;
    const long long total = (long long)nev * nrc;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(q / nrc), i = (int)(q - (long long)e * nrc);
        const RecCell c = cells[i];
        const R *Te = T + (size_t)e * N;
        const double b = base[e];
        float acc = 0.0f;
        for (int j = 1; j <= 2; ++j)
            for (int k = 1; k <= 2; ++k)
                for (int l = 1; l <= 2; ++l) {
                    double produ = (1.0 - fabs(((double)(l - 1) * g.dnz - c.drz) / g.dnz)) *
                                   (1.0 - fabs(((double)(k - 1) * g.dnx - c.drx) / g.dnx));
                    produ = produ * (1.0 - fabs(((double)(j - 1) * g.dnr - c.drr) / g.dnr));
                    const int iz = c.irz - 1 + l, ix = c.irx - 1 + k, ir = c.irr - 1 + j;   // 1-based
                    const double tv = (double)Te[((size_t)(ir - 1) * g.nnx + (ix - 1)) * g.nnz + (iz - 1)] + b;
                    acc = (float)((double)acc + tv * produ);
                }
        out[q] = acc;
    }
}

void launch_receivers(const Geom &g, int prec, const void *T, const double *base, int nev, int nrc,
                      const RecCell *cells, float *out, cudaStream_t st)
{
    const long long n = (long long)nev * nrc;
    int blocks = (int)((n + 127) / 128);
    if (blocks < 1) blocks = 1;
    if (prec == FM3DT_FP64)
        receivers_kernel<double><<<blocks, 128, 0, st>>>(g, (const double *)T, base, nev, nrc, cells, out);
    else
        receivers_kernel<float><<<blocks, 128, 0, st>>>(g, (const float *)T, base, nev, nrc, cells, out);
}

}  // namespace fm3dt
