// receivers.cu -- receiver traveltimes (fm3dt_parallel.f90 srtimes,
// F:7040-7248): trilinear interpolation of the traveltime field inside the
// receiver's cell, accumulated in single precision exactly like the REAL(4)
// trr of the reference (each partial sum rounded to float, F:7098-7106).
// The cell and its offsets are located on the host (F:7066-7097).
// Compiled without FMA contraction.
#include <algorithm>
#include <mutex>
#include <string>

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

// ---------------------------------------------------------------------------
// Receiver times without any allocation (fm3dt_receiver_times_noalloc).
//
// Some hosts cannot allocate device memory once they are running: a serving
// loop or a Fortran driver that sized its device memory at start-up and must
// keep that footprint fixed (an allocation can block on the device, fragment
// a pre-sized pool, or fail under a memory quota).  This variant keeps all of
// its scratch -- the receiver coordinates staged on the device, an error word
// and the output staging -- in one file-scope device array of fixed size, and
// locates each receiver's cell on the device instead of in a host table, so a
// call allocates neither device nor host memory.
//
// The array lives in every GPU that loads the library until the process
// exits (about 1.1 MiB).  All calls share it and it keeps the last call's
// contents, so two calls whose work overlaps on the GPU (different streams or
// contexts, same device) race on it; the error word is cleared on every call.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxReceivers = 4096;
constexpr long long kNoAllocMaxTimes = 262144;        // events x receivers
constexpr size_t kNoAllocCoordBytes = 3 * sizeof(double) * (size_t)kNoAllocMaxReceivers;
constexpr size_t kNoAllocStatusBytes = 256;
constexpr size_t kNoAllocBytes = kNoAllocCoordBytes + kNoAllocStatusBytes + sizeof(float) * (size_t)kNoAllocMaxTimes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Same cell location (F:7066-7097, last-subdomain clamp F:7069-7070) and the
// same single-precision accumulation as the table-driven kernel above.
// (also the kernel of fm3dt_receiver_times_device, whose receivers are in
// device memory)
template <typename R>
__global__ void receivers_noalloc_kernel(Geom g, const R *__restrict__ T, const double *__restrict__ base, int nev,
                                         int nrc, const double *__restrict__ rcr, const double *__restrict__ rcx,
                                         const double *__restrict__ rcz, int *__restrict__ bad,
                                         float *__restrict__ out)
{
    const size_t N = (size_t)g.nnx * g.nnz * g.nnr;
    const long long total = (long long)nev * nrc;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(q / nrc), i = (int)(q - (long long)e * nrc);
        RecCell c;
        if (!locate_receiver(g, rcr[i], rcx[i], rcz[i], c)) {
            atomicMin(bad, i);
            continue;
        }
        const int irr = c.irr, irx = c.irx, irz = c.irz;
        const double drr = c.drr, drx = c.drx, drz = c.drz;
        const R *Te = T + (size_t)e * N;
        const double b = base[e];
        float acc = 0.0f;
        for (int j = 1; j <= 2; ++j)
            for (int k = 1; k <= 2; ++k)
                for (int l = 1; l <= 2; ++l) {
                    double produ = (1.0 - fabs(((double)(l - 1) * g.dnz - drz) / g.dnz)) *
                                   (1.0 - fabs(((double)(k - 1) * g.dnx - drx) / g.dnx));
                    produ = produ * (1.0 - fabs(((double)(j - 1) * g.dnr - drr) / g.dnr));
                    const int iz = irz - 1 + l, ix = irx - 1 + k, ir = irr - 1 + j;   // 1-based
                    const double tv = (double)Te[((size_t)(ir - 1) * g.nnx + (ix - 1)) * g.nnz + (iz - 1)] + b;
                    acc = (float)((double)acc + tv * produ);
                }
        out[q] = acc;
    }
}

void launch_receivers_located(const Geom &g, int prec, const void *T, const double *base, int nev, int nrc,
                              const double *rcr, const double *rcx, const double *rcz, int *bad, float *out,
                              cudaStream_t st)
{
    const long long n = (long long)nev * nrc;
    const int blocks = (int)std::min<long long>((n + 127) / 128, 1LL << 20);
    if (blocks <= 0) return;
    if (prec == FM3DT_FP64)
        receivers_noalloc_kernel<double><<<blocks, 128, 0, st>>>(g, (const double *)T, base, nev, nrc, rcr, rcx, rcz,
                                                                 bad, out);
    else
        receivers_noalloc_kernel<float><<<blocks, 128, 0, st>>>(g, (const float *)T, base, nev, nrc, rcr, rcx, rcz,
                                                                bad, out);
}

}  // namespace fm3dt

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, so the address is looked up once per device
// (with that device current) and cached.  The cache is not dropped when the
// host resets a device (cudaDeviceReset); after a reset the cached address
// belongs to the destroyed context.
cudaError_t noalloc_scratch(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, fm3dt::g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_base[dev] = p;
    }
    *out = g_noalloc_base[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int fm3dt_receiver_times_noalloc(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx,
                                            const double *rcz, float *out)
{
    using namespace fm3dt;
    if (!ctx || nrc < 0 || (nrc > 0 && (!rcr || !rcx || !rcz || !out))) return FM3DT_EINVAL;
    const int nev = ctx->nev_solved;
    if (nev < 1) {
        ctx->err = "no solved events";
        return FM3DT_ESTATE;
    }
    if (nrc == 0) return FM3DT_OK;
    if (nrc > kNoAllocMaxReceivers || (long long)nev * nrc > kNoAllocMaxTimes) {
        ctx->err = "fm3dt_receiver_times_noalloc: at most 4096 receivers and 262144 event x receiver times "
                   "per call (fixed scratch); split the call or use fm3dt_receiver_times";
        return FM3DT_EINVAL;
    }
    void *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    cudaStream_t s = ctx->stream;
    double *coords = (double *)base;
    int *bad = (int *)((unsigned char *)base + kNoAllocCoordBytes);
    float *dout = (float *)((unsigned char *)base + kNoAllocCoordBytes + kNoAllocStatusBytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(coords, rcr, nrc * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(coords + nrc, rcx, nrc * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(coords + 2 * nrc, rcz, nrc * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0x7f, sizeof(int), s);     // 0x7f7f7f7f: no bad receiver
    if (e == cudaSuccess) {
        launch_receivers_located(ctx->g, ctx->prec, ctx->d_T, ctx->d_base, nev, nrc, coords, coords + nrc,
                                 coords + 2 * nrc, bad, dout, s);
        e = cudaGetLastError();
        ctx->launches += 1;
    }
    // the status word first: on a bad receiver `out` is left untouched, like
    // fm3dt_receiver_times, which checks every receiver before any work
    int first_bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&first_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && first_bad != 0x7f7f7f7f) {
        ctx->err = "receiver " + std::to_string(first_bad + 1) + " lies outside the grid";
        return FM3DT_ERANGE;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)nev * nrc * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        ctx->err = std::string("fm3dt_receiver_times_noalloc: ") + cudaGetErrorString(e);
        return FM3DT_ECUDA;
    }
    return FM3DT_OK;
}
