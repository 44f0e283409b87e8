// rays.cu -- kernel (d): ray back-tracing down the traveltime gradient and
// Frechet-row assembly (fm3dt_parallel.f90 parallel_rpaths, F:7250-7777, and
// the writer's row merge, F:6503-6599).
//
// One thread traces one (event, receiver) ray over the whole grid, so the
// reference's ray hand-off between subdomains (F:6464-6501) and the partial
// rows it creates disappear; the global outer faces stop a ray exactly where
// the reference's boundary subdomains stop it (clip to the first face
// crossed, F:7474-7541).  The ray path is double precision like the
// reference's (with the single-precision field, each step's direction is
// formed in single precision, see rays_kernel); the row's weights are single
// precision and accumulate in the same order as the reference's REAL(4) fdm
// (F:7722-7732), including its quirks:
// the segment clipped at the grid face is integrated with the full nominal
// step length (dinc from vrat*dpl), and the start-point B-spline weights of a
// sub-segment that follows a velocity-cell crossing keep the indices of the
// new cell (F:7647-7652, 7717-7732).
// Compiled without FMA contraction.
#include "internal.h"

namespace fm3dt {

// Single-precision Frechet weights: the row is accumulated in REAL(4), so its
// weights need no more; the FP64 pipe (a small fraction of FP32 throughput on
// this GPU) is kept for the ray path itself, whose end points must match.
__device__ __forceinline__ void bsplf(float u, float w[4])
{
    const float sixth = 1.0f / 6.0f;
    const float u2 = u * u, u3 = u * u * u;
    const float om = 1.0f - u;
    w[0] = om * om * om * sixth;
    w[1] = (4.0f - 6.0f * u2 + 3.0f * u3) * sixth;
    w[2] = (1.0f + 3.0f * u + 3.0f * u2 - 3.0f * u3) * sixth;
    w[3] = u3 * sixth;
}

struct RayCtx {
    const Geom *g;
    const double *veln;
};

__device__ __forceinline__ double veln_at(const Geom &g, const double *veln, int iz, int ix, int ir)
{
    return veln[(size_t)(iz + 1) + (size_t)(g.nnz + 3) * ((size_t)(ix + 1) + (size_t)(g.nnx + 3) * (size_t)(ir + 1))];
}

// trilinear velocity at a point of propagation cell (ipz,ipx,ipr) (F:7629-7641),
// in single precision (it only weights the Frechet row); inr/inx/inz: reciprocals
// of the node spacings
__device__ float trilinf(const Geom &g, const double *veln, int ipz, int ipx, int ipr, float drr, float drx, float drz,
                         float dnr, float dnx, float dnz, float inr, float inx, float inz)
{
    float vel = 0.0f;
    for (int k = 1; k <= 2; ++k)
        for (int l = 1; l <= 2; ++l)
            for (int m = 1; m <= 2; ++m) {
                float produ = (1.0f - fabsf(((float)(m - 1) * dnz - drz) * inz));
                produ = produ * (1.0f - fabsf(((float)(l - 1) * dnx - drx) * inx));
                produ = produ * (1.0f - fabsf(((float)(k - 1) * dnr - drr) * inr));
                if (ipz - 1 + m <= g.nnz + 1 && ipx - 1 + l <= g.nnx + 1 && ipr - 1 + k <= g.nnr + 1)
                    vel = vel + (float)veln_at(g, veln, ipz - 1 + m, ipx - 1 + l, ipr - 1 + k) * produ;
            }
    return vel;
}

constexpr int kRayBlock = 64;

template <typename R>
__global__ void __launch_bounds__(kRayBlock) rays_kernel(RayArgs a)
{
    __shared__ float ray_acc[64 * kRayBlock];
    const Geom g = a.g;
    // the rays of a.nlist listed events (a.events), or of all a.nev events;
    // a ray's row, end point and flag index is its event's row e * nrc + i
    const int total = (a.events ? a.nlist : a.nev) * a.nrc;
    const size_t NB = (size_t)g.nnx * g.nnz;
    const size_t N = NB * g.nnr;
    const size_t nmp = (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2);
    const int maxrp = 100000;        // F:7262
    const double dpl = g.dnr;        // F:7290
    const float fnr = (float)g.dnr, fnx = (float)g.dnx, fnz = (float)g.dnz;
    const float inr = 1.0f / fnr, inx = 1.0f / fnx, inz = 1.0f / fnz;
    const double ivr_ = 1.0 / g.dvr, ivx_ = 1.0 / g.dvx, ivz_ = 1.0 / g.dvz;
    // With the single-precision (offset) field the direction of each step --
    // gradient, its norm, sin(colatitude) -- is formed in single precision
    // (G = float), and cells are located by multiplying with the spacings'
    // reciprocals; positions, crossings and clipping stay in double.  With
    // the double-precision field everything is the reference's double
    // arithmetic (G = double, divisions).
    using G = R;
    constexpr bool kFast = sizeof(R) == sizeof(float);
    const double inr_ = 1.0 / g.dnr, inx_ = 1.0 / g.dnx, inz_ = 1.0 / g.dnz;
    auto cellr = [&](double v) { return kFast ? (int)floor((g.rgor - v) * inr_) + 1 : (int)floor((g.rgor - v) / g.dnr) + 1; };
    auto cellx = [&](double v) { return kFast ? (int)floor((v - g.rgox) * inx_) + 1 : (int)floor((v - g.rgox) / g.dnx) + 1; };
    auto cellz = [&](double v) { return kFast ? (int)floor((v - g.rgoz) * inz_) + 1 : (int)floor((v - g.rgoz) / g.dnz) + 1; };
    auto vcellr = [&](double v) { return kFast ? (int)floor((g.gor - v) * ivr_) + 1 : (int)floor((g.gor - v) / g.dvr) + 1; };
    auto vcellx = [&](double v) { return kFast ? (int)floor((v - g.gox) * ivx_) + 1 : (int)floor((v - g.gox) / g.dvx) + 1; };
    auto vcellz = [&](double v) { return kFast ? (int)floor((v - g.goz) * ivz_) + 1 : (int)floor((v - g.goz) / g.dvz) + 1; };
    for (int qq = blockIdx.x * blockDim.x + threadIdx.x; qq < total; qq += gridDim.x * blockDim.x) {
        const int kk = qq / a.nrc, i = qq - kk * a.nrc;
        const int e = a.events ? a.events[kk] : kk;
        const int q = e * a.nrc + i;
        const R *Te = (const R *)a.T + (size_t)e * N;
        float *fdm = a.fdm ? a.fdm + nmp * (size_t)q : nullptr;
        // The row's sums for the velocity cell whose 4 x 4 x 4 B-spline
        // support the ray is in (one slot per support node, in shared memory,
        // this thread's slots strided by the block size so that a warp's
        // threads hit 32 different banks); added to the row when the ray
        // moves to another cell and at its end.  In the row each node's value
        // is the REAL(4) sum of its terms in ray order, grouped per cell visit.
        float *acc = ray_acc + threadIdx.x;
        int acc_r = -1, acc_x = -1, acc_z = -1;
        for (int t = 0; t < 64; ++t) acc[t * kRayBlock] = 0.0f;
        auto flush = [&]() {
            if (acc_r < 0) return;
            const size_t zstride = (size_t)(g.nvr + 2) * (size_t)(g.nvx + 2);
            // a row of four nodes (along phi) at a time: four independent
            // loads, then the four sums stored
#pragma unroll 1
            for (int nm = 0; nm < 16; ++nm) {
                const int n = nm >> 2, m = nm & 3;
                float *p = fdm + (size_t)(acc_r - 1 + n) +
                           (size_t)(g.nvr + 2) * ((size_t)(acc_x - 1 + m) + (size_t)(g.nvx + 2) * (size_t)(acc_z - 1));
                const float o0 = p[0], o1 = p[zstride], o2 = p[2 * zstride], o3 = p[3 * zstride];
                float *c = acc + (nm * 4) * kRayBlock;
                p[0] = c[0] + o0;
                p[zstride] = c[kRayBlock] + o1;
                p[2 * zstride] = c[2 * kRayBlock] + o2;
                p[3 * zstride] = c[3 * kRayBlock] + o3;
                c[0] = 0.0f;
                c[kRayBlock] = 0.0f;
                c[2 * kRayBlock] = 0.0f;
                c[3 * kRayBlock] = 0.0f;
            }
        };
        auto TD = [&](int iz, int ix, int ir) -> G {
            return (G)Te[((size_t)(ir - 1) * g.nnx + (ix - 1)) * g.nnz + (iz - 1)];
        };
        int st = 0;
        double rgr = a.rcr[i], rgx = a.rcx[i], rgz = a.rcz[i];
        // the start cell (F:7320-7333), formed and checked in double precision
        // so that a non-finite or huge coordinate is rejected, not converted
        double fpr = floor((g.rgor - rgr) / g.dnr) + 1.0;
        double fpx = floor((rgx - g.rgox) / g.dnx) + 1.0;
        double fpz = floor((rgz - g.rgoz) / g.dnz) + 1.0;
        if (fpr == (double)g.nnr) fpr -= 1.0;
        if (fpx == (double)g.nnx) fpx -= 1.0;
        if (fpz == (double)g.nnz) fpz -= 1.0;
        const bool inside = fpr >= 1.0 && fpr < (double)g.nnr && fpx >= 1.0 && fpx < (double)g.nnx &&
                            fpz >= 1.0 && fpz < (double)g.nnz;
        int ipr = inside ? (int)fpr : 0, ipx = inside ? (int)fpx : 0, ipz = inside ? (int)fpz : 0;
        int steps = 0;
        if (!inside && a.flags) atomicMin(&a.flags[1], q);
        if (inside) {
            for (int jstep = 1; jstep <= maxrp; ++jstep) {
                ++steps;
                G dtr = 0;
                int temp = 0;
                if (TD(ipz, ipx, ipr + 1) < TD(ipz, ipx, ipr)) { dtr = dtr + TD(ipz, ipx, ipr + 1) - TD(ipz, ipx, ipr); temp++; }
                if (TD(ipz + 1, ipx, ipr + 1) < TD(ipz + 1, ipx, ipr)) { dtr = dtr + TD(ipz + 1, ipx, ipr + 1) - TD(ipz + 1, ipx, ipr); temp++; }
                if (TD(ipz + 1, ipx + 1, ipr + 1) < TD(ipz + 1, ipx + 1, ipr)) { dtr = dtr + TD(ipz + 1, ipx + 1, ipr + 1) - TD(ipz + 1, ipx + 1, ipr); temp++; }
                if (TD(ipz, ipx + 1, ipr + 1) < TD(ipz, ipx + 1, ipr)) { dtr = dtr + TD(ipz, ipx + 1, ipr + 1) - TD(ipz, ipx + 1, ipr); temp++; }
                if (temp != 0) dtr = dtr / ((G)temp * (G)g.dnr);
                const G rcell = (G)(g.earth + g.rgor - (double)(ipr - 1) * g.dnr);
                G dtx = TD(ipz, ipx + 1, ipr) - TD(ipz, ipx, ipr);
                dtx = dtx + TD(ipz + 1, ipx + 1, ipr) - TD(ipz + 1, ipx, ipr);
                dtx = dtx + TD(ipz + 1, ipx + 1, ipr + 1) - TD(ipz + 1, ipx, ipr + 1);
                dtx = dtx + TD(ipz, ipx + 1, ipr + 1) - TD(ipz, ipx, ipr + 1);
                dtx = dtx / ((G)4 * rcell * (G)g.dnx);
                const G sx = sin((G)rgx);
                G dtz = TD(ipz + 1, ipx, ipr) - TD(ipz, ipx, ipr);
                dtz = dtz + TD(ipz + 1, ipx + 1, ipr + 1) - TD(ipz, ipx + 1, ipr + 1);
                dtz = dtz + TD(ipz + 1, ipx + 1, ipr) - TD(ipz, ipx + 1, ipr);
                dtz = dtz + TD(ipz + 1, ipx, ipr + 1) - TD(ipz, ipx, ipr + 1);
                dtz = dtz / ((G)4 * rcell * sx * (G)g.dnz);
                const G crad = (G)(g.earth + rgr);
                const G rd1 = sqrt(dtr * dtr + dtx * dtx + dtz * dtz);
                double nr = rgr + (double)((G)dpl * dtr / rd1);
                double nx = rgx - (double)((G)dpl * dtx / (crad * rd1));
                double nz = rgz - (double)((G)dpl * dtz / (crad * sx * rd1));
                const int ipro = ipr, ipxo = ipx, ipzo = ipz;
                ipr = cellr(nr);
                ipx = cellx(nx);
                ipz = cellz(nz);
                const bool swr = (ipr < 1 || ipr >= g.nnr);
                const bool swx = (ipx < 1 || ipx >= g.nnx);
                const bool swz = (ipz < 1 || ipz >= g.nnz);
                bool stop = false;
                if (swr || swx || swz) {
                    int sw = 0;
                    double atio = 0.0;
                    if (swr) {
                        double ri;
                        if (ipr < 1) { ri = g.rgor; ipr = 1; }
                        else { ri = g.rgor - (double)(g.nnr - 1) * g.dnr; ipr = g.nnr - 1; }
                        atio = (ri - rgr) / (nr - rgr);
                        sw = 1;
                    }
                    if (swx) {
                        double xi;
                        if (ipx < 1) { xi = g.rgox; ipx = 1; }
                        else { xi = g.rgox + (double)(g.nnx - 1) * g.dnx; ipx = g.nnx - 1; }
                        const double r1 = (xi - rgx) / (nx - rgx);
                        if (sw == 1) { if (r1 < atio) { atio = r1; sw = 2; } }
                        else { atio = r1; sw = 2; }
                    }
                    if (swz) {
                        double zi;
                        if (ipz < 1) { zi = g.rgoz; ipz = 1; }
                        else { zi = g.rgoz + (double)(g.nnz - 1) * g.dnz; ipz = g.nnz - 1; }
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
                    stop = true;
                }
                if (fdm) {
                    const int ivr = vcellr(nr);
                    const int ivx = vcellx(nx);
                    const int ivz = vcellz(nz);
                    const int ivro = vcellr(rgr);
                    const int ivxo = vcellx(rgx);
                    const int ivzo = vcellz(rgz);
                    double vrat[4];
                    int chp[4];
                    int nhp = 0;
                    if (ivr != ivro) {
                        const double ri = (ivr > ivro) ? g.gor - (double)(ivr - 1) * g.dvr : g.gor - (double)ivr * g.dvr;
                        vrat[0] = (ri - rgr) / (nr - rgr);
                        chp[0] = 1;
                        nhp = 1;
                    }
                    if (ivx != ivxo) {
                        const double xi = (ivx > ivxo) ? g.gox + (double)(ivx - 1) * g.dvx : g.gox + (double)ivx * g.dvx;
                        const double r1 = (xi - rgx) / (nx - rgx);
                        nhp++;
                        if (nhp == 1) { vrat[0] = r1; chp[0] = 2; }
                        else if (r1 >= vrat[0]) { vrat[1] = r1; chp[1] = 2; }
                        else { vrat[1] = vrat[0]; chp[1] = chp[0]; vrat[0] = r1; chp[0] = 2; }
                    }
                    if (ivz != ivzo) {
                        const double zi = (ivz > ivzo) ? g.goz + (double)(ivz - 1) * g.dvz : g.goz + (double)ivz * g.dvz;
                        const double r1 = (zi - rgz) / (nz - rgz);
                        nhp++;
                        if (nhp == 1) { vrat[0] = r1; chp[0] = 3; }
                        else if (nhp == 2) {
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
                    double drr = (g.rgor - rgr) - (double)(ipro - 1) * g.dnr;
                    double drx = (rgx - g.rgox) - (double)(ipxo - 1) * g.dnx;
                    double drz = (rgz - g.rgoz) - (double)(ipzo - 1) * g.dnz;
                    float vel = trilinf(g, a.veln, ipzo, ipxo, ipro, (float)drr, (float)drx, (float)drz, fnr, fnx, fnz,
                                        inr, inx, inz);
                    float iv2 = 1.0f / (vel * vel);
                    float ui[4], vi[4], wi[4], uio[4], vio[4], wio[4];
                    drr = (g.gor - rgr) - (double)(ivro - 1) * g.dvr;
                    drx = (rgx - g.gox) - (double)(ivxo - 1) * g.dvx;
                    drz = (rgz - g.goz) - (double)(ivzo - 1) * g.dvz;
                    bsplf((float)(drr * ivr_), ui);
                    bsplf((float)(drx * ivx_), vi);
                    bsplf((float)(drz * ivz_), wi);
                    int ivrt = ivro, ivxt = ivxo, ivzt = ivzo;
                    for (int k = 0; k < nhp; ++k) {
                        const float iv2o = iv2;
                        for (int m = 0; m < 4; ++m) { uio[m] = ui[m]; vio[m] = vi[m]; wio[m] = wi[m]; }
                        if (k > 0) {
                            if (chp[k - 1] == 1) ivrt = ivr;
                            else if (chp[k - 1] == 2) ivxt = ivx;
                            else if (chp[k - 1] == 3) ivzt = ivz;
                        }
                        const double rigz = rgz + vrat[k] * (nz - rgz);
                        const double rigx = rgx + vrat[k] * (nx - rgx);
                        const double rigr = rgr + vrat[k] * (nr - rgr);
                        const int iprt = cellr(rigr);
                        const int ipxt = cellx(rigx);
                        const int ipzt = cellz(rigz);
                        drr = (g.rgor - rigr) - (double)(iprt - 1) * g.dnr;
                        drx = (rigx - g.rgox) - (double)(ipxt - 1) * g.dnx;
                        drz = (rigz - g.rgoz) - (double)(ipzt - 1) * g.dnz;
                        vel = trilinf(g, a.veln, ipzt, ipxt, iprt, (float)drr, (float)drx, (float)drz, fnr, fnx, fnz,
                                      inr, inx, inz);
                        iv2 = 1.0f / (vel * vel);
                        drr = (g.gor - rigr) - (double)(ivrt - 1) * g.dvr;
                        drx = (rigx - g.gox) - (double)(ivxt - 1) * g.dvx;
                        drz = (rigz - g.goz) - (double)(ivzt - 1) * g.dvz;
                        bsplf((float)(drr * ivr_), ui);
                        bsplf((float)(drx * ivx_), vi);
                        bsplf((float)(drz * ivz_), wi);
                        const double dinc = (k == 0) ? vrat[k] * dpl : (vrat[k] - vrat[k - 1]) * dpl;
                        const float hd = (float)(0.5 * dinc);
                        if (ivzt - 1 < 0 || ivzt + 2 > g.nvz + 1 || ivxt - 1 < 0 || ivxt + 2 > g.nvx + 1 ||
                            ivrt - 1 < 0 || ivrt + 2 > g.nvr + 1) {
                            st = 1;
                            continue;
                        }
                        // a sub-segment in another support cell: the current
                        // cell's sums go to the row first
                        if (ivrt != acc_r || ivxt != acc_x || ivzt != acc_z) {
                            flush();
                            acc_r = ivrt; acc_x = ivxt; acc_z = ivzt;
                        }
#pragma unroll 1
                        for (int n = 0; n < 4; ++n)
#pragma unroll
                            for (int m = 0; m < 4; ++m) {
                                const float uv = ui[n] * vi[m] * iv2, uvo = uio[n] * vio[m] * iv2o;
#pragma unroll
                                for (int l = 0; l < 4; ++l) {
                                    const float a1 = -(uv * wi[l] + uvo * wio[l]) * hd;
                                    float &c = acc[((n * 4 + m) * 4 + l) * kRayBlock];
                                    c = a1 + c;
                                }
                            }
                    }
                }
                rgr = nr; rgx = nx; rgz = nz;
                if (stop) break;
            }
        }
        if (fdm) flush();
        if (st && a.flags) atomicMin(&a.flags[0], q);
        if (a.endpoints) {
            a.endpoints[3 * (size_t)q] = rgr;
            a.endpoints[3 * (size_t)q + 1] = rgx;
            a.endpoints[3 * (size_t)q + 2] = rgz;
        }
        if (a.nsteps) a.nsteps[q] = steps;
    }
}

// Rows: count and compact entries with |f| >= 1e-6 (F:7739-7765).  One block
// per row; the block scans the row in column order, V consecutive columns per
// thread (V = 4: 16-byte loads, when the row length keeps every row 16-byte
// aligned), so that enough loads are in flight to stream the dense rows at
// HBM speed.
template <int V>
struct RowVec;
template <>
struct RowVec<1> {
    static __device__ __forceinline__ void load(const float *p, float (&v)[1]) { v[0] = __ldcs(p); }
};
template <>
struct RowVec<4> {
    static __device__ __forceinline__ void load(const float *p, float (&v)[4])
    {
        const float4 x = __ldcs(reinterpret_cast<const float4 *>(p));
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    }
};

template <int V>
__global__ void row_counts_kernel(const float *__restrict__ fdm, int nrows, int nmp, int64_t *__restrict__ counts)
{
    const float ftol = 1.0e-6f;
    __shared__ int red[2][32];
    const int nv = nmp / V;                      // whole vectors (nmp % V == 0)
    int it = 0;
    for (int row = blockIdx.x; row < nrows; row += gridDim.x, it ^= 1) {
        const float *f = fdm + (size_t)row * nmp;
        int c = 0;
#pragma unroll 2
        for (int q = threadIdx.x; q < nv; q += blockDim.x) {
            float v[V];
            RowVec<V>::load(f + (size_t)q * V, v);
#pragma unroll
            for (int j = 0; j < V; ++j) c += fabsf(v[j]) >= ftol ? 1 : 0;
        }
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        // (two buffers: a row's sums are not overwritten by the next row's
        // before thread 0 has read them)
        if ((threadIdx.x & 31) == 0) red[it][threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            int sum = 0;
            for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) sum += red[it][w];
            counts[row] = sum;
        }
    }
}

template <int V>
__global__ void row_compact_kernel(const float *__restrict__ fdm, int nrows, int nmp,
                                   const int64_t *__restrict__ row_ptr, int32_t *__restrict__ cols,
                                   float *__restrict__ vals)
{
    const float ftol = 1.0e-6f;
    __shared__ int wsum[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    const int nv = nmp / V;
    int it = 0;
    for (int row = blockIdx.x; row < nrows; row += gridDim.x) {
        const float *f = fdm + (size_t)row * nmp;
        int64_t base = row_ptr[row];
        for (int c0 = 0; c0 < nv; c0 += blockDim.x, it ^= 1) {
            const int q = c0 + threadIdx.x;
            float v[V];
            int k = 0;
            if (q < nv) {
                RowVec<V>::load(f + (size_t)q * V, v);
#pragma unroll
                for (int j = 0; j < V; ++j) k += fabsf(v[j]) >= ftol ? 1 : 0;
            }
            // the thread's first slot: the kept entries of the lower threads
            // of its warp, then of the lower warps
            int incl = k;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) wsum[it][wid] = incl;
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < nw; ++w) {
                const int x = wsum[it][w];
                before += w < wid ? x : 0;
                total += x;
            }
            if (k > 0) {
                int64_t pos = base + before + incl - k;
#pragma unroll
                for (int j = 0; j < V; ++j)
                    if (fabsf(v[j]) >= ftol) {
                        cols[pos] = q * V + j + 1;
                        vals[pos] = v[j];
                        ++pos;
                    }
            }
            base += total;
            // (the next chunk writes the other wsum buffer; the one after it
            // this buffer again, after the next chunk's barrier, which every
            // thread reaches only after reading this one)
        }
    }
}

// Row pointers from row counts: row_ptr[0] = 0, row_ptr[i+1] = row_ptr[i] +
// counts[i].  Each block scans a chunk of kScanChunk rows and writes its total;
// one block then turns the totals into chunk offsets in order (any number of
// chunks, with a running carry) and the chunks add their offset.
constexpr int kScanThreads = 1024;
constexpr int kScanChunk = kScanThreads;

__device__ int64_t block_exclusive_scan(int64_t v, int64_t *total)
{
    __shared__ int64_t warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    const int64_t before = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kScanThreads) scan_chunks_kernel(const int64_t *__restrict__ counts, int n,
                                                                   int64_t *__restrict__ row_ptr,
                                                                   int64_t *__restrict__ chunk_tot)
{
    const int i = blockIdx.x * kScanChunk + threadIdx.x;
    const int64_t v = i < n ? counts[i] : 0;
    int64_t tot;
    const int64_t ex = block_exclusive_scan(v, &tot);
    if (i < n) row_ptr[i + 1] = ex + v;          // inclusive within the chunk
    if (threadIdx.x == 0) chunk_tot[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) scan_totals_kernel(int64_t *__restrict__ chunk_tot, int nchunks)
{
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nchunks; c0 += kScanThreads) {
        const int c = c0 + threadIdx.x;
        const int64_t v = c < nchunks ? chunk_tot[c] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan(v, &tot);
        if (c < nchunks) chunk_tot[c] = carry + ex;  // offset of chunk c
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void scan_add_kernel(int n, int64_t *__restrict__ row_ptr, const int64_t *__restrict__ chunk_off)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) row_ptr[0] = 0;
    if (i < n) row_ptr[i + 1] += chunk_off[i / kScanChunk];
}

int scan_chunks(int nrows) { return (nrows + kScanChunk - 1) / kScanChunk; }

void launch_row_scan(const int64_t *counts, int nrows, int64_t *row_ptr, int64_t *chunk_tmp, cudaStream_t st)
{
    if (nrows <= 0) return;
    const int nc = scan_chunks(nrows);
    scan_chunks_kernel<<<nc, kScanThreads, 0, st>>>(counts, nrows, row_ptr, chunk_tmp);
    scan_totals_kernel<<<1, kScanThreads, 0, st>>>(chunk_tmp, nc);
    scan_add_kernel<<<(nrows + 255) / 256, 256, 0, st>>>(nrows, row_ptr, chunk_tmp);
}

void launch_rays(const RayArgs &a, cudaStream_t st)
{
    const int total = (a.events ? a.nlist : a.nev) * a.nrc;
    const int block = kRayBlock;
    const int blocks = (total + block - 1) / block;
    if (blocks <= 0) return;
    if (a.prec == FM3DT_FP64)
        rays_kernel<double><<<blocks, block, 0, st>>>(a);
    else
        rays_kernel<float><<<blocks, block, 0, st>>>(a);
}

void launch_row_counts(const float *fdm, int nrows, int nmp, int64_t *counts, cudaStream_t st)
{
    if (nrows <= 0) return;
    const int grid = nrows < 152 * 16 ? nrows : 152 * 16;
    if (nmp % 4 == 0)
        row_counts_kernel<4><<<grid, 256, 0, st>>>(fdm, nrows, nmp, counts);
    else
        row_counts_kernel<1><<<grid, 256, 0, st>>>(fdm, nrows, nmp, counts);
}

void launch_row_compact(const float *fdm, int nrows, int nmp, const int64_t *row_ptr, int32_t *cols, float *vals,
                        cudaStream_t st)
{
    if (nrows <= 0) return;
    const int grid = nrows < 152 * 16 ? nrows : 152 * 16;
    if (nmp % 4 == 0)
        row_compact_kernel<4><<<grid, 256, 0, st>>>(fdm, nrows, nmp, row_ptr, cols, vals);
    else
        row_compact_kernel<1><<<grid, 256, 0, st>>>(fdm, nrows, nmp, row_ptr, cols, vals);
}

}  // namespace fm3dt
