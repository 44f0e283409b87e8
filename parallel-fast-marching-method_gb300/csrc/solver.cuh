// solver.cu -- kernel (b): block-parallel fast-iterative eikonal solver.
//
// Replaces the reference's heap-ordered fast marching (local_fmm, F:78-155),
// its cross-subdomain re-march (order_overlap, F:157-416) and the BSP round
// loop with halo exchange (F:6371-6451, 6691-6892) by two device-side passes
// over tiles of the grid:
//
//  1. Sweep.  Tiles are visited in wavefront order of the event's dominant
//     propagation direction (upward from the bottom face, and along +/-theta
//     and +/-phi as the boundary frame's gradient says): one launch per tile
//     hyperplane, every tile's upwind neighbour tiles already done.  Inside a
//     tile the nodes are swept as a pipelined wavefront: at step s the thread
//     owning column (x', z') updates layer r' = s - x' - z' (swept
//     coordinates), so each node sees its upwind neighbours' final values.
//     Where every node's upwind neighbours lie in that octant, one sweep
//     already gives the converged field.
//  2. Rounds.  Every tile starts active; a work item is one (event, tile)
//     pair from a device active list.  The tile plus 2-deep face halos (the
//     second-order stencil reaches two nodes along each axis) are staged in
//     shared memory; each thread owns a (theta, phi) column and sweeps it in r
//     (upward on even passes, downward on odd ones) until a __syncthreads_or
//     vote finds no node changed.  Changed nodes are written back and every
//     face neighbour whose halo changed is queued for the next round (dedup by
//     a per-tile flag).  The solve ends when a round leaves the list empty.
//
// Updates overwrite (T <- F(T)) with the causal octant stencil of
// stencil.cuh.  The fixed point of that map is unique, so the converged field
// does not depend on update order, tile shape, schedule or batch
// composition: racing neighbour reads inside and between tiles, and the
// sweep, only change how fast the fixed point is reached, never its bits.
#pragma once
#include "internal.h"
#include "stencil.cuh"

namespace fm3dt {

__device__ __forceinline__ unsigned long long fbits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long fbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Shared box of a tile: the tile with 2-deep halos in r and theta, and in phi
// (contiguous) 4 columns either side, so that a TMA copy of the box starts on a
// 16-byte boundary (the tile starts at a multiple of TZ; 4 elements before it
// is 16 bytes before in single precision, 32 in double).  Only the 2 columns
// next to the tile are read.
template <typename R, int TR, int TX, int TZ>
struct Tile {
    static constexpr int NT = TX * TZ;
    static constexpr int ZOFF = 4;        // phi index of the tile's first node in the box
    static constexpr int BR = TR + 4, BX = TX + 4, BZ = TZ + 2 * ZOFF;
    static constexpr int SR = BX * BZ;     // shared stride of one r layer
    static constexpr int NBOX = BR * BX * BZ;
    // shared-memory layout after the box: slowness of the tile's nodes, then
    // the spacing tables of its (r, theta) rows and r layers
    static constexpr int OFF_S = NBOX;
    static constexpr int OFF_HZ = OFF_S + TR * TX * TZ;
    static constexpr int OFF_WZ = OFF_HZ + TR * TX;
    static constexpr int OFF_HX = OFF_WZ + TR * TX;
    static constexpr int OFF_WX = OFF_HX + TR;
    static constexpr int NSMEM = OFF_WX + TR;

    // stage tile + face halos (edges/corners are never read by the stencil;
    // outside the grid reads as unset)
    static __device__ void load(R *sm, const R *Te, const FieldArgs<R> &a, int r0, int x0, int z0)
    {
        const R INF = Lim<R>::inf();
        for (int q = threadIdx.x; q < NBOX; q += NT) {
            const int bz = q % BZ, bx = (q / BZ) % BX, br = q / SR;
            const bool zfar = bz < ZOFF - 2 || bz >= TZ + ZOFF + 2;
            const int out = (bz < ZOFF || bz >= TZ + ZOFF) + (bx < 2 || bx >= TX + 2) + (br < 2 || br >= TR + 2);
            R v = INF;
            if (out <= 1 && !zfar) {
                const int gr = r0 + br - 2, gx = x0 + bx - 2, gz = z0 + bz - ZOFF;
                if (gr >= 0 && gr < a.nnr && gx >= 0 && gx < a.nnx && gz >= 0 && gz < a.nnz)
                    v = __ldcg(Te + ((size_t)gr * a.nnx + gx) * a.nnz + gz);
            }
            sm[q] = v;
        }
    }

    // stage the slowness of the tile's nodes and the spacings its rows use
    // (the rounds reuse them over several passes)
    static __device__ void load_params(R *sm, const FieldArgs<R> &a, int r0, int x0, int z0,
                                       bool slowness = true)
    {
        for (int q = threadIdx.x; slowness && q < TR * TX * TZ; q += NT) {
            const int lz = q % TZ, lx = (q / TZ) % TX, lr = q / (TZ * TX);
            const int gr = r0 + lr, gx = x0 + lx, gz = z0 + lz;
            sm[OFF_S + q] = (gr < a.nnr && gx < a.nnx && gz < a.nnz)
                                ? __ldg(a.s + ((size_t)gr * a.nnx + gx) * a.nnz + gz) : R(1);
        }
        for (int q = threadIdx.x; q < TR * TX; q += NT) {
            const int lx = q % TX, lr = q / TX;
            const int gr = r0 + lr, gx = x0 + lx;
            const bool ok = gr < a.nnr && gx < a.nnx;
            sm[OFF_HZ + q] = ok ? __ldg(a.hz + (size_t)gr * a.nnx + gx) : R(1);
            sm[OFF_WZ + q] = ok ? __ldg(a.wz + (size_t)gr * a.nnx + gx) : R(1);
        }
        for (int q = threadIdx.x; q < TR; q += NT) {
            const bool ok = r0 + q < a.nnr;
            sm[OFF_HX + q] = ok ? __ldg(a.hx + r0 + q) : R(1);
            sm[OFF_WX + q] = ok ? __ldg(a.wx + r0 + q) : R(1);
        }
    }

    // node parameters (slowness and spacings) of one node
    struct Params {
        R s;
        Spacing<R> sp;
    };
    static __device__ __forceinline__ Params params_global(const FieldArgs<R> &a, int gr, int gx, int gz)
    {
        Params p;
        p.sp.h[0] = a.hr;
        p.sp.w[0] = a.wr;
        p.sp.h[1] = __ldg(a.hx + gr);
        p.sp.w[1] = __ldg(a.wx + gr);
        const size_t q = (size_t)gr * a.nnx + gx;
        p.sp.h[2] = __ldg(a.hz + q);
        p.sp.w[2] = __ldg(a.wz + q);
        p.s = __ldg(a.s + q * a.nnz + gz);
        return p;
    }
    static __device__ __forceinline__ Params params_shared(const R *sm, const FieldArgs<R> &a, int r, int tx, int tz)
    {
        Params p;
        p.sp.h[0] = a.hr;
        p.sp.w[0] = a.wr;
        p.sp.h[1] = sm[OFF_HX + r];
        p.sp.w[1] = sm[OFF_WX + r];
        p.sp.h[2] = sm[OFF_HZ + r * TX + tx];
        p.sp.w[2] = sm[OFF_WZ + r * TX + tx];
        p.s = sm[OFF_S + (r * TX + tx) * TZ + tz];
        return p;
    }

    // one node update from the shared box with the node's parameters
    static __device__ __forceinline__ R update_with(const R *sm, int c, const FieldArgs<R> &a, int gr, int gx, int gz,
                                                    const Params &p)
    {
        R t1[6], t2[6];
        t1[0] = sm[c - SR];     t2[0] = sm[c - 2 * SR];
        t1[1] = sm[c + SR];     t2[1] = sm[c + 2 * SR];
        t1[2] = sm[c - BZ];     t2[2] = sm[c - 2 * BZ];
        t1[3] = sm[c + BZ];     t2[3] = sm[c + 2 * BZ];
        t1[4] = sm[c - 1];      t2[4] = sm[c - 2];
        t1[5] = sm[c + 1];      t2[5] = sm[c + 2];
        const unsigned inb = (gr > 0 ? 1u : 0u) | (gr < a.nnr - 1 ? 2u : 0u) | (gx > 0 ? 4u : 0u) |
                             (gx < a.nnx - 1 ? 8u : 0u) | (gz > 0 ? 16u : 0u) | (gz < a.nnz - 1 ? 32u : 0u);
        return fm_update<R>(p.s, t1, t2, inb, p.sp, a.order2);
    }

    // one node update (tile-local r, tx, tz) from shared memory; returns the
    // new value
    static __device__ __forceinline__ R update(const R *sm, int c, const FieldArgs<R> &a, int r, int tx, int tz,
                                               int gr, int gx, int gz)
    {
        return update_with(sm, c, a, gr, gx, gz, params_shared(sm, a, r, tx, tz));
    }

    static __device__ __forceinline__ bool frozen(const FieldArgs<R> &a, int e, int gr, int gx, int gz)
    {
        if (a.box) {
            const int *b = a.box + 6 * e;
            return gr >= b[0] && gr <= b[1] && gx >= b[2] && gx <= b[3] && gz >= b[4] && gz <= b[5];
        }
        return gr == a.nnr - 1 && a.frozen[(size_t)e * a.nnx * a.nnz + (size_t)gx * a.nnz + gz] != 0;
    }
};

// Resident 128-thread CTAs per SM that the register allocation must allow.
// The kernels are issue-bound with long dependent chains, so occupancy pays
// until registers spill.
#ifndef FM_ROUND_MINB_F32
#define FM_ROUND_MINB_F32 8
#endif
#ifndef FM_ROUND_MINB_F64
#define FM_ROUND_MINB_F64 4
#endif
#ifndef FM_SWEEP_MINB_F32
#define FM_SWEEP_MINB_F32 6
#endif
#ifndef FM_SWEEP_MINB_F64
#define FM_SWEEP_MINB_F64 4
#endif
template <typename R, int THREADS>
struct MinBlocks {
    static constexpr int round = (sizeof(R) == 4 ? FM_ROUND_MINB_F32 : FM_ROUND_MINB_F64) * 128 / THREADS;
    static constexpr int sweep = (sizeof(R) == 4 ? FM_SWEEP_MINB_F32 : FM_SWEEP_MINB_F64) * 128 / THREADS;
};

// ---------------------------------------------------------------------------
// Rounds (fast-iterative cleanup until the fixed point)
// ---------------------------------------------------------------------------

// TMA (bulk tensor copy) of a tile box: one thread arms the CTA's mbarrier
// with the box's byte count and issues the copy; every thread then waits for
// the barrier's phase.  The wait gives up after ~1 s of clock cycles
// (kTmaWaitCycles) and reports it, so a copy that never completes cannot hang
// the GPU.
constexpr long long kTmaWaitCycles = 2000000000LL;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, unsigned long long *bar, int c0,
                                            int c1, int c2)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// (the caller has armed the barrier with the bytes of every copy of the phase)
__device__ __forceinline__ void tma_load_box(void *dst, const CUtensorMap *map, unsigned long long *bar,
                                             int c0, int c1, int c2, int c3)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// true when the barrier completed phase `phase` before the time limit
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, int phase)
{
    const long long t0 = clock64();
    while (true) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kTmaWaitCycles) return false;
    }
}
template <typename R, int TR, int TX, int TZ>
__global__ void __launch_bounds__(TX * TZ, (MinBlocks<R, TX * TZ>::round))
    round_kernel(const __grid_constant__ RoundArgs<R> a)
{
    using TL = Tile<R, TR, TX, TZ>;
    static_assert(32 % TR == 0, "a column's rows of a tile lie in one certification word");
    // (the TMA destination: 128-byte aligned; a name of its own, since every
    // extern __shared__ declaration of one name in a translation unit must
    // agree on the alignment)
    extern __shared__ __align__(128) unsigned char round_smem[];
    R *box = reinterpret_cast<R *>(round_smem);
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ int s_abort;
    int phase = 0;
    __shared__ int s_face;
    __shared__ int s_w;
    __shared__ unsigned s_chg[2][TX * TZ];        // per column: nodes changed in a pass
    __shared__ unsigned long long s_upd;
    const FieldArgs<R> &f = a.f;
    const int tid = threadIdx.x;
    const int tz = tid % TZ, tx = tid / TZ;
    const int count = *((volatile const int *)a.cur_count);
    const size_t N = (size_t)f.nnx * f.nnz * (size_t)f.nnr;
    unsigned long long my_tiles = 0, my_staged = 0, my_upd = 0;
    if (tid == 0) s_upd = 0;

    __shared__ int s_dirty_faces;
    // a TMA destination must start on a 128-byte boundary: check the box (and
    // the slowness after it, at a multiple of 128 bytes for every tile shape)
    // before the first copy, and report instead of issuing a misaligned one
    static_assert((Tile<R, TR, TX, TZ>::OFF_S * sizeof(R)) % 128 == 0, "slowness box alignment");
    const bool tma = a.tma && (smem_u32(box) & 127u) == 0;
    if (tid == 0) {
        s_abort = 0;
        if (a.tma && !tma) atomicExch(a.err, 2);
        if (tma) mbar_init(&s_bar);
    }
    __syncthreads();
    if (a.tma && !tma) return;
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        if (tid == 0) {
            const int w = a.cur_list[item];
            s_w = w;
            s_face = 0;
            // take the halo faces changed since this tile's last pass; later
            // activations re-queue it
            s_dirty_faces = atomicExch(&a.flag[w], 0) & (kFaceMask | kFull | kCert);
            __threadfence();
        }
        __syncthreads();
        const int w = s_w;
        const int e = w / f.tiles_per_event;
        const int t = w - e * f.tiles_per_event;
        const int tzi = t % f.ntz;
        const int txi = (t / f.ntz) % f.ntx;
        const int tri = t / (f.ntz * f.ntx);
        const int r0 = tri * TR, x0 = txi * TX, z0 = tzi * TZ;
        R *Te = f.T + (size_t)e * N;
        if (tma) {
            // outside the grid the copy fills NaN, which the stencil never
            // uses: an out-of-grid first neighbour is masked, and a NaN second
            // neighbour fails t2 < t1 like +inf
            // one phase: the box and the tile's slowness (a 3-D copy of its
            // own nodes, beside the box); the threads load the spacings
            if (tid == 0) {
                mbar_expect(&s_bar, (unsigned)((TL::NBOX + TR * TX * TZ) * sizeof(R)));
                tma_load_box(box, &a.tmap, &s_bar, z0 - TL::ZOFF, x0 - 2, r0 - 2, e);
                tma_load_3d(box + TL::OFF_S, &a.smap, &s_bar, z0, x0, r0);
            }
            TL::load_params(box, f, r0, x0, z0, false);
            if (!mbar_wait(&s_bar, phase)) atomicExch(&s_abort, 1);
            phase ^= 1;
            __syncthreads();
            if (s_abort) {
                // the copy did not arrive: report it, give it one more bounded
                // wait so that nothing writes into shared memory after exit
                if (tid == 0) {
                    atomicExch(a.err, 1);
                    mbar_wait(&s_bar, phase ^ 1);
                }
                return;
            }
        } else {
            TL::load(box, Te, f, r0, x0, z0);
            TL::load_params(box, f, r0, x0, z0);
        }

        const int gx = x0 + tx, gz = z0 + tz;
        const bool colv = gx < f.nnx && gz < f.nnz;
        unsigned updm = 0;
#pragma unroll
        for (int r = 0; r < TR; ++r) {
            const int gr = r0 + r;
            if (colv && gr < f.nnr && !TL::frozen(f, e, gr, gx, gz)) updm |= 1u << r;
        }
        __syncthreads();

        // Passes.  The tile was at its fixed point for the halo it last saw, so
        // the first pass recomputes only the nodes within two nodes of a halo
        // face that changed since (every node when the tile is new to the
        // solve); later passes only the nodes with a stencil neighbour (+-1,
        // +-2 along each axis) that changed in the previous pass -- a node's
        // update never reads its own value, so nothing else can change.
        unsigned chm = 0;
        bool last_changed = false;
        const int cbase = (2 * TL::BX + (tx + 2)) * TL::BZ + (tz + TL::ZOFF);
        const int df = s_dirty_faces;
        unsigned dirty;
        if (df & kFull) {
            dirty = updm;
        } else {
            constexpr unsigned all = (TR >= 32) ? 0xffffffffu : ((1u << TR) - 1u);
            dirty = 0;
            if (df & kFaceUp) dirty |= 3u;
            if (df & kFaceDown) dirty |= 3u << (TR - 2);
            if ((df & kFaceXm) && tx < 2) dirty = all;
            if ((df & kFaceXp) && tx >= TX - 2) dirty = all;
            if ((df & kFaceZm) && tz < 2) dirty = all;
            if ((df & kFaceZp) && tz >= TZ - 2) dirty = all;
            // a certified tile: the nodes whose sweep value a recomputation
            // could change (TR divides 32, so a column's rows of the tile lie
            // in one bitmap word)
            if ((df & kCert) && colv)
                dirty |= (a.cert[(((size_t)e * f.nnx + gx) * f.nnz + gz) * a.cert_nw + (r0 >> 5)] >> (r0 & 31)) & all;
            dirty &= updm;
        }
        for (int p = 0; p < a.max_passes; ++p) {
            unsigned pch = 0;
            // r changes only shared-memory offsets and mask bits: no unrolling
            const int k0 = (p & 1) ? 0 : TR - 1, dk = (p & 1) ? 1 : -1;
            my_upd += __popc(dirty);
#pragma unroll 1
            for (int i = 0, k = k0; i < TR; ++i, k += dk) {
                if (!((dirty >> k) & 1u)) continue;
                const int c = cbase + k * TL::SR;
                const R nv = TL::update(box, c, f, k, tx, tz, r0 + k, gx, gz);
                if (fbits(nv) != fbits(box[c])) {
                    box[c] = nv;
                    pch |= 1u << k;
                }
            }
            chm |= pch;
            s_chg[p & 1][tid] = pch;
            last_changed = __syncthreads_or(pch != 0) != 0;
            if (!last_changed) break;
            const unsigned *q = s_chg[p & 1];
            unsigned lat = 0;
            if (tx > 0) lat |= q[tid - TZ];
            if (tx > 1) lat |= q[tid - 2 * TZ];
            if (tx < TX - 1) lat |= q[tid + TZ];
            if (tx < TX - 2) lat |= q[tid + 2 * TZ];
            if (tz > 0) lat |= q[tid - 1];
            if (tz > 1) lat |= q[tid - 2];
            if (tz < TZ - 1) lat |= q[tid + 1];
            if (tz < TZ - 2) lat |= q[tid + 2];
            dirty = (lat | (pch << 1) | (pch >> 1) | (pch << 2) | (pch >> 2)) & updm;
        }

#pragma unroll
        for (int r = 0; r < TR; ++r)
            if ((chm >> r) & 1u)
                Te[((size_t)(r0 + r) * f.nnx + gx) * f.nnz + gz] = box[cbase + r * TL::SR];

        int fb = 0;
        if (chm & 3u) fb |= 1;                       // read by the tile above
        if (chm >> (TR - 2)) fb |= 2;                // read by the tile below
        if (chm && tx < 2) fb |= 4;
        if (chm && tx >= TX - 2) fb |= 8;
        if (chm && tz < 2) fb |= 16;
        if (chm && tz >= TZ - 2) fb |= 32;
        if (fb) atomicOr(&s_face, fb);
        __threadfence();
        __syncthreads();
        if (tid < 7) {
            int fl = s_face;
            if (tid == 6 && last_changed) fl |= 64;   // pass cap hit: run again
            if ((fl >> tid) & 1) {
                int nb = -1, bit = kFull;
                const int sl = f.ntx * f.ntz;
                // the neighbour's halo face opposite to the face that changed
                switch (tid) {
                    case 0: nb = tri > 0 ? w - sl : -1; bit = kFaceDown; break;
                    case 1: nb = tri < f.ntr - 1 ? w + sl : -1; bit = kFaceUp; break;
                    case 2: nb = txi > 0 ? w - f.ntz : -1; bit = kFaceXp; break;
                    case 3: nb = txi < f.ntx - 1 ? w + f.ntz : -1; bit = kFaceXm; break;
                    case 4: nb = tzi > 0 ? w - 1 : -1; bit = kFaceZp; break;
                    case 5: nb = tzi < f.ntz - 1 ? w + 1 : -1; bit = kFaceZm; break;
                    default: nb = w; bit = kFull; break;
                }
                if (nb >= 0 && !(atomicOr(&a.flag[nb], bit | kQueued) & kQueued)) {
                    const int pos = atomicAdd(a.next_count, 1);
                    a.next_list[pos] = nb;
                }
            }
        }
        if (tid == 0) {
            const int vr = min(TR, f.nnr - r0), vx = min(TX, f.nnx - x0), vz = min(TZ, f.nnz - z0);
            my_tiles += 1;
            my_staged += (unsigned long long)(vr * vx * vz);
        }
        // every thread's accesses to the box come before the next copy's
        // writes (generic proxy, then async proxy)
        if (tma) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
    }
    if (my_upd) atomicAdd(&s_upd, my_upd);
    __syncthreads();
    if (tid == 0 && my_tiles) {
        atomicAdd(&a.stats[0], my_tiles);
        atomicAdd(&a.stats[1], s_upd);
        atomicAdd(&a.stats[2], my_staged);
        if (a.trace) {
            atomicAdd(&a.trace[2 * a.round], my_tiles);
            atomicAdd(&a.trace[2 * a.round + 1], s_upd);
        }
    }
}

// ---------------------------------------------------------------------------
// Certification after a single sweep
// ---------------------------------------------------------------------------

// A node swept once from an unset field holds F(T) with its three
// downstream neighbours (up, and the lateral directions the sweep runs
// toward) unset; every other input was final when it was computed.  The
// rounds need to recompute it only if one of those neighbours, now set, can
// change F.  It cannot when, with B = T - (earliest upstream neighbour):
//   * every downstream neighbour is first order (its second neighbour is not
//     earlier) and its key is at least B (1 + 1/32), and
//   * no neighbour with a key of B (1 - 1/32) or more is second order.
// Why: adding a first-order causal term with key k to an octant's solve
// gives a root above k (the quadratic is below s^2 at k, or its vertex is
// above k), so every octant that now takes such a term ends above
// B (1 + 1/32) less the solve's rounding, which the margin covers tenfold
// (about 1e-3 of the octant's largest term in single precision); octants
// that take none are unchanged bit for bit; the earliest neighbour stays the
// same, and the terms below B come first in every sort as before.  Nodes
// that fail, and unreached nodes, go into the bitmap.
template <typename R>
__global__ void __launch_bounds__(256, 4) certify_kernel(const CertifyArgs<R> a)
{
    const FieldArgs<R> &f = a.f;
    const R INF = Lim<R>::inf();
    const R margin = R(1.0 / 32.0);
    const size_t layer = (size_t)f.nnx * f.nnz;
    const size_t N = layer * (size_t)f.nnr;
    const long long ncol = (long long)layer;
    const long long total = ncol * a.nev;
    const int tiles_r = 32 / a.tr;    // tiles of the column in one bitmap word
    const unsigned tmask = (a.tr >= 32) ? 0xffffffffu : ((1u << a.tr) - 1u);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q / ncol);
        const int c = (int)(q - (long long)k * ncol);
        const int gx = c / f.nnz, gz = c - gx * f.nnz;
        const int e = a.events[k];
        const R *col = f.T + (size_t)e * N + c;    // this column's node in layer 0
        // lateral neighbours: downstream (the way the sweep runs) and
        // upstream steps in theta (elements of nnz) and phi, and whether the
        // first and second neighbours lie inside the grid
        const int db = a.dir[e];
        const int sx = (db & 1) ? 1 : -1, sz = (db & 2) ? 1 : -1;
        const long long ox = (long long)sx * f.nnz;
        const bool xd1 = (unsigned)(gx + sx) < (unsigned)f.nnx, xd2 = (unsigned)(gx + 2 * sx) < (unsigned)f.nnx;
        const bool xu1 = (unsigned)(gx - sx) < (unsigned)f.nnx, xu2 = (unsigned)(gx - 2 * sx) < (unsigned)f.nnx;
        const bool zd1 = (unsigned)(gz + sz) < (unsigned)f.nnz, zd2 = (unsigned)(gz + 2 * sz) < (unsigned)f.nnz;
        const bool zu1 = (unsigned)(gz - sz) < (unsigned)f.nnz, zu2 = (unsigned)(gz - 2 * sz) < (unsigned)f.nnz;
        const bool frozen_col = f.frozen[(size_t)e * layer + c] != 0;
        auto colv = [&](int gr) -> R { return (gr >= 0 && gr < f.nnr) ? __ldg(col + (size_t)gr * layer) : INF; };
        // the column around the node: v0..v4 = layers gr-2 .. gr+2
        R v0 = INF, v1 = INF, v2 = colv(0), v3 = colv(1), v4 = colv(2);
        // the lateral neighbours of layer gr (unset outside the grid), read a
        // layer ahead: upstream first, downstream first and second
        R nxu, nzu, nxd, nxd2, nzd, nzd2;
        auto lateral = [&](int gr) {
            const bool in = gr < f.nnr;
            const R *p = col + (size_t)(in ? gr : 0) * layer;
            nxu = in && xu1 ? __ldg(p - ox) : INF;
            nzu = in && zu1 ? __ldg(p - sz) : INF;
            nxd = in && xd1 ? __ldg(p + ox) : INF;
            nxd2 = in && xd2 ? __ldg(p + 2 * ox) : INF;
            nzd = in && zd1 ? __ldg(p + sz) : INF;
            nzd2 = in && zd2 ? __ldg(p + 2 * sz) : INF;
        };
        lateral(0);
        for (int w = 0; w < a.cert_nw; ++w) {
            unsigned bits = 0;
            for (int rr = 0; rr < 32; ++rr) {
                const int gr = w * 32 + rr;
                if (gr >= f.nnr) break;
                bool ok = true;
                const R txu = nxu, tzu = nzu, txd = nxd, txd2 = nxd2, tzd = nzd, tzd2 = nzd2;
                lateral(gr + 1);
                if (!(gr == f.nnr - 1 && frozen_col)) {
                    const R *p = col + (size_t)gr * layer;
                    const R T = v2;
                    // upstream first neighbours: down (r+1) and the lateral ones
                    const R td = gr < f.nnr - 1 ? v3 : INF;
                    const R tu = fm_min(td, fm_min(txu, tzu));
                    ok = T < INF && tu < INF;
                    const R B = T - tu;
                    const R hi = B + B * margin, lo = B - B * margin;
                    // a downstream neighbour passes when its key is at least hi
                    // and it is first order (its second neighbour not earlier);
                    // one outside the grid reads unset and passes
                    auto down_ok = [&](R t1, R t2) { return (t1 - tu) >= hi && !(f.order2 && t2 < t1); };
                    ok = ok && down_ok(v1, v0) && down_ok(txd, txd2) && down_ok(tzd, tzd2);
                    // an upstream neighbour at or above lo must be first order
                    if (f.order2) {
                        if (gr < f.nnr - 1 && !((td - tu) < lo) && v4 < td) ok = false;
                        if (xu1 && !((txu - tu) < lo) && xu2 && __ldg(p - 2 * ox) < txu) ok = false;
                        if (zu1 && !((tzu - tu) < lo) && zu2 && __ldg(p - 2 * sz) < tzu) ok = false;
                    }
                }
                if (!ok) bits |= 1u << rr;
                v0 = v1; v1 = v2; v2 = v3; v3 = v4; v4 = colv(gr + 3);
            }
            a.cert[((size_t)e * ncol + c) * a.cert_nw + w] = bits;
            // queue the tiles of this word's rows that hold a marked node
            for (int j = 0; j < tiles_r && bits; ++j) {
                if (!((bits >> (j * a.tr)) & tmask)) continue;
                const int tri = (w * 32) / a.tr + j;
                if (tri >= f.ntr) break;
                const int t = e * f.tiles_per_event + (tri * f.ntx + gx / a.tx) * f.ntz + gz / a.tz;
                if (!(atomicOr(&a.flag[t], kCert | kQueued) & kQueued)) a.list[atomicAdd(a.count, 1)] = t;
            }
        }
    }
}

template <typename R>
void launch_certify(const CertifyArgs<R> &a, cudaStream_t st)
{
    const long long total = (long long)a.f.nnx * a.f.nnz * a.nev;
    if (total <= 0) return;
    const int grid = (int)std::min<long long>((total + 255) / 256, 1LL << 20);
    certify_kernel<R><<<grid, 256, 0, st>>>(a);
}

// ---------------------------------------------------------------------------
// Sweep (one launch per tile hyperplane of the event's dominant direction)
// ---------------------------------------------------------------------------
template <typename R, int TR, int TX, int TZ>
__global__ void __launch_bounds__(TX * TZ, (MinBlocks<R, TX * TZ>::sweep)) sweep_kernel(SweepArgs<R> a)
{
    using TL = Tile<R, TR, TX, TZ>;
    extern __shared__ __align__(16) unsigned char sweep_smem[];
    R *box = reinterpret_cast<R *>(sweep_smem);
    const FieldArgs<R> &f = a.f;
    const int tid = threadIdx.x;
    const int tz = tid % TZ, tx = tid / TZ;
    const long long count = (long long)a.hcount * a.nev;
    const size_t N = (size_t)f.nnx * f.nnz * (size_t)f.nnr;
    for (long long item = blockIdx.x; item < count; item += gridDim.x) {
        const int e = (int)(item / a.hcount);
        const int j = (int)(item - (long long)e * a.hcount);
        const int packed = a.hp_tiles[a.hoff + j];
        const int ap = packed >> 20, bp = (packed >> 10) & 1023, cp = packed & 1023;
        const int dir = a.dir[e];
        const bool sx = dir & 1, sz = (dir >> 1) & 1;
        const int tri = f.ntr - 1 - ap;
        const int txi = sx ? bp : f.ntx - 1 - bp;
        const int tzi = sz ? cp : f.ntz - 1 - cp;
        const int r0 = tri * TR, x0 = txi * TX, z0 = tzi * TZ;
        R *Te = f.T + (size_t)e * N;
        TL::load(box, Te, f, r0, x0, z0);
        const int gx = x0 + tx, gz = z0 + tz;
        const bool colv = gx < f.nnx && gz < f.nnz;
        const int xs = sx ? tx : TX - 1 - tx;
        const int zs = sz ? tz : TZ - 1 - tz;
        const int cbase = (2 * TL::BX + (tx + 2)) * TL::BZ + (tz + TL::ZOFF);
        __syncthreads();
        // pipelined wavefront: layer rp (counted upward from the tile bottom)
        // of column (xs, zs) is updated at step rp + xs + zs
        // The next node's slowness and spacings are fetched one step ahead,
        // so their latency hides behind the barrier.
        typename TL::Params pnext{};
        if (colv && xs + zs == 0 && r0 + TR - 1 < f.nnr) pnext = TL::params_global(f, r0 + TR - 1, gx, gz);
        for (int step = 0; step < TR + TX + TZ - 2; ++step) {
            const int rp = step - xs - zs;
            const typename TL::Params pcur = pnext;
            if (colv && rp + 1 >= 0 && rp + 1 < TR && r0 + TR - 2 - rp < f.nnr)
                pnext = TL::params_global(f, r0 + TR - 2 - rp, gx, gz);
            if (colv && rp >= 0 && rp < TR) {
                const int r = TR - 1 - rp;
                const int gr = r0 + r;
                if (gr < f.nnr && !TL::frozen(f, e, gr, gx, gz)) {
                    const int c = cbase + r * TL::SR;
                    box[c] = TL::update_with(box, c, f, gr, gx, gz, pcur);
                }
            }
            __syncthreads();
        }
        if (colv) {
#pragma unroll
            for (int r = 0; r < TR; ++r) {
                const int gr = r0 + r;
                if (gr < f.nnr) Te[((size_t)gr * f.nnx + gx) * f.nnz + gz] = box[cbase + r * TL::SR];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// launchers (instantiated per precision in solver_f32.cu / solver_f64.cu)
// ---------------------------------------------------------------------------
template <typename R, int S>
struct ShapeKernels {
    static constexpr int TR = kShapes[S].tr, TX = kShapes[S].tx, TZ = kShapes[S].tz;
    // rounds stage the node parameters too; the sweep only the box
    static constexpr size_t SMEM_ROUND = Tile<R, TR, TX, TZ>::NSMEM * sizeof(R);
    static constexpr size_t SMEM_SWEEP = Tile<R, TR, TX, TZ>::NBOX * sizeof(R);
    static void setup()
    {
        static const bool once = [] {
            cudaFuncSetAttribute(round_kernel<R, TR, TX, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SMEM_ROUND);
            cudaFuncSetAttribute(sweep_kernel<R, TR, TX, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SMEM_SWEEP);
            return true;
        }();
        (void)once;
    }
    static void round(int grid, const RoundArgs<R> &a, cudaStream_t st)
    {
        setup();
        round_kernel<R, TR, TX, TZ><<<grid, TX * TZ, SMEM_ROUND, st>>>(a);
    }
    static void sweep(int grid, const SweepArgs<R> &a, cudaStream_t st)
    {
        setup();
        sweep_kernel<R, TR, TX, TZ><<<grid, TX * TZ, SMEM_SWEEP, st>>>(a);
    }
    static int occ_round()
    {
        setup();
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, round_kernel<R, TR, TX, TZ>, TX * TZ, SMEM_ROUND);
        return nb;
    }
    static int occ_sweep()
    {
        setup();
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sweep_kernel<R, TR, TX, TZ>, TX * TZ, SMEM_SWEEP);
        return nb;
    }
};

#define FM_SHAPE_SWITCH(shape, CALL)      \
    switch (shape) {                      \
        case 0: CALL(0); break;           \
        case 1: CALL(1); break;           \
        case 2: CALL(2); break;           \
        case 3: CALL(3); break;           \
        case 4: CALL(4); break;           \
        default: CALL(5); break;          \
    }

}  // namespace fm3dt
