// solver.cu -- kernel (b): block-parallel fast-iterative eikonal solver.
//
// Replaces the reference's heap-ordered fast marching (local_fmm, F:78-155),
// its cross-subdomain re-march (order_overlap, F:157-416) and the BSP round
// loop with halo exchange (F:6371-6451, 6691-6892) by one device-side
// iteration over tiles of the grid:
//
//  * A work item is one (event, tile) pair taken from a device active list.
//  * The tile plus 2-deep face halos (the second-order stencil reaches two
//    nodes along each axis) are staged in shared memory.
//  * Each thread owns a (theta, phi) column of the tile and sweeps it in r
//    (upward on even passes, downward on odd ones); passes repeat until a
//    __syncthreads_or vote finds no node changed.
//  * Changed nodes are written back; every face neighbour whose halo changed
//    is queued for the next round (dedup by a per-tile flag).  The solve ends
//    when a round leaves the list empty.
//
// Updates overwrite (T <- F(T)) with the causal octant stencil of
// stencil.cuh.  The fixed point of that map is unique, so the converged
// field does not depend on update order, tile schedule or batch composition:
// racing neighbour reads inside and between tiles only change how fast the
// fixed point is reached, never which bits it has.
#include "internal.h"
#include "stencil.cuh"

namespace fm3dt {

__device__ __forceinline__ unsigned long long fbits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long fbits(double v) { return (unsigned long long)__double_as_longlong(v); }

template <typename R, int TR, int TX, int TZ>
__global__ void __launch_bounds__(TX * TZ) round_kernel(RoundArgs<R> a)
{
    constexpr int NT = TX * TZ;
    constexpr int BR = TR + 4, BX = TX + 4, BZ = TZ + 4;
    constexpr int SR = BX * BZ;     // shared stride of one r layer
    __shared__ R box[BR * BX * BZ];
    __shared__ int s_face;
    __shared__ int s_w;

    const int tid = threadIdx.x;
    const int tz = tid % TZ, tx = tid / TZ;
    const int count = *((volatile const int *)a.cur_count);
    const size_t NB = (size_t)a.nnx * a.nnz;
    const size_t N = NB * (size_t)a.nnr;
    const R INF = Lim<R>::inf();
    unsigned long long my_tiles = 0, my_nodes = 0, my_staged = 0;

    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        if (tid == 0) {
            const int w = a.cur_list[item];
            s_w = w;
            s_face = 0;
            atomicExch(&a.flag[w], 0);   // later activations re-queue this tile
            __threadfence();
        }
        __syncthreads();
        const int w = s_w;
        const int e = w / a.tiles_per_event;
        const int t = w - e * a.tiles_per_event;
        const int tzi = t % a.ntz;
        const int txi = (t / a.ntz) % a.ntx;
        const int tri = t / (a.ntz * a.ntx);
        const int r0 = tri * TR, x0 = txi * TX, z0 = tzi * TZ;
        R *Te = a.T + (size_t)e * N;

        // stage tile + face halos (edges/corners are never read by the stencil)
        for (int q = tid; q < BR * BX * BZ; q += NT) {
            const int bz = q % BZ, bx = (q / BZ) % BX, br = q / SR;
            const int out = (bz < 2 || bz >= TZ + 2) + (bx < 2 || bx >= TX + 2) + (br < 2 || br >= TR + 2);
            R v = INF;
            if (out <= 1) {
                const int gr = r0 + br - 2, gx = x0 + bx - 2, gz = z0 + bz - 2;
                if (gr >= 0 && gr < a.nnr && gx >= 0 && gx < a.nnx && gz >= 0 && gz < a.nnz)
                    v = __ldcg(Te + ((size_t)gr * a.nnx + gx) * a.nnz + gz);
            }
            box[q] = v;
        }

        // per-column constants
        const int gx = x0 + tx, gz = z0 + tz;
        const bool colv = gx < a.nnx && gz < a.nnz;
        R sv[TR], hxv[TR], hzv[TR];
        unsigned inbv[TR];
        unsigned updm = 0;
#pragma unroll
        for (int r = 0; r < TR; ++r) {
            const int gr = r0 + r;
            const bool v = colv && gr < a.nnr;
            bool fz = false;
            if (v && gr == a.nnr - 1) fz = a.frozen[(size_t)e * NB + (size_t)gx * a.nnz + gz] != 0;
            if (v && !fz) updm |= 1u << r;
            if (v) {
                sv[r] = __ldg(a.s + ((size_t)gr * a.nnx + gx) * a.nnz + gz);
                hxv[r] = __ldg(a.hx + gr);
                hzv[r] = __ldg(a.hz + (size_t)gr * a.nnx + gx);
                inbv[r] = (gr > 0 ? 1u : 0u) | (gr < a.nnr - 1 ? 2u : 0u) | (gx > 0 ? 4u : 0u) |
                          (gx < a.nnx - 1 ? 8u : 0u) | (gz > 0 ? 16u : 0u) | (gz < a.nnz - 1 ? 32u : 0u);
            } else {
                sv[r] = R(0); hxv[r] = R(1); hzv[r] = R(1); inbv[r] = 0u;
            }
        }
        __syncthreads();

        unsigned chm = 0;
        int passes = 0;
        bool last_changed = false;
        const int cbase = (2 * BX + (tx + 2)) * BZ + (tz + 2);
        auto node = [&](int r, bool &ch) {
            if (!((updm >> r) & 1u)) return;
            const int c = cbase + r * SR;
            R t1[6], t2[6];
            t1[0] = box[c - SR];     t2[0] = box[c - 2 * SR];
            t1[1] = box[c + SR];     t2[1] = box[c + 2 * SR];
            t1[2] = box[c - BZ];     t2[2] = box[c - 2 * BZ];
            t1[3] = box[c + BZ];     t2[3] = box[c + 2 * BZ];
            t1[4] = box[c - 1];      t2[4] = box[c - 2];
            t1[5] = box[c + 1];      t2[5] = box[c + 2];
            const R hh[3] = {a.hr, hxv[r], hzv[r]};
            const R nv = fm_update<R>(sv[r], t1, t2, inbv[r], hh, a.order2);
            if (fbits(nv) != fbits(box[c])) {
                box[c] = nv;
                ch = true;
                chm |= 1u << r;
            }
        };
        for (int p = 0; p < a.max_passes; ++p) {
            bool ch = false;
            if (p & 1) {
#pragma unroll
                for (int k = 0; k < TR; ++k) node(k, ch);
            } else {
#pragma unroll
                for (int k = TR - 1; k >= 0; --k) node(k, ch);
            }
            ++passes;
            last_changed = __syncthreads_or(ch) != 0;
            if (!last_changed) break;
        }

        // write back changed nodes
#pragma unroll
        for (int r = 0; r < TR; ++r)
            if ((chm >> r) & 1u)
                Te[((size_t)(r0 + r) * a.nnx + gx) * a.nnz + gz] = box[cbase + r * SR];

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
            int f = s_face;
            if (tid == 6 && last_changed) f |= 64;    // pass cap hit: run again
            if ((f >> tid) & 1) {
                int nb = -1;
                const int sl = a.ntx * a.ntz;
                switch (tid) {
                    case 0: nb = tri > 0 ? w - sl : -1; break;
                    case 1: nb = tri < a.ntr - 1 ? w + sl : -1; break;
                    case 2: nb = txi > 0 ? w - a.ntz : -1; break;
                    case 3: nb = txi < a.ntx - 1 ? w + a.ntz : -1; break;
                    case 4: nb = tzi > 0 ? w - 1 : -1; break;
                    case 5: nb = tzi < a.ntz - 1 ? w + 1 : -1; break;
                    default: nb = w; break;
                }
                if (nb >= 0 && atomicExch(&a.flag[nb], 1) == 0) {
                    const int pos = atomicAdd(a.next_count, 1);
                    a.next_list[pos] = nb;
                }
            }
        }
        if (tid == 0) {
            const int vr = min(TR, a.nnr - r0), vx = min(TX, a.nnx - x0), vz = min(TZ, a.nnz - z0);
            my_tiles += 1;
            my_nodes += (unsigned long long)passes * (unsigned long long)(vr * vx * vz);
            my_staged += (unsigned long long)(vr * vx * vz);
        }
        __syncthreads();
    }
    if (tid == 0 && my_tiles) {
        atomicAdd(&a.stats[0], my_tiles);
        atomicAdd(&a.stats[1], my_nodes);
        atomicAdd(&a.stats[2], my_staged);
    }
}

template <typename R, int S>
static void launch_shape(int grid, const RoundArgs<R> &a, cudaStream_t st)
{
    constexpr int TR = kShapes[S].tr, TX = kShapes[S].tx, TZ = kShapes[S].tz;
    round_kernel<R, TR, TX, TZ><<<grid, TX * TZ, 0, st>>>(a);
}

template <typename R>
static void launch_any(int shape, int grid, const RoundArgs<R> &a, cudaStream_t st)
{
    switch (shape) {
        case 0: launch_shape<R, 0>(grid, a, st); break;
        case 1: launch_shape<R, 1>(grid, a, st); break;
        case 2: launch_shape<R, 2>(grid, a, st); break;
        case 3: launch_shape<R, 3>(grid, a, st); break;
        case 4: launch_shape<R, 4>(grid, a, st); break;
        default: launch_shape<R, 5>(grid, a, st); break;
    }
}

void launch_round_f64(int shape, int grid, const RoundArgs<double> &a, cudaStream_t st) { launch_any<double>(shape, grid, a, st); }
void launch_round_f32(int shape, int grid, const RoundArgs<float> &a, cudaStream_t st) { launch_any<float>(shape, grid, a, st); }

template <typename R, int S>
static int occ_shape()
{
    constexpr int TR = kShapes[S].tr, TX = kShapes[S].tx, TZ = kShapes[S].tz;
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, round_kernel<R, TR, TX, TZ>, TX * TZ, 0);
    return nb;
}

template <typename R>
static int occ_any(int shape)
{
    switch (shape) {
        case 0: return occ_shape<R, 0>();
        case 1: return occ_shape<R, 1>();
        case 2: return occ_shape<R, 2>();
        case 3: return occ_shape<R, 3>();
        case 4: return occ_shape<R, 4>();
        default: return occ_shape<R, 5>();
    }
}

int round_blocks_per_sm(int shape, int prec)
{
    return prec == FM3DT_FP64 ? occ_any<double>(shape) : occ_any<float>(shape);
}

}  // namespace fm3dt
