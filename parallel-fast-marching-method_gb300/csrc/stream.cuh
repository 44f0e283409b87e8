// stream.cuh -- streaming directional sweep (an alternative to the tile sweep
// of solver.cuh).
//
// One warp owns a block of SX x SZ (theta, phi) columns and streams through
// one height segment of the grid (the whole height, or a few tens of layers
// when more parallel work is needed) from the bottom upward.  Lane (x', z')
// updates layer r' at step r' + x' + z' (swept coordinates, as in the tile
// sweep), so each node sees its upwind neighbours' new values; the ramp of
// that wavefront (SX + SZ - 2 steps) is paid once per segment instead of
// once per tile.  The layers the lanes are working on, plus the two layers
// above and below and a two-column halo, sit in a shared-memory ring of RING
// layers.  Work items (segment, column block) go in hyperplanes of the
// event's sweep direction (one launch per hyperplane); an item's upwind
// neighbours are in earlier launches.  Events whose lateral direction is a
// near tie are swept twice more, with that direction reversed and then
// forward again; events still changing on many tiles after a round are swept
// again (flag mode: changed nodes queue their tiles).  The sweep is only a
// good start for the rounds, which reach the same fixed point from
// any start.
#pragma once
#include "solver.cuh"

namespace fm3dt {

// Ring of layers: at step s the lanes read layers s - (SX+SZ) .. s+2 and the
// warp stores layer s+3 (loaded into registers during step s-1), so the
// ring must hold SX + SZ + 4 layers.
template <int SX, int SZ>
struct StreamRing {
    static constexpr int need = SX + SZ + 4;
    static constexpr int value = need <= 16 ? 16 : (need <= 32 ? 32 : 64);
};

// Queue tile w with flag bits `bits` unless it holds them already (flags only
// gain bits while a sweep runs, so a stale read costs one needless atomic);
// the node's new value is made visible before the flag that sends its tile
// to a round.
template <typename R>
__device__ __forceinline__ void stream_queue(const StreamArgs<R> &a, int w, int bits)
{
    const int want = bits | kQueued;
    if ((__ldcg(a.flag + w) & want) == want) return;
    __threadfence();
    if (!(atomicOr(&a.flag[w], want) & kQueued)) a.list[atomicAdd(a.count, 1)] = w;
}

// A node changed in a flag-mode sweep (a verification sweep, a re-sweep, the
// near-tie events' last extra sweep): its tile recomputes every node,
// and each face neighbour whose 2-deep halo holds the node recomputes the
// nodes next to that face (the flag bits of the rounds).
template <typename R>
__device__ void stream_mark(const StreamArgs<R> &a, int e, int gr, int gx, int gz)
{
    const int ti = gr / a.tr, tj = gx / a.tx, tk = gz / a.tz;
    const int ri = gr - ti * a.tr, xi = gx - tj * a.tx, zi = gz - tk * a.tz;
    const int sl = a.ntx * a.ntz;
    const int w = e * a.tiles_per_event + (ti * a.ntx + tj) * a.ntz + tk;
    stream_queue(a, w, kFull);
    if (ri < 2 && ti > 0) stream_queue(a, w - sl, kFaceDown);
    if (ri >= a.tr - 2 && ti < a.ntr - 1) stream_queue(a, w + sl, kFaceUp);
    if (xi < 2 && tj > 0) stream_queue(a, w - a.ntz, kFaceXp);
    if (xi >= a.tx - 2 && tj < a.ntx - 1) stream_queue(a, w + a.ntz, kFaceXm);
    if (zi < 2 && tk > 0) stream_queue(a, w - 1, kFaceZp);
    if (zi >= a.tz - 2 && tk < a.ntz - 1) stream_queue(a, w + 1, kFaceZm);
}

// Activity of a tracked sweep, by chunks of 1 << act_shift layers of an
// item (bit c of a mask: layers [c << act_shift, (c + 1) << act_shift) of the
// item's segment).  Ahead of each launch of a tracked sweep with a previous
// sweep, this kernel writes, for every item of the launch (one thread each),
// the chunks whose nodes can change in this sweep (act_run), given the
// previous sweep's changed chunks (act_prev) and this sweep's (act_cur,
// written by the launches before): a node can change only if a node within
// two layers or columns of it changed since it was last computed -- in this
// item or a face neighbour in the previous sweep, or in an upstream face
// neighbour (below, and before it along theta and phi) in this one.  A
// lateral neighbour's chunk c holds the same layers as this item's chunk c,
// and each changed chunk wakes its own and the adjacent chunks; the items
// above and below meet this one in their (and its) two edge layers.  A
// skipped item's changed chunks are 0.  Items run and skipped are added to
// act_items; a slot beyond the act_n masks is not accessed (bit 2 of *err).
// One of the ten activity masks an item's chunks depend on (which = 0: the
// item, previous sweep; 1 / 2: the items below / above, previous sweep; 3-6:
// the lateral neighbours, previous sweep; 7: the item below, this sweep; 8 /
// 9: the upstream neighbours along theta / phi, this sweep); 0 outside the
// grid of items.  (bx, bz): the item's block in grid order; (sx, sz): the
// sweep's directions.
template <typename R>
__device__ __forceinline__ unsigned stream_mask_read(const StreamArgs<R> &a, int which, int k, int nsegs, int seg,
                                                     int bx, int bz, bool sx, bool sz)
{
    int s_ = seg, x_ = bx, z_ = bz;
    switch (which) {
        case 1: case 7: s_ = seg - 1; break;
        case 2: s_ = seg + 1; break;
        case 3: x_ = bx - 1; break;
        case 4: x_ = bx + 1; break;
        case 5: z_ = bz - 1; break;
        case 6: z_ = bz + 1; break;
        case 8: x_ = bx + (sx ? -1 : 1); break;
        case 9: z_ = bz + (sz ? -1 : 1); break;
        default: break;
    }
    if (s_ < 0 || s_ >= nsegs || x_ < 0 || x_ >= a.nbx || z_ < 0 || z_ >= a.nbz) return 0u;
    const size_t q = ((size_t)(k * nsegs + s_) * a.nbx + x_) * a.nbz + z_;
    if (q >= a.act_n) {
        atomicOr(a.err, 4);
        return 0u;
    }
    return __ldcg((which >= 7 ? a.act_cur : a.act_prev) + q);
}

// The chunks of an item that run, from its ten masks m[] (see
// stream_mask_read); seg_len: layers per segment, nlay: this item's layers.
__device__ __forceinline__ unsigned stream_mask_combine(const unsigned *m, int seg_len, int nlay, int sh)
{
    auto spread = [](unsigned v) { return v | (v << 1) | (v >> 1); };
    unsigned run = spread(m[0] | m[3] | m[4] | m[5] | m[6] | m[8] | m[9]);
    // the item below: its top two layers, next to this item's bottom chunk
    const unsigned below_top2 = (1u << ((seg_len - 1) >> sh)) | (1u << ((seg_len - 2) >> sh));
    if ((m[1] | m[7]) & below_top2) run |= 1u;
    // the item above: its bottom chunk, next to this item's top two layers
    if (m[2] & 1u) run |= (1u << ((nlay - 1) >> sh)) | (nlay >= 2 ? 1u << ((nlay - 2) >> sh) : 0u);
    const int nch = ((nlay - 1) >> sh) + 1;
    if (nch < 32) run &= (1u << nch) - 1u;
    return run;
}

template <typename R>
__global__ void __launch_bounds__(128) stream_activity_kernel(StreamArgs<R> a)
{
    const long long count = (long long)a.hcount * a.nev;
    const int nsegs = (a.f.nnr + a.seg_len - 1) / a.seg_len;
    const int sh = a.act_shift;
    unsigned nrun = 0, nskip = 0;
    for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < count;
         item += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(item / a.hcount);
        const int j = (int)(item - (long long)k * a.hcount);
        const int e = a.events ? a.events[k] : k;
        const int packed = a.hp_blocks[a.hoff + j];
        const int seg = packed >> 24, bxp = (packed >> 12) & 0xfff, bzp = packed & 0xfff;
        int dir = a.dir[e];
        if (a.flip & 4) dir ^= ((dir >> 2) & 1) | (((dir >> 3) & 1) << 1);
        dir ^= a.flip & 3;
        const bool sx = dir & 1, sz = (dir >> 1) & 1;
        const int bx = sx ? bxp : a.nbx - 1 - bxp, bz = sz ? bzp : a.nbz - 1 - bzp;
        const int lo = seg * a.seg_len, nlay = min(a.f.nnr, lo + a.seg_len) - lo;
        unsigned m[10];
#pragma unroll
        for (int w = 0; w < 10; ++w) m[w] = stream_mask_read(a, w, k, nsegs, seg, bx, bz, sx, sz);
        const unsigned run = stream_mask_combine(m, a.seg_len, nlay, sh);
        const size_t self = ((size_t)(k * nsegs + seg) * a.nbx + bx) * a.nbz + bz;
        if (self < a.act_n) {
            a.act_run[self] = run;
            if (!run) a.act_cur[self] = 0;
        } else {
            atomicOr(a.err, 4);
        }
        if (run) ++nrun; else ++nskip;
    }
    if (a.act_items) {
        for (int o = 16; o > 0; o >>= 1) {
            nrun += __shfl_xor_sync(0xffffffffu, nrun, o);
            nskip += __shfl_xor_sync(0xffffffffu, nskip, o);
        }
        if ((threadIdx.x & 31) == 0 && (nrun | nskip)) {
            atomicAdd(&a.act_items[0], (unsigned long long)nrun);
            atomicAdd(&a.act_items[1], (unsigned long long)nskip);
        }
    }
}

// Bounded wait of the one-launch (FLOW) form of a sweep for an upstream
// item's done flag: past this many polls (each an L2 round trip and a
// ~64 ns sleep: about a second in all) the error flag is raised and the item
// goes on.
constexpr unsigned kFlowSpins = 1u << 20;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int *p)
{
    int v;
    asm volatile("ld.volatile.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// A tracked sweep goes straight to the next step that can change a node
// (seating its ring anew) when at least this many quiet steps lie before it.
constexpr int kStreamJump = 4;

// One field element into shared memory by an asynchronous copy (L1-cached:
// the layers an item reads are written in other launches, or by the item
// itself); cp_async_wait_all waits for this thread's copies.
template <typename R>
__device__ __forceinline__ void cp_async_elem(R *smem, const R *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (sizeof(R) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// FRESH: the main sweep of a solve, from an unset field (every node except
// the fixed bottom layer unset).  Each node above the bottom layer then sees
// its downstream neighbours (up, and the lateral ones the sweep runs toward)
// still unset -- later lanes of the block and later launches have not
// written them, and the node's update must not take them -- so it is
// computed by fm_update_upstream, which gives fm_update's value with those
// neighbours unset from the three upstream ones alone.  (Items of the same
// hyperplane may already have written a downstream neighbour in a halo
// column; the upstream form leaves it out, as a sweep from an unset field
// would, and the rounds reach the same fixed point either way.)  The bottom
// layer keeps fm_update: fixed boundary nodes beside an unset one are set.
template <typename R, int SX, int SZ, bool FRESH, bool FLOW>
__device__ __forceinline__ void stream_sweep_body(const StreamArgs<R> &a)
{
    static_assert(SX * SZ == 32, "one warp per column block");
    constexpr int LX = SX + 4, LZ = SZ + 4, LAYER = LX * LZ;
    constexpr int RING = StreamRing<SX, SZ>::value;
    __shared__ R ring[RING * LAYER];
    // tracked sweeps (kept here rather than in registers through the step
    // loop): the item's activity slot, its chunks that changed, and its
    // chunks whose nodes can change (see stream_activity_kernel)
    __shared__ size_t s_aslot;
    __shared__ unsigned s_changed, s_active;
    // FLOW: the item taken from the pass's queue; the activity masks read by
    // lanes 0-9
    __shared__ long long s_item;
    __shared__ size_t s_slot;
    __shared__ unsigned s_m[10];
    using TL = Tile<R, 1, SX, SZ>;
    const FieldArgs<R> &f = a.f;
    const int lane = threadIdx.x;
    const int lx = lane / SZ, lz = lane % SZ;
    const R INF = Lim<R>::inf();
    const size_t N = (size_t)f.nnx * f.nnz * (size_t)f.nnr;
    const long long count = (long long)a.hcount * a.nev;
    for (long long it = blockIdx.x;; it += gridDim.x) {
        // FLOW: one launch per pass; items in the order of their hyperplanes
        // (block-major, then event), each taken from the queue and started
        // when its three upstream neighbours are done
        long long item = it;
        if (FLOW) {
            if (lane == 0) s_item = (long long)atomicAdd(a.next, 1u);
            __syncwarp();
            item = s_item;
            __syncwarp();
        }
        if (item >= count) break;
        int k, packed;
        if (FLOW) {
            const long long fb = item / a.nev;
            k = (int)(item - fb * a.nev);
            packed = a.hp_blocks[fb];
        } else {
            k = (int)(item / a.hcount);
            packed = a.hp_blocks[a.hoff + (int)(item - (long long)k * a.hcount)];
        }
        const int e = a.events ? a.events[k] : k;
        const int seg = packed >> 24, bxp = (packed >> 12) & 0xfff, bzp = packed & 0xfff;
        int dir = a.dir[e];
        if (a.flip & 4) dir ^= ((dir >> 2) & 1) | (((dir >> 3) & 1) << 1);
        dir ^= a.flip & 3;
        const bool sx = dir & 1, sz = (dir >> 1) & 1;
        // this item's layers, counted upward from the bottom: [lo, hi)
        const int lo = seg * a.seg_len, hi = min(f.nnr, lo + a.seg_len);
        const int x0 = (sx ? bxp : a.nbx - 1 - bxp) * SX;
        const int z0 = (sz ? bzp : a.nbz - 1 - bzp) * SZ;
        const int xs = sx ? lx : SX - 1 - lx;
        const int zs = sz ? lz : SZ - 1 - lz;
        const int gx = x0 + lx, gz = z0 + lz;
        const bool colv = gx < f.nnx && gz < f.nnz;
        R *Te = f.T + (size_t)e * N;
        // the item's slot (event ordinal, segment, column block in grid
        // order) in the activity masks and the done flags
        const int nsegs = (f.nnr + a.seg_len - 1) / a.seg_len;
        const size_t slot = ((size_t)(k * nsegs + seg) * a.nbx + x0 / SX) * a.nbz + z0 / SZ;
        if (FLOW) {
            // (kept in shared memory for the item's end)
            __syncwarp();
            if (lane == 0) s_slot = slot;
            // lanes 0-2: the items below, and before this one along theta
            // and phi, done (a bounded wait: past the limit the error flag
            // is raised and the item goes on)
            if (lane < 3) {
                const int s_ = seg - (lane == 0), xq = bxp - (lane == 1), zq = bzp - (lane == 2);
                if (s_ >= 0 && xq >= 0 && zq >= 0) {
                    const int bxq = sx ? xq : a.nbx - 1 - xq, bzq = sz ? zq : a.nbz - 1 - zq;
                    const size_t q = ((size_t)(k * nsegs + s_) * a.nbx + bxq) * a.nbz + bzq;
                    if (q < a.done_n) {
                        // (once any wait of the launch has given up, the
                        // others do too)
                        unsigned spins = 0;
                        while (ld_acquire_u32(a.done + q) == 0u) {
                            if (++spins > kFlowSpins || ((spins & 63u) == 0u && (ld_volatile_i32(a.err) & 16))) {
                                atomicOr(a.err, 16);
                                break;
                            }
                            __nanosleep(64);
                        }
                    } else {
                        atomicOr(a.err, 16);
                    }
                }
            }
            __syncwarp();
        }
        {
        // activity: the chunks that run
        if (!FRESH && a.act_cur) {
            const size_t aslot = slot;
            unsigned run = ~0u;
            if (a.act_prev) {
                if (FLOW) {
                    // from the neighbours' masks, as stream_activity_kernel
                    // computes it for a launch of a hyperplane
                    if (lane < 10) s_m[lane] = stream_mask_read(a, lane, k, nsegs, seg, x0 / SX, z0 / SZ, sx, sz);
                    __syncwarp();
                    run = stream_mask_combine(s_m, a.seg_len, hi - lo, a.act_shift);
                    if (lane == 0) {
                        if (!run && aslot < a.act_n) a.act_cur[aslot] = 0;
                        if (a.act_items) atomicAdd(a.act_items + (run ? 0 : 1), 1ull);
                    }
                } else {
                    // (stream_activity_kernel wrote the chunks that run)
                    run = aslot < a.act_n ? __ldcg(a.act_run + aslot) : 0u;
                }
            }
            if (!run) goto item_done;
            __syncwarp();
            if (lane == 0) {
                s_aslot = aslot;
                s_changed = 0;
                s_active = run;
            }
        }
        // layer rp (counted upward from the bottom) into registers (this
        // lane's share of the layer), unset outside the grid; then into its
        // ring slot
        constexpr int PER = (LAYER + 31) / 32;
        R buf[PER];
        // this lane's share of a layer: offsets in a grid layer (phi
        // fastest), -1 outside the grid; the same for every layer of the item
        const size_t lstride = (size_t)f.nnx * f.nnz;
        int loff[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int q = lane + 32 * k;
            const int qx = x0 + q / LZ - 2, qz = z0 + q % LZ - 2;
            loff[k] = (q < LAYER && qx >= 0 && qx < f.nnx && qz >= 0 && qz < f.nnz) ? qx * f.nnz + qz : -1;
        }
        auto fetch_layer = [&](int rp) {
            const bool rin = rp >= 0 && rp < f.nnr;
            const R *src = Te + (size_t)(f.nnr - 1 - (rin ? rp : 0)) * lstride;
#pragma unroll
            for (int k = 0; k < PER; ++k) buf[k] = (rin && loff[k] >= 0) ? __ldcg(src + loff[k]) : INF;
        };
        auto store_layer = [&](int rp) {
            R *dst = ring + ((rp + RING) & (RING - 1)) * LAYER;
#pragma unroll
            for (int k = 0; k < PER; ++k)
                if (lane + 32 * k < LAYER) dst[lane + 32 * k] = buf[k];
        };
        __syncwarp();
        for (int rp = lo - 2; rp <= lo + 2; ++rp) {
            fetch_layer(rp);
            store_layer(rp);
        }
        fetch_layer(lo + 3);
        const int c = (lx + 2) * LZ + (lz + 2);
        typename TL::Params pnext{};
        if (colv && xs + zs == 0) pnext = TL::params_global(f, f.nnr - 1 - lo, gx, gz);
        const int steps = (hi - lo) + SX + SZ - 2;
        for (int step = 0; step < steps; ++step) {
            // layer lo+step+3 was fetched during the previous step; fetch
            // the next one now, used a step later
            store_layer(lo + step + 3);
            fetch_layer(lo + step + 4);
            __syncwarp();
            const int rp = lo + step - xs - zs;
            const typename TL::Params pcur = pnext;
            // the next node's slowness and spacings, one step ahead
            if (colv && rp + 1 >= lo && rp + 1 < hi) pnext = TL::params_global(f, f.nnr - 2 - rp, gx, gz);
            // (tracked sweeps: the step runs when a lane's node lies in a
            // chunk that can change)
            if (!FRESH && a.act_cur &&
                !__any_sync(0xffffffffu, colv && rp >= lo && rp < hi && ((s_active >> ((rp - lo) >> a.act_shift)) & 1u))) {
                // A quiet step.  The first step from here with a node in a
                // chunk that can change (at step t the lanes hold layers
                // lo + t - (SX + SZ - 2) .. lo + t); none: the item is done.
                // The steps between change nothing and so wake no chunk: far
                // enough ahead, go there directly, the ring seated anew by
                // asynchronous copies (one wait for all of them).
                const int r0 = max(0, step - (SX + SZ - 2));
                const int c0 = r0 >> a.act_shift;
                const unsigned m = c0 < 32 ? s_active & (~0u << c0) : 0u;
                if (!m) break;
                const int t = max((__ffs(m) - 1) << a.act_shift, r0);
                if (t - step >= kStreamJump && t < steps) {
                    __syncwarp();
                    for (int r = max(lo - 2, lo + t - (SX + SZ)); r <= lo + t + 2; ++r) {
                        if (FLOW) {
                            // (other CTAs of this launch wrote these layers:
                            // loads from L2, not a possibly older L1 line)
                            fetch_layer(r);
                            store_layer(r);
                            continue;
                        }
                        const bool rin = r >= 0 && r < f.nnr;
                        const R *src = Te + (size_t)(f.nnr - 1 - (rin ? r : 0)) * lstride;
                        R *dst = ring + ((r + RING) & (RING - 1)) * LAYER;
#pragma unroll
                        for (int k = 0; k < PER; ++k) {
                            const int q = lane + 32 * k;
                            if (q < LAYER) {
                                if (rin && loff[k] >= 0)
                                    cp_async_elem(dst + q, src + loff[k]);
                                else
                                    dst[q] = INF;
                            }
                        }
                    }
                    if (!FLOW) cp_async_wait_all();
                    fetch_layer(lo + t + 3);
                    const int rq = lo + t - xs - zs;
                    if (colv && rq >= lo && rq < hi) pnext = TL::params_global(f, f.nnr - 1 - rq, gx, gz);
                    step = t - 1;
                }
                __syncwarp();
                continue;
            }
            if (colv && rp >= lo && rp < hi) {
                const int gr = f.nnr - 1 - rp;
                if (!TL::frozen(f, e, gr, gx, gz)) {
                    const R *L0 = ring + ((rp + RING) & (RING - 1)) * LAYER;
                    const R *Lu1 = ring + ((rp + 1 + RING) & (RING - 1)) * LAYER;
                    const R *Lu2 = ring + ((rp + 2 + RING) & (RING - 1)) * LAYER;
                    const R *Ld1 = ring + ((rp - 1 + RING) & (RING - 1)) * LAYER;
                    const R *Ld2 = ring + ((rp - 2 + RING) & (RING - 1)) * LAYER;
                    R v;
                    if (FRESH && rp >= 1) {
                        // upstream: down, and x-1 / z-1 when the sweep runs
                        // toward +theta / +phi (else x+1 / z+1)
                        const int ox = sx ? -LZ : LZ, oz = sz ? -1 : 1;
                        const bool xlo = gx > 0, xhi = gx < f.nnx - 1, zlo = gz > 0, zhi = gz < f.nnz - 1;
                        v = fm_update_upstream<R>(pcur.s, Ld1[c], Ld2[c], L0[c + ox], L0[c + 2 * ox], L0[c + oz],
                                                  L0[c + 2 * oz], true, gr > 0, sx ? xlo : xhi, sx ? xhi : xlo,
                                                  sz ? zlo : zhi, sz ? zhi : zlo, pcur.sp, f.order2);
                    } else {
                        R t1[6], t2[6];
                        t1[0] = Lu1[c];       t2[0] = Lu2[c];          // r-1 (up)
                        t1[1] = Ld1[c];       t2[1] = Ld2[c];          // r+1 (down)
                        t1[2] = L0[c - LZ];   t2[2] = L0[c - 2 * LZ];
                        t1[3] = L0[c + LZ];   t2[3] = L0[c + 2 * LZ];
                        t1[4] = L0[c - 1];    t2[4] = L0[c - 2];
                        t1[5] = L0[c + 1];    t2[5] = L0[c + 2];
                        const unsigned inb = (gr > 0 ? 1u : 0u) | (gr < f.nnr - 1 ? 2u : 0u) | (gx > 0 ? 4u : 0u) |
                                             (gx < f.nnx - 1 ? 8u : 0u) | (gz > 0 ? 16u : 0u) |
                                             (gz < f.nnz - 1 ? 32u : 0u);
                        v = fm_update<R>(pcur.s, t1, t2, inb, pcur.sp, f.order2);
                    }
                    const R old = L0[c];
                    if (fbits(v) != fbits(old)) {
                        ring[((rp + RING) & (RING - 1)) * LAYER + c] = v;
                        Te[((size_t)gr * f.nnx + gx) * f.nnz + gz] = v;
                        if (!FRESH && a.act_cur) {
                            // this chunk changed; it and its neighbours can change further
                            const unsigned b = 1u << ((rp - lo) >> a.act_shift);
                            atomicOr(&s_changed, b);
                            atomicOr(&s_active, b | (b << 1) | (b >> 1));
                        }
                        if (a.flag) stream_mark(a, e, gr, gx, gz);
                    }
                }
            }
            __syncwarp();
        }
        if (!FRESH && a.act_cur && lane == 0 && s_aslot < a.act_n) a.act_cur[s_aslot] = s_changed;
        }
    item_done:
        if (FLOW) {
            // the item's writes (field, masks, queued tiles) before its flag
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                const size_t q = s_slot;
                if (q < a.done_n)
                    st_release_u32(a.done + q, 1u);
                else
                    atomicOr(a.err, 16);
            }
        }
    }
}

// The per-hyperplane form (one launch per hyperplane of a pass) and the
// one-launch form, each with its own register budget: the one-launch form
// holds its items' queue state, and is bounded to the resident CTAs of the
// per-hyperplane form's main sweep.
#ifndef FM_FLOW_BLOCKS_F32
#define FM_FLOW_BLOCKS_F32 20
#endif
template <typename R> struct FlowBlocks { static constexpr int value = FM_FLOW_BLOCKS_F32; };
template <> struct FlowBlocks<double> { static constexpr int value = 12; };

template <typename R, int SX, int SZ, bool FRESH>
__global__ void __launch_bounds__(32) stream_sweep_kernel(StreamArgs<R> a)
{
    stream_sweep_body<R, SX, SZ, FRESH, false>(a);
}

template <typename R, int SX, int SZ, bool FRESH>
__global__ void __launch_bounds__(32, FlowBlocks<R>::value) stream_flow_kernel(StreamArgs<R> a)
{
    stream_sweep_body<R, SX, SZ, FRESH, true>(a);
}

template <typename R, int SX, int SZ>
struct StreamKernels {
    static void sweep(int grid, const StreamArgs<R> &a, cudaStream_t st)
    {
        if (a.flow) {
            if (a.fresh)
                stream_flow_kernel<R, SX, SZ, true><<<grid, 32, 0, st>>>(a);
            else
                stream_flow_kernel<R, SX, SZ, false><<<grid, 32, 0, st>>>(a);
            return;
        }
        if (!a.fresh && a.act_cur && a.act_prev) {
            const long long items = (long long)a.hcount * a.nev;
            const int blocks = (int)std::min<long long>((items + 127) / 128, 4096);
            stream_activity_kernel<R><<<blocks, 128, 0, st>>>(a);
        }
        if (a.fresh)
            stream_sweep_kernel<R, SX, SZ, true><<<grid, 32, 0, st>>>(a);
        else
            stream_sweep_kernel<R, SX, SZ, false><<<grid, 32, 0, st>>>(a);
    }
    static int occ(bool fresh, bool flow)
    {
        int nb = 0;
        if (flow) {
            if (fresh)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stream_flow_kernel<R, SX, SZ, true>, 32, 0);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stream_flow_kernel<R, SX, SZ, false>, 32, 0);
        } else if (fresh) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stream_sweep_kernel<R, SX, SZ, true>, 32, 0);
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stream_sweep_kernel<R, SX, SZ, false>, 32, 0);
        }
        return nb;
    }
};

#define FM_STREAM_SWITCH(idx, CALL)       \
    switch (idx) {                        \
        case 0: CALL(4, 8); break;        \
        default: CALL(2, 16); break;      \
    }

}  // namespace fm3dt
