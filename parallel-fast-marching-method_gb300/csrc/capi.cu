// capi.cu -- the C ABI of libfm3dt_gpu (declared in include/fm3dt_gpu.h).
//
// Host-side orchestration of the per-source pipeline that fm3dt_parallel.f90
// runs per source (F:6371-6599): boundary injection, the tile-round solve
// loop, receiver times, rays and Frechet rows.  All device memory is owned by
// the context; all work goes to the context's stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

using namespace fm3dt;

namespace {

thread_local std::string g_create_err;

int fail(fm3dt_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    else g_create_err = msg;
    return code;
}

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? FM3DT_ENOMEM : FM3DT_ECUDA,       \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

#define CKL()                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess)                                                                   \
            return fail(ctx, FM3DT_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

// Device buffers of one call, allocated on the context's stream and freed
// (stream-ordered) on every return path.
struct DeviceScratch {
    cudaStream_t s;
    cudaMemPool_t pool;
    std::vector<void *> bufs;
    // from the context's pool (which keeps its memory between calls) on the
    // context's stream
    explicit DeviceScratch(const fm3dt_ctx *ctx) : s(ctx->stream), pool(ctx->pool) {}
    DeviceScratch(const DeviceScratch &) = delete;
    DeviceScratch &operator=(const DeviceScratch &) = delete;
    template <typename T>
    cudaError_t alloc(T **p, size_t n)
    {
        *p = nullptr;
        if (n == 0) return cudaSuccess;
        cudaError_t e = pool ? cudaMallocFromPoolAsync((void **)p, n * sizeof(T), pool, s)
                             : cudaMallocAsync((void **)p, n * sizeof(T), s);
        if (e == cudaSuccess) bufs.push_back((void *)*p);
        return e;
    }
    ~DeviceScratch()
    {
        for (void *p : bufs) cudaFreeAsync(p, s);
    }
};

// fm3dt_parallel.f90:61 initialises the double-precision pi from a
// default-kind (single precision) literal; the converted angles use that value.
double ref_pi() { return (double)3.1415926535898f; }

Geom convert(const fm3dt_grid_desc &d)
{
    const double pi = ref_pi();
    Geom g;
    g.nvr = d.nvr; g.nvx = d.nvx; g.nvz = d.nvz;
    g.gor = d.gor;
    g.dvr = d.dvr;
    g.dvx = d.dvxd * pi / 180.0;          // F:6110-6117
    g.dvz = d.dvzd * pi / 180.0;
    g.gox = (90.0 - d.goxd) * pi / 180.0;
    g.goz = d.gozd * pi / 180.0;
    g.nnr = d.nnr; g.nnx = d.nnx; g.nnz = d.nnz;
    g.rgor = d.rgor;
    g.dnr = d.dnr;
    g.dnx = d.dnxd * pi / 180.0;
    g.dnz = d.dnzd * pi / 180.0;
    g.rgox = (90.0 - d.rgoxd) * pi / 180.0;
    g.rgoz = d.rgozd * pi / 180.0;
    g.earth = d.earth;
    return g;
}

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

size_t rsize(int prec) { return prec == FM3DT_FP64 ? sizeof(double) : sizeof(float); }

int tiles_per_event(const Geom &g, int shape, int *ntr, int *ntx, int *ntz)
{
    const TileShape s = kShapes[shape];
    *ntr = (g.nnr + s.tr - 1) / s.tr;
    *ntx = (g.nnx + s.tx - 1) / s.tx;
    *ntz = (g.nnz + s.tz - 1) / s.tz;
    return *ntr * *ntx * *ntz;
}

template <typename R>
void fill_geometry(const Geom &g, std::vector<R> &hx, std::vector<R> &hz, std::vector<R> &wx, std::vector<R> &wz)
{
    // spacings at each node as the stencil evaluates them (F:642-644, 712ff):
    // dr, r*dtheta, r*sin(theta)*dphi with r = rgor - (ir-1)*dnr + earth,
    // and their inverse squares
    hx.resize(g.nnr);
    wx.resize(g.nnr);
    hz.resize((size_t)g.nnr * g.nnx);
    wz.resize((size_t)g.nnr * g.nnx);
    for (int ir = 0; ir < g.nnr; ++ir) {
        const double ri = g.rgor - (double)ir * g.dnr + g.earth;
        const double v = ri * g.dnx;
        hx[ir] = (R)v;
        wx[ir] = (R)(1.0 / (v * v));
        for (int ix = 0; ix < g.nnx; ++ix) {
            const double risti = ri * std::sin(g.rgox + (double)ix * g.dnx);
            const double w = risti * g.dnz;
            hz[(size_t)ir * g.nnx + ix] = (R)w;
            wz[(size_t)ir * g.nnx + ix] = (R)(1.0 / (w * w));
        }
    }
}

template <typename R>
int upload_geometry(fm3dt_ctx *ctx)
{
    std::vector<R> hx, hz, wx, wz;
    fill_geometry<R>(ctx->g, hx, hz, wx, wz);
    CK(cudaMemcpy(ctx->d_hx, hx.data(), hx.size() * sizeof(R), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_hz, hz.data(), hz.size() * sizeof(R), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_wx, wx.data(), wx.size() * sizeof(R), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_wz, wz.data(), wz.size() * sizeof(R), cudaMemcpyHostToDevice));
    return FM3DT_OK;
}

// Tile hyperplanes a' + b' + c' = h of the swept tile coordinates of a shape
// (a' counts tile layers upward from the bottom), packed a'<<20 | b'<<10 | c'.
int ensure_planes(fm3dt_ctx *ctx, int shape)
{
    auto &P = ctx->planes[shape];
    if (P.shape == shape) return FM3DT_OK;
    int ntr, ntx, ntz;
    tiles_per_event(ctx->g, shape, &ntr, &ntx, &ntz);
    if (ntr > 2047 || ntx > 1023 || ntz > 1023) return fail(ctx, FM3DT_EINVAL, "too many tiles along one axis");
    const int H = ntr + ntx + ntz - 2;
    std::vector<std::vector<int>> by(H);
    for (int a = 0; a < ntr; ++a)
        for (int b = 0; b < ntx; ++b)
            for (int c = 0; c < ntz; ++c) by[a + b + c].push_back((a << 20) | (b << 10) | c);
    std::vector<int> flat;
    P.off.assign(H, 0);
    P.cnt.assign(H, 0);
    for (int h = 0; h < H; ++h) {
        P.off[h] = (int)flat.size();
        P.cnt[h] = (int)by[h].size();
        flat.insert(flat.end(), by[h].begin(), by[h].end());
    }
    CK(cudaMalloc(&P.d_tiles, flat.size() * sizeof(int)));
    CK(cudaMemcpy(P.d_tiles, flat.data(), flat.size() * sizeof(int), cudaMemcpyHostToDevice));
    P.shape = shape;
    return FM3DT_OK;
}

// Hyperplanes s' + x' + z' = h of a streaming sweep's work items: height
// segment s' (counted upward), column blocks x', z' in swept coordinates,
// packed s'<<24 | x'<<12 | z'.
int ensure_block_planes(fm3dt_ctx *ctx, int sweep_shape, int nseg, const fm3dt_ctx::Planes **out)
{
    for (const auto &P : ctx->block_planes)
        if (P.shape == sweep_shape && P.nseg == nseg) {
            *out = &P;
            return FM3DT_OK;
        }
    const StreamShape ss = kStreamShapes[sweep_shape - kNumShapes];
    const int nbx = (ctx->g.nnx + ss.sx - 1) / ss.sx, nbz = (ctx->g.nnz + ss.sz - 1) / ss.sz;
    if (nbx > 4095 || nbz > 4095 || nseg > 127) return fail(ctx, FM3DT_EINVAL, "too many column blocks or segments");
    fm3dt_ctx::Planes P;
    P.shape = sweep_shape;
    P.nseg = nseg;
    const int H = nseg + nbx + nbz - 2;
    std::vector<int> flat;
    P.off.assign(H, 0);
    P.cnt.assign(H, 0);
    for (int h = 0; h < H; ++h) {
        P.off[h] = (int)flat.size();
        for (int s = 0; s < nseg && s <= h; ++s)
            for (int b = std::max(0, h - s - nbz + 1); b <= std::min(h - s, nbx - 1); ++b)
                flat.push_back((s << 24) | (b << 12) | (h - s - b));
        P.cnt[h] = (int)flat.size() - P.off[h];
    }
    CK(cudaMalloc(&P.d_tiles, flat.size() * sizeof(int)));
    CK(cudaMemcpy(P.d_tiles, flat.data(), flat.size() * sizeof(int), cudaMemcpyHostToDevice));
    ctx->block_planes.push_back(std::move(P));
    *out = &ctx->block_planes.back();
    return FM3DT_OK;
}

// Height segments for a streaming sweep over nitems events: enough work
// items per launch to fill the GPU once, each segment at least 16 layers.
// Height segments for a streaming sweep of nitems events: the count that
// minimises a model of its time.  Hyperplane h of the items (segment s,
// column block (x', z')) with s + x' + z' = h is one launch; its items run in
// ceil(items / sgrid) waves of seg_len + SX + SZ - 2 steps each (the
// wavefront ramp), plus a few steps' worth of launch gap.  More segments give
// a launch more items (fewer idle SMs) but more launches and more ramp.
int stream_segments(const fm3dt_ctx *ctx, int nitems, int nbx, int nbz, int sgrid, int ramp)
{
    const int nnr = ctx->g.nnr;
    constexpr double kLaunchSteps = 4.0;
    // an item fills its ring (five layers and the first prefetch) before its
    // first step: about six steps' worth of loads
    constexpr int kFillSteps = 6;
    // blocks per lateral hyperplane (x' + z' = d)
    std::vector<long long> lat(nbx + nbz - 1, 0);
    for (int d = 0; d < nbx + nbz - 1; ++d)
        lat[d] = std::min(d, nbx - 1) - std::max(0, d - (nbz - 1)) + 1;
    int best = 1;
    double best_t = 0.0;
    for (int nseg = 1; nseg <= std::max(1, nnr / 8); nseg *= 2) {
        const int seg_len = (nnr + nseg - 1) / nseg;
        double t = 0.0;
        for (int h = 0; h < nbx + nbz - 1 + nseg - 1; ++h) {
            long long cnt = 0;
            for (int sg = 0; sg < nseg; ++sg) {
                const int d = h - sg;
                if (d >= 0 && d < nbx + nbz - 1) cnt += lat[d];
            }
            const long long items = cnt * (long long)nitems;
            t += (double)((items + sgrid - 1) / sgrid) * (seg_len + ramp + kFillSteps) + kLaunchSteps;
        }
        if (nseg == 1 || t < best_t) {
            best = nseg;
            best_t = t;
        }
    }
    return best;
}

// The field as a 4-D tensor (phi, theta, r, event) for TMA copies of a round
// tile's box; null when TMA cannot be used (phi rows not a multiple of 16
// bytes, the driver entry point missing, or switched off).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn()
{
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return (EncodeTiledFn)p;
    }();
    return fn;
}

const CUtensorMap *field_tensor_map(fm3dt_ctx *ctx, int shape)
{
    if (!ctx->use_tma) return nullptr;
    if (ctx->tmap_ok[shape]) return &ctx->tmap[shape];
    const Geom &g = ctx->g;
    const size_t es = ctx->prec == FM3DT_FP64 ? 8 : 4;
    if (((size_t)g.nnz * es) % 16 != 0) return nullptr;
    EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return nullptr;
    const cuuint64_t dims[4] = {(cuuint64_t)g.nnz, (cuuint64_t)g.nnx, (cuuint64_t)g.nnr, (cuuint64_t)ctx->maxev};
    const cuuint64_t strides[3] = {(cuuint64_t)g.nnz * es, (cuuint64_t)g.nnz * g.nnx * es,
                                   (cuuint64_t)g.nnz * g.nnx * g.nnr * es};
    // the box of Tile<R, tr, tx, tz>: tz + 8 phi columns, 2-deep halos in theta and r
    const TileShape ts = kShapes[shape];
    const cuuint32_t box[4] = {(cuuint32_t)(ts.tz + 8), (cuuint32_t)(ts.tx + 4), (cuuint32_t)(ts.tr + 4), 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(&ctx->tmap[shape], es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                           ctx->d_T, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA);
    if (r != CUDA_SUCCESS) return nullptr;
    // the slowness [r][theta][phi]: the tile's own nodes, no halo
    const cuuint32_t sbox[3] = {(cuuint32_t)ts.tz, (cuuint32_t)ts.tx, (cuuint32_t)ts.tr};
    const CUresult r2 = enc(&ctx->smap[shape], es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                            3, ctx->d_s, dims, strides, sbox, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA);
    if (r2 != CUDA_SUCCESS) return nullptr;
    ctx->tmap_ok[shape] = true;
    return &ctx->tmap[shape];
}

// Solve schedule.  Per context, at run time (fm3dt_set_schedule; the
// autotuner picks them per workload): the near-tie events' extra sweeps and
// band, the re-sweeps after the first rounds and their threshold.
// Compile-time (the measured best on this GPU):
//   FM_ROUND0_PER_TILE     first round with one CTA per tile when its tile count is known
//   FM_OVERLAP_TIES        near-tie events' sweeps and first round beside the other events' ...
//   FM_OVERLAP_MIN_EVENTS  ... when at least this many other events are in the batch
//   FM_CERTIFY             the other events' first round only where the certification
//                          of their single sweep fails
//   FM_OVERLAP_MAIN        the near-tie events' main sweep on stream2 too, ahead of
//                          their extra sweeps, beside the other events' main sweep
//   FM_FRESH_SWEEP         main sweeps from the unset field with upstream-only node
//                          updates (the same values as the full update there)
//   FM_TIE_QUEUE           the near-tie events' last extra sweep queues the tiles
//                          it changes for their first round, which then takes
//                          those tiles instead of every tile
//   FM_TIE_SKIP            the near-tie events' extra sweeps after the first skip
//                          the items where nothing near them changed (StreamArgs)
#ifndef FM_TIE_QUEUE
#define FM_TIE_QUEUE 1
#endif
#ifndef FM_TIE_SKIP
#define FM_TIE_SKIP 1
#endif
//   FM_TIES_FIRST          in a two-part solve the other events' main sweep waits
//                          for the near-tie events' one
#ifndef FM_TIES_FIRST
#define FM_TIES_FIRST 0
#endif
//   FM_SWEEP_FLOW          a streaming sweep pass as one launch whose items start
//                          when their upstream neighbours are done (instead of
//                          one launch per hyperplane)
#ifndef FM_SWEEP_FLOW
#define FM_SWEEP_FLOW 1
#endif
//   FM_FLOW_FIRST          ... the first tracked sweep of a chain too
#ifndef FM_FLOW_FIRST
#define FM_FLOW_FIRST 1
#endif
//   FM_FLOW_TIE_MAIN       ... and the near-tie events' main sweep (stream2)
#ifndef FM_FLOW_TIE_MAIN
#define FM_FLOW_TIE_MAIN 0
#endif
//   FM_FLOW_SHARE_FIRST    percent of the resident slots a one-launch pass on stream2
//   FM_FLOW_SHARE          takes: the chain's first tracked sweep (beside the other part's
//                          certification), the later ones
#ifndef FM_FLOW_SHARE_FIRST
#define FM_FLOW_SHARE_FIRST 75
#endif
#ifndef FM_FLOW_SHARE
#define FM_FLOW_SHARE 75
#endif
#ifndef FM_FRESH_SWEEP
#define FM_FRESH_SWEEP 1
#endif
#ifndef FM_ROUND0_PER_TILE
#define FM_ROUND0_PER_TILE 1
#endif
#ifndef FM_OVERLAP_MIN_EVENTS
#define FM_OVERLAP_MIN_EVENTS 32
#endif
#ifndef FM_OVERLAP_TIES
#define FM_OVERLAP_TIES 1
#endif
#ifndef FM_CERTIFY
#define FM_CERTIFY 1
#endif
#ifndef FM_OVERLAP_MAIN
#define FM_OVERLAP_MAIN 1
#endif

#ifndef FM_SWEEP_GRAPHS
#define FM_SWEEP_GRAPHS 1
#endif

// How a solve starts: from boundary frames (initialisation, sweep, rounds),
// from the current fields (resume: rounds with every tile active), or from
// point-source boxes the caller already wrote (rounds from the boxes' tiles).
enum SolveMode { kFrames = 0, kResume = 1, kPoint = 2 };

// The rays of nlist listed events (d_events; null: all nev events) from the
// receivers, into the dense rows and end points of a forward call's plan.
void launch_ray_list(fm3dt_ctx *ctx, int nev, const fm3dt_ctx::EarlyRays &er, const int *d_events, int nlist,
                     cudaStream_t s)
{
    RayArgs ra{};
    ra.g = ctx->g;
    ra.prec = ctx->prec;
    ra.T = ctx->d_T;
    ra.veln = ctx->d_veln;
    ra.nev = nev;
    ra.nrc = er.nrc;
    ra.events = d_events;
    ra.nlist = nlist;
    ra.rcr = er.rcr;
    ra.rcx = er.rcx;
    ra.rcz = er.rcz;
    ra.fdm = er.fdm;
    ra.endpoints = er.endpoints;
    ra.nsteps = nullptr;
    ra.flags = er.flags;
    launch_rays(ra, s);
    ctx->launches += 1;
}

int solve_common(fm3dt_ctx *ctx, int nev, fm3dt_status *st, int mode = kFrames)
{
    const bool resume = mode == kResume;
    const bool point = mode == kPoint || (resume && ctx->last_point);
    cudaStream_t s = ctx->stream;
    const Geom &g = ctx->g;
    cudaEvent_t ev0, ev1, sw0, sw1;
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    CK(cudaEventCreate(&sw0));
    CK(cudaEventCreate(&sw1));
    CK(cudaEventRecord(ev0, s));
    CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), s));
    const bool do_sweep = ctx->sweep && mode == kFrames;

    if (mode == kFrames) {
        launch_fill_inf(ctx->d_T, (size_t)nev * ctx->N, ctx->prec, s);
        launch_finalize_frames(g, nev, ctx->prec, ctx->d_frames, ctx->d_T, ctx->d_frozen, ctx->d_base, s);
        launch_sweep_directions(g, nev, ctx->d_frames, ctx->d_dir, ctx->tie_ratio, s);
        ctx->launches += 3;
        CKL();
    }

    const int shape = ctx->shape;
    const TileShape ts = kShapes[shape];
    int ntr, ntx, ntz;
    const int tpe = tiles_per_event(g, shape, &ntr, &ntx, &ntz);

    FieldArgs<double> f64{};
    FieldArgs<float> f32{};
    auto fill_field = [&](auto &f, auto *T, auto *sl, auto *hx, auto *hz, auto *wx, auto *wz) {
        f.T = T; f.s = sl; f.hx = hx; f.hz = hz; f.wx = wx; f.wz = wz;
        f.frozen = ctx->d_frozen;
        f.box = point ? ctx->d_box : nullptr;
        f.nnr = g.nnr; f.nnx = g.nnx; f.nnz = g.nnz;
        f.ntr = ntr; f.ntx = ntx; f.ntz = ntz;
        f.tiles_per_event = tpe;
        f.order2 = ctx->desc.fom ? 1 : 0;
    };
    if (ctx->prec == FM3DT_FP64) {
        fill_field(f64, (double *)ctx->d_T, (const double *)ctx->d_s, (const double *)ctx->d_hx,
                   (const double *)ctx->d_hz, (const double *)ctx->d_wx, (const double *)ctx->d_wz);
        f64.hr = g.dnr;
        f64.wr = 1.0 / (g.dnr * g.dnr);
    } else {
        fill_field(f32, (float *)ctx->d_T, (const float *)ctx->d_s, (const float *)ctx->d_hx,
                   (const float *)ctx->d_hz, (const float *)ctx->d_wx, (const float *)ctx->d_wz);
        f32.hr = (float)g.dnr;
        f32.wr = (float)(1.0 / (g.dnr * g.dnr));
    }

    // 1. directional sweep, one launch per tile hyperplane
    int sweep_launches = 0;
    int64_t sweep_nodes = 0;      // nodes visited by all sweep passes
    int64_t interval_nodes = 0;   // ... by the passes inside the sweep interval
    bool verified = false;
    const bool streaming = ctx->sweep_shape >= kNumShapes;
    const int sidx = streaming ? ctx->sweep_shape - kNumShapes : 0;
    const int nbx = (g.nnx + kStreamShapes[sidx].sx - 1) / kStreamShapes[sidx].sx;
    const int nbz = (g.nnz + kStreamShapes[sidx].sz - 1) / kStreamShapes[sidx].sz;
    // resident one-warp CTAs of the streaming sweep (the main sweep's form and
    // the general form differ in registers)
    auto stream_grid = [&](bool fresh, bool flow = false) {
        return streaming ? std::max(1, ctx->prec == FM3DT_FP64 ? occupancy_stream_f64(sidx, fresh, flow)
                                                               : occupancy_stream_f32(sidx, fresh, flow)) * sm_count()
                         : 1;
    };
    // One streaming sweep of nitems events (events == null: all), lateral
    // directions flipped by `flip`; with `flag`, changed nodes queue their
    // tiles (and face neighbours) on list/count for the rounds.  `fresh`: the
    // events' main sweep, from their unset fields (upstream-only updates).
    // `recurs`: a pass that recurs from solve to solve (kept as a graph).
    // `act`: the item activity of a chain of sweeps (this sweep's, the
    // previous one's or null), see StreamArgs.
    auto stream_pass = [&](int nitems, const int *events, int flip, int nseg, int *flag, int *list,
                           int *count, cudaStream_t st, bool fresh, bool recurs,
                           unsigned *act_cur = nullptr, const unsigned *act_prev = nullptr,
                           unsigned long long *act_items = nullptr) -> int {
        sweep_nodes += (int64_t)nitems * (int64_t)ctx->N;
        const int sgrid = stream_grid(fresh);
        if (nseg <= 0) nseg = stream_segments(ctx, nitems, nbx, nbz, sgrid, kStreamShapes[sidx].sx + kStreamShapes[sidx].sz - 2);
        nseg = std::min(nseg, g.nnr);
        const fm3dt_ctx::Planes *PP = nullptr;
        int rc = ensure_block_planes(ctx, ctx->sweep_shape, nseg, &PP);
        if (rc) return rc;
        const auto &P = *PP;
        const int seg_len = (g.nnr + nseg - 1) / nseg;
        // (items of one layer or column would miss a 2-deep neighbour)
        const bool track = !fresh && act_cur && seg_len >= 2 && kStreamShapes[sidx].sx >= 2;
        // One launch for the whole pass (FM_SWEEP_FLOW): items start as their
        // upstream neighbours finish, with a done flag per item and a queue
        // counter of the pass's stream, both zeroed ahead of the launch.  For
        // the tracked sweeps after a chain's first, whose few active items
        // would leave most of each hyperplane's launch idle; passes that run
        // every item keep one launch per hyperplane, which shares the GPU with
        // the other stream's work (a one-launch pass holds every SM slot).
        const int si = st == ctx->stream2 ? 1 : 0;
        const bool flow = FM_SWEEP_FLOW && streaming &&
                          ((track && (act_prev != nullptr || FM_FLOW_FIRST)) || (fresh && si == 1 && FM_FLOW_TIE_MAIN));
        const int nblocks = P.off.empty() ? 0 : P.off.back() + P.cnt.back();
        const size_t done_n = (size_t)nitems * (size_t)((g.nnr + seg_len - 1) / seg_len) * (size_t)nbx * (size_t)nbz;
        if (flow && done_n * sizeof(unsigned) > ctx->done_bytes[si]) {
            CK(cudaStreamSynchronize(st));
            cudaFree(ctx->d_done[si]);
            ctx->d_done[si] = nullptr;
            ctx->done_bytes[si] = 0;
            CK(cudaMalloc(&ctx->d_done[si], done_n * sizeof(unsigned)));
            ctx->done_bytes[si] = done_n * sizeof(unsigned);
        }
        // (on stream2, beside the other part's work, a share of the resident
        // slots: a one-launch pass holds its slots to the end)
        const int fgrid = flow ? (int)std::min<long long>((long long)nblocks * nitems,
                                                          std::max(1, stream_grid(fresh, true) *
                                                                          (si ? (act_prev ? FM_FLOW_SHARE
                                                                                          : FM_FLOW_SHARE_FIRST)
                                                              : 100) / 100))
                               : 0;
        // the pass's launches: one (flow), else one per hyperplane (two with a
        // tracked previous sweep)
        const int nlaunch = flow ? 1 : (int)P.off.size() * (track && act_prev ? 2 : 1);
        // (returns the first error of the flags' and counter's zeroing; the
        // launches' errors surface at the next check)
        auto enqueue = [&]() -> cudaError_t {
            cudaError_t ez = cudaSuccess;
            if (flow) {
                ez = cudaMemsetAsync(ctx->d_done[si], 0, done_n * sizeof(unsigned), st);
                if (ez == cudaSuccess) ez = cudaMemsetAsync(ctx->d_next + si, 0, sizeof(unsigned), st);
                if (ez != cudaSuccess) return ez;
            }
            for (size_t h = 0; h < (flow ? (size_t)1 : P.off.size()); ++h) {
                const long long items = (long long)P.cnt[h] * nitems;
                const int grid = flow ? fgrid : (int)std::min<long long>(items, sgrid);
                auto fill = [&](auto &a) {
                    a.hp_blocks = P.d_tiles; a.hoff = flow ? 0 : P.off[h]; a.hcount = flow ? nblocks : P.cnt[h];
                    a.flow = flow ? 1 : 0;
                    a.done = flow ? ctx->d_done[si] : nullptr;
                    a.done_n = flow ? done_n : 0;
                    a.next = flow ? ctx->d_next + si : nullptr;
                    a.dir = ctx->d_dir; a.nev = nitems; a.nbx = nbx; a.nbz = nbz;
                    a.events = events;
                    a.flip = flip;
                    a.fresh = fresh ? 1 : 0;
                    a.seg_len = seg_len;
                    a.flag = flag;
                    a.list = list; a.count = count;
                    a.tr = ts.tr; a.tx = ts.tx; a.tz = ts.tz;
                    a.ntr = ntr; a.ntx = ntx; a.ntz = ntz; a.tiles_per_event = tpe;
                    a.act_cur = track ? act_cur : nullptr;
                    a.act_prev = track ? act_prev : nullptr;
                    a.act_run = track && !flow ? ctx->d_act[2] : nullptr;
                    // chunks of at least 4 layers, at most 32 of them per item
                    a.act_shift = 2;
                    while (((seg_len - 1) >> a.act_shift) >= 32) ++a.act_shift;
                    a.act_items = track ? act_items : nullptr;
                    a.act_n = ctx->act_bytes / sizeof(unsigned);
                    a.err = ctx->d_err;
                };
                if (ctx->prec == FM3DT_FP64) {
                    StreamArgs<double> a{};
                    a.f = f64;
                    fill(a);
                    launch_stream_f64(sidx, grid, a, st);
                } else {
                    StreamArgs<float> a{};
                    a.f = f32;
                    fill(a);
                    launch_stream_f32(sidx, grid, a, st);
                }
            }
            return cudaSuccess;
        };
        // Passes that recur from solve to solve (the main sweeps and the
        // near-tie events' extra sweeps; not the re-sweeps, whose event count
        // varies) run as a graph captured on first use: one launch instead of
        // one per hyperplane.
        bool launched = false;
        if (FM_SWEEP_GRAPHS && recurs && !ctx->sweep_graph_off) {
            const long long key[fm3dt_ctx::kSweepKey] = {ctx->prec, sidx, nitems, (long long)(intptr_t)events, flip,
                                                         nseg, fresh ? 1 : 0, (long long)(intptr_t)st, ctx->shape,
                                                         (long long)(intptr_t)flag, (long long)(intptr_t)list,
                                                         (long long)(intptr_t)count, (long long)(intptr_t)act_cur,
                                                         (long long)(intptr_t)act_prev, (long long)(intptr_t)act_items,
                                                         (long long)(intptr_t)(flow ? ctx->d_done[si] : nullptr)};
            cudaGraphExec_t exec = nullptr;
            for (const auto &sg : ctx->sweep_graphs)
                if (memcmp(sg.key, key, sizeof key) == 0) exec = sg.exec;
            if (!exec) {
                cudaGraph_t gr = nullptr;
                cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    const cudaError_t eq = enqueue();
                    e = cudaStreamEndCapture(st, &gr);
                    if (e == cudaSuccess) e = eq;
                }
                if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, gr, 0);
                if (gr) cudaGraphDestroy(gr);
                if (e != cudaSuccess) {
                    // launched one by one from now on in this context
                    (void)cudaGetLastError();
                    ctx->sweep_graph_off = true;
                    exec = nullptr;
                } else {
                    if (ctx->sweep_graphs.size() >= fm3dt_ctx::kSweepGraphs) {
                        cudaGraphExecDestroy(ctx->sweep_graphs.front().exec);
                        ctx->sweep_graphs.erase(ctx->sweep_graphs.begin());
                    }
                    fm3dt_ctx::SweepGraph sg;
                    memcpy(sg.key, key, sizeof key);
                    sg.exec = exec;
                    ctx->sweep_graphs.push_back(sg);
                }
            }
            if (exec) {
                CK(cudaGraphLaunch(exec, st));
                launched = true;
            }
        }
        if (!launched) CK(enqueue());
        sweep_launches += nlaunch;
        ctx->launches += nlaunch;
        return FM3DT_OK;
    };
    CK(cudaEventRecord(sw0, s));
    std::vector<int> ties, others;     // near-tie events and the rest
    bool overlap = false;              // ties' extra sweeps beside the others' first round
    bool tie_queue = false;            // ties' last extra sweep queues their first round's tiles
    bool tie_act = false;              // ties' extra sweeps skip items where nothing changed
    // the activity buffers of extra sweep k: this sweep's and the previous one's
    auto act_cur = [&](int k) { return tie_act ? ctx->d_act[k & 1] : nullptr; };
    auto act_prev = [&](int k) -> const unsigned * { return tie_act && k > 0 ? ctx->d_act[(k - 1) & 1] : nullptr; };
    auto act_items = [&](int k) { return tie_act && k < fm3dt_ctx::kMaxTieSweeps ? ctx->d_act_items + 2 * k : nullptr; };
    ctx->act_sweeps = 0;
    ctx->tie_sweep_n = 0;
    if (do_sweep && streaming) {
        // streaming sweep: one launch per column-block hyperplane
        // the events whose lateral direction is a near tie get two more
        // sweeps, reversed and then forward
        CK(cudaMemcpyAsync(ctx->h_dir, ctx->d_dir, nev * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int e = 0; e < nev; ++e)
            (ctx->h_dir[e] & 12 ? ties : others).push_back(e);
        // (only for large batches: with a few events the first round is short,
        // and contexts that solve side by side, as a service runs them, lose
        // more to the priority stream than they gain)
        overlap = FM_OVERLAP_TIES && !ctx->verify && !ties.empty() && (int)others.size() >= FM_OVERLAP_MIN_EVENTS &&
                  ctx->tie_sweeps > 0;
        // The near-tie events' last extra sweep runs in flag mode: a node it
        // leaves unchanged, with every neighbour that was updated after it
        // unchanged too, is a fixed point of the stencil, and every other node
        // lies in a tile the sweep queues (its own, or a face neighbour's
        // whose halo holds a changed node).  Their first round then takes the
        // queued tiles, not every tile.  (The other events' first round is
        // appended by their certification, so without it they need every
        // tile, which the list cannot hold beside a queue.)
        tie_queue = FM_TIE_QUEUE && !ctx->verify && !ties.empty() && ctx->tie_sweeps > 0 &&
                    (overlap || FM_CERTIFY || others.empty());
        if (tie_queue && !overlap) {
            CK(cudaMemsetAsync(ctx->d_flag, 0, (size_t)nev * tpe * sizeof(int), s));
            CK(cudaMemsetAsync(ctx->d_count[0], 0, sizeof(int), s));
        }
        // item activity of the near-tie events' extra sweeps: one mask per
        // (event, segment, column block), for at most 127 segments
        if (FM_TIE_SKIP && !ties.empty() && ctx->tie_sweeps > 1) {
            const size_t need = ties.size() * (size_t)std::min(127, g.nnr) * (size_t)nbx * (size_t)nbz *
                                sizeof(unsigned);
            if (need > ctx->act_bytes) {
                CK(cudaStreamSynchronize(ctx->stream2));
                for (auto &p : ctx->d_act) {
                    cudaFree(p);
                    p = nullptr;
                }
                ctx->act_bytes = 0;
                for (auto &p : ctx->d_act) CK(cudaMalloc(&p, need));
                ctx->act_bytes = need;
            }
            tie_act = true;
            ctx->act_sweeps = std::min(ctx->tie_sweeps, fm3dt_ctx::kMaxTieSweeps);
            CK(cudaMemsetAsync(ctx->d_act_items, 0, 2 * fm3dt_ctx::kMaxTieSweeps * sizeof(unsigned long long), s));
        }
        if (!ties.empty())
            CK(cudaMemcpyAsync(ctx->d_events, ties.data(), ties.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        // pass 0 sweeps every event from the boundary, pass 1 the near-tie
        // events reversed; pass 2 (verification, optional) sweeps once more
        // and queues the rounds' tiles where a node still changed
        if (ctx->verify) {
            CK(cudaMemsetAsync(ctx->d_flag, 0, (size_t)nev * tpe * sizeof(int), s));
            CK(cudaMemsetAsync(ctx->d_count[0], 0, sizeof(int), s));
        }
        // (ctx->tie_sweeps sweeps of the near-tie events, alternating reversed
        // and forward, stand for pass 1)
        struct PassPlan { int pass, flip; bool queue; int k; };
        std::vector<PassPlan> plan{{0, 0, false, 0}};
        for (int k = 0; k < ctx->tie_sweeps; ++k)
            plan.push_back({1, (k & 1) ? 0 : 4, tie_queue && k == ctx->tie_sweeps - 1, k});
        plan.push_back({2, 0, ctx->verify != 0, 0});
        for (const PassPlan &pl : plan) {
            const int pass = pl.pass;
            if ((pass == 0 && overlap && FM_OVERLAP_MAIN) || (pass == 1 && (ties.empty() || overlap)) ||
                (pass == 2 && !ctx->verify))
                continue;
            const int nitems = pass == 1 ? (int)ties.size() : nev;
            const int rc = stream_pass(nitems, pass == 1 ? ctx->d_events : nullptr, pl.flip,
                                       pass == 1 ? ctx->tie_segments : ctx->sweep_segments,
                                       pl.queue ? ctx->d_flag : nullptr, ctx->d_list[0], ctx->d_count[0], s,
                                       pass == 0 && FM_FRESH_SWEEP, pass != 2, pass == 1 ? act_cur(pl.k) : nullptr,
                                       pass == 1 ? act_prev(pl.k) : nullptr, pass == 1 ? act_items(pl.k) : nullptr);
            if (rc) return rc;
        }
        CKL();
        verified = ctx->verify != 0;
        interval_nodes = sweep_nodes;
    } else if (do_sweep) {
        sweep_nodes = (int64_t)nev * (int64_t)ctx->N;
        interval_nodes = sweep_nodes;
        const int sshape = ctx->sweep_shape;
        int rc = ensure_planes(ctx, sshape);
        if (rc) return rc;
        const auto &P = ctx->planes[sshape];
        const int sgrid = std::max(1, sweep_blocks_per_sm(sshape, ctx->prec)) * sm_count();
        // the sweep tiles the grid with its own shape
        FieldArgs<double> s64 = f64;
        FieldArgs<float> s32 = f32;
        {
            int a, b, c;
            const int t = tiles_per_event(g, sshape, &a, &b, &c);
            s64.ntr = s32.ntr = a;
            s64.ntx = s32.ntx = b;
            s64.ntz = s32.ntz = c;
            s64.tiles_per_event = s32.tiles_per_event = t;
        }
        for (size_t h = 0; h < P.off.size(); ++h) {
            const long long items = (long long)P.cnt[h] * nev;
            const int grid = (int)std::min<long long>(items, sgrid);
            if (ctx->prec == FM3DT_FP64) {
                SweepArgs<double> a{s64, P.d_tiles, P.off[h], P.cnt[h], ctx->d_dir, nev};
                launch_sweep_f64(sshape, grid, a, s);
            } else {
                SweepArgs<float> a{s32, P.d_tiles, P.off[h], P.cnt[h], ctx->d_dir, nev};
                launch_sweep_f32(sshape, grid, a, s);
            }
            ++sweep_launches;
        }
        ctx->launches += sweep_launches;
        CKL();
    }
    // (with the main sweeps in the first round's two parts, the sweep time ends
    // with the other events' main sweep there)
    if (!(overlap && FM_OVERLAP_MAIN)) CK(cudaEventRecord(sw1, s));

    // 2. rounds until no tile changes: all tiles after a sweep, else the
    //    tiles whose nodes or 2-deep halos include the bottom layer
    //    (or, after a verification sweep, the tiles it queued)
    const int tlo = (do_sweep || resume) ? 0 : std::max(0, (g.nnr - 3) / ts.tr);
    const int first = tlo * ntx * ntz;
    const int cnt = (ntr - tlo) * ntx * ntz;
    CK(cudaMemsetAsync(ctx->d_count[1], 0, sizeof(int), s));
    CK(cudaMemsetAsync(ctx->d_stats, 0, 3 * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(ctx->d_trace, 0, 2 * sizeof(unsigned long long) * fm3dt_ctx::kTraceRounds, s));
    // Certification of the events swept exactly once (all but the near-tie
    // events, which had extra sweeps): their first round recomputes only the
    // nodes it marks, on the tiles it appends to list 0
    auto certify = [&](const int *events, int n, cudaStream_t st) {
        auto fill = [&](auto &ca, const auto &f) {
            ca.f = f;
            ca.events = events; ca.nev = n;
            ca.dir = ctx->d_dir;
            ca.cert = ctx->d_cert; ca.cert_nw = ctx->cert_nw;
            ca.tr = ts.tr; ca.tx = ts.tx; ca.tz = ts.tz;
            ca.flag = ctx->d_flag; ca.list = ctx->d_list[0]; ca.count = ctx->d_count[0];
        };
        if (ctx->prec == FM3DT_FP64) {
            CertifyArgs<double> ca{};
            fill(ca, f64);
            launch_certify_f64(ca, st);
        } else {
            CertifyArgs<float> ca{};
            fill(ca, f32);
            launch_certify_f32(ca, st);
        }
        ctx->launches += 1;
    };
    const bool certify_alone = FM_CERTIFY && do_sweep && streaming && !verified && !overlap && !others.empty();
    if (!verified) {
        // (with the near-tie events' tiles queued by their last sweep, the
        // flags and list 0 were cleared before it)
        if (!(tie_queue && !overlap)) CK(cudaMemsetAsync(ctx->d_flag, 0, (size_t)nev * tpe * sizeof(int), s));
        if (overlap) {
            // the first round is launched below, in two parts
        } else if (tie_queue && !certify_alone) {
            // every event a near tie: list 0 holds the tiles their last sweep queued
        } else if (certify_alone) {
            // the near-tie events' tiles first (this sets the count), then the
            // other events' marked tiles appended
            if (tie_queue) {
                // (queued by the near-tie events' last sweep)
            } else if (!ties.empty())
                launch_initial_tiles((int)ties.size(), ctx->d_events, tpe, first, cnt, ctx->d_list[0],
                                     ctx->d_count[0], ctx->d_flag, s);
            else
                CK(cudaMemsetAsync(ctx->d_count[0], 0, sizeof(int), s));
            CK(cudaMemcpyAsync(ctx->d_events_b, others.data(), others.size() * sizeof(int), cudaMemcpyHostToDevice,
                               s));
            certify(ctx->d_events_b, (int)others.size(), s);
        } else if (mode == kPoint)
            launch_initial_tiles_box(nev, tpe, ntx, ntz, ts.tr, ts.tx, ts.tz, ctx->d_box_init, ctx->d_list[0],
                                     ctx->d_count[0], ctx->d_flag, s);
        else
            launch_initial_tiles(nev, nullptr, tpe, first, cnt, ctx->d_list[0], ctx->d_count[0], ctx->d_flag, s);
        ctx->launches += 1;
        CKL();
    }

    const int bps = std::max(1, round_blocks_per_sm(shape, ctx->prec));
    const int grid = bps * sm_count();
    const int max_rounds = ctx->max_rounds > 0 ? ctx->max_rounds : 64 * (ntr + ntx + ntz) + 256;
    const int chunk = 8;
    RoundArgs<double> a64{};
    RoundArgs<float> a32{};
    a64.f = f64;
    a32.f = f32;
    a64.flag = a32.flag = ctx->d_flag;
    a64.max_passes = a32.max_passes = ctx->max_passes;
    a64.stats = a32.stats = ctx->d_stats;
    a64.err = a32.err = ctx->d_err;
    a64.cert = a32.cert = ctx->d_cert;
    a64.cert_nw = a32.cert_nw = ctx->cert_nw;
    {
        const CUtensorMap *map = field_tensor_map(ctx, shape);
        a64.tma = a32.tma = map ? 1 : 0;
        if (map) {
            a64.tmap = a32.tmap = *map;
            a64.smap = a32.smap = ctx->smap[shape];
        }
    }

    int rounds = 0;
    bool done = false;
    double round_ms = 0.0, resweep_ms = 0.0;
    ctx->round_ms_trace.clear();
    for (float &m : ctx->part_ms) m = 0.0f;
    // after the first round of a swept solve, the events that still change
    // on many tiles are swept again (ctx->resweeps times at most): corrections
    // that the first round made deep in the grid then reach the top in one
    // pass instead of one tile layer per round; the sweep queues the tiles
    // it changes for the next round
    int resweeps_left = (do_sweep && streaming && !verified) ? ctx->resweeps : 0;
    int grid_override = 0;   // launch grid other than the persistent one (0: persistent)
    auto launch_round = [&](int round, int *cur_list, int *cur_count, int *next_list, int *next_count,
                            cudaStream_t st) {
        const int gr = grid_override > 0 ? grid_override : grid;
        if (ctx->prec == FM3DT_FP64) {
            a64.trace = round < fm3dt_ctx::kTraceRounds ? ctx->d_trace : nullptr;
            a64.round = round;
            a64.cur_list = cur_list; a64.cur_count = cur_count;
            a64.next_list = next_list; a64.next_count = next_count;
            launch_round_f64(shape, gr, a64, st);
        } else {
            a32.trace = round < fm3dt_ctx::kTraceRounds ? ctx->d_trace : nullptr;
            a32.round = round;
            a32.cur_list = cur_list; a32.cur_count = cur_count;
            a32.next_list = next_list; a32.next_count = next_count;
            launch_round_f32(shape, gr, a32, st);
        }
        ctx->launches += 1;
    };
    // events that still change on many tiles after a round are swept again
    // (see resweeps_left; `left` counts down), on stream st: `list`/`count`
    // is the list the next round takes, `queued` its length, `ev_buf` a
    // device array for the swept events' indices that no other stream reads
    // meanwhile; the list's new length goes to the pinned *h_cnt
    auto maybe_resweep = [&](cudaStream_t st, int *h_cnt, int *list, int *count, int queued, int *ev_buf,
                             int &left) -> int {
        if (left <= 0) return FM3DT_OK;
        --left;
        if (!((double)queued > ctx->resweep_frac * (double)nev * (double)tpe)) return FM3DT_OK;
        std::vector<int> lst(queued);
        CK(cudaMemcpyAsync(lst.data(), list, (size_t)queued * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<int> per(nev, 0);
        for (int w : lst) per[w / tpe] += 1;
        std::vector<int> busy;
        for (int e = 0; e < nev; ++e)
            if ((double)per[e] > ctx->resweep_frac * (double)tpe) busy.push_back(e);
        if (busy.empty()) return FM3DT_OK;
        cudaEvent_t r0, r1;
        CK(cudaEventCreate(&r0));
        CK(cudaEventCreate(&r1));
        CK(cudaMemcpyAsync(ev_buf, busy.data(), busy.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaEventRecord(r0, st));
        const int rc = stream_pass((int)busy.size(), ev_buf, 0, 0, ctx->d_flag, list, count, st, false, false);
        if (rc) return rc;
        interval_nodes += (int64_t)busy.size() * (int64_t)ctx->N;
        CK(cudaEventRecord(r1, st));
        CKL();
        CK(cudaMemcpyAsync(h_cnt, count, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        float m = 0.0f;
        cudaEventElapsedTime(&m, r0, r1);
        resweep_ms += m;
        cudaEventDestroy(r0);
        cudaEventDestroy(r1);
        return FM3DT_OK;
    };
    // A part's rounds, a chunk at a time, so that two parts (on two streams)
    // can alternate: L.list[L.cur] is the list its next round takes; ev_buf
    // and left for its re-sweeps; h_cnt the pinned copy of its list's length;
    // ev its round events (2 per round of a chunk); ready recorded after the
    // chunk's length is read back.
    struct RoundLists { int *list[2]; int *count[2]; int cur; };
    struct Part {
        cudaStream_t st;
        RoundLists L;
        int *ev_buf;
        int left;
        int *h_cnt;
        std::vector<cudaEvent_t> *ev;
        cudaEvent_t ready;
        bool pending, done;
        int first, n;
    };
    auto part_launch = [&](Part &p) -> int {
        const int chunk_now = p.left > 0 ? 1 : chunk;
        while ((int)p.ev->size() < 2 * chunk) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            p.ev->push_back(e);
        }
        p.first = rounds;
        for (int k = 0; k < chunk_now && rounds < max_rounds; ++k, ++rounds) {
            const int cur = p.L.cur, nxt = cur ^ 1;
            CK(cudaMemsetAsync(p.L.count[nxt], 0, sizeof(int), p.st));
            CK(cudaEventRecord((*p.ev)[2 * k], p.st));
            // the first round's tile count is known on the host: one CTA per
            // tile, so blocks free up as they finish
            if (rounds == 0 && FM_ROUND0_PER_TILE && !verified && mode != kPoint && !certify_alone && !tie_queue)
                grid_override = (int)std::min<long long>((long long)nev * cnt, 1LL << 30);
            launch_round(rounds, p.L.list[cur], p.L.count[cur], p.L.list[nxt], p.L.count[nxt], p.st);
            grid_override = 0;
            CK(cudaEventRecord((*p.ev)[2 * k + 1], p.st));
            p.L.cur = nxt;
        }
        p.n = rounds - p.first;
        CKL();
        CK(cudaMemcpyAsync(p.h_cnt, p.L.count[p.L.cur], sizeof(int), cudaMemcpyDeviceToHost, p.st));
        CK(cudaEventRecord(p.ready, p.st));
        p.pending = true;
        return FM3DT_OK;
    };
    // (after the part's ready event) the chunk's times, re-sweeps, and the end
    auto part_finish = [&](Part &p) -> int {
        for (int q = 0; q < p.n; ++q) {
            float m = 0.0f;
            cudaEventElapsedTime(&m, (*p.ev)[2 * q], (*p.ev)[2 * q + 1]);
            round_ms += m;
            if ((int)ctx->round_ms_trace.size() < fm3dt_ctx::kTraceRounds) ctx->round_ms_trace.push_back(m);
        }
        p.pending = false;
        const int rc = maybe_resweep(p.st, p.h_cnt, p.L.list[p.L.cur], p.L.count[p.L.cur], *p.h_cnt, p.ev_buf, p.left);
        if (rc) return rc;
        if (*p.h_cnt == 0) p.done = true;
        return FM3DT_OK;
    };
    // A forward call's early rays: once the other events (part 0 of a
    // two-part solve) have converged, their rays start on the context stream,
    // which that part no longer uses, beside the near-tie events' rounds.
    auto early_rays = [&]() -> int {
        auto &er = ctx->early;
        if (!er.on || !er.events.empty() || others.empty()) return FM3DT_OK;
        er.events = others;
        CK(cudaMemcpyAsync(er.d_events, others.data(), others.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        if (er.fdm) CK(cudaMemsetAsync(er.fdm, 0, er.fdm_bytes, s));
        launch_ray_list(ctx, nev, er, er.d_events, (int)others.size(), s);
        CKL();
        return FM3DT_OK;
    };
    // Rounds of one or two parts until their lists come back empty or the
    // round cap; two parts alternate, each chunk launched as soon as its
    // part's previous one has been read back.
    auto converge = [&](Part *parts, int np) -> int {
        for (;;) {
            bool open = false, progressed = false;
            for (int i = 0; i < np; ++i) {
                Part &p = parts[i];
                if (p.done && i == 0 && np > 1) {
                    const int rc = early_rays();
                    if (rc) return rc;
                }
                if (p.done) continue;
                if (p.pending) {
                    const cudaError_t q = np > 1 ? cudaEventQuery(p.ready) : cudaEventSynchronize(p.ready);
                    if (q == cudaErrorNotReady) {
                        open = true;
                        continue;
                    }
                    CK(q);
                    const int rc = part_finish(p);
                    if (rc) return rc;
                    progressed = true;
                }
                if (!p.done && rounds < max_rounds) {
                    const int rc = part_launch(p);
                    if (rc) return rc;
                    progressed = true;
                }
                if (p.pending) open = true;
            }
            if (!open) break;
            if (!progressed) std::this_thread::yield();
        }
        return FM3DT_OK;
    };
    cudaEvent_t ready_ev[2];
    CK(cudaEventCreateWithFlags(&ready_ev[0], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ready_ev[1], cudaEventDisableTiming));
    struct ReadyGuard {
        cudaEvent_t *e;
        ~ReadyGuard() { cudaEventDestroy(e[0]); cudaEventDestroy(e[1]); }
    } ready_guard{ready_ev};
    if (overlap) {
        // The solve in two parts that run side by side and converge apart
        // (events do not interact).  On stream2, whose higher priority gets
        // its blocks scheduled first: the near-tie events' main sweep, their
        // extra sweeps and their first round (on the tiles the last sweep
        // queued, or every tile), queueing onto list c.  On the context
        // stream: the other events' main sweep, their certification, their
        // first round on the tiles it marks (or, without the certification,
        // every tile, one CTA per tile so that blocks free up as they finish)
        // and their further rounds until they converge, while stream2 still
        // runs the near-tie events' chain; then the near-tie events' rounds.
        cudaEvent_t fork, join, r0, r1;
        CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
        CK(cudaEventCreate(&r0));
        CK(cudaEventCreate(&r1));
        // the parts' phases: near-tie extra sweeps and first round (stream2),
        // the others' certification and first round (context stream)
        cudaEvent_t pe[6];
        for (auto &e : pe) CK(cudaEventCreate(&e));
        CK(cudaMemcpyAsync(ctx->d_events, ties.data(), ties.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->d_events_b, others.data(), others.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        if (!FM_OVERLAP_MAIN) CK(cudaEventRecord(r0, s));
        CK(cudaEventRecord(fork, s));
        cudaStream_t s2 = ctx->stream2;
        CK(cudaStreamWaitEvent(s2, fork, 0));
        if (FM_OVERLAP_MAIN) {
            // each part's main sweep: the near-tie events' on stream2 ahead of
            // their extra sweeps, the others' on the context stream -- after
            // the near-tie events' (FM_TIES_FIRST), which then has the GPU to
            // itself and starts the longer chain sooner, the others' main
            // sweep filling the gaps of its extra sweeps
            int rc = stream_pass((int)ties.size(), ctx->d_events, 0, ctx->tie_segments, nullptr, ctx->d_list[0],
                                 ctx->d_count[0], s2, FM_FRESH_SWEEP, true);
            if (rc) return rc;
            if (FM_TIES_FIRST) {
                CK(cudaEventRecord(pe[0], s2));
                CK(cudaStreamWaitEvent(s, pe[0], 0));
            }
            rc = stream_pass((int)others.size(), ctx->d_events_b, 0, ctx->sweep_segments, nullptr, ctx->d_list[0],
                             ctx->d_count[0], s, FM_FRESH_SWEEP, true);
            if (rc) return rc;
            interval_nodes += (int64_t)nev * (int64_t)ctx->N;
            CK(cudaEventRecord(sw1, s));
            CK(cudaEventRecord(r0, s));
        }
        if (tie_queue) CK(cudaMemsetAsync(ctx->d_count_b, 0, sizeof(int), s2));
        CK(cudaEventRecord(pe[0], s2));
        // the extra sweeps' own times (events between them on stream2)
        const int nts = std::min(ctx->tie_sweeps, fm3dt_ctx::kMaxTieSweeps);
        std::vector<cudaEvent_t> tse(nts + 1);
        for (auto &e : tse) CK(cudaEventCreate(&e));
        for (int k = 0; k < ctx->tie_sweeps; ++k) {
            if (k <= nts) CK(cudaEventRecord(tse[k], s2));
            // (height segments by the time model for the near-tie events alone:
            // their sweeps are the longer chain of the two parts); the last one
            // queues their first round's tiles on list b
            const bool q = tie_queue && k == ctx->tie_sweeps - 1;
            const int rc = stream_pass((int)ties.size(), ctx->d_events, (k & 1) ? 0 : 4,
                                       FM_OVERLAP_MAIN ? ctx->tie_segments : (ctx->tie_segments > 0 ? ctx->tie_segments : 2),
                                       q ? ctx->d_flag : nullptr, ctx->d_list_b, ctx->d_count_b, s2, false, true,
                                       act_cur(k), act_prev(k), act_items(k));
            if (rc) return rc;
        }
        if (ctx->tie_sweeps <= nts) CK(cudaEventRecord(tse[nts], s2));
        if (!tie_queue)
            launch_initial_tiles((int)ties.size(), ctx->d_events, tpe, first, cnt, ctx->d_list_b, ctx->d_count_b,
                                 ctx->d_flag, s2);
        CK(cudaEventRecord(pe[1], s2));
        CK(cudaMemsetAsync(ctx->d_count_c, 0, sizeof(int), s2));
        launch_round(0, ctx->d_list_b, ctx->d_count_b, ctx->d_list_c, ctx->d_count_c, s2);
        CK(cudaEventRecord(pe[2], s2));
        CK(cudaEventRecord(join, s2));
        CK(cudaEventRecord(pe[3], s));
        if (FM_CERTIFY) {
            // the other events were swept once: only the tiles holding a node
            // the certification cannot clear, from those nodes
            CK(cudaMemsetAsync(ctx->d_count[0], 0, sizeof(int), s));
            certify(ctx->d_events_b, (int)others.size(), s);
            CK(cudaEventRecord(pe[4], s));
            launch_round(0, ctx->d_list[0], ctx->d_count[0], ctx->d_list[1], ctx->d_count[1], s);
        } else {
            launch_initial_tiles((int)others.size(), ctx->d_events_b, tpe, first, cnt, ctx->d_list[0],
                                 ctx->d_count[0], ctx->d_flag, s);
            grid_override = (int)std::min<long long>((long long)others.size() * cnt, 1LL << 30);
            CK(cudaEventRecord(pe[4], s));
            launch_round(0, ctx->d_list[0], ctx->d_count[0], ctx->d_list[1], ctx->d_count[1], s);
            grid_override = 0;
        }
        CK(cudaEventRecord(pe[5], s));
        CK(cudaEventRecord(r1, s));
        ctx->launches += 2;
        CKL();
        CK(cudaMemcpyAsync(ctx->h_count, ctx->d_count[1], sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float m = 0.0f;
        cudaEventElapsedTime(&m, r0, r1);
        round_ms += m;
        ctx->round_ms_trace.push_back(m);
        rounds = 1;
        // The two parts' further rounds, alternating: the other events' on
        // the context stream (re-sweeps take their indices in events b, which
        // stream2 does not read), the near-tie events' on stream2 after their
        // chain (lists c and b; their first chunk is queued behind the chain
        // at once).
        Part parts[2] = {
            {s, {{ctx->d_list[1], ctx->d_list[0]}, {ctx->d_count[1], ctx->d_count[0]}, 0}, ctx->d_events_b,
             resweeps_left, ctx->h_count, &ctx->round_events, ready_ev[0], false, false, 0, 0},
            {s2, {{ctx->d_list_c, ctx->d_list_b}, {ctx->d_count_c, ctx->d_count_b}, 0}, ctx->d_events,
             resweeps_left, ctx->h_count + 1, &ctx->round_events_b, ready_ev[1], false, false, 0, 0}};
        int rc = maybe_resweep(s, ctx->h_count, parts[0].L.list[0], parts[0].L.count[0], *ctx->h_count,
                               ctx->d_events_b, parts[0].left);
        if (rc) return rc;
        if (*ctx->h_count == 0) parts[0].done = true;
        rc = converge(parts, 2);
        if (rc) return rc;
        // (the context stream waits for stream2's last chunk)
        CK(cudaEventRecord(join, s2));
        CK(cudaStreamWaitEvent(s, join, 0));
        CK(cudaStreamSynchronize(s));
        cudaEventElapsedTime(&ctx->part_ms[0], pe[0], pe[1]);
        cudaEventElapsedTime(&ctx->part_ms[1], pe[1], pe[2]);
        cudaEventElapsedTime(&ctx->part_ms[2], pe[3], pe[4]);
        cudaEventElapsedTime(&ctx->part_ms[3], pe[4], pe[5]);
        for (int k = 0; k < nts; ++k) cudaEventElapsedTime(&ctx->tie_sweep_ms[k], tse[k], tse[k + 1]);
        ctx->tie_sweep_n = nts;
        for (auto &e : tse) cudaEventDestroy(e);
        for (auto &e : pe) cudaEventDestroy(e);
        cudaEventDestroy(fork);
        cudaEventDestroy(join);
        cudaEventDestroy(r0);
        cudaEventDestroy(r1);
        done = parts[0].done && parts[1].done;
    } else {
        Part part{s, {{ctx->d_list[0], ctx->d_list[1]}, {ctx->d_count[0], ctx->d_count[1]}, 0}, ctx->d_events,
                  resweeps_left, ctx->h_count, &ctx->round_events, ready_ev[0], false, false, 0, 0};
        const int rc = converge(&part, 1);
        if (rc) return rc;
        done = part.done;
    }
    CK(cudaEventRecord(ev1, s));
    CK(cudaMemcpyAsync(ctx->h_stats, ctx->d_stats, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    if (ctx->act_sweeps > 0)
        CK(cudaMemcpyAsync(ctx->h_act_items, ctx->d_act_items, 2 * ctx->act_sweeps * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, s));
    int kerr = 0;
    CK(cudaMemcpyAsync(&kerr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    ctx->h_base.resize(nev);
    CK(cudaMemcpyAsync(ctx->h_base.data(), ctx->d_base, nev * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0.0f, sms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventElapsedTime(&sms, sw0, sw1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaEventDestroy(sw0);
    cudaEventDestroy(sw1);
    ctx->nev_solved = nev;
    ctx->last_rounds = rounds;
    ctx->last_point = point ? 1 : 0;
    if (st) {
        st->rounds = rounds;
        st->converged = done ? 1 : 0;
        st->tile_updates = (int64_t)ctx->h_stats[0];
        st->node_passes = (int64_t)ctx->h_stats[1];
        st->tile_nodes = (int64_t)ctx->h_stats[2];
        st->ms = ms;
        st->round_ms = round_ms;
        st->round_launches = rounds;
        st->sweep_ms = do_sweep ? sms + resweep_ms : 0.0;
        st->sweep_launches = sweep_launches;
        st->sweep_nodes = sweep_nodes;
        st->interval_nodes = interval_nodes;
    }
    if (kerr == 2) return fail(ctx, FM3DT_ECUDA, "a tile copy (TMA) destination was not 128-byte aligned");
    if (kerr & 4) return fail(ctx, FM3DT_ECUDA, "a tracked sweep met an activity slot out of range");
    if (kerr & 16)
        return fail(ctx, FM3DT_ECUDA, "a one-launch sweep pass gave up waiting for an item's upstream neighbours");
    if (kerr) return fail(ctx, FM3DT_ECUDA, "a tile copy (TMA) did not complete in time");
    if (!done) return fail(ctx, FM3DT_ENOCONV, "solver round limit reached before convergence");
    return FM3DT_OK;
}

// Replaces a context's grid geometry (same node counts): the refined source
// grids move with each source.
int set_geometry(fm3dt_ctx *ctx, const Geom &g)
{
    ctx->g = g;
    ctx->hr = g.dnr;
    ctx->have_velocity = 0;
    return ctx->prec == FM3DT_FP64 ? upload_geometry<double>(ctx) : upload_geometry<float>(ctx);
}

// A refined source grid solves with its parent's tuning, without the sweep.
void inherit_tuning(fm3dt_ctx *fc, const fm3dt_ctx *parent)
{
    fc->shape = parent->shape;
    fc->max_passes = parent->max_passes;
    fc->sweep = 0;
}

int check_ready(fm3dt_ctx *ctx, int nev)
{
    if (!ctx) return FM3DT_EINVAL;
    if (!ctx->have_velocity) return fail(ctx, FM3DT_ESTATE, "fm3dt_set_velocity must come first");
    if (nev < 1 || nev > ctx->maxev) return fail(ctx, FM3DT_EINVAL, "nev outside 1..max_events");
    return FM3DT_OK;
}

}  // namespace

extern "C" {

int fm3dt_ctx_create(const fm3dt_grid_desc *desc, fm3dt_ctx **out)
{
    fm3dt_ctx *ctx = nullptr;
    if (!desc || !out) return fail(nullptr, FM3DT_EINVAL, "null argument");
    *out = nullptr;
    const fm3dt_grid_desc &d = *desc;
    if (d.nnr < 3 || d.nnx < 3 || d.nnz < 3 || d.nvr < 1 || d.nvx < 1 || d.nvz < 1)
        return fail(nullptr, FM3DT_EINVAL, "grid dimensions too small (need nn >= 3, nv >= 1)");
    if (d.dnr <= 0 || d.dnxd <= 0 || d.dnzd <= 0 || d.dvr <= 0 || d.dvxd <= 0 || d.dvzd <= 0 || d.earth <= 0)
        return fail(nullptr, FM3DT_EINVAL, "grid spacings and earth radius must be positive");
    if (d.fom != 0 && d.fom != 1) return fail(nullptr, FM3DT_EINVAL, "fom must be 0 or 1");
    if (d.precision != FM3DT_FP64 && d.precision != FM3DT_FP32_OFFSET)
        return fail(nullptr, FM3DT_EINVAL, "unknown precision");
    if (d.max_events < 1) return fail(nullptr, FM3DT_EINVAL, "max_events must be >= 1");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail(nullptr, FM3DT_ENODEV, "no CUDA device");
    }
    ctx = new fm3dt_ctx();
    ctx->desc = d;
    ctx->g = convert(d);
    ctx->prec = d.precision;
    ctx->maxev = d.max_events;
    ctx->N = (size_t)d.nnr * d.nnx * d.nnz;
    ctx->NB = (size_t)d.nnx * d.nnz;
    ctx->hr = ctx->g.dnr;
    const size_t rs = rsize(ctx->prec);
    size_t maxtiles = 0;
    for (int sh = 0; sh < kNumShapes; ++sh) {
        int a, b, c;
        maxtiles = std::max(maxtiles, (size_t)tiles_per_event(ctx->g, sh, &a, &b, &c));
    }
    ctx->flag_capacity = maxtiles * (size_t)ctx->maxev;
    if (ctx->flag_capacity > (size_t)INT32_MAX) {
        delete ctx;
        return fail(nullptr, FM3DT_EINVAL, "too many tiles for 32-bit work items");
    }
    auto cleanup_fail = [&](int code, const std::string &m) {
        g_create_err = m;
        fm3dt_ctx_destroy(ctx);
        return code;
    };
#define CKC(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return cleanup_fail(e_ == cudaErrorMemoryAllocation ? FM3DT_ENOMEM : FM3DT_ECUDA,         \
                                std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)
    CKC(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    {
        // the scratch pool of the context's calls (the dense Frechet rows of
        // a ray call are the largest): its memory is kept between calls
        // rather than returned to the system at every synchronisation
        int dev = 0;
        CKC(cudaGetDevice(&dev));
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = dev;
        CKC(cudaMemPoolCreate(&ctx->pool, &pp));
        uint64_t keep = UINT64_MAX;
        CKC(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    const size_t nvel = (size_t)(d.nvr + 2) * (d.nvx + 2) * (d.nvz + 2);
    const size_t npad = (size_t)(d.nnr + 3) * (d.nnx + 3) * (d.nnz + 3);
    CKC(cudaMalloc(&ctx->d_velv, nvel * sizeof(double)));
    CKC(cudaMalloc(&ctx->d_veln, npad * sizeof(double)));
    CKC(cudaMalloc(&ctx->d_s, ctx->N * rs));
    CKC(cudaMalloc(&ctx->d_hx, (size_t)d.nnr * rs));
    CKC(cudaMalloc(&ctx->d_hz, (size_t)d.nnr * d.nnx * rs));
    CKC(cudaMalloc(&ctx->d_wx, (size_t)d.nnr * rs));
    CKC(cudaMalloc(&ctx->d_wz, (size_t)d.nnr * d.nnx * rs));
    CKC(cudaMalloc(&ctx->d_dir, ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_T, ctx->N * ctx->maxev * rs));
    CKC(cudaMalloc(&ctx->d_frames, ctx->NB * ctx->maxev * sizeof(double)));
    CKC(cudaMalloc(&ctx->d_base, ctx->maxev * sizeof(double)));
    CKC(cudaMalloc(&ctx->d_frozen, ctx->NB * ctx->maxev));
    CKC(cudaMalloc(&ctx->d_flag, ctx->flag_capacity * sizeof(int)));
    ctx->cert_nw = (d.nnr + 31) / 32;
    CKC(cudaMalloc(&ctx->d_cert, (size_t)ctx->maxev * d.nnx * d.nnz * ctx->cert_nw * sizeof(unsigned)));
    CKC(cudaMalloc(&ctx->d_list[0], ctx->flag_capacity * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_list[1], ctx->flag_capacity * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_count[0], sizeof(int)));
    CKC(cudaMalloc(&ctx->d_count[1], sizeof(int)));
    CKC(cudaMalloc(&ctx->d_stats, 3 * sizeof(unsigned long long)));
    CKC(cudaMalloc(&ctx->d_trace, 2 * sizeof(unsigned long long) * fm3dt_ctx::kTraceRounds));
    CKC(cudaMalloc(&ctx->d_params, 4 * ctx->maxev * sizeof(double)));
    CKC(cudaMalloc(&ctx->d_box, 6 * ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_box_init, 6 * ctx->maxev * sizeof(int)));
    CKC(cudaMallocHost(&ctx->h_count, 2 * sizeof(int)));
    CKC(cudaMallocHost(&ctx->h_dir, ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_events, ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_events_b, ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_list_b, ctx->flag_capacity * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_count_b, sizeof(int)));
    CKC(cudaMalloc(&ctx->d_list_c, ctx->flag_capacity * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_act_items, 2 * fm3dt_ctx::kMaxTieSweeps * sizeof(unsigned long long)));
    CKC(cudaMalloc(&ctx->d_next, 2 * sizeof(unsigned)));
    CKC(cudaMalloc(&ctx->d_ray_events, 2 * (size_t)ctx->maxev * sizeof(int)));
    CKC(cudaMalloc(&ctx->d_count_c, sizeof(int)));
    CKC(cudaMalloc(&ctx->d_err, sizeof(int)));
    {
        const char *env = std::getenv("FM3DT_TMA");
        if (env && env[0] == '0') ctx->use_tma = 0;
    }
    {
        int least = 0, greatest = 0;
        CKC(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CKC(cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, greatest));
    }
    CKC(cudaMallocHost(&ctx->h_stats, 3 * sizeof(unsigned long long)));
    CKC(cudaMemset(ctx->d_base, 0, ctx->maxev * sizeof(double)));
    int rc = ctx->prec == FM3DT_FP64 ? upload_geometry<double>(ctx) : upload_geometry<float>(ctx);
    if (rc != FM3DT_OK) return cleanup_fail(rc, ctx->err);
#undef CKC
    *out = ctx;
    return FM3DT_OK;
}

int fm3dt_set_velocity(fm3dt_ctx *ctx, const double *velv)
{
    if (!ctx || !velv) return FM3DT_EINVAL;
    const Geom &g = ctx->g;
    const size_t nvel = (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2);
    for (size_t q = 0; q < nvel; ++q)
        if (!(velv[q] > 0.0) || !std::isfinite(velv[q]))
            return fail(ctx, FM3DT_EINVAL, "velocity values must be positive and finite");
    CK(cudaMemcpyAsync(ctx->d_velv, velv, nvel * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    launch_gridder(g, ctx->d_velv, ctx->d_veln, ctx->stream);
    launch_slowness(g, ctx->d_veln, ctx->d_s, ctx->prec, ctx->stream);
    ctx->launches += 2;
    CKL();
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->have_velocity = 1;
    return FM3DT_OK;
}

int fm3dt_solve(fm3dt_ctx *ctx, int nev, const double *boundary, fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!boundary) return fail(ctx, FM3DT_EINVAL, "null boundary");
    CK(cudaMemcpyAsync(ctx->d_frames, boundary, (size_t)nev * ctx->NB * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    return solve_common(ctx, nev, st);
}

int fm3dt_solve_device(fm3dt_ctx *ctx, int nev, const double *d_boundary, fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!d_boundary) return fail(ctx, FM3DT_EINVAL, "null boundary");
    CK(cudaMemcpyAsync(ctx->d_frames, d_boundary, (size_t)nev * ctx->NB * sizeof(double), cudaMemcpyDeviceToDevice,
                       ctx->stream));
    return solve_common(ctx, nev, st);
}

int fm3dt_solve_resume(fm3dt_ctx *ctx, fm3dt_status *st)
{
    if (!ctx) return FM3DT_EINVAL;
    if (ctx->nev_solved < 1) return fail(ctx, FM3DT_ESTATE, "no solved events to resume");
    return solve_common(ctx, ctx->nev_solved, st, kResume);
}

int fm3dt_solve_planewave(fm3dt_ctx *ctx, int nev, const double *params, fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!params) return fail(ctx, FM3DT_EINVAL, "null params");
    const Geom &g = ctx->g;
    PlaneWaveGeom pg;
    pg.rb = g.earth + (g.rgor - (double)(g.nnr - 1) * g.dnr);
    pg.thc = g.rgox + (double)(g.nnx - 1) * g.dnx * 0.5;
    pg.phc = g.rgoz + (double)(g.nnz - 1) * g.dnz * 0.5;
    pg.rbs = pg.rb * std::sin(pg.thc);
    CK(cudaMemcpyAsync(ctx->d_params, params, (size_t)nev * 4 * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    launch_planewave_frames(g, pg, nev, ctx->d_params, ctx->d_frames, ctx->stream);
    ctx->launches += 1;
    CKL();
    return solve_common(ctx, nev, st);
}

int fm3dt_solve_point(fm3dt_ctx *ctx, int nev, const double *src, int refine, int extent, fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!src) return fail(ctx, FM3DT_EINVAL, "null sources");
    if (refine != 0 && (refine < 2 || refine > 16)) return fail(ctx, FM3DT_EINVAL, "refine must be 0 or 2..16");
    if (extent < (refine ? 2 : 1) || extent > 16)
        return fail(ctx, FM3DT_EINVAL, refine ? "extent must be 2..16 with a refined grid" : "extent must be 1..16");
    const Geom &g = ctx->g;
    cudaStream_t s = ctx->stream;
    std::vector<PointSource> ps(nev);
    std::vector<int> box(6 * (size_t)nev), fixed(6 * (size_t)nev);
    for (int e = 0; e < nev; ++e) {
        const PointSource p{src[3 * e], src[3 * e + 1], src[3 * e + 2]};
        const double f[3] = {(g.rgor - p.h) / g.dnr, (p.th - g.rgox) / g.dnx, (p.ph - g.rgoz) / g.dnz};
        const int n[3] = {g.nnr, g.nnx, g.nnz};
        for (int a = 0; a < 3; ++a) {
            if (!(f[a] >= 0.0 && f[a] < (double)(n[a] - 1)))
                return fail(ctx, FM3DT_ERANGE, "source " + std::to_string(e + 1) + " lies outside the grid");
            const int c = (int)std::floor(f[a]);
            const int lo = std::max(0, c - extent + 1), hi = std::min(n[a] - 1, c + extent);
            box[6 * e + 2 * a] = lo;
            box[6 * e + 2 * a + 1] = hi;
            // with a refined grid the box's outer layer is left to the coarse
            // solve (the fine solve saw nothing outside the box), except on
            // the faces of the grid itself
            fixed[6 * e + 2 * a] = (refine && lo > 0) ? lo + 1 : lo;
            fixed[6 * e + 2 * a + 1] = (refine && hi < n[a] - 1) ? hi - 1 : hi;
        }
        ps[e] = p;
    }
    const size_t rs = rsize(ctx->prec);
    launch_fill_inf(ctx->d_T, (size_t)nev * ctx->N, ctx->prec, s);
    CK(cudaMemsetAsync(ctx->d_base, 0, (size_t)nev * sizeof(double), s));
    ctx->launches += 1;
    if (!refine) {
        PointSource *d_src = nullptr;
        DeviceScratch sc(ctx);
        CK(sc.alloc(&d_src, (size_t)nev));
        CK(cudaMemcpyAsync(d_src, ps.data(), nev * sizeof(PointSource), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->d_box, box.data(), box.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->d_box_init, box.data(), box.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        launch_point_analytic(g, ctx->prec, ctx->d_veln, nev, d_src, ctx->d_box, ctx->d_T, s);
        ctx->launches += 1;
        CKL();
    } else {
        CK(cudaStreamSynchronize(s));
        for (int e = 0; e < nev; ++e) {
            const int *b = &box[6 * e];
            const int fn[3] = {(b[1] - b[0]) * refine + 1, (b[3] - b[2]) * refine + 1, (b[5] - b[4]) * refine + 1};
            fm3dt_ctx *fc = nullptr;
            for (auto &fe : ctx->fine)
                if (fe.nnr == fn[0] && fe.nnx == fn[1] && fe.nnz == fn[2]) fc = fe.ctx;
            if (!fc) {
                fm3dt_grid_desc fd = ctx->desc;
                fd.nnr = fn[0];
                fd.nnx = fn[1];
                fd.nnz = fn[2];
                fd.max_events = 1;
                rc = fm3dt_ctx_create(&fd, &fc);
                if (rc != FM3DT_OK) return fail(ctx, rc, std::string("refined grid: ") + fm3dt_last_error(nullptr));
                inherit_tuning(fc, ctx);
                ctx->fine.push_back({fn[0], fn[1], fn[2], fc});
            }
            // the refined grid: node (0,0,0) on the box corner, 1/refine spacing
            Geom fg = g;
            fg.nnr = fn[0];
            fg.nnx = fn[1];
            fg.nnz = fn[2];
            fg.rgor = g.rgor - (double)b[0] * g.dnr;
            fg.rgox = g.rgox + (double)b[2] * g.dnx;
            fg.rgoz = g.rgoz + (double)b[4] * g.dnz;
            fg.dnr = g.dnr / refine;
            fg.dnx = g.dnx / refine;
            fg.dnz = g.dnz / refine;
            rc = set_geometry(fc, fg);
            if (rc != FM3DT_OK) return fail(ctx, rc, std::string("refined grid: ") + fc->err);
            CK(cudaMemcpyAsync(fc->d_velv, ctx->d_velv,
                               (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2) * sizeof(double),
                               cudaMemcpyDeviceToDevice, fc->stream));
            launch_gridder(fg, fc->d_velv, fc->d_veln, fc->stream);
            launch_slowness(fg, fc->d_veln, fc->d_s, fc->prec, fc->stream);
            fc->have_velocity = 1;
            // straight-ray start within two fine cells of the source
            int fb[6];
            const double ff[3] = {(fg.rgor - ps[e].h) / fg.dnr, (ps[e].th - fg.rgox) / fg.dnx,
                                  (ps[e].ph - fg.rgoz) / fg.dnz};
            for (int a = 0; a < 3; ++a) {
                const int c = std::min(std::max((int)std::floor(ff[a]), 0), fn[a] - 2);
                fb[2 * a] = std::max(0, c - 1);
                fb[2 * a + 1] = std::min(fn[a] - 1, c + 2);
            }
            launch_fill_inf(fc->d_T, fc->N, fc->prec, fc->stream);
            CK(cudaMemsetAsync(fc->d_base, 0, sizeof(double), fc->stream));
            CK(cudaMemcpyAsync(fc->d_box, fb, sizeof fb, cudaMemcpyHostToDevice, fc->stream));
            CK(cudaMemcpyAsync(fc->d_box_init, fb, sizeof fb, cudaMemcpyHostToDevice, fc->stream));
            PointSource *d_src = nullptr;
            DeviceScratch sc(fc);
            CK(sc.alloc(&d_src, 1));
            CK(cudaMemcpyAsync(d_src, &ps[e], sizeof(PointSource), cudaMemcpyHostToDevice, fc->stream));
            launch_point_analytic(fg, fc->prec, fc->d_veln, 1, d_src, fc->d_box, fc->d_T, fc->stream);
            fc->launches += 4;
            fm3dt_status fst{};
            rc = solve_common(fc, 1, &fst, kPoint);
            ctx->launches += fc->launches;
            fc->launches = 0;
            if (rc != FM3DT_OK) return fail(ctx, rc, std::string("refined grid solve: ") + fc->err);
            launch_point_sample(ctx->prec, fc->d_T, fn[1], fn[2], refine, b, g.nnx, g.nnz,
                                (char *)ctx->d_T + (size_t)e * ctx->N * rs, s);
            ctx->launches += 1;
            CKL();
        }
        // fixed: the box without its outer layer; active at the start: every
        // tile the sampled box touches
        CK(cudaMemcpyAsync(ctx->d_box, fixed.data(), fixed.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->d_box_init, box.data(), box.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    return solve_common(ctx, nev, st, kPoint);
}

int fm3dt_receiver_times(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx, const double *rcz,
                         float *out)
{
    if (!ctx || nrc < 0 || (nrc > 0 && (!rcr || !rcx || !rcz || !out))) return FM3DT_EINVAL;
    if (ctx->nev_solved < 1) return fail(ctx, FM3DT_ESTATE, "no solved events");
    if (nrc == 0) return FM3DT_OK;
    const Geom &g = ctx->g;
    std::vector<RecCell> cells(nrc);
    for (int i = 0; i < nrc; ++i) {
        RecCell c;
        if (!locate_receiver(g, rcr[i], rcx[i], rcz[i], c))
            return fail(ctx, FM3DT_ERANGE, "receiver " + std::to_string(i + 1) + " lies outside the grid");
        cells[i] = c;
    }
    RecCell *d_cells = nullptr;
    float *d_out = nullptr;
    const int nev = ctx->nev_solved;
    DeviceScratch sc(ctx);
    CK(sc.alloc(&d_cells, (size_t)nrc));
    CK(sc.alloc(&d_out, (size_t)nev * nrc));
    CK(cudaMemcpyAsync(d_cells, cells.data(), nrc * sizeof(RecCell), cudaMemcpyHostToDevice, ctx->stream));
    launch_receivers(g, ctx->prec, ctx->d_T, ctx->d_base, nev, nrc, d_cells, d_out, ctx->stream);
    ctx->launches += 1;
    CKL();
    CK(cudaMemcpyAsync(out, d_out, (size_t)nev * nrc * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FM3DT_OK;
}

int fm3dt_receiver_times_device(fm3dt_ctx *ctx, int nrc, const double *d_rcr, const double *d_rcx,
                                const double *d_rcz, float *d_out)
{
    if (!ctx || nrc < 0 || (nrc > 0 && (!d_rcr || !d_rcx || !d_rcz || !d_out))) return FM3DT_EINVAL;
    if (ctx->nev_solved < 1) return fail(ctx, FM3DT_ESTATE, "no solved events");
    if (nrc == 0) return FM3DT_OK;
    cudaStream_t s = ctx->stream;
    DeviceScratch sc(ctx);
    int *d_bad = nullptr;
    CK(sc.alloc(&d_bad, 1));
    CK(cudaMemsetAsync(d_bad, 0x7f, sizeof(int), s));           // 0x7f7f7f7f: none
    launch_receivers_located(ctx->g, ctx->prec, ctx->d_T, ctx->d_base, ctx->nev_solved, nrc, d_rcr, d_rcx, d_rcz,
                             d_bad, d_out, s);
    ctx->launches += 1;
    CKL();
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (bad != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "receiver " + std::to_string(bad + 1) + " lies outside the grid");
    return FM3DT_OK;
}

// Rays of every solved event from receivers in device memory.  Traces the
// rays (end points to d_end when not null) and, when rows are wanted, forms
// the row pointers on the device (d_row_ptr, nrows + 1) and returns the entry
// count in *total; the caller then compacts the rows with rays_compact.
static int rays_trace(fm3dt_ctx *ctx, DeviceScratch &sc, int nrc, const double *d_rcr, const double *d_rcx,
               const double *d_rcz, bool want_rows, double *d_end, int64_t *d_row_ptr, int64_t *total,
               float **d_fdm_out)
{
    const Geom &g = ctx->g;
    const int nev = ctx->nev_solved;
    const int nrows = nev * nrc;
    const size_t nmp = (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2);
    cudaStream_t s = ctx->stream;
    float *d_fdm = nullptr;
    int *d_flags = nullptr;
    CK(sc.alloc(&d_flags, 2));
    CK(cudaMemsetAsync(d_flags, 0x7f, 2 * sizeof(int), s));     // 0x7f7f7f7f: no ray flagged
    if (want_rows) {
        // the dense rows: the context's own buffer, kept between calls (a
        // pool allocation of this size was not always reused once smaller
        // allocations had come and gone)
        const size_t need = (size_t)nrows * nmp * sizeof(float);
        if (need > ctx->dense_bytes) {
            CK(cudaStreamSynchronize(s));
            cudaFree(ctx->d_dense);
            ctx->d_dense = nullptr;
            ctx->dense_bytes = 0;
            CK(cudaMalloc(&ctx->d_dense, need));
            ctx->dense_bytes = need;
        }
        d_fdm = ctx->d_dense;
        CK(cudaMemsetAsync(d_fdm, 0, need, s));
    }
    RayArgs ra{};
    ra.g = g;
    ra.prec = ctx->prec;
    ra.T = ctx->d_T;
    ra.veln = ctx->d_veln;
    ra.nev = nev;
    ra.nrc = nrc;
    ra.rcr = d_rcr;
    ra.rcx = d_rcx;
    ra.rcz = d_rcz;
    ra.fdm = d_fdm;
    ra.endpoints = d_end;
    ra.nsteps = nullptr;
    ra.flags = d_flags;
    launch_rays(ra, s);
    ctx->launches += 1;
    CKL();
    *total = 0;
    if (want_rows) {
        int64_t *d_counts = nullptr, *d_chunks = nullptr;
        CK(sc.alloc(&d_counts, (size_t)nrows));
        CK(sc.alloc(&d_chunks, (size_t)scan_chunks(nrows)));
        launch_row_counts(d_fdm, nrows, (int)nmp, d_counts, s);
        launch_row_scan(d_counts, nrows, d_row_ptr, d_chunks, s);
        ctx->launches += 4;
        CKL();
        CK(cudaMemcpyAsync(total, d_row_ptr + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    }
    int flags[2] = {0, 0};
    CK(cudaMemcpyAsync(flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (flags[1] != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "ray " + std::to_string(flags[1]) + ": receiver " +
                                           std::to_string(flags[1] % nrc + 1) + " lies outside the grid");
    if (flags[0] != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "ray " + std::to_string(flags[0]) +
                                           ": B-spline support outside the velocity grid");
    *d_fdm_out = d_fdm;
    return FM3DT_OK;
}

// The address through which this device's kernels reach host memory at p,
// or null when there is none (pageable memory).
static void *mapped_host(const void *p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// How a host forward call moves page-locked data over this host's link: a
// kernel through the device mapping (*kernel = 1) or a copy-engine transfer
// (0), whichever moved up to 64 MB of the call's own buffers faster (the
// second of two tries of each; h2d: host -> dev, else dev -> host).  Hosts
// differ: measured on GB300 machines, 30 GB/s by copy against ~150 GB/s by
// kernel writes on one, 175 against 55 on another.  Transfers below 1 MB
// take the copy.
static int link_choice(fm3dt_ctx *ctx, double *dev, void *host, double *mapped, size_t bytes, bool h2d, int *kernel)
{
    *kernel = 0;
    bytes = std::min(bytes, (size_t)64 << 20) & ~(size_t)15;
    if (bytes < ((size_t)1 << 20)) return FM3DT_OK;
    const size_t n = bytes / sizeof(double);
    cudaStream_t s = ctx->stream;
    cudaEvent_t ev[3];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() { for (int i = 0; i < 3; ++i) cudaEventDestroy(e[i]); }
    } ev_guard{ev};
    float tk = 0.0f, tc = 0.0f;
    for (int rep = 0; rep < 2; ++rep) {
        CK(cudaEventRecord(ev[0], s));
        if (h2d)
            launch_link_copy(mapped, dev, n, s);
        else
            launch_link_copy(dev, mapped, n, s);
        ctx->launches += 1;
        CKL();
        CK(cudaEventRecord(ev[1], s));
        CK(cudaMemcpyAsync(h2d ? (void *)dev : host, h2d ? host : (void *)dev, bytes,
                           h2d ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(ev[2], s));
        CK(cudaStreamSynchronize(s));
        CK(cudaEventElapsedTime(&tk, ev[0], ev[1]));
        CK(cudaEventElapsedTime(&tc, ev[1], ev[2]));
    }
    *kernel = tk < tc ? 1 : 0;
    return FM3DT_OK;
}

// A host forward call's boundary frames into ctx->d_frames: read by a kernel
// through the device mapping when they are page-locked and the link favours
// it, else copied.
static int upload_frames(fm3dt_ctx *ctx, const double *boundary, int nev)
{
    const size_t n = (size_t)nev * ctx->NB;
    const double *m = (const double *)mapped_host(boundary);
    if (m && ctx->link_frames < 0) {
        int k = 0;
        const int rc = link_choice(ctx, ctx->d_frames, (void *)boundary, (double *)m, n * sizeof(double), true, &k);
        if (rc != FM3DT_OK) return rc;
        ctx->link_frames = k;
    }
    if (m && ctx->link_frames == 1) {
        launch_link_copy(m, ctx->d_frames, n, ctx->stream);
        ctx->launches += 1;
        CKL();
        return FM3DT_OK;
    }
    CK(cudaMemcpyAsync(ctx->d_frames, boundary, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return FM3DT_OK;
}

// Before a host forward call's rows exist: with page-locked cols and vals and
// no choice made yet, how its rows will leave (ctx->link_rows), measured on
// its own cols array (overwritten later) and device scratch.
static int choose_rows_link(fm3dt_ctx *ctx, DeviceScratch &sc, int32_t *cols, float *vals, int64_t cap)
{
    if (ctx->link_rows >= 0 || cap <= 0) return FM3DT_OK;
    double *m_cols = (double *)mapped_host(cols);
    if (!m_cols || !mapped_host(vals)) return FM3DT_OK;
    const size_t bytes = std::min((size_t)cap * sizeof(int32_t), (size_t)64 << 20) & ~(size_t)15;
    if (bytes < ((size_t)1 << 20)) return FM3DT_OK;
    if ((uintptr_t)cols % 16 != 0) return FM3DT_OK;
    double *tmp = nullptr;
    CK(sc.alloc(&tmp, bytes / sizeof(double)));
    int k = 0;
    const int rc = link_choice(ctx, tmp, (void *)cols, m_cols, bytes, false, &k);
    if (rc != FM3DT_OK) return rc;
    ctx->link_rows = k;
    return FM3DT_OK;
}

// Compacted rows of a host entry point into the caller's cols/vals: compacted
// into the context's buffer, then moved out by a kernel through the device
// mapping when both arrays are page-locked (16-byte aligned) and the link
// favours it, else by copy-engine transfers on stream s.
static int rays_compact(fm3dt_ctx *ctx, const float *d_fdm, int nrows, const int64_t *d_row_ptr, int32_t *d_cols,
                        float *d_vals);
static int rays_compact_to_host(fm3dt_ctx *ctx, const float *d_fdm, int nrows, const int64_t *d_rowptr,
                                int64_t total, int32_t *cols, float *vals, cudaStream_t s)
{
    // (the values at a 256-byte boundary after the columns)
    const size_t cbytes = (size_t)total * sizeof(int32_t), vbytes = (size_t)total * sizeof(float);
    const size_t voff = (cbytes + 255) & ~(size_t)255;
    const size_t need = voff + vbytes;
    if (need > ctx->compact_bytes) {
        CK(cudaStreamSynchronize(s));
        cudaFree(ctx->d_compact);
        ctx->d_compact = nullptr;
        ctx->compact_bytes = 0;
        CK(cudaMalloc(&ctx->d_compact, need));
        ctx->compact_bytes = need;
    }
    int32_t *d_cols = (int32_t *)ctx->d_compact;
    float *d_vals = (float *)((char *)ctx->d_compact + voff);
    const int rc = rays_compact(ctx, d_fdm, nrows, d_rowptr, d_cols, d_vals);
    if (rc != FM3DT_OK) return rc;
    void *m_cols = mapped_host(cols), *m_vals = mapped_host(vals);
    if (m_cols && m_vals && ctx->link_rows == 1 && (uintptr_t)m_cols % 16 == 0 && (uintptr_t)m_vals % 16 == 0) {
        launch_link_copy_bytes(d_cols, m_cols, cbytes, s);
        launch_link_copy_bytes(d_vals, m_vals, vbytes, s);
        ctx->launches += 2;
        CKL();
        return FM3DT_OK;
    }
    CK(cudaMemcpyAsync(cols, d_cols, cbytes, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(vals, d_vals, vbytes, cudaMemcpyDeviceToHost, s));
    return FM3DT_OK;
}

static int rays_compact(fm3dt_ctx *ctx, const float *d_fdm, int nrows, const int64_t *d_row_ptr, int32_t *d_cols,
                 float *d_vals)
{
    const Geom &g = ctx->g;
    const size_t nmp = (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2);
    launch_row_compact(d_fdm, nrows, (int)nmp, d_row_ptr, d_cols, d_vals, ctx->stream);
    ctx->launches += 1;
    CKL();
    return FM3DT_OK;
}

static int rays_ready(fm3dt_ctx *ctx)
{
    if (ctx->nev_solved < 1) return fail(ctx, FM3DT_ESTATE, "no solved events");
    if (!ctx->have_velocity) return fail(ctx, FM3DT_ESTATE, "no velocity model");
    if (ctx->last_point)
        return fail(ctx, FM3DT_ESTATE, "rays are traced through teleseismic (boundary-frame) solves only");
    return FM3DT_OK;
}

int fm3dt_rays_frechet(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx, const double *rcz,
                       int64_t *row_ptr, int32_t *cols, float *vals, int64_t cap, double *endpoints)
{
    if (!ctx || nrc < 0 || (nrc > 0 && (!rcr || !rcx || !rcz))) return FM3DT_EINVAL;
    int rc = rays_ready(ctx);
    if (rc != FM3DT_OK) return rc;
    const bool want_rows = cols != nullptr && vals != nullptr;
    if (want_rows && !row_ptr) return FM3DT_EINVAL;
    if (nrc == 0) return FM3DT_OK;
    for (int i = 0; i < nrc; ++i) {
        RecCell c;
        if (!locate_receiver(ctx->g, rcr[i], rcx[i], rcz[i], c))
            return fail(ctx, FM3DT_ERANGE, "receiver " + std::to_string(i + 1) + " lies outside the grid");
    }
    const int nrows = ctx->nev_solved * nrc;
    cudaStream_t s = ctx->stream;
    const auto h0 = std::chrono::steady_clock::now();
    cudaEvent_t pev[4];
    for (auto &e : pev) CK(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() { for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]); }
    } ev_guard{pev};
    CK(cudaEventRecord(pev[0], s));
    DeviceScratch sc(ctx);
    double *d_rec = nullptr, *d_end = nullptr;
    int64_t *d_rowptr = nullptr;
    CK(sc.alloc(&d_rec, 3 * (size_t)nrc));
    if (endpoints) CK(sc.alloc(&d_end, 3 * (size_t)nrows));
    if (want_rows) CK(sc.alloc(&d_rowptr, (size_t)nrows + 1));
    CK(cudaMemcpyAsync(d_rec, rcr, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_rec + nrc, rcx, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_rec + 2 * nrc, rcz, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
    int64_t total = 0;
    float *d_fdm = nullptr;
    rc = rays_trace(ctx, sc, nrc, d_rec, d_rec + nrc, d_rec + 2 * nrc, want_rows, d_end, d_rowptr, &total, &d_fdm);
    if (rc != FM3DT_OK) return rc;
    CK(cudaEventRecord(pev[1], s));
    CK(cudaEventRecord(pev[2], s));
    if (endpoints)
        CK(cudaMemcpyAsync(endpoints, d_end, 3 * (size_t)nrows * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (want_rows) {
        CK(cudaMemcpyAsync(row_ptr, d_rowptr, ((size_t)nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        if (total > cap) {
            CK(cudaStreamSynchronize(s));
            return fail(ctx, FM3DT_ERANGE, "Frechet rows need " + std::to_string(total) + " entries, capacity " +
                                               std::to_string(cap));
        }
        if (total > 0) {
            // (the compacted rows in the context's buffer, kept between calls)
            const size_t need = (size_t)total * (sizeof(int32_t) + sizeof(float));
            if (need > ctx->compact_bytes) {
                CK(cudaStreamSynchronize(s));
                cudaFree(ctx->d_compact);
                ctx->d_compact = nullptr;
                ctx->compact_bytes = 0;
                CK(cudaMalloc(&ctx->d_compact, need));
                ctx->compact_bytes = need;
            }
            int32_t *d_cols = (int32_t *)ctx->d_compact;
            float *d_vals = (float *)((char *)ctx->d_compact + (size_t)total * sizeof(int32_t));
            rc = rays_compact(ctx, d_fdm, nrows, d_rowptr, d_cols, d_vals);
            if (rc != FM3DT_OK) return rc;
            CK(cudaEventRecord(pev[2], s));
            CK(cudaMemcpyAsync(cols, d_cols, (size_t)total * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(vals, d_vals, (size_t)total * sizeof(float), cudaMemcpyDeviceToHost, s));
        }
    } else if (row_ptr) {
        for (int q = 0; q <= nrows; ++q) row_ptr[q] = 0;
    }
    CK(cudaEventRecord(pev[3], s));
    CK(cudaStreamSynchronize(s));
    cudaEventElapsedTime(&ctx->rays_ms[0], pev[0], pev[1]);
    cudaEventElapsedTime(&ctx->rays_ms[1], pev[1], pev[2]);
    cudaEventElapsedTime(&ctx->rays_ms[2], pev[2], pev[3]);
    ctx->rays_ms[3] = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - h0).count();
    return FM3DT_OK;
}

int fm3dt_rays_frechet_device(fm3dt_ctx *ctx, int nrc, const double *d_rcr, const double *d_rcx,
                              const double *d_rcz, int64_t *d_row_ptr, int32_t *d_cols, float *d_vals, int64_t cap,
                              int64_t *total, double *d_endpoints)
{
    if (!ctx || nrc < 0 || (nrc > 0 && (!d_rcr || !d_rcx || !d_rcz))) return FM3DT_EINVAL;
    int rc = rays_ready(ctx);
    if (rc != FM3DT_OK) return rc;
    const bool want_rows = d_cols != nullptr && d_vals != nullptr;
    if (want_rows && (!d_row_ptr || !total)) return FM3DT_EINVAL;
    if (total) *total = 0;
    if (nrc == 0) return FM3DT_OK;
    const int nrows = ctx->nev_solved * nrc;
    DeviceScratch sc(ctx);
    int64_t n = 0;
    float *d_fdm = nullptr;
    rc = rays_trace(ctx, sc, nrc, d_rcr, d_rcx, d_rcz, want_rows, d_endpoints, d_row_ptr, &n, &d_fdm);
    if (rc != FM3DT_OK) return rc;
    if (!want_rows) {
        CK(cudaStreamSynchronize(ctx->stream));
        return FM3DT_OK;
    }
    *total = n;
    if (n > cap)
        return fail(ctx, FM3DT_ERANGE, "Frechet rows need " + std::to_string(n) + " entries, capacity " +
                                           std::to_string(cap));
    if (n > 0) {
        rc = rays_compact(ctx, d_fdm, nrows, d_row_ptr, d_cols, d_vals);
        if (rc != FM3DT_OK) return rc;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return FM3DT_OK;
}

// The forward step of a batch whose boundary frames are in ctx->d_frames:
// the solve, with the rays of the part that converges first traced inside
// it (ctx->early), then the receiver times (d_times) and the remaining rays;
// with rows, the row pointers on the device (d_row_ptr) and the entry count
// in *total, the dense rows in *d_fdm_out for rays_compact.
static int forward_common(fm3dt_ctx *ctx, DeviceScratch &sc, int nev, int nrc, const double *d_rcr,
                          const double *d_rcx, const double *d_rcz, float *d_times, bool want_rows, double *d_end,
                          int64_t *d_row_ptr, int64_t *total, float **d_fdm_out, fm3dt_status *st)
{
    const Geom &g = ctx->g;
    const int nrows = nev * nrc;
    const size_t nmp = (size_t)(g.nvr + 2) * (g.nvx + 2) * (g.nvz + 2);
    cudaStream_t s = ctx->stream;
    int *d_flags = nullptr;   // [0], [1] as RayArgs::flags; [2] the first receiver outside the grid
    CK(sc.alloc(&d_flags, 3));
    CK(cudaMemsetAsync(d_flags, 0x7f, 3 * sizeof(int), s));      // 0x7f7f7f7f: none
    float *d_fdm = nullptr;
    const size_t need = want_rows ? (size_t)nrows * nmp * sizeof(float) : 0;
    if (need > ctx->dense_bytes) {
        CK(cudaStreamSynchronize(s));
        cudaFree(ctx->d_dense);
        ctx->d_dense = nullptr;
        ctx->dense_bytes = 0;
        CK(cudaMalloc(&ctx->d_dense, need));
        ctx->dense_bytes = need;
    }
    if (want_rows) d_fdm = ctx->d_dense;
    auto &er = ctx->early;
    er.nrc = nrc;
    er.rcr = d_rcr;
    er.rcx = d_rcx;
    er.rcz = d_rcz;
    er.fdm = d_fdm;
    er.fdm_bytes = need;
    er.endpoints = d_end;
    er.flags = d_flags;
    er.d_events = ctx->d_ray_events;
    er.events.clear();
    er.on = nrc > 0;
    struct Off {
        fm3dt_ctx::EarlyRays &e;
        ~Off() { e.on = false; }
    } off{er};
    int rc = solve_common(ctx, nev, st);
    er.on = false;
    ctx->early_events = (int)er.events.size();
    if (rc != FM3DT_OK) return rc;
    *total = 0;
    if (nrc == 0) return FM3DT_OK;
    launch_receivers_located(g, ctx->prec, ctx->d_T, ctx->d_base, nev, nrc, d_rcr, d_rcx, d_rcz, d_flags + 2,
                             d_times, s);
    ctx->launches += 1;
    // the rays of the events not traced inside the solve
    if (er.events.empty()) {
        if (d_fdm) CK(cudaMemsetAsync(d_fdm, 0, need, s));
        launch_ray_list(ctx, nev, er, nullptr, 0, s);
    } else if ((int)er.events.size() < nev) {
        std::vector<char> early(nev, 0);
        for (int e : er.events) early[e] = 1;
        std::vector<int> rest;
        for (int e = 0; e < nev; ++e)
            if (!early[e]) rest.push_back(e);
        int *d_rest = ctx->d_ray_events + ctx->maxev;
        CK(cudaMemcpyAsync(d_rest, rest.data(), rest.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        launch_ray_list(ctx, nev, er, d_rest, (int)rest.size(), s);
    }
    CKL();
    if (want_rows) {
        int64_t *d_counts = nullptr, *d_chunks = nullptr;
        CK(sc.alloc(&d_counts, (size_t)nrows));
        CK(sc.alloc(&d_chunks, (size_t)scan_chunks(nrows)));
        launch_row_counts(d_fdm, nrows, (int)nmp, d_counts, s);
        launch_row_scan(d_counts, nrows, d_row_ptr, d_chunks, s);
        ctx->launches += 4;
        CKL();
        CK(cudaMemcpyAsync(total, d_row_ptr + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    }
    int flags[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (flags[2] != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "receiver " + std::to_string(flags[2] + 1) + " lies outside the grid");
    if (flags[1] != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "ray " + std::to_string(flags[1]) + ": receiver " +
                                           std::to_string(flags[1] % nrc + 1) + " lies outside the grid");
    if (flags[0] != 0x7f7f7f7f)
        return fail(ctx, FM3DT_ERANGE, "ray " + std::to_string(flags[0]) +
                                           ": B-spline support outside the velocity grid");
    *d_fdm_out = d_fdm;
    return FM3DT_OK;
}

int fm3dt_forward_device(fm3dt_ctx *ctx, int nev, const double *d_boundary, int nrc, const double *d_rcr,
                         const double *d_rcx, const double *d_rcz, float *d_times, int64_t *d_row_ptr,
                         int32_t *d_cols, float *d_vals, int64_t cap, int64_t *total, double *d_endpoints,
                         fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!d_boundary || nrc < 0 || (nrc > 0 && (!d_rcr || !d_rcx || !d_rcz || !d_times)))
        return fail(ctx, FM3DT_EINVAL, "null argument");
    const bool want_rows = d_cols != nullptr && d_vals != nullptr;
    if (want_rows && (!d_row_ptr || !total)) return fail(ctx, FM3DT_EINVAL, "rows need d_row_ptr and total");
    if (total) *total = 0;
    CK(cudaMemcpyAsync(ctx->d_frames, d_boundary, (size_t)nev * ctx->NB * sizeof(double), cudaMemcpyDeviceToDevice,
                       ctx->stream));
    DeviceScratch sc(ctx);
    int64_t n = 0;
    float *d_fdm = nullptr;
    rc = forward_common(ctx, sc, nev, nrc, d_rcr, d_rcx, d_rcz, d_times, want_rows, d_endpoints, d_row_ptr, &n,
                        &d_fdm, st);
    if (rc != FM3DT_OK || !want_rows || nrc == 0) return rc;
    *total = n;
    if (n > cap)
        return fail(ctx, FM3DT_ERANGE, "Frechet rows need " + std::to_string(n) + " entries, capacity " +
                                           std::to_string(cap));
    if (n > 0) {
        rc = rays_compact(ctx, d_fdm, nev * nrc, d_row_ptr, d_cols, d_vals);
        if (rc != FM3DT_OK) return rc;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return FM3DT_OK;
}

int fm3dt_forward(fm3dt_ctx *ctx, int nev, const double *boundary, int nrc, const double *rcr, const double *rcx,
                  const double *rcz, float *times, int64_t *row_ptr, int32_t *cols, float *vals, int64_t cap,
                  double *endpoints, fm3dt_status *st)
{
    int rc = check_ready(ctx, nev);
    if (rc) return rc;
    if (!boundary || nrc < 0 || (nrc > 0 && (!rcr || !rcx || !rcz || !times)))
        return fail(ctx, FM3DT_EINVAL, "null argument");
    const bool want_rows = cols != nullptr && vals != nullptr;
    if (want_rows && !row_ptr) return fail(ctx, FM3DT_EINVAL, "rows need row_ptr");
    cudaStream_t s = ctx->stream;
    const int nrows = nev * nrc;
    DeviceScratch sc(ctx);
    double *d_rec = nullptr, *d_end = nullptr;
    float *d_times = nullptr;
    int64_t *d_rowptr = nullptr;
    if (nrc > 0) {
        CK(sc.alloc(&d_rec, 3 * (size_t)nrc));
        CK(sc.alloc(&d_times, (size_t)nrows));
        if (endpoints) CK(sc.alloc(&d_end, 3 * (size_t)nrows));
        if (want_rows) CK(sc.alloc(&d_rowptr, (size_t)nrows + 1));
        CK(cudaMemcpyAsync(d_rec, rcr, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_rec + nrc, rcx, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_rec + 2 * nrc, rcz, nrc * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    rc = upload_frames(ctx, boundary, nev);
    if (rc != FM3DT_OK) return rc;
    if (want_rows && nrc > 0) {
        rc = choose_rows_link(ctx, sc, cols, vals, cap);
        if (rc != FM3DT_OK) return rc;
    }
    int64_t total = 0;
    float *d_fdm = nullptr;
    rc = forward_common(ctx, sc, nev, nrc, d_rec, d_rec + nrc, d_rec + 2 * nrc, d_times, want_rows, d_end, d_rowptr,
                        &total, &d_fdm, st);
    if (rc != FM3DT_OK || nrc == 0) return rc;
    CK(cudaMemcpyAsync(times, d_times, (size_t)nrows * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (endpoints)
        CK(cudaMemcpyAsync(endpoints, d_end, 3 * (size_t)nrows * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (want_rows) {
        CK(cudaMemcpyAsync(row_ptr, d_rowptr, ((size_t)nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        if (total > cap) {
            CK(cudaStreamSynchronize(s));
            return fail(ctx, FM3DT_ERANGE, "Frechet rows need " + std::to_string(total) + " entries, capacity " +
                                               std::to_string(cap));
        }
        if (total > 0) {
            rc = rays_compact_to_host(ctx, d_fdm, nrows, d_rowptr, total, cols, vals, s);
            if (rc != FM3DT_OK) return rc;
        }
    }
    CK(cudaStreamSynchronize(s));
    return FM3DT_OK;
}

int fm3dt_forward_early_events(const fm3dt_ctx *ctx)
{
    return ctx ? ctx->early_events : 0;
}

int fm3dt_set_host_link(fm3dt_ctx *ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) return FM3DT_EINVAL;
    const int v = mode == 0 ? -1 : mode - 1;
    ctx->link_frames = ctx->link_rows = v;
    return FM3DT_OK;
}

int fm3dt_host_link(const fm3dt_ctx *ctx, int *frames, int *rows)
{
    if (!ctx || !frames || !rows) return FM3DT_EINVAL;
    *frames = ctx->link_frames;
    *rows = ctx->link_rows;
    return FM3DT_OK;
}

int fm3dt_get_times(fm3dt_ctx *ctx, int event, double *ttn)
{
    if (!ctx || !ttn) return FM3DT_EINVAL;
    if (event < 0 || event >= ctx->nev_solved) return fail(ctx, FM3DT_EINVAL, "event not solved");
    double *d_out = nullptr;
    DeviceScratch sc(ctx);
    CK(sc.alloc(&d_out, ctx->N));
    const double base = ctx->prec == FM3DT_FP64 ? 0.0 : ctx->h_base[event];
    launch_to_absolute(ctx->g, ctx->prec, ctx->d_T, (size_t)event * ctx->N, base, d_out, ctx->stream);
    ctx->launches += 1;
    CKL();
    CK(cudaMemcpyAsync(ttn, d_out, ctx->N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FM3DT_OK;
}

int fm3dt_get_velocity(fm3dt_ctx *ctx, double *veln)
{
    if (!ctx || !veln) return FM3DT_EINVAL;
    if (!ctx->have_velocity) return fail(ctx, FM3DT_ESTATE, "no velocity model");
    const Geom &g = ctx->g;
    const size_t npad = (size_t)(g.nnr + 3) * (g.nnx + 3) * (g.nnz + 3);
    CK(cudaMemcpyAsync(veln, ctx->d_veln, npad * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FM3DT_OK;
}

int fm3dt_set_times(fm3dt_ctx *ctx, int event, int nev_total, const double *ttn)
{
    if (!ctx || !ttn) return FM3DT_EINVAL;
    if (nev_total < 1 || nev_total > ctx->maxev || event < 0 || event >= nev_total)
        return fail(ctx, FM3DT_EINVAL, "event index outside 1..max_events");
    double base = 0.0;
    if (ctx->prec != FM3DT_FP64) {
        double m = INFINITY;
        for (size_t q = 0; q < ctx->N; ++q)
            if (ttn[q] > 0.0 && ttn[q] < m) m = ttn[q];
        base = std::isfinite(m) ? m : 0.0;
    }
    if ((int)ctx->h_base.size() < nev_total) ctx->h_base.resize(nev_total, 0.0);
    ctx->h_base[event] = base;
    double *d_in = nullptr;
    DeviceScratch sc(ctx);
    CK(sc.alloc(&d_in, ctx->N));
    CK(cudaMemcpyAsync(d_in, ttn, ctx->N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    launch_from_absolute(ctx->g, ctx->prec, d_in, base, ctx->d_T, (size_t)event * ctx->N, ctx->stream);
    ctx->launches += 1;
    CKL();
    CK(cudaMemcpyAsync(ctx->d_base + event, &ctx->h_base[event], sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->nev_solved = nev_total;
    return FM3DT_OK;
}

int fm3dt_set_tuning(fm3dt_ctx *ctx, int tile_shape, int max_passes, int max_rounds, int sweep)
{
    if (!ctx) return FM3DT_EINVAL;
    if (tile_shape < 0 || tile_shape >= kNumShapes) return fail(ctx, FM3DT_EINVAL, "tile shape out of range");
    ctx->shape = tile_shape;
    if (max_passes > 0) ctx->max_passes = max_passes;
    if (max_rounds > 0) ctx->max_rounds = max_rounds;
    if (sweep >= 0) {
        ctx->sweep = sweep ? 1 : 0;
        ctx->verify = sweep == 2 ? 1 : 0;
    }
    return FM3DT_OK;
}

int fm3dt_set_schedule(fm3dt_ctx *ctx, int tie_sweeps, double tie_ratio, int resweeps, double resweep_frac)
{
    if (!ctx) return FM3DT_EINVAL;
    if (tie_sweeps > 16 || resweeps > 16 || tie_ratio > 1.0 || resweep_frac > 1.0 || tie_ratio != tie_ratio ||
        resweep_frac != resweep_frac)
        return fail(ctx, FM3DT_EINVAL, "schedule: tie_sweeps and resweeps <= 16, ratios <= 1");
    if (tie_sweeps >= 0) ctx->tie_sweeps = tie_sweeps;
    if (tie_ratio >= 0.0) ctx->tie_ratio = tie_ratio;
    if (resweeps >= 0) ctx->resweeps = resweeps;
    if (resweep_frac >= 0.0) ctx->resweep_frac = resweep_frac;
    return FM3DT_OK;
}

int fm3dt_set_sweep_shape(fm3dt_ctx *ctx, int tile_shape)
{
    if (!ctx) return FM3DT_EINVAL;
    if (tile_shape < 0 || tile_shape >= kNumSweepShapes)
        return fail(ctx, FM3DT_EINVAL, "sweep shape out of range");
    ctx->sweep_shape = tile_shape;
    return FM3DT_OK;
}

int fm3dt_set_sweep_segments(fm3dt_ctx *ctx, int segments, int tie_segments)
{
    if (!ctx) return FM3DT_EINVAL;
    if (segments < 0 || tie_segments < 0 || segments > 127 || tie_segments > 127)
        return fail(ctx, FM3DT_EINVAL, "segments outside 0..127");
    ctx->sweep_segments = segments;
    ctx->tie_segments = tie_segments;
    return FM3DT_OK;
}

int fm3dt_round_trace(fm3dt_ctx *ctx, int cap, int64_t *tiles, int64_t *updates)
{
    if (!ctx || cap < 0) return FM3DT_EINVAL;
    const int n = std::min(std::min(cap, ctx->last_rounds), fm3dt_ctx::kTraceRounds);
    if (n > 0 && tiles && updates) {
        std::vector<unsigned long long> h(2 * (size_t)n);
        CK(cudaMemcpy(h.data(), ctx->d_trace, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; ++i) {
            tiles[i] = (int64_t)h[2 * i];
            updates[i] = (int64_t)h[2 * i + 1];
        }
    }
    return ctx->last_rounds;
}

int fm3dt_tie_sweep_items(fm3dt_ctx *ctx, int cap, int64_t *run, int64_t *skipped)
{
    if (!ctx || cap < 0) return FM3DT_EINVAL;
    const int n = std::min(cap, ctx->act_sweeps);
    for (int i = 0; i < n; ++i) {
        if (run) run[i] = (int64_t)ctx->h_act_items[2 * i];
        if (skipped) skipped[i] = (int64_t)ctx->h_act_items[2 * i + 1];
    }
    return ctx->act_sweeps;
}

int fm3dt_tie_sweep_ms(fm3dt_ctx *ctx, int cap, float *ms)
{
    if (!ctx || cap < 0) return FM3DT_EINVAL;
    for (int i = 0; i < std::min(cap, ctx->tie_sweep_n) && ms; ++i) ms[i] = ctx->tie_sweep_ms[i];
    return ctx->tie_sweep_n;
}

int fm3dt_rays_ms(fm3dt_ctx *ctx, float *ms)
{
    if (!ctx || !ms) return FM3DT_EINVAL;
    for (int i = 0; i < 4; ++i) ms[i] = ctx->rays_ms[i];
    return FM3DT_OK;
}

int fm3dt_part_ms(fm3dt_ctx *ctx, float *ms)
{
    if (!ctx || !ms) return FM3DT_EINVAL;
    for (int i = 0; i < 4; ++i) ms[i] = ctx->part_ms[i];
    return FM3DT_OK;
}

int fm3dt_round_trace_ms(fm3dt_ctx *ctx, int cap, float *ms)
{
    if (!ctx || cap < 0) return FM3DT_EINVAL;
    const int n = std::min(cap, (int)ctx->round_ms_trace.size());
    for (int i = 0; i < n && ms; ++i) ms[i] = ctx->round_ms_trace[i];
    return (int)ctx->round_ms_trace.size();
}

int fm3dt_tile_shapes(int *count)
{
    if (!count) return FM3DT_EINVAL;
    *count = kNumShapes;
    return FM3DT_OK;
}

int fm3dt_tile_shape(int index, int *tr, int *tx, int *tz)
{
    if (index < 0 || index >= kNumShapes || !tr || !tx || !tz) return FM3DT_EINVAL;
    *tr = kShapes[index].tr;
    *tx = kShapes[index].tx;
    *tz = kShapes[index].tz;
    return FM3DT_OK;
}

int64_t fm3dt_launch_count(const fm3dt_ctx *ctx) { return ctx ? ctx->launches : 0; }

const char *fm3dt_last_error(const fm3dt_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

void fm3dt_ctx_destroy(fm3dt_ctx *ctx)
{
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &sg : ctx->sweep_graphs) cudaGraphExecDestroy(sg.exec);
    for (auto e : ctx->round_events) cudaEventDestroy(e);
    for (auto e : ctx->round_events_b) cudaEventDestroy(e);
    cudaFree(ctx->d_velv);
    cudaFree(ctx->d_veln);
    cudaFree(ctx->d_s);
    cudaFree(ctx->d_hx);
    cudaFree(ctx->d_hz);
    cudaFree(ctx->d_wx);
    cudaFree(ctx->d_wz);
    cudaFree(ctx->d_dir);
    for (auto &P : ctx->planes) cudaFree(P.d_tiles);
    for (auto &P : ctx->block_planes) cudaFree(P.d_tiles);
    cudaFree(ctx->d_events);
    cudaFree(ctx->d_events_b);
    cudaFree(ctx->d_list_b);
    cudaFree(ctx->d_count_b);
    cudaFree(ctx->d_list_c);
    cudaFree(ctx->d_act_items);
    cudaFree(ctx->d_next);
    cudaFree(ctx->d_ray_events);
    for (auto p : ctx->d_done) cudaFree(p);
    cudaFree(ctx->d_dense);
    cudaFree(ctx->d_compact);
    cudaFree(ctx->d_count_c);
    for (auto p : ctx->d_act) cudaFree(p);
    cudaFree(ctx->d_err);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->h_dir) cudaFreeHost(ctx->h_dir);
    cudaFree(ctx->d_T);
    cudaFree(ctx->d_frames);
    cudaFree(ctx->d_base);
    cudaFree(ctx->d_frozen);
    cudaFree(ctx->d_flag);
    cudaFree(ctx->d_cert);
    cudaFree(ctx->d_list[0]);
    cudaFree(ctx->d_list[1]);
    cudaFree(ctx->d_count[0]);
    cudaFree(ctx->d_count[1]);
    cudaFree(ctx->d_stats);
    cudaFree(ctx->d_trace);
    cudaFree(ctx->d_params);
    cudaFree(ctx->d_box);
    cudaFree(ctx->d_box_init);
    for (auto &f : ctx->fine) fm3dt_ctx_destroy(f.ctx);
    if (ctx->h_count) cudaFreeHost(ctx->h_count);
    if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    delete ctx;
}

}  // extern "C"
