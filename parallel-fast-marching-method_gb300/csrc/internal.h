// internal.h -- device data layout and kernel launchers of libfm3dt_gpu.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fm3dt_gpu.h"

namespace fm3dt {

// Grid in solver units (converted like fm3dt_parallel.f90:6110-6117).
struct Geom {
    int nvr, nvx, nvz;
    double gor, gox, goz, dvr, dvx, dvz;
    int nnr, nnx, nnz;
    double rgor, rgox, rgoz, dnr, dnx, dnz;
    double earth;
};

// Tile shapes of the solver kernel (r, theta, phi extents; phi is the
// contiguous axis).  One thread owns one (theta, phi) column of TR nodes.
struct TileShape { int tr, tx, tz; };
constexpr int kNumShapes = 6;
constexpr TileShape kShapes[kNumShapes] = {{4, 8, 32}, {8, 8, 32}, {16, 8, 32}, {8, 4, 32}, {16, 4, 32}, {32, 4, 32}};

// Field, model and tiling shared by the solver kernels.
template <typename R>
struct FieldArgs {
    R *T;                       // [E][nnr][nnx][nnz]
    const R *s;                 // [nnr][nnx][nnz] slowness
    const R *hx, *wx;           // [nnr]      r*dtheta and its inverse square
    const R *hz, *wz;           // [nnr*nnx]  r*sin(theta)*dphi and its inverse square
    R hr, wr;                   // dr and 1/dr^2
    const uint8_t *frozen;      // [E][nnx*nnz] fixed bottom-layer nodes
    const int *box;             // [E][6] fixed node box r0,r1,x0,x1,z0,z1 (inclusive) of point
                                // sources, or null
    int nnr, nnx, nnz;
    int ntr, ntx, ntz;          // tiles per axis
    int tiles_per_event;
    int order2;
};

// Per-tile flag of the rounds: the halo faces changed since the tile's last
// pass (up = r-1 side, down = r+1 side, then -/+ theta and -/+ phi), "recompute
// every node", and "in the next round's list".
constexpr int kFaceUp = 1, kFaceDown = 2, kFaceXm = 4, kFaceXp = 8, kFaceZm = 16, kFaceZp = 32;
constexpr int kFaceMask = 63, kFull = 64, kQueued = 128;
// A tile queued by the certification after a sweep: its first pass
// recomputes only the nodes the certification bitmap marks.
constexpr int kCert = 256;

// Arguments of one solver round.
template <typename R>
struct RoundArgs {
    FieldArgs<R> f;
    int *flag;                  // [E*tiles] 1 while a tile is queued
    const int *cur_list;
    const int *cur_count;
    int *next_list;
    int *next_count;
    int max_passes;
    unsigned long long *stats;  // [0] tiles processed, [1] node updates, [2] staged nodes
    unsigned long long *trace;  // per round: [2*round] tiles, [2*round+1] node updates (or null)
    int round;
    // nodes a certified tile recomputes first: bit r%32 of word
    // ((e*nnx + x)*nnz + z)*cert_nw + r/32 (or null)
    const unsigned *cert;
    int cert_nw;
    // tile + halo box by one TMA copy (tma != 0): the field as a 4-D tensor
    // (phi, theta, r, event) with the box of the tile shape; err is raised if
    // a copy does not complete in time
    int tma;
    int *err;
    alignas(64) CUtensorMap tmap;
    alignas(64) CUtensorMap smap;   // the slowness as a 3-D tensor, the box of a tile's nodes
};

// Arguments of one sweep launch (one tile hyperplane).
template <typename R>
struct SweepArgs {
    FieldArgs<R> f;
    const int *hp_tiles;        // swept tile coordinates (r' << 20 | x' << 10 | z'), by hyperplane
    int hoff, hcount;           // this hyperplane's slice of hp_tiles
    const int *dir;             // [E] bit 0: sweep +theta, bit 1: sweep +phi
    int nev;
};

// Streaming sweep (stream.cuh): one warp per column block of SX x SZ
// columns streamed over the whole height; sweep shape indices kNumShapes and
// up select these blocks.
struct StreamShape { int sx, sz; };
constexpr int kNumStream = 2;
constexpr StreamShape kStreamShapes[kNumStream] = {{4, 8}, {2, 16}};
constexpr int kNumSweepShapes = kNumShapes + kNumStream;

template <typename R>
struct StreamArgs {
    FieldArgs<R> f;
    const int *hp_blocks;       // swept (segment, x block, z block): s << 24 | x' << 12 | z', by hyperplane
    int hoff, hcount;
    const int *dir;             // [E] bit 0: sweep +theta, bit 1: sweep +phi, bits 2/3: near ties
    const int *events;          // the events swept (indices), or null for events 0..nev-1
    int nev;
    int flip;                   // bit 0 / 1: reverse theta / phi; bit 2: reverse each near-tie lateral direction
    int fresh;                  // the main sweep from an unset field: upstream-only node updates
    int nbx, nbz;               // column blocks per axis
    int seg_len;                // layers per height segment
    // verification sweep: when flag is set, every node whose value changes
    // queues its round tile (recompute all) and, near a tile face, the face
    // neighbour (that face changed) -- the first round's work list
    int *flag, *list, *count;
    int tr, tx, tz;             // the rounds' tile shape and tile counts
    int ntr, ntx, ntz, tiles_per_event;
    // activity (a chain of sweeps of the same events and height segments):
    // per item (event ordinal, segment, column block in grid order) a mask of
    // its chunks of 1 << act_shift layers in which a node changed in this
    // sweep (act_cur) and in the previous one (act_prev).  A step of an item
    // runs when one of its nodes lies in a chunk that can change: one near a
    // chunk that changed in the previous sweep (in the item or a face
    // neighbour), or earlier in this one (an upstream neighbour, or the item
    // itself); act_cur null: no tracking, act_prev null: everything runs.
    unsigned *act_cur;
    const unsigned *act_prev;
    unsigned *act_run;          // the chunks of each item that run (stream_activity_kernel)
    int act_shift;
    size_t act_n;               // masks in each activity buffer
    int *err;                   // bit 2 raised: an activity slot out of range (not accessed)
    // with tracking and a previous sweep (or null): [0] items that ran,
    // [1] items skipped
    unsigned long long *act_items;
    // one launch for the whole pass (flow): items taken in order from the
    // counter *next (zero at the start), hp_blocks holding every hyperplane's
    // blocks in order (hcount: all of them, hoff 0); an item starts when the
    // done flags (zero at the start, done_n of them, same slots as the
    // activity masks) of its three upstream neighbours are set
    int flow;
    unsigned *done;
    size_t done_n;
    unsigned *next;
};

void launch_stream_f32(int idx, int grid, const StreamArgs<float> &a, cudaStream_t st);
void launch_stream_f64(int idx, int grid, const StreamArgs<double> &a, cudaStream_t st);
int occupancy_stream_f32(int idx, bool fresh, bool flow = false);
int occupancy_stream_f64(int idx, bool fresh, bool flow = false);

// After a single sweep from an unset field: mark the nodes a recomputation
// could change (certification bitmap) and queue their tiles (kCert).
template <typename R>
struct CertifyArgs {
    FieldArgs<R> f;
    const int *events;          // the events (indices), all swept once
    int nev;
    const int *dir;             // [E] sweep directions (bit 0: +theta, bit 1: +phi)
    unsigned *cert;
    int cert_nw;
    int tr, tx, tz;             // the rounds' tile shape
    int *flag, *list, *count;
};
void launch_certify_f32(const CertifyArgs<float> &a, cudaStream_t st);
void launch_certify_f64(const CertifyArgs<double> &a, cudaStream_t st);

void launch_round_f64(int shape, int grid, const RoundArgs<double> &a, cudaStream_t st);
void launch_round_f32(int shape, int grid, const RoundArgs<float> &a, cudaStream_t st);
void launch_sweep_f64(int shape, int grid, const SweepArgs<double> &a, cudaStream_t st);
void launch_sweep_f32(int shape, int grid, const SweepArgs<float> &a, cudaStream_t st);
int occupancy_round_f32(int shape);
int occupancy_round_f64(int shape);
int occupancy_sweep_f32(int shape);
int occupancy_sweep_f64(int shape);
inline int round_blocks_per_sm(int shape, int prec)
{
    return prec == FM3DT_FP64 ? occupancy_round_f64(shape) : occupancy_round_f32(shape);
}
inline int sweep_blocks_per_sm(int shape, int prec)
{
    return prec == FM3DT_FP64 ? occupancy_sweep_f64(shape) : occupancy_sweep_f32(shape);
}

// model.cu
void launch_gridder(const Geom &g, const double *velv, double *veln, cudaStream_t st);
void launch_slowness(const Geom &g, const double *veln, void *s, int prec, cudaStream_t st);

// boundary.cu
struct PlaneWaveGeom { double rb, thc, phc, rbs; };
void launch_planewave_frames(const Geom &g, const PlaneWaveGeom &pg, int nev, const double *params,
                             double *frames, cudaStream_t st);
void launch_finalize_frames(const Geom &g, int nev, int prec, const double *frames, void *T,
                            uint8_t *frozen, double *base, cudaStream_t st);
void launch_fill_inf(void *T, size_t n, int prec, cudaStream_t st);
// n doubles between device memory and the device mapping of page-locked host
// memory (either way round), by a kernel
void launch_link_copy(const double *src, double *dst, size_t n, cudaStream_t st);
// the same for `bytes` bytes between 16-byte aligned addresses
void launch_link_copy_bytes(const void *src, void *dst, size_t bytes, cudaStream_t st);
void launch_sweep_directions(const Geom &g, int nev, const double *frames, int *dir, double tie_ratio,
                             cudaStream_t st);
// (events: the event of each of the nev entries; null = 0..nev-1)
void launch_initial_tiles(int nev, const int *events, int tiles_per_event, int first_tile, int count_per_event,
                          int *list, int *count, int *flag, cudaStream_t st);
void launch_initial_tiles_box(int nev, int tiles_per_event, int ntx, int ntz, int tr, int tx, int tz,
                              const int *box, int *list, int *count, int *flag, cudaStream_t st);
void launch_to_absolute(const Geom &g, int prec, const void *T, size_t offset, double base, double *out,
                        cudaStream_t st);
void launch_from_absolute(const Geom &g, int prec, const double *in, double base, void *T, size_t offset,
                          cudaStream_t st);

// point.cu -- point sources
struct PointSource { double h, th, ph; };   // height km, colatitude rad, longitude rad
void launch_point_analytic(const Geom &g, int prec, const double *veln, int nev, const PointSource *src,
                           const int *box, void *T, cudaStream_t st);
void launch_point_sample(int prec, const void *Tf, int nnx_f, int nnz_f, int refine, const int box[6], int nnx,
                         int nnz, void *T_event, cudaStream_t st);

// receivers.cu
struct RecCell { int irr, irx, irz, pad; double drr, drx, drz; };
// Cell of a receiver and its offsets in it (F:7066-7097, with the
// last-subdomain clamp of F:7069-7070).  The cell indices are formed and
// range-checked in double precision before any conversion to int, so a NaN,
// infinite or huge coordinate is rejected (false) instead of converting with
// undefined behaviour.
__host__ __device__ inline bool locate_receiver(const Geom &g, double rcr, double rcx, double rcz, RecCell &c)
{
    const double fr = floor((g.rgor - rcr) / g.dnr) + 1.0;
    double fx = floor((rcx - g.rgox) / g.dnx) + 1.0;
    double fz = floor((rcz - g.rgoz) / g.dnz) + 1.0;
    if (fx == (double)g.nnx) fx -= 1.0;
    if (fz == (double)g.nnz) fz -= 1.0;
    // (every comparison with NaN is false)
    if (!(fr >= 1.0 && fr < (double)g.nnr && fx >= 1.0 && fx < (double)g.nnx && fz >= 1.0 && fz < (double)g.nnz))
        return false;
    c.irr = (int)fr;
    c.irx = (int)fx;
    c.irz = (int)fz;
    c.pad = 0;
    c.drx = (rcx - g.rgox) - (double)(c.irx - 1) * g.dnx;
    c.drz = (rcz - g.rgoz) - (double)(c.irz - 1) * g.dnz;
    c.drr = (g.rgor - rcr) - (double)(c.irr - 1) * g.dnr;
    return true;
}
void launch_receivers(const Geom &g, int prec, const void *T, const double *base, int nev, int nrc,
                      const RecCell *cells, float *out, cudaStream_t st);
// receivers located on the device (rcr/rcx/rcz in device memory); *bad gets
// the lowest index of a receiver outside the grid (atomicMin; preset it)
void launch_receivers_located(const Geom &g, int prec, const void *T, const double *base, int nev, int nrc,
                              const double *rcr, const double *rcx, const double *rcz, int *bad, float *out,
                              cudaStream_t st);

// rays.cu
struct RayArgs {
    Geom g;
    int prec;
    const void *T;              // [E][N] traveltimes (R)
    const double *veln;         // padded velocity (-1..n+1)
    int nev, nrc;
    const int *events;          // the events traced (nlist of them), or null for all nev
    int nlist;
    const double *rcr, *rcx, *rcz;
    float *fdm;                 // [E*nrc][nmp] dense rows, or nullptr
    double *endpoints;          // [E*nrc][3], or nullptr
    int *nsteps;                // [E*nrc], or nullptr
    // first ray (atomicMin) whose B-spline support left the velocity grid [0]
    // and whose receiver lies outside the propagation grid [1]; INT_MAX if none
    int *flags;
};
void launch_rays(const RayArgs &a, cudaStream_t st);
// row_ptr (nrows+1) from per-row counts; chunk_tmp holds scan_chunks(nrows) values
int scan_chunks(int nrows);
void launch_row_scan(const int64_t *counts, int nrows, int64_t *row_ptr, int64_t *chunk_tmp, cudaStream_t st);
void launch_row_counts(const float *fdm, int nrows, int nmp, int64_t *counts, cudaStream_t st);
void launch_row_compact(const float *fdm, int nrows, int nmp, const int64_t *row_ptr, int32_t *cols,
                        float *vals, cudaStream_t st);

}  // namespace fm3dt

struct fm3dt_ctx {
    fm3dt_grid_desc desc;
    fm3dt::Geom g;
    int prec = 0;
    int maxev = 0;
    size_t N = 0;       // nodes per event
    size_t NB = 0;      // bottom-frame nodes per event
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;   // scratch of the context's calls, kept between them
    // device buffers
    double *d_velv = nullptr;
    double *d_veln = nullptr;
    void *d_s = nullptr;
    void *d_hx = nullptr;
    void *d_hz = nullptr;
    void *d_wx = nullptr;
    void *d_wz = nullptr;
    int *d_dir = nullptr;
    void *d_T = nullptr;
    double *d_frames = nullptr;
    double *d_base = nullptr;
    uint8_t *d_frozen = nullptr;
    int *d_flag = nullptr;
    unsigned *d_cert = nullptr;   // [maxev][nnx][nnz][cert_nw] certification bitmap
    int cert_nw = 0;
    int *d_list[2] = {nullptr, nullptr};
    int *d_count[2] = {nullptr, nullptr};
    unsigned long long *d_stats = nullptr;
    double *d_params = nullptr;
    int *h_count = nullptr;       // pinned [2]: the list lengths of a solve's (up to) two parts
    unsigned long long *h_stats = nullptr;  // pinned
    std::vector<double> h_base;
    double hr = 0.0;
    int have_velocity = 0;
    int nev_solved = 0;
    // tuning
    int shape = 0;
    int max_passes = 64;
    int max_rounds = 0;           // 0 = automatic
    int sweep = 1;                // directional sweep before the rounds
    int sweep_shape = fm3dt::kNumShapes;   // the sweep's shape: streaming 4x8 column blocks
    int verify = 0;               // follow a streaming sweep by a verifying sweep (off: slower)
    unsigned long long *d_trace = nullptr;   // per-round tiles / node updates
    static constexpr int kTraceRounds = 8192;
    int last_rounds = 0;
    // tile hyperplanes of each shape (device list + host offsets)
    struct Planes { int shape = -1; int nseg = 1; int *d_tiles = nullptr; std::vector<int> off, cnt; };
    std::vector<Planes> block_planes;   // streaming sweeps, by (shape, height segments)
    int sweep_segments = 0;       // height segments of the streaming sweep (0: automatic)
    // solve schedule (fm3dt_set_schedule): extra sweeps of the near-tie events,
    // the near-tie band, re-sweeps after the first rounds and their threshold
    int tie_sweeps = 2;
    double tie_ratio = 0.1;
    int resweeps = 4;
    double resweep_frac = 0.01;
    int tie_segments = 0;         // the same for the reversed sweep of near-tie events
    int *h_dir = nullptr;         // pinned [maxev] sweep directions of the last solve
    int *d_events = nullptr;      // [maxev] the near-tie events of the last solve
    // the first round of the other events runs on stream2 while the near-tie
    // events get their extra sweeps; their first round then takes list_b
    cudaStream_t stream2 = nullptr;
    int *d_events_b = nullptr;    // [maxev] the other events
    int *d_ray_events = nullptr;  // [2 * maxev] a forward call's early ray events, then the rest
    int *d_list_b = nullptr;      // [flag_capacity]
    int *d_count_b = nullptr;
    int *d_list_c = nullptr;      // [flag_capacity] what the near-tie events' first round queues
    int *d_count_c = nullptr;
    // item activity of the near-tie events' extra sweeps (this sweep's and
    // the previous one's, alternating), grown on demand
    unsigned *d_act[3] = {nullptr, nullptr, nullptr};   // [2]: the chunks that run
    size_t act_bytes = 0;
    // items run / skipped by each of the last solve's near-tie extra sweeps
    static constexpr int kMaxTieSweeps = 16;
    unsigned long long *d_act_items = nullptr;   // [2 * kMaxTieSweeps]
    // one-launch sweep passes: done flags and queue counters, per stream
    // (context stream, stream2), the flags grown on demand
    unsigned *d_done[2] = {nullptr, nullptr};
    size_t done_bytes[2] = {0, 0};
    unsigned *d_next = nullptr;                  // [2]
    // the rays' dense rows and (host entry point) compacted rows, grown on demand
    float *d_dense = nullptr;
    size_t dense_bytes = 0;
    void *d_compact = nullptr;
    size_t compact_bytes = 0;
    // A forward call's rays traced inside its solve: when the part of a
    // two-part solve that converges first is done, its events' rays start on
    // the context stream while the other part still solves (see
    // fm3dt_forward_device).  Set for the length of that call only.
    struct EarlyRays {
        bool on = false;
        int nrc = 0;
        const double *rcr = nullptr, *rcx = nullptr, *rcz = nullptr;
        float *fdm = nullptr;        // dense rows (zeroed before the first launch), or null
        size_t fdm_bytes = 0;
        double *endpoints = nullptr;
        int *flags = nullptr;        // [2], as RayArgs::flags
        int *d_events = nullptr;     // [2 * maxev]: the early list, then the rest
        std::vector<int> events;     // host copy of the early list (empty: none launched)
    } early;
    unsigned long long h_act_items[2 * kMaxTieSweeps] = {};
    int act_sweeps = 0;
    float tie_sweep_ms[kMaxTieSweeps] = {};      // device time of each (two-part solves)
    int tie_sweep_n = 0;
    // TMA tensor maps of the field, by round tile shape (encoded on first use)
    int *d_err = nullptr;         // raised by a kernel whose bounded wait gave up
    bool tmap_ok[fm3dt::kNumShapes] = {};
    CUtensorMap tmap[fm3dt::kNumShapes];
    CUtensorMap smap[fm3dt::kNumShapes];
    int use_tma = 1;
    Planes planes[fm3dt::kNumSweepShapes];   // tile hyperplanes, then column-block hyperplanes
    size_t flag_capacity = 0;     // tiles allocated for flags/lists
    int64_t launches = 0;
    std::string err;
    // sweep passes captured as graphs, keyed by precision, sweep shape, event
    // count, event list, flip, height segments, form, stream, tile shape,
    // (flag mode) the flags and queue it writes, the activity it tracks and
    // (one-launch passes) its done flags
    static constexpr int kSweepKey = 16;
    static constexpr size_t kSweepGraphs = 24;
    struct SweepGraph { long long key[kSweepKey]; cudaGraphExec_t exec; };
    std::vector<SweepGraph> sweep_graphs;
    bool sweep_graph_off = false;
    std::vector<cudaEvent_t> round_events;   // start/stop pairs of round kernels
    std::vector<cudaEvent_t> round_events_b; // ... of a second part's rounds (stream2)
    std::vector<float> round_ms_trace;       // device time of each round of the last solve
    float part_ms[4] = {};                   // the first round's two parts (fm3dt_part_ms)
    float rays_ms[4] = {};                   // the last host-buffer ray call's phases (fm3dt_rays_ms)
    int early_events = 0;                    // events whose rays the last forward call traced early
    // how a host forward call moves page-locked frames in and rows out: through
    // the device mapping by kernels (1) or by copy-engine transfers (0);
    // -1 until measured on the context's first such call (fm3dt_set_host_link)
    int link_frames = -1, link_rows = -1;
    // point sources: fixed node boxes, and the refined source grids' contexts
    int *d_box = nullptr;         // [maxev][6] fixed nodes
    int *d_box_init = nullptr;    // [maxev][6] nodes whose tiles start active
    int last_point = 0;           // the last solve started from point sources
    struct Fine { int nnr, nnx, nnz; fm3dt_ctx *ctx; };
    std::vector<Fine> fine;
};
