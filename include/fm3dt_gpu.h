/*
 * fm3dt_gpu.h -- C ABI of the GB300 forward teleseismic traveltime solver.
 *
 * Drop-in replacement for the forward-solve path of the Parallel Fast
 * Marching Method program fm3dt_parallel (fm3dt_parallel.f90, "F" below).
 * The reference is one monolithic Fortran/MPI program with no library
 * interface; each entry point here replaces one stage of its per-source loop
 * (F:6371-6599) and takes plain host pointers, so a Fortran host binds it with
 * ISO_C_BINDING and a C/C++ or Python host with a prototype or ctypes.
 *
 * Conventions
 *  - The caller owns every host buffer; the library owns device memory.
 *  - Every function returns FM3DT_OK (0) or a negative FM3DT_E* code and never
 *    exits the process; fm3dt_last_error() gives a message for the last
 *    failure of that context (or of a failed create when ctx is NULL).
 *  - One context per host thread; each context has its own CUDA stream.
 *    Distinct contexts may be used concurrently from different threads.
 *  - Layouts follow the reference: traveltime fields and boundary frames are
 *    phi-fastest (F:6191 ttn(iz,ix,ir)), velocity nodes r-fastest (F:6118-6125).
 *  - Grid index ir = 1 is the top layer and ir = nnr the bottom layer, where
 *    the teleseismic wavefront is injected (F:6908-6913).
 */
#ifndef FM3DT_GPU_H
#define FM3DT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FM3DT_OK = 0,
    FM3DT_EINVAL = -1,        /* bad argument or dimension */
    FM3DT_ENOMEM = -2,        /* device allocation failed */
    FM3DT_ECUDA = -3,         /* CUDA runtime error */
    FM3DT_ENOCONV = -4,       /* solver round limit reached before convergence */
    FM3DT_ERANGE = -5,        /* receiver or ray support outside the grids */
    FM3DT_ESTATE = -6,        /* call out of order (e.g. solve before velocity) */
    FM3DT_ENODEV = -7         /* no CUDA device */
};

enum {
    FM3DT_FP64 = 0,           /* double-precision stencils (plain drop-in) */
    FM3DT_FP32_OFFSET = 1     /* single-precision stencils on times stored as
                                 offsets from each event's earliest boundary time */
};

/* Grid header exactly as the six .vtx header lines give it (F:6103-6108):
 * heights in km, latitude/longitude and angular steps in degrees.  The
 * library converts units like F:6110-6117.  fom is line 10 of
 * fm3dt_parallel.in (0 first order, 1 mixed order; F:100-111). */
typedef struct {
    int nvr, nvx, nvz;
    double gor, goxd, gozd;
    double dvr, dvxd, dvzd;
    int nnr, nnx, nnz;
    double rgor, rgoxd, rgozd;
    double dnr, dnxd, dnzd;
    double earth;
    int fom;
    int precision;            /* FM3DT_FP64 or FM3DT_FP32_OFFSET */
    int max_events;           /* events solved together per fm3dt_solve call */
} fm3dt_grid_desc;

/* Per-solve report. */
typedef struct {
    int rounds;               /* tile rounds until no tile was active */
    int converged;            /* 1 when every event reached its fixed point */
    int64_t tile_updates;     /* tile activations processed */
    int64_t node_passes;      /* node updates (tile nodes x in-tile passes) */
    int64_t tile_nodes;       /* grid nodes staged by all tile activations */
    double ms;                /* device time of the whole solve */
    double round_ms;          /* device time of the rounds: from the end of the sweep interval
                                 to the last round (in batches solved in two parts it also
                                 covers the near-tie events' extra sweeps and the
                                 certification, which run beside the first round) */
    int round_launches;       /* tile-round kernel launches */
    int sweep_launches;       /* directional-sweep kernel launches (all passes) */
    double sweep_ms;          /* device time of the sweep interval: the main sweep (in
                                 batches solved in two parts, until the other events' main
                                 sweep ends) plus any re-sweeps */
    int64_t sweep_nodes;      /* grid nodes staged by all sweep passes */
    int64_t interval_nodes;   /* of those, the nodes swept inside the sweep interval (the main
                                 sweeps and any re-sweeps; in batches solved in two parts the
                                 near-tie events' main sweep counts, their extra sweeps not) */
} fm3dt_status;

typedef struct fm3dt_ctx fm3dt_ctx;

/* Replaces F:6050-6191 (topology, input conversion, allocation).  Allocates
 * the device fields for desc->max_events events.  The context keeps the
 * rays' dense rows (nev*nrc*(nvr+2)*(nvx+2)*(nvz+2)*4 bytes, from the first
 * fm3dt_rays_frechet* call with rows, grown by a larger one) and the host
 * entry point's compacted rows until fm3dt_ctx_destroy; the other scratch of
 * its calls comes from a memory pool of the context that keeps its memory
 * until then too. */
int fm3dt_ctx_create(const fm3dt_grid_desc *desc, fm3dt_ctx **out);

/* Replaces F:6172 gridder (F:6989-7038): cubic B-spline interpolation of the
 * velocity nodes onto every propagation node, including the one-node ghost
 * ring.  velv: (nvz+2)(nvx+2)(nvr+2) doubles in .vtx order (r fastest). */
int fm3dt_set_velocity(fm3dt_ctx *ctx, const double *velv);

/* Replaces start_fmm (F:6894-6961) and the BSP fast-marching loop
 * (F:6371-6451) for nev <= max_events sources.  boundary: nev frames of
 * nnz*nnx doubles, phi fastest -- the itimes.out records of these sources;
 * values <= 0 mean "no time" (F:6935-6936), positive values are fixed. */
int fm3dt_solve(fm3dt_ctx *ctx, int nev, const double *boundary, fm3dt_status *st);

/* Same as fm3dt_solve with the boundary frames already in device memory
 * (d_boundary is a device pointer, e.g. frames kept resident between
 * tomography iterations). */
int fm3dt_solve_device(fm3dt_ctx *ctx, int nev, const double *d_boundary, fm3dt_status *st);

/* Continues the fast-iterative rounds from the current fields of the last
 * solved (or uploaded) events, every tile active, until no node changes.
 * On a converged solve it changes nothing (a fixed-point check); after
 * fm3dt_set_times with a field of a nearby model it is a warm start. */
int fm3dt_solve_resume(fm3dt_ctx *ctx, fm3dt_status *st);

/* Same solve with the boundary frames generated on the device from a
 * synthetic teleseismic plane wave per event: params is nev x 4 doubles
 * (t0 s, p s/km, cos az, sin az); time at a bottom node = t0 + p * d, d the
 * distance of the node from the section centre along the propagation azimuth
 * in the tangent plane of the bottom surface. */
int fm3dt_solve_planewave(fm3dt_ctx *ctx, int nev, const double *params, fm3dt_status *st);

/* Point sources (local events).  No counterpart in the reference, whose
 * sources are teleseismic boundary frames; the serving workload's local
 * events need it.  src: nev x 3 doubles (height km -- negative below the
 * surface --, colatitude rad, longitude rad; the receiver convention).
 * Around each source a box of 2*extent nodes per axis centred on the source
 * cell is started before the rounds run:
 *   refine = 0:  straight-ray times (Cartesian chord times the mean of the
 *                source's trilinear slowness and the node's), the whole box
 *                fixed;  extent 1..16;
 *   refine = k:  (2..16) a k-times finer grid over the box, started with
 *                straight-ray times within two fine cells of the source and
 *                solved to its fixed point, sampled at the coarse nodes; the
 *                box without its outer layer fixed;  extent 2..16.
 * Times are seconds after the origin time.  Receiver times work as after
 * fm3dt_solve; rays and Frechet rows are teleseismic only (FM3DT_ESTATE).
 * FM3DT_ERANGE if a source lies outside the grid. */
int fm3dt_solve_point(fm3dt_ctx *ctx, int nev, const double *src, int refine, int extent, fm3dt_status *st);

/* Replaces srtimes (F:7040-7248): trilinear receiver times of every solved
 * event, accumulated in single precision like REAL(4) trr (F:47, 7098-7106).
 * rcr: receiver height km; rcx: colatitude rad; rcz: longitude rad
 * (converted like F:6313-6314).  out: nev x nrc floats, event-major (the
 * rtravel.out order, F:7174-7176). */
int fm3dt_receiver_times(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx,
                         const double *rcz, float *out);

/* Same receiver times as fm3dt_receiver_times for callers that cannot
 * allocate memory after start-up -- e.g. a serving loop or a Fortran driver
 * that fixed its device footprint when it began and must keep it (an
 * allocation can block, fragment a pre-sized pool or fail under a quota).
 * This entry point has no counterpart in the reference.  It allocates
 * nothing: its scratch is one fixed device array of about 1.1 MiB inside the
 * library, held by every GPU that loads the library until the process ends.
 * Limits: nrc <= 4096 and nev * nrc <= 262144 per call, else FM3DT_EINVAL.
 * The first call on a device looks up that array's device address (once per
 * device, with the device current); make that first call before capturing
 * any stream.  The looked-up address is kept for the life of the process and
 * is not refreshed after cudaDeviceReset: a host that resets a device must not
 * call this entry point on that device again.  All calls share the array:
 * calls whose GPU work overlaps (other streams or contexts on the same device)
 * race on it.  A receiver outside the grid (or with a non-finite coordinate)
 * gives FM3DT_ERANGE and leaves `out` unwritten, as fm3dt_receiver_times does. */
int fm3dt_receiver_times_noalloc(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx,
                                 const double *rcz, float *out);

/* Replaces parallel_rpaths and the Frechet writer merge (F:6456-6599,
 * F:7250-7777): one ray per (event, receiver), traced from the receiver down
 * the traveltime gradient with step dnr until it leaves the grid, and its
 * Frechet row -integral(B/v^2 ds) accumulated in single precision.
 * Rows are returned as CSR over nev*nrc rows (event-major): row_ptr has
 * nev*nrc+1 entries; cols are the reference's 1-based velocity-node columns
 * ((iz*(nvx+2)+ix)*(nvr+2)+ir+1), ascending; vals single precision.  Only
 * entries with |value| >= 1e-6 are kept (F:7263).  cap is the capacity of
 * cols/vals; if the rows need more, FM3DT_ERANGE is returned with
 * row_ptr[nev*nrc] = the required count.  endpoints (nullable): nev*nrc*3
 * doubles (height km, colat rad, lon rad).  Pass cols = vals = NULL and
 * cap = 0 to trace rays only.  FM3DT_ERANGE if a receiver lies outside the
 * grid (or has a non-finite coordinate) or a ray's B-spline support leaves
 * the velocity grid. */
int fm3dt_rays_frechet(fm3dt_ctx *ctx, int nrc, const double *rcr, const double *rcx,
                       const double *rcz, int64_t *row_ptr, int32_t *cols, float *vals,
                       int64_t cap, double *endpoints);

/* Device-memory forms of fm3dt_receiver_times and fm3dt_rays_frechet, for a
 * tomography loop that keeps receivers, times and the Frechet matrix on the
 * GPU between iterations (the reference writes them to rtravel.out and
 * frechet.out, F:6503-6599, 7174-7176).  Every array argument is a device
 * pointer except *total.  fm3dt_receiver_times_device writes nev x nrc floats
 * to d_out.  fm3dt_rays_frechet_device writes nev*nrc+1 row pointers to
 * d_row_ptr (formed on the device), the entry count to *total, and the rows
 * to d_cols/d_vals when *total <= cap (FM3DT_ERANGE otherwise, rows not
 * written); d_endpoints is nullable; d_cols = d_vals = NULL traces rays only.
 * Both return after the GPU work has finished. */
int fm3dt_receiver_times_device(fm3dt_ctx *ctx, int nrc, const double *d_rcr, const double *d_rcx,
                                const double *d_rcz, float *d_out);
int fm3dt_rays_frechet_device(fm3dt_ctx *ctx, int nrc, const double *d_rcr, const double *d_rcx,
                              const double *d_rcz, int64_t *d_row_ptr, int32_t *d_cols, float *d_vals,
                              int64_t cap, int64_t *total, double *d_endpoints);

/* One forward step of a batch, as the reference's per-source loop runs it
 * (F:6273-6370: local_fmm, then srtimes F:7040-7248 and parallel_rpaths
 * F:7250-7777 on the field): fm3dt_solve, fm3dt_receiver_times and
 * fm3dt_rays_frechet in one call, with the same arguments, results and
 * errors as those three called in turn.  In a batch solved in two parts
 * (near-tie events and the others), the rays of the part that converges
 * first are traced while the other part still solves.
 * fm3dt_forward: host buffers (boundary frames, receivers in; times nev x nrc,
 * rows and nullable endpoints out; cols = vals = NULL traces rays only); when
 * cols and vals are page-locked memory mapped for the device (cudaHostAlloc,
 * cudaHostRegister), the compaction kernel can write the rows into them
 * directly, and a kernel can read page-locked boundary frames through their
 * mapping, where this host's link favours that (fm3dt_set_host_link).
 * fm3dt_forward_device: every array a device pointer (d_boundary frames
 * are copied into the context), *total on the host as in
 * fm3dt_rays_frechet_device.  st is nullable.  Both return after the GPU work
 * has finished. */
int fm3dt_forward(fm3dt_ctx *ctx, int nev, const double *boundary, int nrc, const double *rcr,
                  const double *rcx, const double *rcz, float *times, int64_t *row_ptr, int32_t *cols,
                  float *vals, int64_t cap, double *endpoints, fm3dt_status *st);
int fm3dt_forward_device(fm3dt_ctx *ctx, int nev, const double *d_boundary, int nrc, const double *d_rcr,
                         const double *d_rcx, const double *d_rcz, float *d_times, int64_t *d_row_ptr,
                         int32_t *d_cols, float *d_vals, int64_t cap, int64_t *total, double *d_endpoints,
                         fm3dt_status *st);
/* Events whose rays the last forward call traced inside its solve (0 when
 * the batch was solved in one part). */
int fm3dt_forward_early_events(const fm3dt_ctx *ctx);

/* How fm3dt_forward moves page-locked host buffers: mode 0 measures it on the
 * context's next such call (the default: a kernel through the device mapping
 * against a copy-engine transfer of up to 64 MB of that call's own buffers,
 * for the frames in and the rows out, the faster kept), 1 always copies, 2
 * always uses the mapping.  fm3dt_host_link reports the current choice for
 * the frames and the rows (-1 not yet measured, 0 copies, 1 mapping).
 * Results do not depend on it. */
int fm3dt_set_host_link(fm3dt_ctx *ctx, int mode);
int fm3dt_host_link(const fm3dt_ctx *ctx, int *frames, int *rows);

/* Copies the solved traveltime field of one event to the host: nnr*nnx*nnz
 * doubles, phi fastest (absolute seconds in both precisions; unreached nodes
 * are 0.0 like the reference's ttn). */
int fm3dt_get_times(fm3dt_ctx *ctx, int event, double *ttn);

/* Copies the gridded velocity (the reference's veln, F:6993) to the host:
 * (nnr+3)(nnx+3)(nnz+3) doubles, phi fastest, node indices -1..n+1. */
int fm3dt_get_velocity(fm3dt_ctx *ctx, double *veln);

/* Uploads a traveltime field for one event (nnr*nnx*nnz doubles, phi
 * fastest), e.g. to trace rays through a field computed elsewhere. */
int fm3dt_set_times(fm3dt_ctx *ctx, int event, int nev_total, const double *ttn);

/* Solver tuning: tile shape index, in-tile pass cap and round cap (0 keeps
 * the current value), directional sweep before the rounds (1 on, 0 off,
 * -1 keep; 2 on, and a streaming sweep is followed by a second, verifying
 * sweep that queues only the tiles still changing instead of starting the
 * rounds with every tile).  None of these changes the converged field. */
int fm3dt_set_tuning(fm3dt_ctx *ctx, int tile_shape, int max_passes, int max_rounds, int sweep);

/* Solve schedule (a negative value keeps the current one): extra sweeps of the
 * near-tie events, alternating reversed and forward (0..16, default 2); the
 * near-tie band, a lateral component below tie_ratio times the other (0..1,
 * default 0.1: within ~6 degrees of an axis); re-sweeps after the first rounds
 * (0..16, default 4) of the events with more than resweep_frac of their tiles
 * still queued (default 0.01).  None of these changes the converged field;
 * the best values depend on the model's heterogeneity. */
int fm3dt_set_schedule(fm3dt_ctx *ctx, int tie_sweeps, double tie_ratio, int resweeps, double resweep_frac);

/* Shape of the directional sweep (independent of the rounds' shape): a tile
 * shape index 0..count-1 of fm3dt_tile_shapes (tile sweep), or count +
 * 0 / 1 for the streaming sweep, one warp per 4x8 / 2x16 block of
 * (theta, phi) columns streamed over the whole height.  None of these
 * changes the converged field. */
int fm3dt_set_sweep_shape(fm3dt_ctx *ctx, int tile_shape);

/* Height segments of the streaming sweep (its work items are column blocks
 * of one segment; more segments give more parallel items per launch and a
 * longer pipeline ramp), for the sweep of every event and for the two extra
 * sweeps of the events whose lateral direction is a near tie (within ~6
 * degrees of an axis).  0 = automatic: chosen from the batch size for the
 * main sweep, two segments for the extra sweeps (they run beside the other
 * events' first round). */
int fm3dt_set_sweep_segments(fm3dt_ctx *ctx, int segments, int tie_segments);

/* Per-round trace of the last solve: tiles processed and node updates of
 * each round (up to cap rounds).  Returns the number of rounds, or a negative
 * error. */
int fm3dt_round_trace(fm3dt_ctx *ctx, int cap, int64_t *tiles, int64_t *updates);

/* Device time (ms, CUDA events around each launch) of each round of the last
 * solve, up to cap rounds.  Returns the number of rounds recorded. */
int fm3dt_round_trace_ms(fm3dt_ctx *ctx, int cap, float *ms);

/* Device times (ms) of the last solve's first round when it ran in two parts
 * side by side: ms[0] the near-tie events' extra sweeps, ms[1] their first
 * round, ms[2] the other events' certification, ms[3] their first round;
 * zeros when the solve ran in one part. */
int fm3dt_part_ms(fm3dt_ctx *ctx, float *ms);

/* Times (ms) of the last fm3dt_rays_frechet call: ms[0] device time of the
 * receivers' copy in, the rays and the row pointers; ms[1] of the rows'
 * compaction; ms[2] of the copies out; ms[3] the call's wall time. */
int fm3dt_rays_ms(fm3dt_ctx *ctx, float *ms);

/* The last solve's near-tie extra sweeps after the first skip the work items
 * (a height segment of a block of columns of one event) where nothing near
 * them changed: run[k] / skipped[k] the items extra sweep k ran and skipped,
 * for up to cap sweeps (sweep 0 runs every item and counts none).  Returns
 * the number of extra sweeps recorded (0 when none tracked activity). */
int fm3dt_tie_sweep_items(fm3dt_ctx *ctx, int cap, int64_t *run, int64_t *skipped);

/* Device time (ms) of each near-tie extra sweep of the last solve when it ran
 * in two parts (up to cap of them); returns their number (0 otherwise). */
int fm3dt_tie_sweep_ms(fm3dt_ctx *ctx, int cap, float *ms);

/* Number of available tile shapes and the shape (TR, TX, TZ) of one. */
int fm3dt_tile_shapes(int *count);
int fm3dt_tile_shape(int index, int *tr, int *tx, int *tz);

/* Kernel launches made by this context since creation. */
int64_t fm3dt_launch_count(const fm3dt_ctx *ctx);

const char *fm3dt_last_error(const fm3dt_ctx *ctx);

void fm3dt_ctx_destroy(fm3dt_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
