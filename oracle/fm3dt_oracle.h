/*
 * fm3dt_oracle.h -- CPU oracle for the forward teleseismic traveltime path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the serial
 * (1x1x1-subdomain) path of fm3dt_parallel.f90 of the Parallel Fast Marching
 * Method.  Only tests/, the smoke() entry and bench.py's CPU-baseline leg may
 * load it, and only as the checker.  The GPU library never links it.
 *
 * Parity status: UNPINNED by reference outputs.  The reference is Fortran 90 +
 * MPI; no Fortran compiler or MPI exists in this image, the reference ships no
 * tests and no golden vectors, and its one end-to-end input (itimes.out) is
 * missing from the repository.  The restatement is pinned instead by analytic
 * known-answer cases (homogeneous plane wave, linear gradient, straight ray)
 * in tests/test_oracle.py.
 *
 * Units follow the reference after its input conversion (F = fm3dt_parallel.f90):
 *   heights in km (positive up, r = earth + height), colatitude and longitude
 *   in radians, traveltimes in seconds.
 * Layouts:
 *   velv  (nvz+2)(nvx+2)(nvr+2) doubles, r fastest (the .vtx value order,
 *         F:6118-6125), index k + (nvr+2)*(j + (nvx+2)*i).
 *   veln  (nnr+3)(nnx+3)(nnz+3) doubles, phi fastest, node indices -1..n+1
 *         (F:6993), index (iz+1) + (nnz+3)*((ix+1) + (nnx+3)*(ir+1)) with
 *         1-based iz,ix,ir.
 *   ttn   nnr*nnx*nnz doubles, phi fastest, index (iz-1)+nnz*((ix-1)+nnx*(ir-1)).
 *         ir = 1 is the top layer, ir = nnr the bottom layer.
 *   bottom  nnz*nnx doubles, phi fastest: the boundary-time frame of one
 *         source (one itimes.out record, F:6908-6913).
 */
#ifndef FM3DT_ORACLE_H
#define FM3DT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nvr, nvx, nvz;
    double gor, gox, goz, dvr, dvx, dvz;
    int nnr, nnx, nnz;
    double rgor, rgox, rgoz, dnr, dnx, dnz;
    double earth;
} orc_grid;

/* Synthetic teleseismic plane wave on the bottom face (test input generator). */
typedef struct {
    double t0;      /* arrival time under the section centre, s */
    double p;       /* horizontal slowness along the bottom surface, s/km */
    double cos_az;  /* cosine / sine of the propagation azimuth (from north) */
    double sin_az;
} orc_planewave;

double orc_pi(void);

/* .vtx header (degrees, latitude) -> solver units (F:6103-6117). */
void orc_grid_from_header(const int nv[3], const double vorig[3], const double vstep[3],
                          const int nn[3], const double norig[3], const double nstep[3],
                          double earth, orc_grid *g);

/* receivers.dat / sources.dat latitude, longitude (degrees) -> colatitude,
 * longitude in radians (F:6283-6284, 6313-6314). */
void orc_latlon_to_rad(int n, const double *lat, const double *lon,
                       double *colat, double *lonr);

/* Cubic B-spline gridder (F:6989-7038).  Returns 0, or -1 if a velocity
 * index falls outside 0..nv+1 (the reference reads out of bounds there;
 * the oracle clamps and reports it). */
int orc_gridder(const orc_grid *g, const double *velv, double *veln, int *nclamped);

/* Serial narrow-band fast marching of one source: start_fmm seeding
 * (F:6894-6961) followed by local_fmm (F:78-155) with fouds1_all (fom=0,
 * F:535-633) or fouds2_all (fom=1, F:635-1004) and the binary heap of
 * F:1006-1098.  Unset nodes come back as 0.0 like the reference.  Returns
 * the number of heap pops in *npops.  Returns 0 or a negative error. */
int orc_fmm(const orc_grid *g, const double *veln, int fom, const double *bottom,
            double *ttn, long long *npops);

/* The reference's decomposed run (its mpirun -np 9 layout with nr = nx = nz
 * = 2, F:6052-6056): the grid split into nr x nx x nz blocks like F:6127-6168,
 * each block an emulated rank with its own gridder call (F:6172), start_fmm
 * on the bottom blocks (the block holding the earliest boundary time seeds
 * and marches), then bulk-synchronous rounds (F:6371-6451): exchange of the
 * two boundary layers with the neighbours that changed (F:6691-6795),
 * order_overlap with the face stencils fouds2_left .. fouds2_down and the
 * reopen pass (F:157-416, 1100-2825, 5747-6009), local_fmm, until no node
 * moved by more than the single-precision literal 1e-5 s (F:6403,
 * 6963-6987).  velv (not the gridded velocity): every block grids its own
 * nodes with its offsets.  Returns 0, -4 after max_rounds, -2 for blocks
 * thinner than two nodes, -3 out of memory; *rounds the rounds run. */
int orc_fmm_decomposed(const orc_grid *g, const double *velv, int fom, const double *bottom, int nr, int nx,
                       int nz, int max_rounds, double *ttn, int *rounds);

/* Fixed point of the reference's stencil: the same octant formulas
 * (fouds1_all / fouds2_all) with the heap's "alive" test restated as
 * "earlier than the node", iterated by Gauss-Seidel sweeps in alternating
 * directions until a sweep changes no bit.  Order independent; equals the
 * fast-marching result wherever the heap order is causal (e.g. a full
 * teleseismic frame on a smooth model).  Returns 0, or -4 if max_sweeps was
 * reached first. */
int orc_fixed_point(const orc_grid *g, const double *veln, int fom, const double *bottom,
                    double *ttn, int max_sweeps, int *sweeps);

/* The same fixed point from an arbitrary start: init (ttn layout, INFINITY =
 * unset) and fixed (one byte per node, 1 = keep the init value). */
int orc_fixed_point_field(const orc_grid *g, const double *veln, int fom, const double *init,
                          const unsigned char *fixed, double *ttn, int max_sweeps, int *sweeps);

/* Start of a point-source solve (no reference counterpart: a restatement of
 * the GPU library's fm3dt_solve_point): a box of 2*extent nodes per axis
 * around the source cell with straight-ray times (refine = 0, all fixed) or
 * the times of a refine-times finer grid over the box solved from a
 * straight-ray start (the box without its outer layer fixed).  Source at
 * height h km, colatitude th, longitude ph (radians).  Returns -5 if the
 * source lies outside the grid. */
int orc_point_start(const orc_grid *g, const double *velv, const double *veln, int fom, double h, double th,
                    double ph, int refine, int extent, double *init, unsigned char *fixed);

/* Receiver traveltimes (F:7040-7248): trilinear interpolation accumulated
 * in single precision.  Returns 0, or -(1+k) if receiver k lies outside the
 * propagation grid. */
int orc_srtimes(const orc_grid *g, const double *ttn, int nrc, const double *rcr,
                const double *rcx, const double *rcz, float *trr);

/* Ray back-tracing and Frechet rows (F:7250-7777) with the reference's global
 * boundary behaviour (rays stop, clipped, at the outer faces of the whole
 * grid).  fdm is nrc*nmp floats, nmp=(nvr+2)(nvx+2)(nvz+2), column order r
 * fastest (F:7753-7763); pass NULL to skip the Frechet accumulation (cfd=0).
 * endpoints gets 3 doubles (height km, colat, lon) per ray; nsteps the step
 * count per ray (0 when the start cell is outside the grid).  Returns 0 or a
 * negative error (-2: B-spline support outside the velocity grid). */
int orc_rays(const orc_grid *g, const double *ttn, const double *veln, int nrc,
             const double *rcr, const double *rcx, const double *rcz,
             float *fdm, double *endpoints, int *nsteps);

/* Sparsify one dense Frechet row like F:7739-7765 (|f| >= 1e-6 in single
 * precision).  Writes up to cap (col, val) pairs with 1-based columns and
 * returns the count. */
int orc_sparsify(int nmp, const float *row, int cap, int *cols, float *vals);

/* Synthetic plane-wave boundary frame: t = t0 + p * d, d the distance of the
 * bottom node from the section centre along the propagation azimuth in the
 * local tangent plane of the bottom surface.  frame is nnz*nnx, phi fastest. */
void orc_planewave_frame(const orc_grid *g, const orc_planewave *pw, double *frame);

/* Event parameters of the synthetic plane wave from an epicentral distance
 * and back-azimuth (degrees). */
void orc_planewave_params(const orc_grid *g, double delta_deg, double baz_deg,
                          orc_planewave *pw);

#ifdef __cplusplus
}
#endif
#endif
