/*
 * orbit_gb300 -- C ABI of the GB300-native PyORBIT 2.5D space-charge and
 * TEAPOT tracking hot path.
 *
 * One shared library (liborbit_gb300.so) exports these entry points.  All
 * signatures use plain C types and pointers; no framework types cross the
 * boundary.  Every function returns an int status (ORBIT_OK == 0, negative on
 * error) and records a message retrievable with orbit_last_error().  The
 * reference aborts the process on these conditions (ORBIT_MPI_Finalize, e.g.
 * src/spacecharge/SpaceChargeCalc2p5D.cc:131-143, Grid2D.cc:38-52,
 * PoissonSolverFFT2D.cc:30-42); this library reports them instead.
 *
 * Execution model: each bunch owns one CUDA stream.  Compute calls enqueue
 * work on the bunch's stream and return; orbit_bunch_sync() and the
 * download calls wait for it and report any error the kernels recorded in
 * the bunch's device status word.  Coordinates stay resident in HBM as six
 * FP64 arrays (x, xp, y, yp, z, dE) between calls.
 */
#ifndef ORBIT_GB300_H
#define ORBIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status codes                                                        */
/* ------------------------------------------------------------------ */
#define ORBIT_OK 0
#define ORBIT_ERR_ARG (-1)      /* bad handle, size or parameter */
#define ORBIT_ERR_EXTENT (-2)   /* zero beam extent (SpaceChargeCalc2p5D.cc:131-143) */
#define ORBIT_ERR_GRID (-3)     /* grid too small (Grid2D.cc:40-51, Grid1D.cc:70-82) */
#define ORBIT_ERR_CUDA (-4)     /* CUDA runtime error */
#define ORBIT_ERR_NAN (-5)      /* non-finite coordinate met by the extrema scan */
#define ORBIT_ERR_DEVICE (-6)   /* device-side check failed (range check, bounded barrier wait ran out) */
#define ORBIT_ERR_NOMEM (-8)    /* device allocation failed */
#define ORBIT_ERR_UNSUPPORTED (-9)

/* Copies the calling thread's last error message (NUL terminated) into buf.
 * Returns the message length. */
int orbit_last_error(char* buf, int len);

/* Library version string, e.g. "orbit_gb300 0.1 sm_103a". */
const char* orbit_version(void);

/* Measures this GPU's FP64 FMA throughput (TFLOP/s, independent DFMA
 * chains) and streaming copy bandwidth (GB/s, read + write), the roofs the
 * benchmark reports against.  No counterpart in the reference. */
int orbit_device_peaks(double* fp64_tflops, double* copy_gbs);
/* Binary64 multiply rates in G multiplies/s over all SMs: on the FP64 pipe
 * alone, on the integer pipes alone (the library's correctly rounded
 * integer multiply) and half on each; no counterpart in the reference. */
int orbit_device_mul_rates(double* fp64_gmul, double* int_gmul, double* mixed_gmul);
/* Checks the integer-pipe binary64 multiply, add, fused multiply-add,
 * x 2^+-1 and the double-to-float and float-to-double conversions against
 * the hardware instructions on n generated cases (random normal operands
 * over several exponent spreads, cancellations, rounding ties, zeros and
 * random bit patterns); mismatches[0..5] receives the number of results
 * whose bits differ, per operation.  No counterpart in the reference. */
int orbit_softf64_check(long long n, unsigned long long seed, long long* mismatches);

/* ------------------------------------------------------------------ */
/* Bunch: device-resident SoA macroparticle container                 */
/* replaces Bunch (src/orbit/Bunch.hh:60-136, AoS double[6] rows) and  */
/* SyncPart kinematics (src/orbit/SyncPart.cc:236-306)                 */
/* ------------------------------------------------------------------ */
typedef struct orbit_bunch orbit_bunch_t;

/* Reference-particle data the maps and the SC kick read. `time` is advanced
 * by drift/quad1/bend1 exactly as SyncPart::setTime is in teapotbase.cc:164-165,
 * 638-642, 1109-1113. */
typedef struct {
  double beta, gamma, momentum, mass, charge, classical_radius, macrosize, time;
} orbit_sync_t;

int orbit_bunch_create(orbit_bunch_t** out, int capacity);
int orbit_bunch_destroy(orbit_bunch_t* b);
/* Host SoA -> device: soa[c] points at n doubles for c = x,xp,y,yp,z,dE. */
int orbit_bunch_upload(orbit_bunch_t* b, const double* const* soa, int n);
/* Device -> host, same layout; waits for pending work. */
int orbit_bunch_download(orbit_bunch_t* b, double* const* soa);
/* Device SoA -> device: for callers that already hold device arrays. */
int orbit_bunch_upload_device(orbit_bunch_t* b, const double* const* dev_soa, int n);
int orbit_bunch_size(const orbit_bunch_t* b, int* n);
int orbit_bunch_set_sync(orbit_bunch_t* b, const orbit_sync_t* s);
int orbit_bunch_get_sync(const orbit_bunch_t* b, orbit_sync_t* s);
/* Per-particle "macrosize" attribute (Grid2D.cc:123-131); NULL removes it. */
int orbit_bunch_set_macrosizes(orbit_bunch_t* b, const double* m, int n);
/* The six device coordinate arrays (valid until the next upload/resize). */
int orbit_bunch_device_coords(orbit_bunch_t* b, double** dev_soa);
/* Waits for the bunch's stream and reports device-side errors. */
int orbit_bunch_sync(orbit_bunch_t* b);
/* The bunch's CUDA stream as an opaque pointer (cudaStream_t). */
int orbit_bunch_stream(orbit_bunch_t* b, void** stream);

/* ------------------------------------------------------------------ */
/* SpaceChargeCalc2p5D (src/spacecharge/SpaceChargeCalc2p5D.cc:25-234) */
/* ------------------------------------------------------------------ */
typedef struct orbit_sc2p5d orbit_sc2p5d_t;

#define ORBIT_FORM_PLAIN 0   /* FP64 throughout: the drop-in */
#define ORBIT_FORM_FP32 1    /* deposit/FFT/gradient FP32, coordinates and kick FP64 */

/* SpaceChargeCalc2p5D(xSize, ySize, zSize[, xy_ratio]); xy_ratio <= 0 means
 * the 3-argument constructor (wrap_spacechargecalc2p5d.cc:38-52). */
int orbit_sc2p5d_create(orbit_sc2p5d_t** out, int nx, int ny, int nz, double xy_ratio, int form);
int orbit_sc2p5d_destroy(orbit_sc2p5d_t* c);
/* trackBunch(bunch, length) without a boundary (SpaceChargeCalc2p5D.cc:77-120).
 * Enqueued on the bunch's stream. */
int orbit_sc2p5d_track(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length);

#define ORBIT_GRID_RHO 0
#define ORBIT_GRID_PHI 1
#define ORBIT_GRID_LONG 2
#define ORBIT_GRID_LONG_DERIV 3 /* 2.5Drb only: getLongDerivativeGrid */
/* getRhoGrid / getPhiGrid (nx*ny, row-major [ix][iy]) and getLongGrid (nz)
 * copied to host (wrap_spacechargecalc2p5d.cc:55-115).  Waits for the last
 * stream the calculator ran on. */
int orbit_sc2p5d_get_grid(orbit_sc2p5d_t* c, int which, double* host_out);
/* lim = {xmin,xmax,ymin,ymax,zmin,zmax,dx,dy,dz,xy_ratio,total_macrosize} */
int orbit_sc2p5d_get_limits(orbit_sc2p5d_t* c, double* lim);
int orbit_sc2p5d_get_sizes(const orbit_sc2p5d_t* c, int* nx, int* ny, int* nz, int* form);
/* The Green rebuild and the convolution of each kick (forward rows with the
 * line-density finalization, columns with the Green multiply, backward
 * rows) as one cooperative launch with two grid-wide barriers (on = 1, the
 * default where the device supports cooperative launches), or as separate
 * kernels (on = 0; always for SpaceChargeCalc2p5Drb).  *active (optional)
 * receives whether the fused launch will run.  Applies to kicks enqueued
 * afterwards: a program keeps the form its graph was recorded with.  The
 * same results either way.  No counterpart in the reference (the solve of
 * PoissonSolverFFT2D.cc:174-256). */
int orbit_sc2p5d_set_fused_conv(orbit_sc2p5d_t* c, int on, int* active);
/* The fused convolution's barrier waits: the limit in polls (>= 1; default
 * 2^20, about 0.1 s), and a block withheld from the first barrier (-1:
 * none), a test hook with which the other blocks' waits run out: they
 * return, and the next status check of the bunch reports ORBIT_ERR_DEVICE. */
int orbit_sc2p5d_set_conv_wait(orbit_sc2p5d_t* c, long long polls, int withhold);
/* ---- bunch diagnostics on the device (src/orbit/BunchDiagnostics) ---- */
/* BunchTwissAnalysis::analyzeBunch (BunchTwissAnalysis.cc:49-140): out[29] =
 * {count, total macrosize, <c_i> [6], <c_i c_j> for i >= j [21, row i holds
 * j = 0..i]}, macrosize-weighted with per-particle macrosizes; the
 * coordinates stay on the device.  Waits for the bunch's stream. */
int orbit_bunch_moments(orbit_bunch_t* b, double* out);
/* BunchTuneAnalysis::analyzeBunch (BunchTuneAnalysis.cc:36-108) with
 * twiss = {betax, alphax, etax, etapx, betay, alphay} and etot = kinetic
 * energy + mass: per-particle phases, tunes and actions kept on the device
 * (zero before the first call, as the attribute the reference adds).
 * Enqueued on the bunch's stream; the first call allocates. */
int orbit_bunch_tune_analysis(orbit_bunch_t* b, const double* twiss, double etot);
/* BunchTwissAnalysis::computeBunchMoments (BunchTwissAnalysis.cc:146-340)
 * summed on the device: out[(order+1)^2] = the moment table getBunchMoment
 * (i, j) reads (row i: power of x), with the reference's recurrences,
 * normalisation and fixed cells; params = {D, E_kin + mass, beta^2, xAvg,
 * yAvg, xbetaterm, ybetaterm} from analyzeBunch's getters (D = 0 without the
 * dispersion term).  2 <= order <= 16.  Waits for the bunch's stream. */
int orbit_bunch_xy_moments(orbit_bunch_t* b, int order, const double* params, double* out);
/* The six attribute rows {xLastPhase, yLastPhase, xLastTune, yLastTune,
 * xAction, yAction}, each of n values, to or from the host. */
int orbit_bunch_phase_get(orbit_bunch_t* b, double* host);
int orbit_bunch_phase_set(orbit_bunch_t* b, const double* host);

/* ---- conducting boundaries (Boundary2D: src/spacecharge/BaseBoundary2D.cc,
 * ShapedBoundary2D.cc, wrap_boundary2d.cc) ---- */
typedef struct orbit_boundary orbit_boundary_t;
#define ORBIT_SHAPE_POINTS 0    /* points given with orbit_boundary_set_point */
#define ORBIT_SHAPE_CIRCLE 1
#define ORBIT_SHAPE_ELLIPSE 2
#define ORBIT_SHAPE_RECTANGLE 3
/* Boundary2D(nPoints, nModes): points set one by one, then initialized
 * (BaseBoundary2D.cc:21-97, 190-229).  2*nModes+1 < nPoints; at most 63
 * modes and 4096 points. */
int orbit_boundary_create(orbit_boundary_t** out, int n_points, int n_modes);
/* Boundary2D(nPoints, nModes, shape, xDim, yDim): circle of diameter xDim
 * (xDim == yDim), ellipse with axes xDim, yDim, rectangle xDim x yDim; the
 * number of points is rounded down to a multiple of 4; initialized
 * (ShapedBoundary2D.cc:18-145). */
int orbit_boundary_create_shape(orbit_boundary_t** out, int n_points, int n_modes, int shape, double xdim,
                                double ydim);
int orbit_boundary_destroy(orbit_boundary_t* b);
/* setBoundaryPoint / initialize / getBoundaryPoint (BaseBoundary2D.cc:154-229) */
int orbit_boundary_set_point(orbit_boundary_t* b, int i, double x, double y);
int orbit_boundary_initialize(orbit_boundary_t* b);
int orbit_boundary_get_point(const orbit_boundary_t* b, int i, double* x, double* y);
/* n_points, n_modes, shape (ORBIT_SHAPE_*), lim = {xmin, xmax, ymin, ymax}, initialized */
int orbit_boundary_info(const orbit_boundary_t* b, int* n_points, int* n_modes, int* shape, double* lim,
                        int* initialized);
/* isInside: 1 inside, -1 outside (ShapedBoundary2D.cc:284-304) */
int orbit_boundary_is_inside(const orbit_boundary_t* b, double x, double y);
/* The least-squares matrix ((2 n_modes + 1) x n_points, row-major) and the
 * normalising radius, for addBoundaryPotential on host grids. */
int orbit_boundary_lsq(const orbit_boundary_t* b, double* out);
int orbit_boundary_rnorm(const orbit_boundary_t* b, double* rnorm);
/* SpaceChargeCalc2p5D::trackBunch(bunch, length, boundary)
 * (SpaceChargeCalc2p5D.cc:77-234): grid on the boundary's extents, the
 * boundary potential subtracted from phi, particles outside the boundary
 * not kicked.  Enqueued on the bunch's stream. */
int orbit_sc2p5d_track_boundary(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, const orbit_boundary_t* bnd);

/* SpaceChargeCalc2p5Drb(xSize, ySize, zSize[, xy_ratio]), plain FP64 form
 * (src/spacecharge/wrap_spacechargecalc2p5d_rb.cc:37-50): the 2.5D kick
 * plus a longitudinal kick of dE from the smoothed derivative of the line
 * density and a pipe radius; the grid keeps the calculator's ratio and the
 * Poisson solver grid is never reshaped (SpaceChargeCalc2p5Drb.cc:107-306).
 * Destroyed with orbit_sc2p5d_destroy; grids, limits and counters through
 * the orbit_sc2p5d_* calls (lim[10] is the rho-grid sum the kick divides
 * by), the derivative grid as ORBIT_GRID_LONG_DERIV. */
int orbit_sc2p5drb_create(orbit_sc2p5d_t** out, int nx, int ny, int nz, double xy_ratio);
/* trackBunch(bunch, length, pipe_radius) (SpaceChargeCalc2p5Drb.cc:107-155) */
int orbit_sc2p5drb_track(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, double pipe_radius);
/* setLongAveragingPointsN / getLongAveragingPointsN (:309-318) */
int orbit_sc2p5drb_set_long_avg(orbit_sc2p5d_t* c, int n);
int orbit_sc2p5drb_get_long_avg(const orbit_sc2p5d_t* c, int* n);
/* No counterpart in the reference (its values stay local to trackBunch):
 * abx = {a_bunch, x_center, y_center} of the last kick. */
int orbit_sc2p5drb_beam(orbit_sc2p5d_t* c, double* abx);

/* No counterpart in the reference (diagnostic).  Kicks solved and Green
 * spectra rebuilt (PoissonSolverFFT2D::setGridXY followed by the Green
 * transform, PoissonSolverFFT2D.cc:103-172) since the calculator was
 * created.  Waits for the last stream the calculator ran on. */
int orbit_sc2p5d_counters(orbit_sc2p5d_t* c, long long* kicks, long long* green_rebuilds);
/* Grid2D::calcGradient + Grid1D::getValue at n host points with the current
 * grids (Grid2D.cc:212-256, Grid1D.cc:191-211). */
int orbit_sc2p5d_fields(orbit_sc2p5d_t* c, int n, const double* x, const double* y, const double* z,
                        double* ex, double* ey, double* lam);

/* No counterpart in the reference.  One trackBunch of a freshly constructed
 * plain FP64 calculator (the result of orbit_sc2p5d_create + _track on the
 * same inputs) that allocates nothing: for callers that cannot call
 * cudaMalloc -- code running inside another framework's memory pool or
 * under a fixed memory budget, loops that must not allocate after start-up,
 * hosts that cannot afford the device synchronisation an allocation or free
 * can cause.  All scratch (solver state, grids, FFT spectra, Green
 * function) lives in one static device array of about 2.1 MB that every GPU
 * loading the library holds until the process exits; grids are limited to
 * nx, ny <= 128 and nz <= 256 (larger sizes return ORBIT_ERR_UNSUPPORTED).
 * dev_coords: device SoA, coordinate c (x, xp, y, yp, z, dE) at
 * dev_coords + c*stride, stride >= n; xp and yp are updated in place.
 * stream: a cudaStream_t (NULL = default stream).  Every call copies the
 * fresh calculator's state from host memory into the array and waits for
 * the stream before it returns.  The first call on a device looks up the
 * array's device address (once per device, under a lock).  Calls share the
 * array: calls that overlap on the GPU race. */
int orbit_sc2p5d_track_static(double* dev_coords, int n, int stride, int nx, int ny, int nz, double xy_ratio,
                              double length, const orbit_sync_t* sync, void* stream);

/* ------------------------------------------------------------------ */
/* teapot_base maps (src/teapot/teapotbase.cc; Python names in         */
/* src/teapot/wrap_teapotbase.cc:488-512).  The useCharge argument of  */
/* the reference is accepted by the Python layer and ignored there too */
/* ------------------------------------------------------------------ */
int orbit_tpb_rotatexy(orbit_bunch_t* b, double angle);
int orbit_tpb_drift(orbit_bunch_t* b, double length);
int orbit_tpb_wrapbunch(orbit_bunch_t* b, double length);
int orbit_tpb_kick(orbit_bunch_t* b, double kx, double ky, double kE);
int orbit_tpb_multp(orbit_bunch_t* b, int pole, double kl, int skew);
int orbit_tpb_multpfringeIN(orbit_bunch_t* b, int pole, double kl, int skew);
int orbit_tpb_multpfringeOUT(orbit_bunch_t* b, int pole, double kl, int skew);
int orbit_tpb_quad1(orbit_bunch_t* b, double length, double kq);
int orbit_tpb_quad2(orbit_bunch_t* b, double length);
int orbit_tpb_quadfringeIN(orbit_bunch_t* b, double kq);
int orbit_tpb_quadfringeOUT(orbit_bunch_t* b, double kq);
int orbit_tpb_wedgerotate(orbit_bunch_t* b, double e, int frinout);
int orbit_tpb_wedgedrift(orbit_bunch_t* b, double e, int inout);
int orbit_tpb_wedgebend(orbit_bunch_t* b, double e, int inout, double rho, int nsteps);
int orbit_tpb_bend1(orbit_bunch_t* b, double length, double th);
int orbit_tpb_bend2(orbit_bunch_t* b, double length);
int orbit_tpb_bend3(orbit_bunch_t* b, double th);
int orbit_tpb_bend4(orbit_bunch_t* b, double th);
int orbit_tpb_bendfringeIN(orbit_bunch_t* b, double rho);
int orbit_tpb_bendfringeOUT(orbit_bunch_t* b, double rho);

/* ------------------------------------------------------------------ */
/* Lattice programs: a recorded node sequence replayed on the device   */
/* (AccNode.trackActions order, py/orbit/lattice/AccNode.py:302-350)   */
/* ------------------------------------------------------------------ */
#define ORBIT_OP_DRIFT 1      /* d0 = length */
#define ORBIT_OP_QUAD1 2      /* d0 = length, d1 = kq */
#define ORBIT_OP_QUAD2 3      /* d0 = length */
#define ORBIT_OP_QFRIN 4      /* d0 = kq */
#define ORBIT_OP_QFROUT 5     /* d0 = kq */
#define ORBIT_OP_BEND1 6      /* d0 = length, d1 = theta */
#define ORBIT_OP_BEND2 7      /* d0 = length */
#define ORBIT_OP_BEND3 8      /* d0 = theta */
#define ORBIT_OP_BEND4 9      /* d0 = theta */
#define ORBIT_OP_BFRIN 10     /* d0 = rho */
#define ORBIT_OP_BFROUT 11    /* d0 = rho */
#define ORBIT_OP_MULTP 12     /* i0 = pole, i1 = skew, d0 = kl */
#define ORBIT_OP_MPFRIN 13    /* i0 = pole, i1 = skew, d0 = kl */
#define ORBIT_OP_MPFROUT 14   /* i0 = pole, i1 = skew, d0 = kl */
#define ORBIT_OP_ROTXY 15     /* d0 = angle */
#define ORBIT_OP_WRAP 16      /* d0 = ring length */
#define ORBIT_OP_KICK 17      /* d0 = kx, d1 = ky, d2 = kE */
#define ORBIT_OP_WEDGEROT 18  /* d0 = e, i0 = frinout */
#define ORBIT_OP_WEDGEDRIFT 19 /* d0 = e, i0 = inout */
#define ORBIT_OP_WEDGEBEND 20 /* d0 = e, i0 = inout, d1 = rho, i1 = nsteps */
#define ORBIT_OP_SC 32        /* i0 = calculator index, d0 = sc length, d1 = pipe radius (2.5Drb calculators),
                                 i1 = 1 + boundary index (0: none; orbit_program_set_boundaries) */

typedef struct {
  int32_t code, i0, i1, i2;
  double d[6];
} orbit_op_t;

typedef struct orbit_program orbit_program_t;

/* Compiles ops into fused device passes: all maps between two SC kicks run
 * in one particle pass together with the previous kick and the next extrema
 * scan.  calcs[i] serves ORBIT_OP_SC ops with i0 == i. */
int orbit_program_create(orbit_program_t** out, const orbit_op_t* ops, int nops,
                         orbit_sc2p5d_t* const* calcs, int ncalcs);
int orbit_program_destroy(orbit_program_t* p);
/* Boundaries for SC ops with i1 = 1 + index (the boundary passed to the
 * node's trackBunch); the program keeps the pointers, which must outlive it. */
int orbit_program_set_boundaries(orbit_program_t* p, orbit_boundary_t* const* bnds, int n);
/* Runs the program `turns` times on the bunch (captured once per bunch as a
 * CUDA graph and replayed) and advances the bunch's sync time. Waits for
 * completion and reports device errors. */
int orbit_program_run(orbit_program_t* p, orbit_bunch_t* b, int turns);
/* As orbit_program_run, but only enqueues the graphs on the bunch's stream;
 * orbit_bunch_sync() waits and reports device errors. */
int orbit_program_enqueue(orbit_program_t* p, orbit_bunch_t* b, int turns);
/* Number of kernel launches one pass of the program issues. */
int orbit_program_launches(const orbit_program_t* p, int* launches);
/* Runs one turn without graph capture, timing every launch with CUDA events
 * on the bunch's stream; per kernel kind k < *nkinds: names[32*k] (NUL
 * terminated), total milliseconds and launch count.  Advances the bunch like
 * orbit_program_run(p, b, 1). */
int orbit_program_profile(orbit_program_t* p, orbit_bunch_t* b, int max_kinds, char* names, double* total_ms,
                          int* launches, int* nkinds);

/* ---- batched tracking of many bunches (scans) ----
 * No single counterpart in the reference: a scan there is a Python loop
 * over bunches, each tracked by its own lattice (AccLattice.trackBunch,
 * py/orbit/lattice/AccLattice.py:243-255).  Here member i is programs[i]
 * tracking bunches[i]; all members advance together, one kernel launch per
 * stage per grid class, each class on its own stream in one CUDA graph per
 * turn.  The programs must share one node structure (same op codes, SC
 * nodes in the same places), each use one plain-form 2.5D calculator of
 * its own (no boundary, no 2.5Drb), and every bunch needs >= 2 particles.
 * The first run times candidate launch shapes per class (autotuner); its
 * choice can be read and fixed with orbit_batch_class / _set_tuning. */
typedef struct orbit_batch orbit_batch_t;
int orbit_batch_create(orbit_batch_t** out, orbit_program_t* const* programs, orbit_bunch_t* const* bunches, int n);
int orbit_batch_destroy(orbit_batch_t* b);
/* Enqueues `turns` turns of every member and advances each bunch's sync
 * time; orbit_batch_sync waits and reports the first device error of any
 * member.  orbit_batch_run = enqueue + sync. */
int orbit_batch_enqueue(orbit_batch_t* b, int turns);
int orbit_batch_sync(orbit_batch_t* b);
int orbit_batch_run(orbit_batch_t* b, int turns);
/* Number of grid classes, and kernel launches per captured turn. */
int orbit_batch_info(const orbit_batch_t* b, int* n_classes, int* launches_per_turn);
/* The cudaStream_t the batch's turns are enqueued on (as void*). */
int orbit_batch_stream(orbit_batch_t* b, void** stream);
/* One turn without graph capture, the classes one after another on the
 * batch stream, every launch timed by CUDA events (as
 * orbit_program_profile); advances the members like orbit_batch_run(b, 1).
 * Needs a first run (the autotuned shapes). */
int orbit_batch_profile(orbit_batch_t* b, int max_kinds, char* names, double* total_ms, int* launches,
                        int* nkinds);
/* Class cls: grid[3] = nx, ny, nz; members; tuning[6] = deposit threads,
 * deposit particles per block, pass threads, pass particles per block, FFT
 * schedule (1: radix-2 stages, 0: radix-4 stages), tuned (0/1). */
int orbit_batch_class(const orbit_batch_t* b, int cls, int* grid, int* members, int* tuning);
/* Fixes class cls's shapes (tuning[0..4], one of the candidates); no
 * autotuning runs afterwards. */
int orbit_batch_set_tuning(orbit_batch_t* b, int cls, const int* tuning);

/* ---- NVTX ranges (no counterpart in the reference) ----
 * A named NVTX range pushed and popped by the host layer: with
 * ORBIT_NVTX=1 in the environment the Python lattice walk
 * (AccNode.trackActions) opens one per node, so Nsight Systems timelines and
 * ncu --nvtx filters show the lattice structure; the C entry points
 * (teapot_base maps, trackBunch, program and batch turns) always open their
 * own.  Without an attached tool a range costs a branch. */
int orbit_nvtx_push(const char* name);
int orbit_nvtx_pop(void);

/* ---- learned denoising closure (no counterpart in the reference) ----
 * A 4-level convolutional encoder-decoder (channels 16-64, 302,561
 * parameters; BF16 convolution weights, FP32 activations and accumulation)
 * mapping the normalised charge density of a few-macroparticle deposit to
 * the density of a deposit with many more macroparticles on the same grid.
 * Images are NCHW FP32 device arrays of h x w (multiples of 8). */
typedef struct orbit_denoiser orbit_denoiser_t;
/* Training beams (transverse positions): kind 0 Gaussian with rms sx, sy;
 * 1 KV projection (uniform ellipse, semi-axes 2 sx, 2 sy); 2 waterbag
 * projection (shadow of a uniform 4D ball, semi-axes sqrt(6) sx, sqrt(6) sy).
 * Particle i depends only on (seed, i).  orbit_beam_sample writes n
 * positions to device arrays; orbit_beam_deposit deposits n particles of unit
 * weight (Grid2D's 9-point weights, FP32) on the node grid
 * lim = {xmin, xmax, ymin, ymax} of nx x ny into dev_grid (cleared first),
 * dropping particles outside it.  Both wait for completion. */
int orbit_beam_sample(double* dev_x, double* dev_y, int n, int kind, double sx, double sy, unsigned long long seed);
int orbit_beam_deposit(float* dev_grid, int nx, int ny, const double* lim, long long n, int kind, double sx,
                       double sy, unsigned long long seed);
/* The same deposit of n given positions (device arrays), e.g. a tracked
 * bunch's x and y (waits). */
int orbit_grid_deposit(float* dev_grid, int nx, int ny, const double* lim, const double* dev_x, const double* dev_y,
                       long long n);
int orbit_denoiser_create(orbit_denoiser_t** out, int max_batch, int h, int w, unsigned long long seed);
int orbit_denoiser_destroy(orbit_denoiser_t* d);
int orbit_denoiser_info(const orbit_denoiser_t* d, int* nparam, int* h, int* w, int* max_batch);
/* FP32 parameters (the master copy Adam updates) to/from host memory;
 * setting them resets the Adam moments. */
int orbit_denoiser_get_params(orbit_denoiser_t* d, float* host);
int orbit_denoiser_set_params(orbit_denoiser_t* d, const float* host);
/* dev_out = network(dev_in) for nb images on `stream` (NULL: the
 * denoiser's own stream, a blocking stream ordered with the legacy default
 * stream). */
int orbit_denoiser_forward(orbit_denoiser_t* d, const float* dev_in, float* dev_out, int nb, void* stream);
/* Single-image forwards (the kick's closure) run their 3x3 layers on the
 * tensor cores (tcgen05, TF32 operands, FP32 accumulation) unless `on` is
 * 0; batches and training use the CUDA-core layers. */
int orbit_denoiser_set_tensor_cores(orbit_denoiser_t* d, int on);
/* Batches (training steps, gradients and batched forwards) run their 3x3
 * layers' forward, data gradient and weight gradient on the tensor cores
 * when `on` (TF32 operands, FP32 accumulation in tensor memory).  Off by
 * default.  A synchronised step that finds a tensor-core
 * wait gave up returns ORBIT_ERR_DEVICE and the network falls back to the
 * CUDA cores (see orbit_denoiser_tensor_status). */
int orbit_denoiser_set_batch_tensor_cores(orbit_denoiser_t* d, int on);
/* Synchronises; *on = whether single-image forwards use the tensor cores
 * now; *err = the error bits of the tensor-core layers since the last call
 * (then reset): 1 = a bounded wait on an MMA gave up, 2 = the MMA had not
 * completed after a second wait either and its tensor memory was released
 * all the same.  After any error this network runs its single-image
 * forwards on the CUDA-core layers; after bit 2 no network of the process
 * uses the tensor cores again.  A learned closure whose network reported
 * an error falls back to the plain deposit. */
int orbit_denoiser_tensor_status(orbit_denoiser_t* d, int* on, int* err);
/* Training loss (no counterpart in the reference): levels = 0, the mean
 * squared error of the output against the target (the default); levels L
 * in 1..7, the multi-scale loss sum_{s=0..L} weights[s] mean((P^s y -
 * P^s t)^2) with P the 2x2 average pooling (h and w divisible by 2^L).
 * Weights 4^s make it a stand-in for the force error (the squared error of
 * the field of y - t), which weights an error of wavenumber k by 1/k^2:
 * pooling s times keeps the modes below k_max / 2^s.  Waits for the device. */
int orbit_denoiser_set_loss(orbit_denoiser_t* d, int levels, const float* weights);
/* The tensor-core layers' bounded waits: each gives up after `cycles` SM
 * clock cycles (default 2e9, about one second).  withhold_mma != 0 (for
 * testing the failure path only) issues no MMA, so every wait runs out
 * with nothing in flight.  No counterpart in the reference. */
int orbit_denoiser_set_wait_limit(orbit_denoiser_t* d, long long cycles, int withhold_mma);
/* One Adam step (learning rate lr) on the mean squared error of nb pairs,
 * on `stream` (NULL: the denoiser's own stream; pass the stream that wrote
 * the inputs); *loss (if not NULL) receives the loss before the step
 * (waits). */
int orbit_denoiser_train_step(orbit_denoiser_t* d, const float* dev_in, const float* dev_target, int nb, float lr,
                              float* loss, void* stream);
/* Loss, parameter gradients (host, nparam floats) and, if dev_out is not
 * NULL, the network output for nb pairs, without an update (waits). */
int orbit_denoiser_gradients(orbit_denoiser_t* d, const float* dev_in, const float* dev_target, int nb, float* grads,
                             float* loss, float* dev_out, void* stream);
/* The learned closure of a 2.5D calculator, plain or FP32 form (nx x ny =
 * the network's image size; bunches with a uniform macrosize; not the
 * 2.5Drb calculator, not with a boundary): each kick the network
 * denoises the deposit (clamped at zero, rescaled to the deposit's total
 * charge) before the FFT solve; every check_every-th kick the raw deposit is
 * solved as well and, if the relative rms difference of the two potentials
 * exceeds `bound`, the calculator falls back to the plain deposit until
 * orbit_sc2p5d_denoiser_reset.  dn NULL removes the closure.  A denoiser
 * serves one calculator at a time (its buffers are shared). */
int orbit_sc2p5d_set_denoiser(orbit_sc2p5d_t* c, orbit_denoiser_t* dn, int check_every, double bound);
int orbit_sc2p5d_denoiser_state(orbit_sc2p5d_t* c, int* fallback, long long* checks, long long* trips,
                                double* last_err);
int orbit_sc2p5d_denoiser_reset(orbit_sc2p5d_t* c);

#ifdef __cplusplus
}
#endif

#endif
