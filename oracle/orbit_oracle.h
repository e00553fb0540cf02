/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the PyORBIT 2.5D space-charge + TEAPOT hot path,
 * used as the CPU reference of the CUDA path's tests and as the timed CPU baseline
 * ("port").  Every function cites the reference file:line it restates.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference legs may load it.  It is never linked into the product library.
 *
 * Coordinates are SoA: soa[c*n + i], c = 0..5 -> x, xp, y, yp, z, dE.
 */
#ifndef ORBIT_ORACLE_H
#define ORBIT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference-particle kinematics needed by the maps and the SC kick
 * (src/orbit/SyncPart.cc:236-306). */
typedef struct {
  double beta, gamma, momentum, mass, charge, classical_radius, macrosize;
  double time;
} oracle_sync_t;

typedef struct oracle_sc oracle_sc_t;

/* SpaceChargeCalc2p5D(xSize, ySize, zSize[, xy_ratio]) -- xy_ratio <= 0
 * selects the 3-argument constructor (ratio 1.0), as
 * src/spacecharge/wrap_spacechargecalc2p5d.cc:38-52. */
oracle_sc_t* oracle_sc_new(int nx, int ny, int nz, double xy_ratio);
void oracle_sc_free(oracle_sc_t* sc);

/* SpaceChargeCalc2p5D::trackBunch(bunch, length, NULL)
 * (src/spacecharge/SpaceChargeCalc2p5D.cc:77-234).  `msize` is an optional
 * per-particle macrosize array (NULL -> sync->macrosize for every particle).
 * nthreads > 1 splits the particles into that many slices with private grids
 * summed afterwards, the same decomposition the reference uses across MPI
 * ranks (Grid2D.cc:443-477, Grid1D.cc:762-798, BunchExtremaCalculator.cc:68).
 * Returns 0, or -2 for a zero-extent bunch (the reference aborts there,
 * SpaceChargeCalc2p5D.cc:131-143). */
int oracle_sc_track(oracle_sc_t* sc, double* soa, int n, const double* msize,
                    const oracle_sync_t* sync, double length, int nthreads);

/* Copy out rho[nx*ny], phi[nx*ny], zgrid[nz] and
 * lim = {xmin,xmax,ymin,ymax,zmin,zmax,dx,dy,dz,xy_ratio,total_macrosize}. */
void oracle_sc_grids(const oracle_sc_t* sc, double* rho, double* phi, double* zg, double* lim);

/* Evaluate the SC field at particles with the current grids:
 * ex, ey = Grid2D::calcGradient (Grid2D.cc:212-256), lam = Grid1D::getValue
 * (Grid1D.cc:191-211). */
void oracle_sc_fields(const oracle_sc_t* sc, int n, const double* x, const double* y,
                      const double* z, double* ex, double* ey, double* lam);

/* SpaceChargeCalc2p5Drb(xSize, ySize, zSize[, xy_ratio]) -- 2.5D transverse
 * kick plus the longitudinal kick from the smoothed derivative of the line
 * density and a pipe radius (src/spacecharge/SpaceChargeCalc2p5Drb.cc).
 * Freed with oracle_sc_free; grids read with oracle_sc_grids (lim[10] is
 * the rho-grid sum the kick uses). */
oracle_sc_t* oracle_scrb_new(int nx, int ny, int nz, double xy_ratio);
void oracle_scrb_set_long_avg(oracle_sc_t* sc, int n);
int oracle_scrb_track(oracle_sc_t* sc, double* soa, int n, const double* msize, const oracle_sync_t* sync,
                      double length, double pipe_radius, int nthreads);
/* derivative grid [nz]; abx = {a_bunch, x_center, y_center} */
void oracle_scrb_extra(const oracle_sc_t* sc, double* zderiv, double* abx);

/* Conducting boundary: BaseBoundary2D(nPoints, nModes) with points set by
 * the caller then initialized, or ShapedBoundary2D(nPoints, nModes, shape,
 * xDim, yDim) with shape 1 circle, 2 ellipse, 3 rectangle
 * (src/spacecharge/BaseBoundary2D.cc, ShapedBoundary2D.cc). */
typedef struct oracle_bnd oracle_bnd_t;
oracle_bnd_t* oracle_bnd_new(int np, int nm);
oracle_bnd_t* oracle_bnd_new_shape(int np, int nm, int shape, double xdim, double ydim);
void oracle_bnd_free(oracle_bnd_t* b);
void oracle_bnd_set_point(oracle_bnd_t* b, int i, double x, double y);
int oracle_bnd_initialize(oracle_bnd_t* b);
int oracle_bnd_is_inside(const oracle_bnd_t* b, double x, double y);
void oracle_bnd_get(const oracle_bnd_t* b, double* head, double* bx, double* by, double* lsq);
/* SpaceChargeCalc2p5D::trackBunch(bunch, length, boundary): grid on the
 * boundary's extents, boundary potential subtracted, particles outside the
 * boundary not kicked.  Returns -3 when the boundary does not fit the grid. */
int oracle_sc_track_bnd(oracle_sc_t* s, double* soa, int n, const double* msize, const oracle_sync_t* sync,
                        double length, oracle_bnd_t* b, int nthreads);

/* ---- bunch diagnostics (src/orbit/BunchDiagnostics) ---- */
/* BunchTwissAnalysis::analyzeBunch: out[29] = {count, total macrosize,
 * <c_i> [6], <c_i c_j> i >= j [21]}. */
void oracle_twiss_moments(const double* soa, int n, const double* msize, double* out);
/* BunchTuneAnalysis::analyzeBunch: ph = 6 SoA rows of n {xLastPhase,
 * yLastPhase, xLastTune, yLastTune, xAction, yAction}, updated in place. */
void oracle_tune_analysis(const double* soa, int n, double beta, double etot, const double* twiss, double* ph);

/* ---- TEAPOT maps (src/teapot/teapotbase.cc) ---- */
void oracle_rotatexy(double* soa, int n, double angle);
void oracle_drift(double* soa, int n, oracle_sync_t* s, double length);
void oracle_wrapbunch(double* soa, int n, double length);
void oracle_kick(double* soa, int n, double kx, double ky, double kE);
void oracle_multp(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew);
void oracle_multpfringeIN(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew);
void oracle_multpfringeOUT(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew);
void oracle_quad1(double* soa, int n, oracle_sync_t* s, double length, double kq);
void oracle_quad2(double* soa, int n, const oracle_sync_t* s, double length);
void oracle_quadfringeIN(double* soa, int n, const oracle_sync_t* s, double kq);
void oracle_quadfringeOUT(double* soa, int n, const oracle_sync_t* s, double kq);
void oracle_wedgerotate(double* soa, int n, const oracle_sync_t* s, double e, int frinout);
void oracle_wedgedrift(double* soa, int n, const oracle_sync_t* s, double e, int inout);
void oracle_wedgebend(double* soa, int n, const oracle_sync_t* s, double e, int inout, double rho, int nsteps);
void oracle_bend1(double* soa, int n, oracle_sync_t* s, double length, double th);
void oracle_bend2(double* soa, int n, const oracle_sync_t* s, double length);
void oracle_bend3(double* soa, int n, const oracle_sync_t* s, double th);
void oracle_bend4(double* soa, int n, const oracle_sync_t* s, double th);
void oracle_bendfringeIN(double* soa, int n, const oracle_sync_t* s, double rho);
void oracle_bendfringeOUT(double* soa, int n, const oracle_sync_t* s, double rho);

/* ---- recorded lattice programs ----
 * An op is {code, i0, i1, i2, d0..d5}; the codes and parameter meanings are
 * shared with the product's program format (include/orbit_gb300.h,
 * ORBIT_OP_*).  SC ops index into `calcs`. */
typedef struct {
  int32_t code, i0, i1, i2;
  double d[6];
} oracle_op_t;

/* Runs ops[0..nops) in order, `turns` times.  Returns 0 or the first
 * non-zero status of an SC op. */
int oracle_run_program(const oracle_op_t* ops, int nops, int turns, double* soa, int n,
                       const double* msize, oracle_sync_t* sync, oracle_sc_t** calcs,
                       int nthreads);

/* rms emittances of (x,xp) and (y,yp) (BunchTwissAnalysis.cc:372-390). */
void oracle_rms_emittance(const double* soa, int n, double* ex, double* ey);

#ifdef __cplusplus
}
#endif

#endif
