// 2.5D space-charge calculator: device state and kernel entry points shared
// by the eager trackBunch path (sc2p5d.cu) and the lattice programs
// (program.cu).
#pragma once

#include "common.cuh"

namespace orbit {

// Device-resident per-calculator state, written by the setup kernel so
// that a whole kick runs without a host round trip (and can be captured in
// a CUDA graph).  Field meanings follow SpaceChargeCalc2p5D::bunchAnalysis
// (src/spacecharge/SpaceChargeCalc2p5D.cc:122-234) and PoissonSolverFFT2D.
struct ScState {
  double xmin, xmax, ymin, ymax, dx, dy, inv_dx, inv_dy;  // rho/phi grid (Grid2D)
  double zmin, zmax, dz, inv_dz;                          // line-density grid (Grid1D)
  double xy_ratio;                                        // calculator's xy_ratio (persists)
  double sxmin, sxmax, symin, symax, sdx, sdy;            // Poisson-solver grid
  double re00;                                            // Re G~[0][0] (PoissonSolverFFT2D.cc:164)
  double scale;                                           // log(dx_solver/dx_rho) (:213)
  double total_m;                                         // sum of the line density (:229-233)
  double inv_qscale;                                      // macrosize per unit of the fixed-point deposit
  int green_dirty;                                        // Green spectrum must be rebuilt
  int skip;                                               // this kick is skipped (zero extent)
  unsigned long long key[6];                              // extrema accumulators (ordered keys)
  unsigned long long phi_absmax;                          // bits of max |phi| (non-negative doubles
  unsigned long long lam_absmax;                          //  order like their bit patterns), max |lambda|
  int dep_k;                                              // fraction bits of the integer deposit (0: FP64 path)
  unsigned ext_count;                                     // blocks done with the extrema scan (last one sets up)
  // 2.5Drb: beam centre, a_bunch^2 and the two pipe-radius terms of the
  // longitudinal kick (SpaceChargeCalc2p5Drb.cc:124-136, 226-254)
  double rb_xc, rb_yc, rb_a2, rb_lin, rb_lout;
  unsigned long long n_kicks, n_green;                    // kicks solved, Green spectra rebuilt
  // learned closure: fallen back to the plain deposit (sticky), the last
  // check's relative rms potential difference, checks and fall-backs
  int dn_fallback;
  double dn_err;
  unsigned long long dn_checks, dn_trips;
  // arrival counters of the fused convolution's two grid-wide barriers,
  // zeroed by every kick's set-up
  unsigned conv_bar[2];
};

// Inside test of a conducting boundary (BaseBoundary2D.cc:144-151,
// ShapedBoundary2D.cc:284-304): type -1 none (every particle is inside),
// 0 the extents of arbitrary points (p = xmin, xmax, ymin, ymax), 1 circle
// (p0 = radius), 2 ellipse (p0, p1 = semi-axes), 3 rectangle (p0, p1 =
// full sides).
struct BndShape {
  int type;
  double p0, p1, p2, p3;
};

__host__ __device__ __forceinline__ bool bnd_inside(const BndShape& b, double x, double y) {
  switch (b.type) {
    case 0: return x > b.p0 && x < b.p1 && y > b.p2 && y < b.p3;
    case 1: return x * x + y * y < b.p0 * b.p0;
    case 2: {
      double xx = x / b.p0, yy = y / b.p1;
      return (xx * xx + yy * yy) < 1.0;
    }
    case 3: return fabs(x / b.p0) < 0.5 && fabs(y / b.p1) < 0.5;
    default: return true;
  }
}

// Arguments of the grid set-up run at the end of the extrema scan.
struct SetupArgs {
  double inv_qscale;  // macrosize per unit of the fixed-point deposit (1 for the fp32 form)
  int nx, ny, nz;
  int rb;             // SpaceChargeCalc2p5Drb set-up: fixed ratio, solver grid never reshaped
  int bnd;            // a conducting boundary fixes the transverse grid to its extents
  double bxmin, bxmax, bymin, bymax;
  cudaGraphConditionalHandle cond;  // inside a graph: the Green-rebuild branch of this kick (0: none)
};

// Units of the plain-form deposit for one bunch: K > 0 (uniform macrosize)
// deposits unit weights in units of 2^-K, else macrosize * S through FP64.
struct DepScales {
  int K;
  double S, inv_q, ms_uniform;
};

struct FftPlan {
  int n;
  int nst;
  int pow2;  // n is a power of two: radix-4 stages and at most one radix-2
  int rad[24];
};

}  // namespace orbit

struct orbit_boundary;
struct orbit_denoiser;

namespace orbit {
// The denoiser's device error flag (tensor-core waits that gave up).
int* dn_error_flag(orbit_denoiser* d);
// Forward of one image in place for the learned closure: the caller writes
// the image into *in and reads the output from *out (the network's own
// input and output activations: no copies); dn_forward_inplace also writes
// *nparts per-block sums of the output clamped at zero into parts.
int dn_closure_io(orbit_denoiser* d, float** in, const float** out, int* nparts);
int dn_forward_inplace(orbit_denoiser* d, cudaStream_t st, double* parts);
// The network's parameter version (bumped by every change) and, before a
// stream capture that runs it, the packing of its tensor-core weights done
// eagerly when a change left them stale (a packing captured into one graph
// would not run where another graph is replayed).
unsigned long long dn_version(const orbit_denoiser* d);
int dn_prepare_capture(orbit_denoiser* d);
constexpr int kDnMaxParts = 4096;  // sums the closure's buffer holds
}  // namespace orbit

struct orbit_sc2p5d {
  int nx = 0, ny = 0, nz = 0, form = 0;
  int nx2 = 0, ny2 = 0, H = 0;   // doubled grid, H = ny2/2 + 1
  double xy_ratio0 = 1.0;
  orbit::ScState* d_st = nullptr;
  unsigned long long* d_rho_q = nullptr;  // fixed-point deposit (both forms)
  unsigned long long* d_z_q = nullptr;
  double* d_rho = nullptr;                // user-visible rho (nx*ny)
  double* d_phi = nullptr;                // user-visible phi (nx*ny)
  double* d_lam = nullptr;                // user-visible line density (nz)
  float* d_phi_f = nullptr;               // fp32-form phi
  float* d_lam_f = nullptr;
  long long* d_phi_fix = nullptr;         // plain form: phi, lambda as scaled 64-bit integers
  long long* d_lam_fix = nullptr;
  void* d_hat = nullptr;                  // nx2 * H complex work spectrum (T = double or float)
  void* d_green = nullptr;                // nx2 * H complex Green spectrum
  double* d_gbuf = nullptr;               // nx2 * ny2 real Green function
  void* d_gscratch = nullptr;             // nx2 * H complex: Green row spectra inside a graph
  void* d_tw_x = nullptr;                 // twiddles for N = nx2
  void* d_tw_y = nullptr;                 // twiddles for N = ny2
  orbit::FftPlan plan_x{}, plan_y{};
  cudaEvent_t done = nullptr;    // recorded after the last work that used the buffers
  bool used = false;
  cudaStream_t aux = nullptr;    // captures the Green-rebuild graph branch
  // branch handle created with the set-up of the next kick while a graph is
  // captured, and the graph it belongs to
  cudaGraphConditionalHandle pending_cond = 0;
  cudaGraph_t pending_graph = nullptr;
  bool smem_deposit = false, smem_kick = false;
  bool band_deposit = false;              // plain form: the grid in row bands (too large for one block)
  // the Green rebuild and the convolution in one cooperative launch (0
  // blocks: the separate kernels), the barrier wait limit in polls and a
  // block withheld from the first barrier (test hook, -1: none)
  bool fused_conv = true;
  int conv_blocks = 0;
  long long conv_wait_polls = 1ll << 20;
  int conv_withhold = -1;
  // SpaceChargeCalc2p5Drb (plain form): longitudinal kick from the smoothed
  // derivative of the line density
  bool rb = false;
  int n_long_avg = 3;
  double* d_lamd = nullptr;               // derivative grid (nz)
  int dep_threads = 512, kick_threads = 512;
  // learned closure (both forms): the network, the check period and bound,
  // the host kick counter, and the output-sum, raw-density and check-solve
  // buffers (the image and the output are the network's own)
  orbit_denoiser* dn = nullptr;
  int dn_every = 10;
  double dn_bound = 0.05;
  long long dn_count = 0;
  double* d_dn_parts = nullptr;  // the network's per-block sums of its clamped output
  double* d_dn_raw = nullptr;
  void* d_dn_hat = nullptr;
  double* d_dn_phi = nullptr;
  orbit::ScState* d_dn_st = nullptr;
  // bumped by every setter that changes what an enqueued kick launches or
  // reads (closure, fused convolution and its waits): lattice programs
  // captured before it are captured again
  unsigned long long cfg_gen = 0;
};

namespace orbit {

// Enqueues one full trackBunch (extrema .. kick) for the bunch on `st`.
// `do_extrema` = false when the extrema keys were already accumulated by a
// fused pass; `do_kick` = false when the kick is deferred to the next fused
// pass.  Returns the number of kernel launches added through *launches.
int sc_enqueue_kick(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, cudaStream_t st,
                    bool do_extrema, bool do_kick, int* launches, double pipe_radius = 0.0,
                    const orbit_boundary* bnd = nullptr);
// Cross-stream ordering of a calculator's buffers: work on stream s waits
// for the last recorded use, then records a new one.
cudaError_t sc_order_before(orbit_sc2p5d_t* c, cudaStream_t s);
cudaError_t sc_mark_used(orbit_sc2p5d_t* c, cudaStream_t s);
DepScales sc_dep_scales(const orbit_sc2p5d_t* c, const orbit_bunch_t* b);
SetupArgs sc_setup_args(const orbit_sc2p5d_t* c, const DepScales& d, const orbit_boundary* bnd = nullptr);
// The boundary's inside test (type -1 for none).
BndShape bnd_shape_of(const orbit_boundary* bnd);
// Subtracts the boundary potential from phi (BaseBoundary2D::addBoundaryPotential)
// on stream s and recomputes max |phi|; returns launches added.
int bnd_enqueue_potential(const orbit_boundary* bnd, orbit_sc2p5d_t* c, cudaStream_t s, int* launches);
// Uploads the boundary's points and least-squares matrix if not yet on the
// device (outside any stream capture).
int bnd_ensure_device(orbit_boundary* bnd);
// While s is being captured into a graph (and the calculator can branch):
// a conditional handle on that graph for the Green rebuild of the kick
// whose set-up is about to be enqueued; with `pending` it is kept for that
// kick's sc_enqueue_kick.  0 otherwise.
cudaGraphConditionalHandle sc_green_cond(orbit_sc2p5d_t* c, cudaStream_t s, bool pending);
// Forgets a pending handle (start of a new capture).
void sc_clear_pending(orbit_sc2p5d_t* c);
// Band deposit of grids too large for one block's shared memory: rows per
// band and the number of bands.
int band_rows(int nx, int ny, int nz, int* nbands);
// Kick factor 2 L r_c / (beta^2 gamma^3) computed on the host exactly as
// SpaceChargeCalc2p5D.cc:96 does (libm pow).
double sc_host_factor(const orbit_sync_t& s, double length);
// Longitudinal kick factor of the 2.5Drb calculator, -L r_c m / gamma^2
// (SpaceChargeCalc2p5Drb.cc:128).
double sc_rb_long_factor(const orbit_sync_t& s, double length);

// Per-particle SC kick and extrema helpers used inside fused passes.
struct KickArgs {
  const ScState* st;
  const double* phi;      // plain form
  const double* lam;
  const float* phi_f;     // fp32 form
  const float* lam_f;
  const long long* phi_fix;  // plain form, fixed point
  const long long* lam_fix;
  double host_factor;
  int nx, ny, nz, form;
  const double* lamd;     // 2.5Drb: derivative grid, else null
  double rb_lsf;          // 2.5Drb: -L r_c m / gamma^2
  BndShape bnd;           // particles outside a conducting boundary are not kicked
};

}  // namespace orbit
