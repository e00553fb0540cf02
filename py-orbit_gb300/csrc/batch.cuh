// Batched tracking of many independent bunches (intensity and quadrupole
// scans): the members of one grid class share every kernel launch of a
// lattice turn.  Particle kernels find their member through a block table
// (members have different particle counts); grid kernels take the member
// from blockIdx.y (one class = one grid size).
#pragma once

#include "sc2p5d.cuh"
#include "teapot.cuh"

namespace orbit {

// One member's share of a fused pass (kick + maps + extrema scan).
struct PassJob {
  double* c[6];
  int n;
  int pad;
  const DevOp* ops;     // the member's compiled ops (same layout for all members)
  MapCtx m;
  KickArgs ka;
  ScState* ext;
  unsigned* status;
  SetupArgs sa;
  double* knl;          // per-particle 1/(1+dp_p)
};

// One member's deposit (plain form).
struct DepJob {
  const double* x;
  const double* y;
  const double* z;
  const double* msize;
  int n;
  int K;
  const ScState* st;
  unsigned long long* g_rho;
  unsigned long long* g_z;
  double ms_uniform, qscale;
};

// One member's grids for the Poisson solve (plain form).
struct SolveJob {
  ScState* st;
  unsigned long long* rho_q;
  unsigned long long* z_q;
  double* rho;
  double* lam;
  double* phi;
  double* gbuf;
  double2* hat;
  double2* green;
  const double2* tw_x;
  const double2* tw_y;
  long long* phi_fix;
  long long* lam_fix;
};

// Launch shapes of one class, chosen by the autotuner.
struct ClassTuning {
  int dep_threads, dep_chunk;    // deposit: threads per block, particles per block
  int pass_threads, pass_chunk;  // fused pass
  int fft_wide;                  // 1: radix-2 stages, N/2 threads; 0: radix-4 stages, N/4 threads
};

// Block layout of a batched particle launch: blk_job[block] is the member a
// block works for, mblk[member] = {first block, number of blocks}.
struct BlockMap {
  unsigned short* blk_job = nullptr;  // device
  int2* mblk = nullptr;               // device
  int nblk = 0;
};

// Batched launches of one class (sc2p5d.cu); jobs are device arrays of nm
// members; `proto` is any calculator of the class (sizes, plans).
int batch_enqueue_green(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* proto, int fft_wide, cudaStream_t s);
// `tag` names the launch for orbit_batch_profile.
int batch_enqueue_deposit(const DepJob* jobs, const BlockMap& bm, const orbit_sc2p5d_t* proto, int threads,
                          cudaStream_t s, const char* tag);
int batch_enqueue_solve(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* proto, int fft_wide, bool phi_fix,
                        cudaStream_t s);
// The columns (forward, Green multiply, backward) and backward rows alone,
// for timing the FFT schedules: they write only the work spectra, the
// potentials and max |phi|, which the next solve and grid set-up replace.
int batch_enqueue_fft_probe(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* proto, int fft_wide, cudaStream_t s);
int batch_init_attrs(const orbit_sc2p5d_t* proto);
// Shared-memory bytes of the plain deposit grids of the class, and whether
// they fit in shared memory.
bool batch_deposit_smem(const orbit_sc2p5d_t* proto);
// Blocks per particle chunk of the class's deposit: the number of row bands
// of a grid too large for one block's shared memory, else 1.
int batch_deposit_bands(const orbit_sc2p5d_t* proto);

// Batched fused pass (program.cu).  kf: 0 no kick, 1 plain kick; ksmem: the
// kick keeps a fixed-point copy of the potential of `smem` bytes in shared
// memory.
int batch_enqueue_pass(const PassJob* jobs, const BlockMap& bm, int threads, int kf, bool ext, bool ksmem,
                       size_t smem, int a, int b, int km, cudaStream_t s, const char* tag);
// Largest pass-kick copy of the potential kept in shared memory.
size_t batch_pass_smem_limit();

}  // namespace orbit
