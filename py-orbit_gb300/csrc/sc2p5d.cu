// SpaceChargeCalc2p5D on the GPU: extrema, grid set-up, deposit, FFT Poisson
// solve and kick as a chain of kernels on the bunch's stream with no host
// round trip (src/spacecharge/SpaceChargeCalc2p5D.cc:77-234,
// PoissonSolverFFT2D.cc:115-256, Grid2D.cc, Grid1D.cc).
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "sc2p5d.cuh"
#include "sc_device.cuh"
#include "batch.cuh"

namespace orbit {

static const int kMaxSmem = 220 * 1024;

// Thread bound of the single-bunch shared-memory deposit (one block per SM
// holds the 128x128 grid): 65536 / ORBIT_DEP_THREADS registers per thread.
#ifndef ORBIT_DEP_THREADS
#define ORBIT_DEP_THREADS 768
#endif

bool make_fft_plan(int n, FftPlan& pl) {
  pl.n = n;
  pl.nst = 0;
  int m = n;
  while (m % 4 == 0 && pl.nst < 24) { pl.rad[pl.nst++] = 4; m /= 4; }
  const int primes[] = {2, 3, 5, 7, 11, 13};
  for (int p : primes)
    while (m % p == 0 && pl.nst < 24) { pl.rad[pl.nst++] = p; m /= p; }
  pl.pow2 = (n & (n - 1)) == 0;
  return m == 1;
}

double sc_host_factor(const orbit_sync_t& s, double length) {
  return 2 * length * s.classical_radius / (std::pow(s.beta, 2) * std::pow(s.gamma, 3));
}

// -L r_c m / gamma^2 (SpaceChargeCalc2p5Drb.cc:128), libm pow as the reference.
double sc_rb_long_factor(const orbit_sync_t& s, double length) {
  return -length * s.classical_radius * s.mass / (std::pow(s.gamma, 2));
}

// ---------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------
// Extrema scan; the last block sets up the grids for the kick.  The
// accumulation grids start at zero: the kernels that read them clear them.
__global__ void k_extrema(const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ z, int n, ScState* st, unsigned* status, SetupArgs sa) {
  ExtAcc a;
  a.init();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a.add(x[i], y[i], z[i]);
  ext_commit_and_setup(a, st, status, sa, gridDim.x);
}

// Green function of the doubled grid (PoissonSolverFFT2D.cc:115-152): the
// quadrant 0 <= iX <= nx2/2, 0 <= iY <= ny2/2 is evaluated and written to
// its mirror images, as the reference copies it.  gate: run only when the
// Green spectrum is marked dirty (0 inside a graph branch taken on that
// flag).
__device__ __forceinline__ void green_fill_body(const ScState* st, double* g, int nx2, int ny2, int gate, int blk,
                                                int nblk) {
  if ((gate && !st->green_dirty) || st->skip) return;
  double sdx = st->sdx, sdy = st->sdy;
  const int hx = nx2 / 2, hy = ny2 / 2;
  const int qy = hy + 1;
  int tot = (hx + 1) * qy;
  for (int idx = blk * blockDim.x + threadIdx.x; idx < tot; idx += nblk * blockDim.x) {
    int iX = idx / qy, iY = idx % qy;
    double v = 0.0;
    if (iX != 0 || iY != 0) {
      double rX = __dmul_rn((double)iX, sdx), rY = __dmul_rn((double)iY, sdy);
      double r2 = __dadd_rn(__dmul_rn(rX, rX), __dmul_rn(rY, rY));
      v = __ddiv_rn(-log(r2), 2.0);
    }
    int mX = nx2 - iX, mY = ny2 - iY;
    g[(size_t)iX * ny2 + iY] = v;
    if (iY > 0 && mY != iY) g[(size_t)iX * ny2 + mY] = v;
    if (iX > 0 && mX != iX) {
      g[(size_t)mX * ny2 + iY] = v;
      if (iY > 0 && mY != iY) g[(size_t)mX * ny2 + mY] = v;
    }
  }
}

__global__ void k_green_fill(const ScState* st, double* g, int nx2, int ny2, int gate) {
  green_fill_body(st, g, nx2, ny2, gate, blockIdx.x, gridDim.x);
}

// Line density to doubles, total macrosize and the Green-rebuild flag
// reset, run by one extra block of the forward row transforms (the deposit
// is complete; an eager Green rebuild ran before it, a graph branch reads
// no flag).  The line density accumulator is cleared for the next deposit.
template <typename G>
__device__ __noinline__ void finalize_block(ScState* st, G* zacc, int nz, double* lam, float* lam_f,
                                            bool reset_dirty = true) {
  if (threadIdx.x == 0) {
    if (reset_dirty) st->green_dirty = 0;
    st->n_kicks += 1;
  }
  __shared__ double s_part[32];
  double iq = st->inv_qscale;
  double acc = 0.0;
  long long iacc = 0;
  unsigned long long amax = 0ull;
  for (int k = threadIdx.x; k < nz; k += blockDim.x) {
    G g = zacc[k];
    zacc[k] = (G)0;
    double v;
    if (sizeof(G) == 8) {
      long long q = (long long)g;
      iacc += q;
      v = (double)q * iq;
    } else {
      v = (double)g;
      acc += v;
    }
    lam[k] = v;
    if (lam_f) lam_f[k] = (float)v;
    unsigned long long bv = (unsigned long long)__double_as_longlong(fabs(v));
    amax = bv > amax ? bv : amax;
  }
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, amax, off);
    amax = o > amax ? o : amax;
  }
  if ((threadIdx.x & 31) == 0 && amax) atomicMax(&st->lam_absmax, amax);
  if (sizeof(G) == 8) {
    // exact integer sum, one rounding
    __shared__ long long s_i[32];
    for (int off = 16; off > 0; off >>= 1) iacc += __shfl_xor_sync(0xffffffffu, iacc, off);
    if ((threadIdx.x & 31) == 0) s_i[threadIdx.x >> 5] = iacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long t = 0;
      for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) t += s_i[w];
      st->total_m = (double)t * iq;
    }
  } else {
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) t += s_part[w];
      st->total_m = t;
    }
  }
}

// Loads of data that other blocks of the same launch wrote (the fused
// convolution): from L2, never from a stale L1 line.
template <bool CG, typename C>
__device__ __forceinline__ C ldx(const C* p) {
  if (CG) return __ldcg(p);
  return *p;
}

// Green function value of the doubled grid at row iX <= nx2/2, column j
// (mirrored as green_fill_body writes it): the same operations, so the
// same bits.
__device__ __forceinline__ double green_value(double sdx, double sdy, int iX, int j, int ny2) {
  const int iY = j <= ny2 / 2 ? j : ny2 - j;
  if (iX == 0 && iY == 0) return 0.0;
  double rX = __dmul_rn((double)iX, sdx), rY = __dmul_rn((double)iY, sdy);
  double r2 = __dadd_rn(__dmul_rn(rX, rX), __dmul_rn(rY, rY));
  return __ddiv_rn(-log(r2), 2.0);
}

// Row transforms along y (length N = ny2) of two real rows per block:
// z = a + i b, Z = FFT(z), A_k = (Z_k + conj Z_{N-k})/2, B_k = (Z_k - conj Z_{N-k})/(2i).
// SRC 0: Green rows (double, full length; rows 0..nx2/2 transformed, the
//        rest mirrored; nrows = nx2/2 + 1)
// SRC 1: rho from the fixed-point grid (first ny columns, first nx rows;
//        both forms)
// SRC 3: a double grid of nrows x ncols, read only (the raw density of a
//        learned-closure check)
// SRC 4: Green rows as SRC 0, the function evaluated in place (the fused
//        convolution)
// The deposit grid (SRC 1) is cleared as it is read, ready for the next
// deposit, and one extra block (the last) finalizes the line density.
// gate (SRC 0): as for k_green_fill.  sa, stw_in: the block's work buffers
// and its staged twiddles (the fused convolution stages them once);
// otherwise the dynamic shared memory and a copy made here.
template <typename T, int SRC, int LOGN = 0>
__device__ __forceinline__ void rows_fwd_body(ScState* st, void* src, double* rho_out, typename CT<T>::t* hat,
                                              const typename CT<T>::t* __restrict__ tw, const FftPlan& pl,
                                              int nrows, int ncols, int H, int gate, void* zacc, int nz,
                                              double* lam, float* lam_f, int blk, int nblk,
                                              typename CT<T>::t* sa = nullptr,
                                              const typename CT<T>::t* stw_in = nullptr, bool reset_dirty = true) {
  typedef typename CT<T>::t C;
  if (SRC == 0 && gate && !st->green_dirty) return;
  if (st->skip) return;
  if (SRC == 1 && blk == nblk - 1) {
    finalize_block(st, (unsigned long long*)zacc, nz, lam, lam_f, reset_dirty);
    return;
  }
  extern __shared__ unsigned char smem_raw[];
  C* a = sa ? sa : reinterpret_cast<C*>(smem_raw);
  C* b = a + pl.n;
  const int N = pl.n;
  const C* stw = stw_in;
  if (!stw) {
    load_twiddles(b + N, tw, N);
    stw = b + N;
  }
  int r0 = 2 * blk, r1 = r0 + 1;
  double iq = st->inv_qscale;
  double gsx = 0.0, gsy = 0.0;
  if (SRC == 4) {
    gsx = st->sdx;
    gsy = st->sdy;
  }
  // deposit rows: columns ncols..N-1 are the zero padding
  const bool hz = SRC != 0 && SRC != 4 && fft_halfzero_ok<T>(pl, ncols);
  for (int j = threadIdx.x; j < (hz ? N / 2 : N); j += blockDim.x) {
    T va = (T)0, vb = (T)0;
    if (j < ncols) {
      if (SRC == 0) {
        const double* g = (const double*)src;
        va = (T)g[(size_t)r0 * N + j];
        if (r1 < nrows) vb = (T)g[(size_t)r1 * N + j];
      } else if (SRC == 3) {
        const double* g = (const double*)src;
        va = (T)g[(size_t)r0 * ncols + j];
        if (r1 < nrows) vb = (T)g[(size_t)r1 * ncols + j];
      } else if (SRC == 4) {
        va = (T)green_value(gsx, gsy, r0, j, N);
        if (r1 < nrows) vb = (T)green_value(gsx, gsy, r1, j, N);
      } else if (SRC == 1) {
        long long* q = (long long*)src;
        double da = (double)q[(size_t)r0 * ncols + j] * iq;
        q[(size_t)r0 * ncols + j] = 0;
        rho_out[(size_t)r0 * ncols + j] = da;
        va = (T)da;
        if (r1 < nrows) {
          double db = (double)q[(size_t)r1 * ncols + j] * iq;
          q[(size_t)r1 * ncols + j] = 0;
          rho_out[(size_t)r1 * ncols + j] = db;
          vb = (T)db;
        }
      }
    }
    C v;
    v.x = va;
    v.y = vb;
    if (hz) {
      a[2 * j] = v;
      a[2 * j + 1] = v;
    } else {
      a[j] = v;
    }
  }
  __syncthreads();
  C* Z;
  if constexpr (LOGN > 0) Z = block_fft_fixed<T, false, LOGN>(a, b, stw, hz ? 1 : 0);
  else Z = hz ? block_fft_pow2<T, false>(a, b, pl, stw, 1) : block_fft<T>(a, b, pl, stw, false);
  for (int k = threadIdx.x; k < H; k += blockDim.x) {
    C zk = Z[k], zc = c_conj(Z[(N - k) % N]);
    C A, B;
    A.x = (zk.x + zc.x) * (T)0.5;
    A.y = (zk.y + zc.y) * (T)0.5;
    // (zk - zc) / (2i) = -i/2 (zk - zc)
    B.x = (zk.y - zc.y) * (T)0.5;
    B.y = -(zk.x - zc.x) * (T)0.5;
    hat[(size_t)r0 * H + k] = A;
    if (r1 < nrows) hat[(size_t)r1 * H + k] = B;
    if (SRC == 0 || SRC == 4) {
      // Green rows 0..nrows-1 = 0..nx2/2; row nx2 - r repeats row r
      const int nfull = 2 * (nrows - 1);
      if (r0 > 0 && r0 < nrows - 1) hat[(size_t)(nfull - r0) * H + k] = A;
      if (r1 < nrows - 1) hat[(size_t)(nfull - r1) * H + k] = B;
    }
  }
}

template <typename T, int SRC>
__global__ void k_rows_fwd(ScState* st, void* src, double* rho_out, typename CT<T>::t* hat,
                           const typename CT<T>::t* __restrict__ tw, FftPlan pl, int nrows, int ncols, int H,
                           int gate, void* zacc, int nz, double* lam, float* lam_f) {
  rows_fwd_body<T, SRC>(st, src, rho_out, hat, tw, pl, nrows, ncols, H, gate, zacc, nz, lam, lam_f, blockIdx.x,
                        gridDim.x);
}

// Column transforms along x (length N = nx2), one column k per block.
// The Green spectrum is stored column by column (green[k * N + r]).
// MODE 0: forward transform of the Green columns (when dirty), hat -> green.
// MODE 1: forward, multiply by the Green spectrum with the log-scale
//         correction (PoissonSolverFFT2D.cc:212-242), backward; rows >= nin
//         are zero on input and only rows < nin are kept on output.
// CG: hat and green were written by other blocks of the same launch (the
// fused convolution); sa, stw_in as for rows_fwd_body.
template <typename T, int MODE, bool CG = false, int LOGN = 0>
__device__ __forceinline__ void cols_body(ScState* st, typename CT<T>::t* hat, typename CT<T>::t* __restrict__ green,
                                          const typename CT<T>::t* __restrict__ tw, const FftPlan& pl, int nin,
                                          int H, int ny2, int gate, int k, typename CT<T>::t* sa = nullptr,
                                          const typename CT<T>::t* stw_in = nullptr) {
  typedef typename CT<T>::t C;
  if (MODE == 0 && gate && !st->green_dirty) return;
  if (st->skip) return;
  extern __shared__ unsigned char smem_raw[];
  C* a = sa ? sa : reinterpret_cast<C*>(smem_raw);
  C* b = a + pl.n;
  const int N = pl.n;
  const C* stw = stw_in;
  if (!stw) {
    load_twiddles(b + N, tw, N);
    stw = b + N;
  }
  const bool hz = MODE == 1 && fft_halfzero_ok<T>(pl, nin);
  for (int r = threadIdx.x; r < (hz ? N / 2 : N); r += blockDim.x) {
    C v;
    if (r < nin) v = ldx<CG>(hat + (size_t)r * H + k);
    else { v.x = (T)0; v.y = (T)0; }
    if (hz) {
      a[2 * r] = v;
      a[2 * r + 1] = v;
    } else {
      a[r] = v;
    }
  }
  __syncthreads();
  C* F;
  if constexpr (LOGN > 0) F = block_fft_fixed<T, false, LOGN>(a, b, stw, hz ? 1 : 0);
  else F = hz ? block_fft_pow2<T, false>(a, b, pl, stw, 1) : block_fft<T>(a, b, pl, stw, false);
  if (MODE == 0) {
    for (int r = threadIdx.x; r < N; r += blockDim.x) green[(size_t)k * N + r] = F[r];
    if (k == 0 && threadIdx.x == 0) st->n_green += 1;
    return;
  }
  double s = st->scale;
  for (int r = threadIdx.x; r < N; r += blockDim.x) {
    C g = ldx<CG>(green + (size_t)k * N + r);
    T gr;
    if (r == 0 && k == 0) {
      double re00 = (double)g.x;
      gr = (T)((re00 + s * (double)(N * ny2)) - s);
    } else {
      gr = (T)((double)g.x - s);
    }
    T gi = g.y;
    C o = F[r], res;
    res.x = o.x * gr - o.y * gi;
    res.y = o.x * gi + o.y * gr;
    F[r] = res;
  }
  __syncthreads();
  C* other = (F == a) ? b : a;
  C* R;
  if constexpr (LOGN > 0) R = block_fft_fixed<T, true, LOGN>(F, other, stw, 0);
  else R = block_fft<T>(F, other, pl, stw, true);
  for (int r = threadIdx.x; r < nin; r += blockDim.x) hat[(size_t)r * H + k] = R[r];
}

template <typename T, int MODE>
__global__ void k_cols(ScState* st, typename CT<T>::t* hat, typename CT<T>::t* __restrict__ green,
                       const typename CT<T>::t* __restrict__ tw, FftPlan pl, int nin, int H, int ny2, int gate) {
  cols_body<T, MODE>(st, hat, green, tw, pl, nin, H, ny2, gate, blockIdx.x);
}

// Backward row transforms (c2r, two rows per block) and the 1/(4 nx ny)
// normalisation onto the nx x ny potential (PoissonSolverFFT2D.cc:244-255).
// Imaginary parts at the self-conjugate k = 0 and k = N/2 are ignored.
template <typename T, bool CG = false, int LOGN = 0>
__device__ __forceinline__ void rows_inv_body(ScState* st, const typename CT<T>::t* __restrict__ hat,
                                              const typename CT<T>::t* __restrict__ tw, const FftPlan& pl,
                                              int nrows, int ny, int H, double denom, double* phi, float* phi_f,
                                              int blk, typename CT<T>::t* sa = nullptr,
                                              const typename CT<T>::t* stw_in = nullptr) {
  typedef typename CT<T>::t C;
  if (st->skip) return;
  extern __shared__ unsigned char smem_raw[];
  C* a = sa ? sa : reinterpret_cast<C*>(smem_raw);
  C* b = a + pl.n;
  const int N = pl.n;
  const C* stw = stw_in;
  if (!stw) {
    load_twiddles(b + N, tw, N);
    stw = b + N;
  }
  int r0 = 2 * blk, r1 = r0 + 1;
  bool has1 = r1 < nrows;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    C A, B;
    if (k < H) {
      A = ldx<CG>(hat + (size_t)r0 * H + k);
      B = has1 ? ldx<CG>(hat + (size_t)r1 * H + k) : C{(T)0, (T)0};
      if (k == 0 || 2 * k == N) { A.y = (T)0; B.y = (T)0; }
    } else {
      A = c_conj(ldx<CG>(hat + (size_t)r0 * H + (N - k)));
      B = has1 ? c_conj(ldx<CG>(hat + (size_t)r1 * H + (N - k))) : C{(T)0, (T)0};
    }
    C z;  // A + i B
    z.x = A.x - B.y;
    z.y = A.y + B.x;
    a[k] = z;
  }
  __syncthreads();
  C* R;
  if constexpr (LOGN > 0) R = block_fft_fixed<T, true, LOGN>(a, b, stw, 0);
  else R = block_fft<T>(a, b, pl, stw, true);
  unsigned long long amax = 0ull;  // bits of max |phi| (non-negative doubles order like their bits)
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    double va = denom * (double)R[j].x;
    phi[(size_t)r0 * ny + j] = va;
    if (phi_f) phi_f[(size_t)r0 * ny + j] = (float)va;
    unsigned long long ba = (unsigned long long)__double_as_longlong(fabs(va));
    amax = ba > amax ? ba : amax;
    if (has1) {
      double vb = denom * (double)R[j].y;
      phi[(size_t)r1 * ny + j] = vb;
      if (phi_f) phi_f[(size_t)r1 * ny + j] = (float)vb;
      unsigned long long bb = (unsigned long long)__double_as_longlong(fabs(vb));
      amax = bb > amax ? bb : amax;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, amax, off);
    amax = o > amax ? o : amax;
  }
  if ((threadIdx.x & 31) == 0 && amax) atomicMax(&st->phi_absmax, amax);
}

template <typename T>
__global__ void k_rows_inv(ScState* st, const typename CT<T>::t* __restrict__ hat,
                           const typename CT<T>::t* __restrict__ tw, FftPlan pl, int nrows, int ny, int H,
                           double denom, double* phi, float* phi_f) {
  rows_inv_body<T>(st, hat, tw, pl, nrows, ny, H, denom, phi, phi_f, blockIdx.x);
}

// ---------------------------------------------------------------------
// Fused convolution: the Green rebuild (when the set-up marked it), the
// forward rows of the deposit with the line-density finalization, the
// column transforms with the Green multiply and the backward rows in one
// cooperative launch (all blocks resident), the phases separated by two
// grid-wide barriers.  Every block stages both twiddle tables once.
// ---------------------------------------------------------------------
struct ConvArgs {
  ScState* st;
  unsigned* status;         // the bunch's status word (ST_SYNC)
  void* src;                // the deposit grid (fixed point or FP32)
  double* rho;
  void* hat;                // nx2 x H complex work spectrum
  void* green;              // nx2 x H complex Green spectrum
  void* gscr;               // nx2 x H complex: the Green row spectra
  const void* twx;
  const void* twy;
  FftPlan plx, ply;
  int nx, ny, nz, H, nx2, ny2;
  void* zacc;               // line-density accumulator
  double* lam;
  float* lam_f;
  double* phi;
  float* phi_f;
  double denom;             // 1 / (nx2 ny2)
  long long wait_polls;     // barrier wait limit
  int withhold;             // test hook: this block skips the first barrier (-1: none)
};

// Grid-wide barrier on a counter zeroed by the kick's set-up: every block
// arrives once (its earlier writes fenced) and waits until all have; the
// wait is bounded by `polls`, after which the block sets ST_SYNC and
// returns false.
__device__ __forceinline__ bool conv_barrier(unsigned* cnt, unsigned nblk, long long polls, unsigned* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(cnt, 1u);
    int ok = 1;
    long long i = 0;
    for (;;) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
      if (v >= nblk) break;
      if (++i > polls) {
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    if (!ok) atomicOr(status, (unsigned)ST_SYNC);
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// T double: plain form; float: FP32 form (both read the fixed-point
// deposit).  LOGN > 0:
// square power-of-two doubled grid nx2 = ny2 = 2^LOGN, transforms
// specialised at compile time (block_fft_fixed); 0: any supported size.
template <typename T, int LOGN>
__global__ void k_conv_fused(ConvArgs A) {
  typedef typename CT<T>::t C;
  constexpr int SRC = 1;  // both forms deposit in fixed point
  extern __shared__ unsigned char smem_raw[];
  ScState* st = A.st;
  if (st->skip) return;  // set by the set-up: the same in every block
  const int nmax = A.nx2 > A.ny2 ? A.nx2 : A.ny2;
  C* a = reinterpret_cast<C*>(smem_raw);  // a, b: nmax each
  C* stx = a + 2 * nmax;
  C* sty = stx + A.nx2;
  load_twiddles(stx, (const C*)A.twx, A.nx2);
  load_twiddles(sty, (const C*)A.twy, A.ny2);
  const int dirty = st->green_dirty;  // read before the first barrier, reset after it
  __syncthreads();
  C* hat = (C*)A.hat;
  C* green = (C*)A.green;
  C* gscr = (C*)A.gscr;
  // phase 1: deposit rows (+ the finalization item), Green rows
  const int nrp = (A.nx + 1) / 2, ngp = dirty ? (A.nx + 2) / 2 : 0;
  for (int it = blockIdx.x; it < nrp + 1 + ngp; it += gridDim.x) {
    if (it <= nrp)
      rows_fwd_body<T, SRC, LOGN>(st, A.src, A.rho, hat, nullptr, A.ply, A.nx, A.ny, A.H, 1, A.zacc, A.nz, A.lam,
                                  A.lam_f, it, nrp + 1, a, sty, false);
    else
      rows_fwd_body<T, 4, LOGN>(st, nullptr, nullptr, gscr, nullptr, A.ply, A.nx + 1, A.ny2, A.H, 0, nullptr, 0,
                                nullptr, nullptr, it - nrp - 1, ngp, a, sty);
    __syncthreads();
  }
  if ((int)blockIdx.x == A.withhold) return;
  if (!conv_barrier(&st->conv_bar[0], gridDim.x, A.wait_polls, A.status)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0 && dirty) st->green_dirty = 0;
  // phase 2: per column, the Green column (when rebuilt), then the deposit's
  // forward transform, the multiply and the backward transform
  for (int k = blockIdx.x; k < A.H; k += gridDim.x) {
    if (dirty) {
      cols_body<T, 0, true, LOGN>(st, gscr, green, nullptr, A.plx, A.nx2, A.H, A.ny2, 0, k, a, stx);
      __syncthreads();
    }
    cols_body<T, 1, true, LOGN>(st, hat, green, nullptr, A.plx, A.nx, A.H, A.ny2, 1, k, a, stx);
    __syncthreads();
  }
  if (!conv_barrier(&st->conv_bar[1], gridDim.x, A.wait_polls, A.status)) return;
  // phase 3: backward rows onto phi
  for (int it = blockIdx.x; it < nrp; it += gridDim.x) {
    rows_inv_body<T, true, LOGN>(st, hat, nullptr, A.ply, A.nx, A.ny, A.H, A.denom, A.phi, A.phi_f, it, a, sty);
    __syncthreads();
  }
}

// Plain form: phi and lambda as 64-bit integers phi * 2^sphi, lambda *
// 2^slam with the scales chosen from their maxima (below 2^61), read by the
// fixed-point kick.
__device__ __forceinline__ void phi_fix_body(const ScState* st, const double* __restrict__ phi,
                                             const double* __restrict__ lam, long long* phi_fix, long long* lam_fix,
                                             int ng, int nz, int blk) {
  if (st->skip) return;
  int sphi = scale_bits(st->phi_absmax), slam = scale_bits(st->lam_absmax);
  int i = blk * blockDim.x + threadIdx.x;
  if (i < ng) phi_fix[i] = phi_fixed(phi[i], sphi);
  if (i < nz) lam_fix[i] = phi_fixed(lam[i], slam);
}

__global__ void k_phi_fix(const ScState* st, const double* __restrict__ phi, const double* __restrict__ lam,
                          long long* phi_fix, long long* lam_fix, int ng, int nz) {
  phi_fix_body(st, phi, lam, phi_fix, lam_fix, ng, nz, blockIdx.x);
}

// 2.5Drb: one cell of the smoothed line-density derivative
// (SpaceChargeCalc2p5Drb::calculateLongDerivative, SpaceChargeCalc2p5Drb.cc:257-306),
// a quadratic least-squares fit over navg cells solved by Cramer's rule,
// with the reference's operation order and explicit rounding.
__device__ double rb_deriv_cell(const double* lam, int nz, int navg, double zmin, double dz, int iz) {
  if (nz < navg) navg = nz;
  double zc = __dadd_rn(zmin, __dmul_rn(iz + 0.5, dz));
  int i0 = iz - navg / 2;
  if (i0 < 0) i0 = 0;
  if (i0 + navg >= nz) i0 = nz - navg;
  double m[5], q[5];
  for (int j = 0; j < 5; ++j) {
    m[j] = 0.0;
    q[j] = 0.0;
    for (int i = i0; i < i0 + navg; ++i) {
      double t = (double)(i - i0 + 1), tj = 1.0;
      for (int e = 0; e < j; ++e) tj = __dmul_rn(tj, t);  // t^j, exact for these small integers
      m[j] = __dadd_rn(m[j], tj);
      q[j] = __dadd_rn(q[j], __dmul_rn(tj, lam[i]));
    }
  }
#define M(a, b) __dmul_rn(a, b)
  double det = __dsub_rn(__dadd_rn(__dsub_rn(__dsub_rn(M(M(m[0], m[2]), m[4]), M(M(m[1], m[1]), m[4])),
                                             M(M(m[0], m[3]), m[3])),
                                   M(M(M(2.0, m[1]), m[2]), m[3])),
                         M(M(m[2], m[2]), m[2]));
  double an = __dsub_rn(__dadd_rn(__dadd_rn(__dsub_rn(__dsub_rn(M(M(q[0], m[1]), m[3]), M(M(q[1], m[0]), m[3])),
                                                      M(M(q[0], m[2]), m[2])),
                                            M(M(q[1], m[1]), m[2])),
                                  M(M(q[2], m[0]), m[2])),
                        M(M(q[2], m[1]), m[1]));
  double bn = __dadd_rn(__dsub_rn(__dsub_rn(__dadd_rn(__dsub_rn(M(M(q[1], m[0]), m[4]), M(M(q[0], m[1]), m[4])),
                                                      M(M(q[0], m[2]), m[3])),
                                            M(M(q[2], m[0]), m[3])),
                                  M(M(q[1], m[2]), m[2])),
                        M(M(q[2], m[1]), m[2]));
#undef M
  double a = __ddiv_rn(an, det), b = __ddiv_rn(bn, det);
  double z0 = __dadd_rn(zmin, __dmul_rn(i0 + 0.5, dz));
  double y = __dadd_rn(__ddiv_rn(__dmul_rn(__dmul_rn(2.0, a), __dadd_rn(__dsub_rn(zc, z0), dz)), dz), b);
  y = __ddiv_rn(y, dz);
  return __ddiv_rn(y, dz);
}

// 2.5Drb analysis on the finished grids (one block): the rho-grid moments
// that give the beam centre and a_bunch = sqrt(2 (<x^2> + <y^2>))
// (SpaceChargeCalc2p5Drb.cc:226-254; the reference takes y from the x grid,
// kept), the total macrosize the kick divides by, the pipe-radius terms of
// the longitudinal kick (:124-136) and the derivative grid.
__global__ void k_rb_analysis(ScState* st, const double* __restrict__ rho, const double* __restrict__ lam,
                              double* lamd, int nx, int ny, int nz, int navg, double pipe_radius) {
  if (st->skip) return;
  const double xmin = st->xmin, dx = st->dx;
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int idx = threadIdx.x; idx < nx * ny; idx += blockDim.x) {
    int ix = idx / ny, iy = idx - ix * ny;
    double val = rho[idx];
    double x = __dadd_rn(xmin, __dmul_rn((double)ix, dx));
    double y = __dadd_rn(xmin, __dmul_rn((double)iy, dx));
    s[0] += val;
    s[1] += x * val;
    s[2] += x * x * val;
    s[3] += y * val;
    s[4] += y * y * val;
  }
  __shared__ double red[32][5];
  for (int c = 0; c < 5; ++c)
    for (int off = 16; off > 0; off >>= 1) s[c] += __shfl_xor_sync(0xffffffffu, s[c], off);
  if ((threadIdx.x & 31) == 0)
    for (int c = 0; c < 5; ++c) red[threadIdx.x >> 5][c] = s[c];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      for (int c = 0; c < 5; ++c) t[c] += red[w][c];
    double total = t[0];
    double xa = t[1] / total, x2 = t[2] / total, ya = t[3] / total, y2 = t[4] / total;
    x2 = fabs(x2 - xa * xa);
    y2 = fabs(y2 - ya * ya);
    double a = sqrt(2 * (x2 + y2));
    st->rb_xc = xa;
    st->rb_yc = ya;
    st->rb_a2 = a * a;
    st->rb_lin = 1.0 + 2 * log(pipe_radius / a);
    st->rb_lout = 2 * log(pipe_radius);
    st->total_m = total;
  }
  const double zmin = st->zmin, dz = st->dz;
  if (nz == 1) {
    if (threadIdx.x == 0) lamd[0] = 0.0;
  } else if (nz == 2) {
    if (threadIdx.x == 0) {
      // Grid1D::calcGradient at the midpoint (Grid1D.cc:520-534, 568-627)
      double g0 = __dadd_rn(zmin, __dmul_rn(0.5, dz)), g1 = __dadd_rn(zmin, __dmul_rn(1.5, dz));
      double zm = __dmul_rn(__dadd_rn(g0, g1), 0.5);
      double d = 0.0;
      if (!(zm < zmin || zm > st->zmax)) {
        double ind = __dsub_rn(__ddiv_rn(__dsub_rn(zm, zmin), dz), 0.5);
        int i0 = (int)ind, ip;
        double gz = __dadd_rn(zmin, __dmul_rn(i0 + 0.5, dz));
        double frac = __ddiv_rn(__dsub_rn(zm, gz), dz);
        if (i0 == 0 && frac < 0.) { i0 = 1; ip = 0; }
        else if (i0 == 1) { if (frac > 0.) { ip = 0; } else { ip = 1; i0 = 0; } }
        else { ip = i0 + 1; }
        d = __ddiv_rn(__dsub_rn(lam[ip], lam[i0]), dz);
      }
      lamd[0] = __ddiv_rn(d, dz);
      lamd[1] = __ddiv_rn(d, dz);
    }
  } else {
    for (int iz = threadIdx.x; iz < nz; iz += blockDim.x) lamd[iz] = rb_deriv_cell(lam, nz, navg, zmin, dz, iz);
  }
}

// Deposit, plain form.  SMEM: block-private fixed-point grids in shared
// memory, flushed with one 64-bit atomic per non-zero cell.  With K > 0
// (uniform macrosize) each particle deposits unit weight in units of 2^-K
// through the integer path (deposit_fixed); otherwise, and for the rare
// particle the integer path declines, macrosize * qscale through FP64.
// Blocks of up to 768 threads (80 registers: 24 warps per SM) cover the
// latency of the shared-memory atomics; 1024 threads at 64 registers spill
// and ran slower.
template <bool SMEM>
__device__ __forceinline__ void deposit_plain_body(const double* __restrict__ x, const double* __restrict__ y,
                                                   const double* __restrict__ z, const double* __restrict__ msize,
                                                   int n, const ScState* st, unsigned long long* g_rho,
                                                   unsigned long long* g_z, double ms_uniform, double qscale, int nx,
                                                   int ny, int nz, int K, int blk, int nblk) {
  DepConst d;
  load_dep_const(d, st, nx, ny, nz);
  if (d.skip) return;
  DepFix df;
  if (K > 0) load_dep_fix(df, st, nx, ny, nz, K);
  // shared: low words of the nx*ny + nz cells, then their high words
  extern __shared__ unsigned s_acc32[];
  const int ncell = nx * ny + nz;
  GridAcc<SMEM> rho, zg;
  if constexpr (SMEM) {
    rho.lo = s_acc32;
    rho.hi_off = ncell;
    zg.lo = s_acc32 + nx * ny;
    zg.hi_off = ncell;
    for (int i = threadIdx.x; i < 2 * ncell; i += blockDim.x) s_acc32[i] = 0u;
    __syncthreads();
  } else {
    rho.p = g_rho;
    zg.p = g_z;
  }
  for (int i = blk * blockDim.x + threadIdx.x; i < n; i += nblk * blockDim.x) {
    double xi = x[i], yi = y[i], zi = z[i];
    if (K > 0 && deposit_fixed(df, rho, zg, xi, yi, zi)) continue;
    double ms = msize ? msize[i] * qscale : ms_uniform;
    deposit_plain(d, rho, zg, xi, yi, zi, ms);
  }
  if constexpr (SMEM) {
    __syncthreads();
    for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
      unsigned long long v = rho.get(i);
      if (v) atomicAdd(i < nx * ny ? g_rho + i : g_z + (i - nx * ny), v);
    }
  }
}

template <bool SMEM>
__global__ void __launch_bounds__(ORBIT_DEP_THREADS) k_deposit_plain(const double* __restrict__ x, const double* __restrict__ y,
                                const double* __restrict__ z, const double* __restrict__ msize, int n,
                                const ScState* st, unsigned long long* g_rho, unsigned long long* g_z,
                                double ms_uniform, double qscale, int nx, int ny, int nz, int K) {
  deposit_plain_body<SMEM>(x, y, z, msize, n, st, g_rho, g_z, ms_uniform, qscale, nx, ny, nz, K, blockIdx.x,
                           gridDim.x);
}

// Band deposit (plain form) for grids whose two 32-bit words per cell do
// not fit in one block's shared memory.  Block (chunk, band) keeps rows
// r0-1..r1 of the grid (band rows [r0, r1) plus one halo row on each side)
// and the whole line density in shared memory, reads the chunk's
// particles and deposits those whose centre row lies in its band (band 0
// also those outside the transverse grid); the halo rows reach the global
// grid through the same exact 64-bit integer adds as every other cell.
__device__ __forceinline__ void deposit_band_body(const double* __restrict__ x, const double* __restrict__ y,
                                                  const double* __restrict__ z, const double* __restrict__ msize,
                                                  int n, const ScState* st, unsigned long long* g_rho,
                                                  unsigned long long* g_z, double ms_uniform, double qscale, int nx,
                                                  int ny, int nz, int K, int rpb, int band, int chunk, int nchunk) {
  DepConst d;
  load_dep_const(d, st, nx, ny, nz);
  if (d.skip) return;
  DepFix df;
  if (K > 0) load_dep_fix(df, st, nx, ny, nz, K);
  const int r0 = band * rpb, r1 = min(nx, r0 + rpb);
  const int lr0 = max(r0 - 1, 0), lr1 = min(r1 + 1, nx);
  const int nloc = (lr1 - lr0) * ny;
  const int ncell = nloc + nz;
  extern __shared__ unsigned s_band32[];
  BandAcc rho;
  rho.lo = s_band32;
  rho.hi_off = ncell;
  rho.base = lr0 * ny;
  rho.r0 = r0;
  rho.r1 = r1;
  rho.first = band == 0;
  GridAcc<true> zg;
  zg.lo = s_band32 + nloc;
  zg.hi_off = ncell;
  for (int i = threadIdx.x; i < 2 * ncell; i += blockDim.x) s_band32[i] = 0u;
  __syncthreads();
  for (int i = chunk * blockDim.x + threadIdx.x; i < n; i += nchunk * blockDim.x) {
    double xi = x[i], yi = y[i], zi = z[i];
    if (K > 0 && deposit_fixed(df, rho, zg, xi, yi, zi)) continue;
    double ms = msize ? msize[i] * qscale : ms_uniform;
    deposit_plain(d, rho, zg, xi, yi, zi, ms);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
    unsigned long long v = ((unsigned long long)s_band32[ncell + i] << 32) | s_band32[i];
    if (v) atomicAdd(i < nloc ? g_rho + (size_t)lr0 * ny + i : g_z + (i - nloc), v);
  }
}

// nb bands; blocks blockIdx.x = chunk * nb + band.
__global__ void __launch_bounds__(768) k_deposit_band(const double* __restrict__ x, const double* __restrict__ y,
                                                      const double* __restrict__ z, const double* __restrict__ msize,
                                                      int n, const ScState* st, unsigned long long* g_rho,
                                                      unsigned long long* g_z, double ms_uniform, double qscale,
                                                      int nx, int ny, int nz, int K, int rpb, int nb) {
  deposit_band_body(x, y, z, msize, n, st, g_rho, g_z, ms_uniform, qscale, nx, ny, nz, K, rpb, blockIdx.x % nb,
                    blockIdx.x / nb, gridDim.x / nb);
}

// Kick (SpaceChargeCalc2p5D.cc:104-119): fixed-point gradient and line
// density (kick_fixed), FP64 routine for the particles it declines.  With
// lamd (2.5Drb) also the longitudinal kick of dE.
template <bool SMEM>
__global__ void k_kick_plain(const double* __restrict__ x, double* __restrict__ xp, const double* __restrict__ y,
                             double* __restrict__ yp, const double* __restrict__ z, int n, const ScState* st,
                             const double* __restrict__ phi, const double* __restrict__ lam,
                             const long long* __restrict__ phi_fix, const long long* __restrict__ lam_fix,
                             double host_factor, int nx, int ny, int nz, const double* __restrict__ lamd,
                             double rb_lsf, double* __restrict__ dE, BndShape bnd) {
  KickConst k;
  KickFix kf;
  load_kick_block(k, &kf, st, host_factor, nx, ny, nz);
  if (k.skip) return;
  extern __shared__ long long s_phix[];
  const long long* P = phi_fix;
  const long long* Lm = lam_fix;
  if (SMEM) {
    // the shared copy is converted here; phi_fix, lam_fix are not read
    for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) s_phix[i] = phi_fixed(phi[i], kf.sphi);
    for (int i = threadIdx.x; i < nz; i += blockDim.x) s_phix[nx * ny + i] = phi_fixed(lam[i], kf.slam);
    __syncthreads();
    P = s_phix;
    Lm = s_phix + nx * ny;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double a = xp[i], b = yp[i];
    double xi = x[i], yi = y[i], zi = z[i];
    if (!bnd_inside(bnd, xi, yi)) continue;  // SpaceChargeCalc2p5D.cc:110
    if (!kick_fixed(kf, P, Lm, xi, yi, zi, a, b)) kick_plain(k, phi, lam, xi, yi, zi, a, b);
    xp[i] = a;
    yp[i] = b;
    if (lamd) {
      RbConst r;
      load_rb_const(r, st, rb_lsf);
      double e = dE[i];
      kick_rb_long(k, r, lamd, xi, yi, zi, e);
      dE[i] = e;
    }
  }
}

template <bool SMEM>
__global__ void k_kick_fp32(const double* __restrict__ x, double* __restrict__ xp, const double* __restrict__ y,
                            double* __restrict__ yp, const double* __restrict__ z, int n, const ScState* st,
                            const float* __restrict__ phi, const float* __restrict__ lam, double host_factor,
                            int nx, int ny, int nz, BndShape bnd) {
  KickConst k;
  load_kick_const(k, st, host_factor, nx, ny, nz);
  if (k.skip) return;
  extern __shared__ float s_phif[];
  const float* P = phi;
  const float* Lm = lam;
  if (SMEM) {
    for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) s_phif[i] = phi[i];
    for (int i = threadIdx.x; i < nz; i += blockDim.x) s_phif[nx * ny + i] = lam[i];
    __syncthreads();
    P = s_phif;
    Lm = s_phif + nx * ny;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!bnd_inside(bnd, x[i], y[i])) continue;
    double a = xp[i], b = yp[i];
    kick_fp32(k, P, Lm, x[i], y[i], z[i], a, b);
    xp[i] = a;
    yp[i] = b;
  }
}

// Field evaluation at arbitrary points (Grid2D::calcGradient, Grid1D::getValue).
__global__ void k_fields(const ScState* st, const double* __restrict__ phi, const double* __restrict__ lam,
                         int nx, int ny, int nz, int n, const double* x, const double* y, const double* z,
                         double* ex, double* ey, double* lv) {
  KickConst k;
  load_kick_const(k, st, 0.0, nx, ny, nz);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // With fac = -1 the kick adds gx/dx * lambda... evaluate the pieces directly.
  int ix, iy;
  double fx, fy;
  tsc_index<double>((x[i] - k.xmin) * k.inv_dx, nx, ix, fx);
  tsc_index<double>((y[i] - k.ymin) * k.inv_dy, ny, iy, fy);
  double wxm, wx0, wxp, wym, wy0, wyp;
  tsc_weights<double>(fx, wxm, wx0, wxp);
  tsc_weights<double>(fy, wym, wy0, wyp);
  double dxw[3] = {fx - 0.5, -2.0 * fx, 0.5 + fx};
  double dyw[3] = {fy - 0.5, -2.0 * fy, 0.5 + fy};
  double wxw[3] = {wxm, wx0, wxp}, wyw[3] = {wym, wy0, wyp};
  double gx = 0, gy = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double v = phi[(ix - 1 + a) * ny + (iy - 1 + b)];
      gx += dxw[a] * wyw[b] * v;
      gy += wxw[a] * dyw[b] * v;
    }
  ex[i] = gx * k.inv_dx;
  ey[i] = gy * k.inv_dy;
  double l = 0.0;
  if (!(z[i] < k.zmin || z[i] > k.zmax)) {
    int i0, ip;
    double w0, wp;
    g1_index<double>(z[i], k.zmin, k.inv_dz, nz, i0, ip, w0, wp);
    l = (nz > 1) ? (w0 * lam[i0] + wp * lam[ip]) : lam[0];
  }
  lv[i] = l;
}

// ---------------------------------------------------------------------
// learned closure (plain form)
// ---------------------------------------------------------------------
// The fixed-point deposit as the network's image (density * scale, scale =
// nx ny / total macrosize: unit mean) and, on check kicks, the raw density.
__global__ void k_learn_in(const ScState* st, const unsigned long long* __restrict__ rho_q,
                           float* __restrict__ img, double* __restrict__ raw, int n, double scale) {
  if (st->skip) return;
  const double iq = st->inv_qscale;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = (double)(long long)rho_q[i] * iq;
    if (raw) raw[i] = v;
    img[i] = (float)(v * scale);
  }
}

// The network output clamped at zero (a density is not negative), rescaled
// to the deposit's total charge (n in image units) and written back as the
// fixed-point deposit the solve reads.  The output's sum is the network's
// per-block sums (`parts`) added in block order by warp 0 of every block:
// the same on every run.  A network that reported a failed tensor-core wait
// (net_err != 0) produced no valid output: the closure falls back to the
// plain deposit for good; nothing is written once it has fallen back.
__global__ void k_learn_out(ScState* st, const float* __restrict__ out, unsigned long long* __restrict__ rho_q, int n,
                            double scale, const double* __restrict__ parts, int nparts,
                            const int* __restrict__ net_err) {
  if (st->skip) return;
  if (*net_err) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && !st->dn_fallback) {
      st->dn_fallback = 1;
      st->dn_trips += 1;
    }
    return;
  }
  if (st->dn_fallback) return;
  __shared__ double s_sum;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int k = threadIdx.x; k < nparts; k += 32) t += parts[k];
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (threadIdx.x == 0) s_sum = t;
  }
  __syncthreads();
  const double sum = s_sum;
  if (!(sum > 0.0)) return;
  const double back = ((double)n / sum) / (scale * st->inv_qscale);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rho_q[i] = (unsigned long long)llrint((double)fmaxf(out[i], 0.f) * back);
}

// State of the check solve: the kick's skip flag and log-scale term.
__global__ void k_learn_chk_prep(const ScState* st, ScState* chk) {
  chk->skip = st->skip;
  chk->scale = st->scale;
  chk->phi_absmax = 0ull;
}

// The closure's check: relative rms difference of the potential from the
// denoised density and the potential from the raw deposit; above `bound`
// the closure falls back to the plain deposit for the following kicks.
__global__ void __launch_bounds__(1024) k_learn_compare(ScState* st, const double* __restrict__ phi, const double* __restrict__ phi_raw, int n,
                                double bound) {
  if (st->skip) return;
  __shared__ double s_d[32], s_r[32];
  double d2 = 0.0, r2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double a = phi[i], b = phi_raw[i];
    d2 += (a - b) * (a - b);
    r2 += b * b;
  }
  for (int off = 16; off > 0; off >>= 1) {
    d2 += __shfl_xor_sync(0xffffffffu, d2, off);
    r2 += __shfl_xor_sync(0xffffffffu, r2, off);
  }
  if ((threadIdx.x & 31) == 0) {
    s_d[threadIdx.x >> 5] = d2;
    s_r[threadIdx.x >> 5] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double D = 0.0, R = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      D += s_d[w];
      R += s_r[w];
    }
    double e = R > 0.0 ? sqrt(D / R) : 0.0;
    st->dn_err = e;
    st->dn_checks += 1;
    if (!(e <= bound)) {
      st->dn_fallback = 1;
      st->dn_trips += 1;
    }
  }
}

// ---------------------------------------------------------------------
// batched kernels (plain form): the members of one grid class in one
// launch; grid kernels take the member from blockIdx.y, particle kernels
// from the block table
// ---------------------------------------------------------------------
__global__ void kb_green_fill(const SolveJob* __restrict__ jobs, int nx2, int ny2) {
  const SolveJob& J = jobs[blockIdx.y];
  green_fill_body(J.st, J.gbuf, nx2, ny2, 1, blockIdx.x, gridDim.x);
}

template <int SRC>
__global__ void kb_rows_fwd(const SolveJob* __restrict__ jobs, FftPlan pl, int nrows, int ncols, int H, int nz) {
  const SolveJob& J = jobs[blockIdx.y];
  if (SRC == 0)
    rows_fwd_body<double, 0>(J.st, J.gbuf, nullptr, J.hat, J.tw_y, pl, nrows, ncols, H, 1, nullptr, 0, nullptr,
                             nullptr, blockIdx.x, gridDim.x);
  else
    rows_fwd_body<double, 1>(J.st, J.rho_q, J.rho, J.hat, J.tw_y, pl, nrows, ncols, H, 1, J.z_q, nz, J.lam, nullptr,
                             blockIdx.x, gridDim.x);
}

template <int MODE>
__global__ void kb_cols(const SolveJob* __restrict__ jobs, FftPlan pl, int nin, int H, int ny2) {
  const SolveJob& J = jobs[blockIdx.y];
  cols_body<double, MODE>(J.st, J.hat, J.green, J.tw_x, pl, nin, H, ny2, 1, blockIdx.x);
}

__global__ void kb_rows_inv(const SolveJob* __restrict__ jobs, FftPlan pl, int nrows, int ny, int H, double denom) {
  const SolveJob& J = jobs[blockIdx.y];
  rows_inv_body<double>(J.st, J.hat, J.tw_y, pl, nrows, ny, H, denom, J.phi, nullptr, blockIdx.x);
}

__global__ void kb_phi_fix(const SolveJob* __restrict__ jobs, int ng, int nz) {
  const SolveJob& J = jobs[blockIdx.y];
  phi_fix_body(J.st, J.phi, J.lam, J.phi_fix, J.lam_fix, ng, nz, blockIdx.x);
}

// Members' blocks: chunk * nb + band.
__global__ void __launch_bounds__(768) kb_deposit_band(const DepJob* __restrict__ jobs,
                                                       const unsigned short* __restrict__ blk_job,
                                                       const int2* __restrict__ mblk, int nx, int ny, int nz, int rpb,
                                                       int nb) {
  const int j = blk_job[blockIdx.x];
  const DepJob& J = jobs[j];
  const int2 mb = mblk[j];
  const int lb = blockIdx.x - mb.x;
  deposit_band_body(J.x, J.y, J.z, J.msize, J.n, J.st, J.g_rho, J.g_z, J.ms_uniform, J.qscale, nx, ny, nz, J.K, rpb,
                    lb % nb, lb / nb, mb.y / nb);
}

template <bool SMEM>
__global__ void __launch_bounds__(768) kb_deposit(const DepJob* __restrict__ jobs,
                                                  const unsigned short* __restrict__ blk_job,
                                                  const int2* __restrict__ mblk, int nx, int ny, int nz) {
  const int j = blk_job[blockIdx.x];
  const DepJob& J = jobs[j];
  const int2 mb = mblk[j];
  deposit_plain_body<SMEM>(J.x, J.y, J.z, J.msize, J.n, J.st, J.g_rho, J.g_z, J.ms_uniform, J.qscale, nx, ny, nz,
                           J.K, blockIdx.x - mb.x, mb.y);
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
// W_N^e = exp(-2 pi i e / N), e = 0..n-1, from long-double cos/sin, with the
// quadrant points exact.
template <typename T>
static void fill_twiddles_host(int n, typename CT<T>::t* h) {
  for (int e = 0; e < n; ++e) {
    long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)e / (long double)n;
    h[e].x = (T)cosl(a);
    h[e].y = (T)(-sinl(a));
  }
  if (n % 4 == 0) {
    h[0].x = 1; h[0].y = 0;
    h[n / 4].x = 0; h[n / 4].y = -1;
    h[n / 2].x = -1; h[n / 2].y = 0;
    h[3 * n / 4].x = 0; h[3 * n / 4].y = 1;
  } else if (n % 2 == 0) {
    h[n / 2].x = -1; h[n / 2].y = 0;
  }
}

template <typename T>
static void* make_twiddles(int n, cudaError_t* err) {
  typedef typename CT<T>::t C;
  std::vector<C> h(n);
  fill_twiddles_host<T>(n, h.data());
  void* d = nullptr;
  *err = cudaMalloc(&d, sizeof(C) * n);
  if (*err == cudaSuccess) *err = cudaMemcpy(d, h.data(), sizeof(C) * n, cudaMemcpyHostToDevice);
  return d;
}

// Power-of-two lengths: one thread per radix-2 butterfly (N/2, at least a
// warp, at most 1024, above which the stages are radix 4); other lengths: a
// fixed block for the generic stages.
static int fft_threads(const FftPlan& pl) {
  int n = pl.n;
  if (pl.pow2) return n / 2 >= 32 ? (n / 2 > 1024 ? 1024 : n / 2) : 32;
  return n >= 1024 ? 512 : (n >= 256 ? 256 : 128);
}

template <typename T>
static size_t fft_smem(int n) { return 3 * sizeof(typename CT<T>::t) * (size_t)n; }  // a, b, twiddles

template <typename T>
static int set_fft_attrs(int nmax) {
  int bytes = (int)fft_smem<T>(nmax);
  if (bytes <= 48 * 1024) return ORBIT_OK;
  ORBIT_CUDA(cudaFuncSetAttribute(k_rows_fwd<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  ORBIT_CUDA(cudaFuncSetAttribute(k_rows_fwd<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  ORBIT_CUDA(cudaFuncSetAttribute(k_rows_fwd<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  ORBIT_CUDA(cudaFuncSetAttribute(k_cols<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  ORBIT_CUDA(cudaFuncSetAttribute(k_cols<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  ORBIT_CUDA(cudaFuncSetAttribute(k_rows_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  return ORBIT_OK;
}

static int ext_blocks(int n) {
  int b = (n + 255) / 256;
  int cap = num_sms() * 4;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

// launch geometry for particle kernels that keep a grid copy in shared memory
static void particle_geometry(size_t smem, int n, int max_threads, int* blocks, int* threads) {
  int bps = smem > 0 ? (int)(kMaxSmem / smem) : 8;
  if (bps < 1) bps = 1;
  if (bps > 4) bps = 4;
  *threads = (bps == 1) ? 1024 : 512;
  if (*threads > max_threads) *threads = max_threads & ~31;  // register-limited kernels
  int b = num_sms() * bps;
  int need = (n + *threads - 1) / *threads;
  *blocks = need < b ? (need < 1 ? 1 : need) : b;
}

// Rows per band of the band deposit: shared memory (two 32-bit words per
// cell of the band, its halo rows and the line density) within 200 KB (the
// deposit's 80 registers at 768 threads already keep one block per SM, so
// fewer, taller bands re-read fewer coordinates); bands of equal height.
int band_rows(int nx, int ny, int nz, int* nbands) {
  long long cells = 200 * 1024 / 8 - nz;
  int rmax = (int)(cells / ny) - 2;
  if (rmax < 1) rmax = 1;
  int nb = (nx + rmax - 1) / rmax;
  int rpb = (nx + nb - 1) / nb;
  *nbands = (nx + rpb - 1) / rpb;
  return rpb;
}

static size_t band_smem(int nx, int ny, int nz) {
  int nb;
  int rpb = band_rows(nx, ny, nz, &nb);
  return 8 * ((size_t)(rpb + 2) * ny + nz);
}

// Fused convolution geometry: threads for the longer transform, shared
// memory for two work buffers and both twiddle tables, and the largest
// number of work items of a phase (deposit rows + finalization + Green
// rows; columns; backward rows).
static int conv_threads(const orbit_sc2p5d_t* c) {
  int tx = fft_threads(c->plan_x), ty = fft_threads(c->plan_y);
  return tx > ty ? tx : ty;
}

template <typename T>
static size_t conv_smem(const orbit_sc2p5d_t* c) {
  int nmax = c->nx2 > c->ny2 ? c->nx2 : c->ny2;
  return sizeof(typename CT<T>::t) * (size_t)(2 * nmax + c->nx2 + c->ny2);
}

static int conv_items(const orbit_sc2p5d_t* c) {
  int rows = (c->nx + 1) / 2 + 1 + (c->nx + 2) / 2;
  return rows > c->H ? rows : c->H;
}

// The fused kernel for the calculator's grid: specialised transforms for
// square power-of-two doubled grids of 128 to 1024 points, else generic.
template <typename T>
static void (*conv_kernel(const orbit_sc2p5d_t* c))(ConvArgs) {
  if (c->nx2 == c->ny2 && c->plan_x.pow2) {
    switch (c->nx2) {
      case 128: return k_conv_fused<T, 7>;
      case 256: return k_conv_fused<T, 8>;
      case 512: return k_conv_fused<T, 9>;
      case 1024: return k_conv_fused<T, 10>;
      default: break;
    }
  }
  return k_conv_fused<T, 0>;
}

// The co-resident block count of the fused convolution (0: it cannot run
// and the separate kernels are used).
template <typename T>
static int init_conv_fused(orbit_sc2p5d_t* c) {
  const void* fn = (const void*)conv_kernel<T>(c);
  size_t sm = conv_smem<T>(c);
  c->conv_blocks = 0;
  int coop = 0, dev = 0;
  ORBIT_CUDA(cudaGetDevice(&dev));
  ORBIT_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop || sm > (size_t)kMaxSmem) return ORBIT_OK;
  if (sm > 48 * 1024) ORBIT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int per_sm = 0;
  ORBIT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, conv_threads(c), sm));
  c->conv_blocks = per_sm * num_sms();
  return ORBIT_OK;
}

static bool use_conv_fused(const orbit_sc2p5d_t* c) {
  return c->fused_conv && c->conv_blocks > 0 && !c->rb && c->d_gscratch && c->d_hat && c->d_green;
}

// The Green rebuild, the forward rows, the convolution and the backward
// rows as one cooperative launch (k_conv_fused).
template <typename T>
static int enqueue_conv_fused(orbit_sc2p5d_t* c, orbit_bunch_t* b, cudaStream_t s, int* nl) {
  ConvArgs A;
  std::memset(&A, 0, sizeof(A));
  A.st = c->d_st;
  A.status = b->d_status;
  A.rho = c->d_rho;
  A.hat = c->d_hat;
  A.green = c->d_green;
  A.gscr = c->d_gscratch;
  A.twx = c->d_tw_x;
  A.twy = c->d_tw_y;
  A.plx = c->plan_x;
  A.ply = c->plan_y;
  A.nx = c->nx; A.ny = c->ny; A.nz = c->nz; A.H = c->H; A.nx2 = c->nx2; A.ny2 = c->ny2;
  A.lam = c->d_lam;
  A.phi = c->d_phi;
  A.denom = 1.0 / (c->nx2 * c->ny2);
  A.wait_polls = c->conv_wait_polls;
  A.withhold = c->conv_withhold;
  A.src = c->d_rho_q;
  A.zacc = c->d_z_q;
  A.lam_f = c->d_lam_f;  // FP32 form: float copies for its kick (null otherwise)
  A.phi_f = c->d_phi_f;
  int items = conv_items(c);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(items < c->conv_blocks ? items : c->conv_blocks);
  cfg.blockDim = dim3(conv_threads(c));
  cfg.dynamicSmemBytes = conv_smem<T>(c);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  ORBIT_PB("fft_conv_fused", s);
  cudaError_t e = cudaLaunchKernelEx(&cfg, conv_kernel<T>(c), A);
  ORBIT_PE(s);
  if (e != cudaSuccess) return cuda_error(e, "sc2p5d fused convolution");
  ++*nl;
  return ORBIT_OK;
}

// Forward row transforms of the deposit (plus one block finalizing the line
// density).
template <typename T>
static int enqueue_rows_fwd(orbit_sc2p5d_t* c, cudaStream_t s, int* nl) {
  typedef typename CT<T>::t C;
  C* hat = (C*)c->d_hat;
  const C* twy = (const C*)c->d_tw_y;
  int thy = fft_threads(c->plan_y);
  size_t smy = fft_smem<T>(c->ny2);
  int blocks = (c->nx + 1) / 2 + 1;
  ORBIT_PB("fft_rows_fwd", s);
  k_rows_fwd<T, 1><<<blocks, thy, smy, s>>>(c->d_st, c->d_rho_q, c->d_rho, hat, twy, c->plan_y, c->nx, c->ny,
                                            c->H, 1, c->d_z_q, c->nz, c->d_lam, c->d_lam_f);
  ORBIT_PE(s);
  ++*nl;
  ORBIT_LAUNCH_CHECK("sc2p5d rows");
  return ORBIT_OK;
}

// Column transforms with the Green multiply, then the backward rows.
template <typename T>
static int enqueue_conv(orbit_sc2p5d_t* c, cudaStream_t s, int* nl) {
  typedef typename CT<T>::t C;
  C* hat = (C*)c->d_hat;
  C* green = (C*)c->d_green;
  const C* twx = (const C*)c->d_tw_x;
  const C* twy = (const C*)c->d_tw_y;
  int thx = fft_threads(c->plan_x), thy = fft_threads(c->plan_y);
  size_t smx = fft_smem<T>(c->nx2), smy = fft_smem<T>(c->ny2);
  double denom = 1.0 / (c->nx2 * c->ny2);
  ORBIT_PB("fft_cols_conv", s);
  k_cols<T, 1><<<c->H, thx, smx, s>>>(c->d_st, hat, green, twx, c->plan_x, c->nx, c->H, c->ny2, 1);
  ORBIT_PE(s);
  ORBIT_PB("fft_rows_inv", s);
  k_rows_inv<T><<<(c->nx + 1) / 2, thy, smy, s>>>(c->d_st, hat, twy, c->plan_y, c->nx, c->ny, c->H, denom,
                                                   c->d_phi, c->d_phi_f);
  ORBIT_PE(s);
  *nl += 2;
  ORBIT_LAUNCH_CHECK("sc2p5d solve");
  return ORBIT_OK;
}

// Green spectrum rebuild.  gate = 1: the kernels return unless the spectrum
// is marked dirty (eager calls); 0: unconditional (the body of a graph
// branch taken on the flag).  `scratch` (nx2 x H complex) holds the row
// spectra.  The Green function is even in x and y: one quadrant is
// evaluated and mirrored, and rows 0..nx are transformed and mirrored.
template <typename T>
static int enqueue_green(orbit_sc2p5d_t* c, cudaStream_t s, int gate, void* scratch, int* nl) {
  typedef typename CT<T>::t C;
  C* green = (C*)c->d_green;
  const C* twx = (const C*)c->d_tw_x;
  const C* twy = (const C*)c->d_tw_y;
  int thx = fft_threads(c->plan_x), thy = fft_threads(c->plan_y);
  size_t smx = fft_smem<T>(c->nx2), smy = fft_smem<T>(c->ny2);
  int quad = (c->nx + 1) * (c->ny + 1);
  int gb = (quad + 255) / 256;
  if (gb > num_sms() * 4) gb = num_sms() * 4;
  ORBIT_PB("green_fill", s);
  k_green_fill<<<gb, 256, 0, s>>>(c->d_st, c->d_gbuf, c->nx2, c->ny2, gate);
  ORBIT_PE(s);
  ORBIT_PB("green_rows", s);
  C* hat = (C*)scratch;
  k_rows_fwd<T, 0><<<(c->nx + 2) / 2, thy, smy, s>>>(c->d_st, c->d_gbuf, nullptr, hat, twy, c->plan_y,
                                                      c->nx + 1, c->ny2, c->H, gate, nullptr, 0, nullptr, nullptr);
  ORBIT_PE(s);
  ORBIT_PB("green_cols", s);
  k_cols<T, 0><<<c->H, thx, smx, s>>>(c->d_st, hat, green, twx, c->plan_x, c->nx2, c->H, c->ny2, gate);
  ORBIT_PE(s);
  *nl += 3;
  ORBIT_LAUNCH_CHECK("sc2p5d green");
  return ORBIT_OK;
}

// FFT block size of a batch class: power-of-two lengths N/2 threads
// (radix-2 stages) or N/4 (radix-4 stages); other lengths the generic block.
static int batch_fft_threads(const FftPlan& pl, int wide) {
  if (!pl.pow2) return fft_threads(pl);
  int t = wide ? pl.n / 2 : pl.n / 4;
  if (t < 32) t = 32;
  if (t > 1024) t = 1024;
  return t;
}

bool batch_deposit_smem(const orbit_sc2p5d_t* c) {
  return 8 * ((size_t)c->nx * c->ny + c->nz) <= (size_t)kMaxSmem;
}

int batch_deposit_bands(const orbit_sc2p5d_t* c) {
  if (batch_deposit_smem(c) || !c->band_deposit) return 1;
  int nb;
  band_rows(c->nx, c->ny, c->nz, &nb);
  return nb;
}

int batch_init_attrs(const orbit_sc2p5d_t* c) {
  int bytes = (int)fft_smem<double>(c->nx2 > c->ny2 ? c->nx2 : c->ny2);
  if (bytes > 48 * 1024) {
    ORBIT_CUDA(cudaFuncSetAttribute(kb_rows_fwd<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    ORBIT_CUDA(cudaFuncSetAttribute(kb_rows_fwd<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    ORBIT_CUDA(cudaFuncSetAttribute(kb_cols<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    ORBIT_CUDA(cudaFuncSetAttribute(kb_cols<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    ORBIT_CUDA(cudaFuncSetAttribute(kb_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  }
  size_t dep = 8 * ((size_t)c->nx * c->ny + c->nz);
  if (dep <= (size_t)kMaxSmem && dep > 48 * 1024)
    ORBIT_CUDA(cudaFuncSetAttribute(kb_deposit<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
  if (c->band_deposit && band_smem(c->nx, c->ny, c->nz) > 48 * 1024)
    ORBIT_CUDA(cudaFuncSetAttribute(kb_deposit_band, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
  return ORBIT_OK;
}

// Green spectra of the members whose solver grid changed (each member's
// blocks return unless its spectrum is dirty); the work spectra hold the
// row transforms, before the deposit.
int batch_enqueue_green(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* c, int fft_wide, cudaStream_t s) {
  int thx = batch_fft_threads(c->plan_x, fft_wide), thy = batch_fft_threads(c->plan_y, fft_wide);
  size_t smx = fft_smem<double>(c->nx2), smy = fft_smem<double>(c->ny2);
  int quad = (c->nx + 1) * (c->ny + 1);
  int gb = (quad + 255) / 256;
  if (gb > 64) gb = 64;
  ORBIT_PB("batch_green_fill", s);
  kb_green_fill<<<dim3(gb, nm), 256, 0, s>>>(jobs, c->nx2, c->ny2);
  ORBIT_PE(s);
  ORBIT_PB("batch_green_rows", s);
  kb_rows_fwd<0><<<dim3((c->nx + 2) / 2, nm), thy, smy, s>>>(jobs, c->plan_y, c->nx + 1, c->ny2, c->H, 0);
  ORBIT_PE(s);
  ORBIT_PB("batch_green_cols", s);
  kb_cols<0><<<dim3(c->H, nm), thx, smx, s>>>(jobs, c->plan_x, c->nx2, c->H, c->ny2);
  ORBIT_PE(s);
  ORBIT_LAUNCH_CHECK("batch green");
  return ORBIT_OK;
}

int batch_enqueue_deposit(const DepJob* jobs, const BlockMap& bm, const orbit_sc2p5d_t* c, int threads,
                          cudaStream_t s, const char* tag) {
  size_t sm = 8 * ((size_t)c->nx * c->ny + c->nz);
  ORBIT_PB(tag, s);
  if (batch_deposit_smem(c)) {
    kb_deposit<true><<<bm.nblk, threads, sm, s>>>(jobs, bm.blk_job, bm.mblk, c->nx, c->ny, c->nz);
  } else if (c->band_deposit) {
    int nb;
    int rpb = band_rows(c->nx, c->ny, c->nz, &nb);
    kb_deposit_band<<<bm.nblk, threads, band_smem(c->nx, c->ny, c->nz), s>>>(jobs, bm.blk_job, bm.mblk, c->nx, c->ny,
                                                                           c->nz, rpb, nb);
  } else {
    kb_deposit<false><<<bm.nblk, threads, 0, s>>>(jobs, bm.blk_job, bm.mblk, c->nx, c->ny, c->nz);
  }
  ORBIT_PE(s);
  ORBIT_LAUNCH_CHECK("batch deposit");
  return ORBIT_OK;
}

int batch_enqueue_fft_probe(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* c, int fft_wide, cudaStream_t s) {
  int thx = batch_fft_threads(c->plan_x, fft_wide), thy = batch_fft_threads(c->plan_y, fft_wide);
  size_t smx = fft_smem<double>(c->nx2), smy = fft_smem<double>(c->ny2);
  kb_cols<1><<<dim3(c->H, nm), thx, smx, s>>>(jobs, c->plan_x, c->nx, c->H, c->ny2);
  kb_rows_inv<<<dim3((c->nx + 1) / 2, nm), thy, smy, s>>>(jobs, c->plan_y, c->nx, c->ny, c->H,
                                                          1.0 / (c->nx2 * c->ny2));
  ORBIT_LAUNCH_CHECK("batch FFT probe");
  return ORBIT_OK;
}

// Forward rows (+ line-density finalize), columns with the Green multiply,
// backward rows, and the fixed-point potential for kicks that read it from
// global memory.
int batch_enqueue_solve(const SolveJob* jobs, int nm, const orbit_sc2p5d_t* c, int fft_wide, bool phi_fix,
                        cudaStream_t s) {
  int thx = batch_fft_threads(c->plan_x, fft_wide), thy = batch_fft_threads(c->plan_y, fft_wide);
  size_t smx = fft_smem<double>(c->nx2), smy = fft_smem<double>(c->ny2);
  ORBIT_PB("batch_rows_fwd", s);
  kb_rows_fwd<1><<<dim3((c->nx + 1) / 2 + 1, nm), thy, smy, s>>>(jobs, c->plan_y, c->nx, c->ny, c->H, c->nz);
  ORBIT_PE(s);
  ORBIT_PB("batch_cols_conv", s);
  kb_cols<1><<<dim3(c->H, nm), thx, smx, s>>>(jobs, c->plan_x, c->nx, c->H, c->ny2);
  ORBIT_PE(s);
  ORBIT_PB("batch_rows_inv", s);
  kb_rows_inv<<<dim3((c->nx + 1) / 2, nm), thy, smy, s>>>(jobs, c->plan_y, c->nx, c->ny, c->H,
                                                          1.0 / (c->nx2 * c->ny2));
  ORBIT_PE(s);
  if (phi_fix) {
    int ng = c->nx * c->ny;
    int m = ng > c->nz ? ng : c->nz;
    ORBIT_PB("batch_phi_fix", s);
    kb_phi_fix<<<dim3((m + 255) / 256, nm), 256, 0, s>>>(jobs, ng, c->nz);
    ORBIT_PE(s);
  }
  ORBIT_LAUNCH_CHECK("batch solve");
  return ORBIT_OK;
}

// Largest block the kernel can launch with (its registers per thread).
template <typename K>
static int max_threads_of(K kernel) {
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, (const void*)kernel) != cudaSuccess) return 256;
  return a.maxThreadsPerBlock;
}

// Block-size limits of the particle kernels: deposit (shared, global), kick
// plain (shared, global), kick fp32 (shared, global).  Queried once,
// outside any stream capture (init_attrs).
static const int* particle_kernel_threads() {
  static const int mt[6] = {max_threads_of(k_deposit_plain<true>), max_threads_of(k_deposit_plain<false>),
                            max_threads_of(k_kick_plain<true>), max_threads_of(k_kick_plain<false>),
                            max_threads_of(k_kick_fp32<true>), max_threads_of(k_kick_fp32<false>)};
  return mt;
}

static double qscale_for(double msum_abs) {
  double M = msum_abs;
  if (!(M > 0.0) || !std::isfinite(M)) return 1.0;
  int e = 0;
  std::frexp(M, &e);  // M < 2^e
  return std::ldexp(1.0, 61 - e);
}

// Fixed-point units of the plain deposit.  Uniform macrosize: unit weight
// in units of 2^-K with 4 n 2^K < 2^62 (a particle's |weights| sum to at
// most 4), the macrosize multiplies the grid afterwards.  Per-particle
// macrosizes: macrosize * S with S * sum|m| <= 2^61.
DepScales sc_dep_scales(const orbit_sc2p5d_t* c, const orbit_bunch_t* b) {
  (void)c;
  DepScales d;
  d.K = 0;
  d.S = 1.0;
  d.inv_q = 1.0;
  d.ms_uniform = 0.0;
  if (!b->has_msize) {
    int e = 0;
    std::frexp(4.0 * (double)(b->n > 0 ? b->n : 1), &e);  // 4n < 2^e
    d.K = 62 - e;
    if (d.K > 55) d.K = 55;
    d.ms_uniform = std::ldexp(1.0, d.K);
    d.inv_q = std::ldexp(b->sync.macrosize, -d.K);
  } else {
    d.S = qscale_for(b->msize_abs_sum);
    d.inv_q = 1.0 / d.S;
  }
  return d;
}

SetupArgs sc_setup_args(const orbit_sc2p5d_t* c, const DepScales& d, const orbit_boundary* bnd) {
  SetupArgs sa;
  sa.inv_qscale = d.inv_q;  // both forms deposit in fixed point
  sa.nx = c->nx;
  sa.ny = c->ny;
  sa.nz = c->nz;
  sa.rb = c->rb ? 1 : 0;
  sa.cond = 0;
  sa.bnd = 0;
  sa.bxmin = sa.bxmax = sa.bymin = sa.bymax = 0.0;
  if (bnd) {
    int np, nm, shape, init;
    double lim[4];
    orbit_boundary_info(bnd, &np, &nm, &shape, lim, &init);
    sa.bnd = 1;
    sa.bxmin = lim[0]; sa.bxmax = lim[1]; sa.bymin = lim[2]; sa.bymax = lim[3];
  }
  return sa;
}

cudaGraphConditionalHandle sc_green_cond(orbit_sc2p5d_t* c, cudaStream_t s, bool pending) {
  if (!c->aux || !c->d_gscratch || use_conv_fused(c)) return 0;  // the fused convolution rebuilds in place
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess) return 0;
  if (cs != cudaStreamCaptureStatusActive) return 0;
  cudaGraphConditionalHandle h = 0;
  if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return 0;
  if (pending) {
    c->pending_cond = h;
    c->pending_graph = g;
  }
  return h;
}

void sc_clear_pending(orbit_sc2p5d_t* c) {
  c->pending_cond = 0;
  c->pending_graph = nullptr;
}

// Inside a stream capture: a conditional graph node, depending on what the
// stream's next work would depend on (the deposit), whose body rebuilds the
// Green spectrum into its own scratch.  The set-up took the branch when the
// spectrum is dirty; the stream's dependencies are left as they were, so
// the forward rows run beside the branch and the caller joins it before
// the column transforms.
static int add_green_branch(orbit_sc2p5d_t* c, cudaStream_t s, cudaGraphConditionalHandle cond,
                            cudaGraphNode_t* node_out) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  ORBIT_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  ORBIT_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  ORBIT_CUDA(cudaStreamBeginCaptureToGraph(c->aux, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int bl = 0;
  int rc = c->form == ORBIT_FORM_PLAIN ? enqueue_green<double>(c, c->aux, 0, c->d_gscratch, &bl)
                                       : enqueue_green<float>(c, c->aux, 0, c->d_gscratch, &bl);
  cudaGraph_t out = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->aux, &out);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_error(e, "sc2p5d: Green branch capture");
  *node_out = node;
  return ORBIT_OK;
}

// The learned closure's check: the raw deposit (FP64 copy) solved into its
// own buffers with the calculator's Green spectrum, in its precision.
template <typename T>
static void enqueue_check_solve(orbit_sc2p5d_t* c, cudaStream_t s) {
  typedef typename CT<T>::t C;
  const int thx = fft_threads(c->plan_x), thy = fft_threads(c->plan_y);
  const size_t smx = fft_smem<T>(c->nx2), smy = fft_smem<T>(c->ny2);
  k_rows_fwd<T, 3><<<(c->nx + 1) / 2, thy, smy, s>>>(c->d_dn_st, c->d_dn_raw, nullptr, (C*)c->d_dn_hat,
                                                       (const C*)c->d_tw_y, c->plan_y, c->nx, c->ny, c->H, 1,
                                                       nullptr, 0, nullptr, nullptr);
  k_cols<T, 1><<<c->H, thx, smx, s>>>(c->d_dn_st, (C*)c->d_dn_hat, (C*)c->d_green, (const C*)c->d_tw_x, c->plan_x,
                                        c->nx, c->H, c->ny2, 1);
  k_rows_inv<T><<<(c->nx + 1) / 2, thy, smy, s>>>(c->d_dn_st, (const C*)c->d_dn_hat, (const C*)c->d_tw_y,
                                                    c->plan_y, c->nx, c->ny, c->H, 1.0 / (c->nx2 * c->ny2),
                                                    c->d_dn_phi, nullptr);
}

int sc_enqueue_kick(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, cudaStream_t s, bool do_extrema,
                    bool do_kick, int* launches, double pipe_radius, const orbit_boundary* bnd) {
  int nl = 0;
  const int n = b->n;
  const double* msz = b->has_msize ? b->d_msize : nullptr;
  const bool plain = c->form == ORBIT_FORM_PLAIN;
  const DepScales ds = sc_dep_scales(c, b);
  // Inside a graph the Green rebuild is a conditional branch beside the
  // forward rows, taken by the set-up (run by the extrema scan here, or by
  // the fused pass that created the pending handle); otherwise its kernels
  // run first and return unless the spectrum is dirty.
  cudaGraphConditionalHandle cond = 0;
  if (do_extrema) {
    SetupArgs sa = sc_setup_args(c, ds, bnd);
    sa.cond = cond = sc_green_cond(c, s, false);
    ORBIT_PB("extrema", s);
    k_extrema<<<ext_blocks(n), 256, 0, s>>>(b->coord(0), b->coord(2), b->coord(4), n, c->d_st, b->d_status, sa);
    ORBIT_PE(s);
    ++nl;
  } else if (c->pending_cond) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    ORBIT_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, nullptr, nullptr, nullptr));
    if (cs == cudaStreamCaptureStatusActive && cg == c->pending_graph) cond = c->pending_cond;
  }
  sc_clear_pending(c);
  cudaGraphNode_t branch_node = nullptr;
  int rc;
  const bool fused = use_conv_fused(c);
  if (!cond && !fused) {
    // before the deposit: the work spectrum is free to hold the row spectra
    rc = plain ? enqueue_green<double>(c, s, 1, c->d_hat, &nl) : enqueue_green<float>(c, s, 1, c->d_hat, &nl);
    if (rc) return rc;
  }
  // both forms: the exact fixed-point deposit
  size_t sm = sizeof(unsigned long long) * ((size_t)c->nx * c->ny + c->nz);
  int blocks, threads;
  const int* mt_dep = particle_kernel_threads();
  particle_geometry(c->smem_deposit ? sm : 0, n, mt_dep[c->smem_deposit ? 0 : 1], &blocks, &threads);
  ORBIT_PB("deposit", s);
  {
    if (c->smem_deposit) {
      k_deposit_plain<true><<<blocks, threads, sm, s>>>(b->coord(0), b->coord(2), b->coord(4), msz, n, c->d_st,
                                                        c->d_rho_q, c->d_z_q, ds.ms_uniform, ds.S, c->nx, c->ny,
                                                        c->nz, ds.K);
    } else if (c->band_deposit) {
      // the grid in row bands, each block one band of one particle chunk
      int nb;
      int rpb = band_rows(c->nx, c->ny, c->nz, &nb);
      // one block per SM (each holds a band of the grid): at most one wave,
      // so that no block starts after the others have finished
      int chunks = (n + 2047) / 2048, cap = num_sms() / nb > 0 ? num_sms() / nb : 1;
      chunks = chunks < 1 ? 1 : (chunks > cap ? cap : chunks);
      int bt = max_threads_of(k_deposit_band);
      bt = bt > 768 ? 768 : (bt & ~31);
      k_deposit_band<<<chunks * nb, bt, band_smem(c->nx, c->ny, c->nz), s>>>(
          b->coord(0), b->coord(2), b->coord(4), msz, n, c->d_st, c->d_rho_q, c->d_z_q, ds.ms_uniform, ds.S, c->nx,
          c->ny, c->nz, ds.K, rpb, nb);
    } else {
      k_deposit_plain<false><<<blocks, threads, 0, s>>>(b->coord(0), b->coord(2), b->coord(4), msz, n, c->d_st,
                                                        c->d_rho_q, c->d_z_q, ds.ms_uniform, ds.S, c->nx, c->ny,
                                                        c->nz, ds.K);
    }
  }
  ORBIT_PE(s);
  ++nl;
  ORBIT_LAUNCH_CHECK("sc2p5d deposit");
  // learned closure: the network denoises the deposit before the solve
  bool dn_check = false;
  double dn_scale = 0.0;
  if (c->dn && !c->rb && !bnd) {
    if (b->has_msize)
      return set_error(ORBIT_ERR_UNSUPPORTED, "the learned closure needs a uniform macrosize");
    const double M = (double)n * b->sync.macrosize;
    if (M > 0.0) {
      const int ng = c->nx * c->ny;
      dn_check = (c->dn_count++ % c->dn_every) == 0;
      dn_scale = (double)ng / M;
      int gb = (ng + 255) / 256;
      if (gb > num_sms() * 2) gb = num_sms() * 2;
      ORBIT_PB("learn_in", s);
      float* img = nullptr;
      const float* out = nullptr;
      int nparts = 0;
      rc = dn_closure_io(c->dn, &img, &out, &nparts);
      if (rc) return rc;
      if (nparts > kDnMaxParts) return set_error(ORBIT_ERR_UNSUPPORTED, "the learned closure's grid is too large");
      k_learn_in<<<gb, 256, 0, s>>>(c->d_st, c->d_rho_q, img, dn_check ? c->d_dn_raw : nullptr, ng, dn_scale);
      ORBIT_PE(s);
      ORBIT_PB("learn_network", s);
      rc = dn_forward_inplace(c->dn, s, c->d_dn_parts);
      ORBIT_PE(s);
      if (rc) return rc;
      ORBIT_PB("learn_out", s);
      k_learn_out<<<gb, 256, 0, s>>>(c->d_st, out, c->d_rho_q, ng, dn_scale, c->d_dn_parts, nparts,
                                     dn_error_flag(c->dn));
      ORBIT_PE(s);
      nl += 2;
      ORBIT_LAUNCH_CHECK("sc2p5d learned closure");
    }
  }
  if (cond) {
    // beside the forward rows, which leave most SMs free (the deposit fills them)
    rc = add_green_branch(c, s, cond, &branch_node);
    if (rc) return rc;
  }
  if (fused) {
    rc = plain ? enqueue_conv_fused<double>(c, b, s, &nl) : enqueue_conv_fused<float>(c, b, s, &nl);
    if (rc) return rc;
  } else {
    rc = plain ? enqueue_rows_fwd<double>(c, s, &nl) : enqueue_rows_fwd<float>(c, s, &nl);
    if (rc) return rc;
  }
  if (c->rb) {
    // beam centre, a_bunch and the derivative grid from the finished grids
    ORBIT_PB("rb_analysis", s);
    k_rb_analysis<<<1, 512, 0, s>>>(c->d_st, c->d_rho, c->d_lam, c->d_lamd, c->nx, c->ny, c->nz, c->n_long_avg,
                                     pipe_radius);
    ORBIT_PE(s);
    ++nl;
    ORBIT_LAUNCH_CHECK("sc2p5drb analysis");
  }
  if (branch_node)  // the column transforms read the Green spectrum
    ORBIT_CUDA(cudaStreamUpdateCaptureDependencies(s, &branch_node, nullptr, 1, cudaStreamAddCaptureDependencies));
  if (!fused) {
    rc = plain ? enqueue_conv<double>(c, s, &nl) : enqueue_conv<float>(c, s, &nl);
    if (rc) return rc;
  }
  if (dn_check) {
    // the raw deposit solved beside the denoised one (in the calculator's
    // own precision: its Green spectrum and twiddles), and the check
    ORBIT_PB("learn_check", s);
    k_learn_chk_prep<<<1, 1, 0, s>>>(c->d_st, c->d_dn_st);
    if (plain)
      enqueue_check_solve<double>(c, s);
    else
      enqueue_check_solve<float>(c, s);
    k_learn_compare<<<1, 1024, 0, s>>>(c->d_st, c->d_phi, c->d_dn_phi, c->nx * c->ny, c->dn_bound);
    ORBIT_PE(s);
    nl += 5;
    ORBIT_LAUNCH_CHECK("sc2p5d learned closure check");
  }
  if (bnd) {
    rc = bnd_enqueue_potential(bnd, c, s, &nl);
    if (rc) return rc;
  }
  if (plain && !c->smem_kick) {
    // kicks that read the potential from global memory take it converted
    // once; the shared-memory kicks convert their own copy
    int ng = c->nx * c->ny;
    int m = ng > c->nz ? ng : c->nz;
    ORBIT_PB("phi_fix", s);
    k_phi_fix<<<(m + 255) / 256, 256, 0, s>>>(c->d_st, c->d_phi, c->d_lam, c->d_phi_fix, c->d_lam_fix, ng, c->nz);
    ORBIT_PE(s);
    ++nl;
    ORBIT_LAUNCH_CHECK("sc2p5d phi_fix");
  }
  if (do_kick) {
    double hf = sc_host_factor(b->sync, length);
    const double* lamd = c->rb ? c->d_lamd : nullptr;
    double lsf = c->rb ? sc_rb_long_factor(b->sync, length) : 0.0;
    BndShape bshape = bnd_shape_of(bnd);
    size_t smk = (plain ? sizeof(double) : sizeof(float)) * ((size_t)c->nx * c->ny + c->nz);
    const int* mt_kick = particle_kernel_threads() + 2;
    particle_geometry(c->smem_kick ? smk : 0, n, mt_kick[(plain ? 0 : 2) + (c->smem_kick ? 0 : 1)], &blocks,
                      &threads);
    ORBIT_PB("kick", s);
    if (plain) {
      if (c->smem_kick)
        k_kick_plain<true><<<blocks, threads, smk, s>>>(b->coord(0), b->coord(1), b->coord(2), b->coord(3),
                                                        b->coord(4), n, c->d_st, c->d_phi, c->d_lam, c->d_phi_fix,
                                                        c->d_lam_fix, hf, c->nx, c->ny, c->nz, lamd, lsf,
                                                        b->coord(5), bshape);
      else
        k_kick_plain<false><<<blocks, threads, 0, s>>>(b->coord(0), b->coord(1), b->coord(2), b->coord(3),
                                                       b->coord(4), n, c->d_st, c->d_phi, c->d_lam, c->d_phi_fix,
                                                       c->d_lam_fix, hf, c->nx, c->ny, c->nz, lamd, lsf,
                                                       b->coord(5), bshape);
    } else {
      if (c->smem_kick)
        k_kick_fp32<true><<<blocks, threads, smk, s>>>(b->coord(0), b->coord(1), b->coord(2), b->coord(3),
                                                       b->coord(4), n, c->d_st, c->d_phi_f, c->d_lam_f, hf, c->nx,
                                                       c->ny, c->nz, bshape);
      else
        k_kick_fp32<false><<<blocks, threads, 0, s>>>(b->coord(0), b->coord(1), b->coord(2), b->coord(3),
                                                      b->coord(4), n, c->d_st, c->d_phi_f, c->d_lam_f, hf, c->nx,
                                                      c->ny, c->nz, bshape);
    }
    ORBIT_PE(s);
    ++nl;
    ORBIT_LAUNCH_CHECK("sc2p5d kick");
  }

  if (launches) *launches += nl;
  return ORBIT_OK;
}

cudaError_t sc_order_before(orbit_sc2p5d_t* c, cudaStream_t s) {
  return c->used ? cudaStreamWaitEvent(s, c->done, 0) : cudaSuccess;
}

cudaError_t sc_mark_used(orbit_sc2p5d_t* c, cudaStream_t s) {
  c->used = true;
  return cudaEventRecord(c->done, s);
}

static int init_attrs(orbit_sc2p5d_t* c) {
  particle_kernel_threads();
  // both forms deposit into the exact fixed-point grids (two 32-bit words
  // per cell in shared memory); the FP32 form's kick reads a float copy
  size_t dep = 8 * ((size_t)c->nx * c->ny + c->nz);
  size_t kick = (c->form == ORBIT_FORM_PLAIN ? 8 : 4) * ((size_t)c->nx * c->ny + c->nz);
  c->smem_deposit = dep <= (size_t)kMaxSmem;
  c->smem_kick = kick <= (size_t)kMaxSmem;
  size_t bs = band_smem(c->nx, c->ny, c->nz);
  c->band_deposit = !c->smem_deposit && bs <= (size_t)kMaxSmem;
  if (c->band_deposit && bs > 48 * 1024)
    ORBIT_CUDA(cudaFuncSetAttribute(k_deposit_band, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
  if (c->smem_deposit && dep > 48 * 1024)
    ORBIT_CUDA(cudaFuncSetAttribute(k_deposit_plain<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
  if (c->form == ORBIT_FORM_PLAIN) {
    if (c->smem_kick && kick > 48 * 1024)
      ORBIT_CUDA(cudaFuncSetAttribute(k_kick_plain<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
    int nmax = c->nx2 > c->ny2 ? c->nx2 : c->ny2;
    int rc = set_fft_attrs<double>(nmax);
    return rc ? rc : init_conv_fused<double>(c);
  }
  if (c->smem_kick && kick > 48 * 1024)
    ORBIT_CUDA(cudaFuncSetAttribute(k_kick_fp32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem));
  int nmax = c->nx2 > c->ny2 ? c->nx2 : c->ny2;
  int rc = set_fft_attrs<float>(nmax);
  return rc ? rc : init_conv_fused<float>(c);
}

}  // namespace orbit

using namespace orbit;

extern "C" {

int orbit_sc2p5d_create(orbit_sc2p5d_t** out, int nx, int ny, int nz, double xy_ratio, int form) {
  if (!out) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_create: null output");
  if (nx < 3 || ny < 3)
    return set_error(ORBIT_ERR_GRID, "Grid2D: the grid size too small (should be more than 3)");
  if (nz < 1) return set_error(ORBIT_ERR_GRID, "Grid1D: the grid size is too small (should be more than 0)");
  if (form != ORBIT_FORM_PLAIN && form != ORBIT_FORM_FP32)
    return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_create: unknown form");
  if (nx > 2048 || ny > 2048)
    return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_sc2p5d_create: nx, ny above 2048 are not supported");
  orbit_sc2p5d_t* c = new orbit_sc2p5d_t();
  c->nx = nx; c->ny = ny; c->nz = nz; c->form = form;
  c->nx2 = 2 * nx; c->ny2 = 2 * ny; c->H = ny + 1;
  c->xy_ratio0 = xy_ratio > 0. ? xy_ratio : 1.0;
  if (!make_fft_plan(c->nx2, c->plan_x) || !make_fft_plan(c->ny2, c->plan_y)) {
    delete c;
    return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_sc2p5d_create: grid sizes must have no prime factor above 13");
  }
  size_t ng = (size_t)nx * ny;
  size_t nhat = (size_t)c->nx2 * c->H;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
  };
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
  A((void**)&c->d_st, sizeof(ScState));
  A((void**)&c->d_rho, sizeof(double) * ng);
  A((void**)&c->d_phi, sizeof(double) * ng);
  A((void**)&c->d_lam, sizeof(double) * nz);
  A((void**)&c->d_lamd, sizeof(double) * nz);
  A((void**)&c->d_gbuf, sizeof(double) * (size_t)c->nx2 * c->ny2);
  // both forms: the fixed-point deposit grids
  A((void**)&c->d_rho_q, sizeof(unsigned long long) * ng);
  A((void**)&c->d_z_q, sizeof(unsigned long long) * nz);
  if (form == ORBIT_FORM_PLAIN) {
    A((void**)&c->d_phi_fix, sizeof(long long) * ng);
    A((void**)&c->d_lam_fix, sizeof(long long) * nz);
    A(&c->d_hat, sizeof(double2) * nhat);
    A(&c->d_green, sizeof(double2) * nhat);
    A(&c->d_gscratch, sizeof(double2) * nhat);
    if (e == cudaSuccess) c->d_tw_x = make_twiddles<double>(c->nx2, &e);
    if (e == cudaSuccess) c->d_tw_y = make_twiddles<double>(c->ny2, &e);
  } else {
    A((void**)&c->d_phi_f, sizeof(float) * ng);
    A((void**)&c->d_lam_f, sizeof(float) * nz);
    A(&c->d_hat, sizeof(float2) * nhat);
    A(&c->d_green, sizeof(float2) * nhat);
    A(&c->d_gscratch, sizeof(float2) * nhat);
    if (e == cudaSuccess) c->d_tw_x = make_twiddles<float>(c->nx2, &e);
    if (e == cudaSuccess) c->d_tw_y = make_twiddles<float>(c->ny2, &e);
  }
  if (e != cudaSuccess) {
    orbit_sc2p5d_destroy(c);
    return cuda_error(e, "orbit_sc2p5d_create");
  }
  // constructor state (SpaceChargeCalc2p5D.cc:25-43): solver on (-r,r,-1,1),
  // grids on (-1,1)^2 and (-0.5,0.5); the Green spectrum is built lazily on
  // the first kick (green_dirty).
  ScState h;
  std::memset(&h, 0, sizeof(h));
  double r = c->xy_ratio0;
  h.xy_ratio = r;
  h.sxmin = -r; h.sxmax = r; h.symin = -1.0; h.symax = 1.0;
  h.sdx = (r - (-r)) / (nx - 1);
  h.sdy = (1.0 - (-1.0)) / (ny - 1);
  h.xmin = -1.0; h.xmax = 1.0; h.ymin = -1.0; h.ymax = 1.0;
  h.dx = 2.0 / (nx - 1); h.dy = 2.0 / (ny - 1); h.inv_dx = 1.0 / h.dx; h.inv_dy = 1.0 / h.dy;
  h.zmin = -0.5; h.zmax = 0.5; h.dz = 1.0 / nz; h.inv_dz = 1.0 / h.dz;
  h.green_dirty = 1;
  h.skip = 0;
  for (int k = 0; k < 3; ++k) { h.key[2 * k] = ~0ull; h.key[2 * k + 1] = 0ull; }
  e = cudaMemcpy(c->d_st, &h, sizeof(h), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    orbit_sc2p5d_destroy(c);
    return cuda_error(e, "orbit_sc2p5d_create");
  }
  int rc = init_attrs(c);
  if (rc) {
    orbit_sc2p5d_destroy(c);
    return rc;
  }
  *out = c;
  return ORBIT_OK;
}

int orbit_sc2p5d_destroy(orbit_sc2p5d_t* c) {
  if (!c) return ORBIT_OK;
  if (c->used) cudaEventSynchronize(c->done);
  if (c->done) cudaEventDestroy(c->done);
  if (c->aux) cudaStreamDestroy(c->aux);
  void* ptrs[] = {c->d_st, c->d_rho_q, c->d_z_q, c->d_rho, c->d_phi, c->d_lam, c->d_lamd,
                  c->d_phi_f, c->d_lam_f, c->d_hat, c->d_green, c->d_gbuf, c->d_gscratch, c->d_tw_x, c->d_tw_y,
                  c->d_phi_fix, c->d_lam_fix, c->d_dn_parts, c->d_dn_raw, c->d_dn_hat, c->d_dn_phi,
                  c->d_dn_st};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete c;
  return ORBIT_OK;
}

int orbit_sc2p5d_set_denoiser(orbit_sc2p5d_t* c, orbit_denoiser_t* dn, int check_every, double bound) {
  if (!c || (dn && (check_every < 1 || !(bound > 0.0))))
    return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_set_denoiser: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ++c->cfg_gen;
  if (!dn) {
    c->dn = nullptr;
    return ORBIT_OK;
  }
  if (c->rb)
    return set_error(ORBIT_ERR_UNSUPPORTED, "the learned closure is built for the 2.5D calculator (plain or FP32 form)");
  int h = 0, w = 0, mb = 0;
  int rc = orbit_denoiser_info(dn, nullptr, &h, &w, &mb);
  if (rc) return rc;
  if (h != c->nx || w != c->ny)
    return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_set_denoiser: the network's image size differs from the grid");
  const size_t ng = (size_t)c->nx * c->ny;
  if (!c->d_dn_parts) {
    ORBIT_CUDA(cudaMalloc(&c->d_dn_parts, sizeof(double) * kDnMaxParts));
    ORBIT_CUDA(cudaMalloc(&c->d_dn_raw, sizeof(double) * ng));
    ORBIT_CUDA(cudaMalloc(&c->d_dn_hat, sizeof(double2) * (size_t)c->nx2 * c->H));
    ORBIT_CUDA(cudaMalloc(&c->d_dn_phi, sizeof(double) * ng));
    ORBIT_CUDA(cudaMalloc(&c->d_dn_st, sizeof(ScState)));
    ORBIT_CUDA(cudaMemset(c->d_dn_st, 0, sizeof(ScState)));
  }
  c->dn = dn;
  c->dn_every = check_every;
  c->dn_bound = bound;
  c->dn_count = 0;
  return orbit_sc2p5d_denoiser_reset(c);
}

int orbit_sc2p5d_denoiser_state(orbit_sc2p5d_t* c, int* fallback, long long* checks, long long* trips,
                                double* last_err) {
  if (!c) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_denoiser_state: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ScState h;
  ORBIT_CUDA(cudaMemcpy(&h, c->d_st, sizeof(h), cudaMemcpyDeviceToHost));
  if (fallback) *fallback = h.dn_fallback;
  if (checks) *checks = (long long)h.dn_checks;
  if (trips) *trips = (long long)h.dn_trips;
  if (last_err) *last_err = h.dn_err;
  return ORBIT_OK;
}

int orbit_sc2p5d_denoiser_reset(orbit_sc2p5d_t* c) {
  if (!c) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_denoiser_reset: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ScState h;
  ORBIT_CUDA(cudaMemcpy(&h, c->d_st, sizeof(h), cudaMemcpyDeviceToHost));
  h.dn_fallback = 0;
  h.dn_err = 0.0;
  h.dn_checks = 0;
  h.dn_trips = 0;
  ORBIT_CUDA(cudaMemcpy(c->d_st, &h, sizeof(h), cudaMemcpyHostToDevice));
  return ORBIT_OK;
}

int orbit_sc2p5d_track_boundary(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, const orbit_boundary_t* bnd) {
  ORBIT_NVTX("SpaceChargeCalc2p5D.trackBunch(boundary)");
  if (!c || !b) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_track_boundary: null handle");
  if (c->rb) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_track_boundary: a 2.5Drb calculator has no boundary");
  if (!bnd) return orbit_sc2p5d_track(c, b, length);
  int np, nm, shape, init;
  double lim[4];
  orbit_boundary_info(bnd, &np, &nm, &shape, lim, &init);
  if (!init)  // BaseBoundary2D.cc:354-363
    return set_error(ORBIT_ERR_ARG, "Boundary2D: the boundary was not initialized, call initialize()");
  if (b->n < 2) return ORBIT_OK;
  int rc = bnd_ensure_device(const_cast<orbit_boundary_t*>(bnd));
  if (rc) return rc;
  ORBIT_CUDA(sc_order_before(c, b->stream));
  rc = sc_enqueue_kick(c, b, length, b->stream, true, true, nullptr, 0.0, bnd);
  if (rc) return rc;
  ORBIT_CUDA(sc_mark_used(c, b->stream));
  return ORBIT_OK;
}

int orbit_sc2p5drb_create(orbit_sc2p5d_t** out, int nx, int ny, int nz, double xy_ratio) {
  int rc = orbit_sc2p5d_create(out, nx, ny, nz, xy_ratio, ORBIT_FORM_PLAIN);
  if (rc) return rc;
  (*out)->rb = true;
  (*out)->n_long_avg = 3;  // SpaceChargeCalc2p5Drb.cc:42
  return ORBIT_OK;
}

int orbit_sc2p5drb_set_long_avg(orbit_sc2p5d_t* c, int n) {
  if (!c || !c->rb || n < 1) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5drb_set_long_avg: bad argument");
  c->n_long_avg = n;
  return ORBIT_OK;
}

int orbit_sc2p5drb_get_long_avg(const orbit_sc2p5d_t* c, int* n) {
  if (!c || !c->rb || !n) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5drb_get_long_avg: bad argument");
  *n = c->n_long_avg;
  return ORBIT_OK;
}

int orbit_sc2p5drb_track(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length, double pipe_radius) {
  ORBIT_NVTX("SpaceChargeCalc2p5Drb.trackBunch");
  if (!c || !b || !c->rb) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5drb_track: null or non-2.5Drb handle");
  if (b->n < 2) return ORBIT_OK;  // SpaceChargeCalc2p5Drb.cc:109-110
  ORBIT_CUDA(sc_order_before(c, b->stream));
  int rc = sc_enqueue_kick(c, b, length, b->stream, true, true, nullptr, pipe_radius);
  if (rc) return rc;
  ORBIT_CUDA(sc_mark_used(c, b->stream));
  return ORBIT_OK;
}

int orbit_sc2p5drb_beam(orbit_sc2p5d_t* c, double* abx) {
  if (!c || !c->rb || !abx) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5drb_beam: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ScState h;
  ORBIT_CUDA(cudaMemcpy(&h, c->d_st, sizeof(h), cudaMemcpyDeviceToHost));
  abx[0] = std::sqrt(h.rb_a2);
  abx[1] = h.rb_xc;
  abx[2] = h.rb_yc;
  return ORBIT_OK;
}

int orbit_sc2p5d_track(orbit_sc2p5d_t* c, orbit_bunch_t* b, double length) {
  ORBIT_NVTX("SpaceChargeCalc2p5D.trackBunch");
  if (!c || !b) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_track: null handle");
  if (c->rb) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_track: a 2.5Drb calculator needs orbit_sc2p5drb_track");
  if (b->n < 2) return ORBIT_OK;  // SpaceChargeCalc2p5D.cc:79-80
  ORBIT_CUDA(sc_order_before(c, b->stream));
  int rc = sc_enqueue_kick(c, b, length, b->stream, true, true, nullptr);
  if (rc) return rc;
  ORBIT_CUDA(sc_mark_used(c, b->stream));
  return ORBIT_OK;
}

int orbit_sc2p5d_get_grid(orbit_sc2p5d_t* c, int which, double* host_out) {
  if (!c || !host_out) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_get_grid: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  size_t ng = (size_t)c->nx * c->ny;
  if (which == ORBIT_GRID_RHO) ORBIT_CUDA(cudaMemcpy(host_out, c->d_rho, sizeof(double) * ng, cudaMemcpyDeviceToHost));
  else if (which == ORBIT_GRID_PHI) ORBIT_CUDA(cudaMemcpy(host_out, c->d_phi, sizeof(double) * ng, cudaMemcpyDeviceToHost));
  else if (which == ORBIT_GRID_LONG) ORBIT_CUDA(cudaMemcpy(host_out, c->d_lam, sizeof(double) * c->nz, cudaMemcpyDeviceToHost));
  else if (which == ORBIT_GRID_LONG_DERIV && c->rb)
    ORBIT_CUDA(cudaMemcpy(host_out, c->d_lamd, sizeof(double) * c->nz, cudaMemcpyDeviceToHost));
  else return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_get_grid: unknown grid");
  return ORBIT_OK;
}

int orbit_sc2p5d_get_limits(orbit_sc2p5d_t* c, double* lim) {
  if (!c || !lim) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_get_limits: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ScState h;
  ORBIT_CUDA(cudaMemcpy(&h, c->d_st, sizeof(h), cudaMemcpyDeviceToHost));
  lim[0] = h.xmin; lim[1] = h.xmax; lim[2] = h.ymin; lim[3] = h.ymax; lim[4] = h.zmin; lim[5] = h.zmax;
  lim[6] = h.dx; lim[7] = h.dy; lim[8] = h.dz; lim[9] = h.xy_ratio; lim[10] = h.total_m;
  return ORBIT_OK;
}

int orbit_sc2p5d_counters(orbit_sc2p5d_t* c, long long* kicks, long long* green_rebuilds) {
  if (!c || !kicks || !green_rebuilds) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_counters: bad argument");
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  ScState h;
  ORBIT_CUDA(cudaMemcpy(&h, c->d_st, sizeof(h), cudaMemcpyDeviceToHost));
  *kicks = (long long)h.n_kicks;
  *green_rebuilds = (long long)h.n_green;
  return ORBIT_OK;
}

int orbit_sc2p5d_get_sizes(const orbit_sc2p5d_t* c, int* nx, int* ny, int* nz, int* form) {
  if (!c) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_get_sizes: null handle");
  if (nx) *nx = c->nx;
  if (ny) *ny = c->ny;
  if (nz) *nz = c->nz;
  if (form) *form = c->form;
  return ORBIT_OK;
}

int orbit_sc2p5d_set_fused_conv(orbit_sc2p5d_t* c, int on, int* active) {
  if (!c) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_set_fused_conv: null handle");
  c->fused_conv = on != 0;
  ++c->cfg_gen;
  if (active) *active = use_conv_fused(c) ? 1 : 0;
  return ORBIT_OK;
}

int orbit_sc2p5d_set_conv_wait(orbit_sc2p5d_t* c, long long polls, int withhold) {
  if (!c || polls < 1 || withhold < -1) return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_set_conv_wait: bad argument");
  c->conv_wait_polls = polls;
  c->conv_withhold = withhold;
  ++c->cfg_gen;
  return ORBIT_OK;
}

int orbit_sc2p5d_fields(orbit_sc2p5d_t* c, int n, const double* x, const double* y, const double* z, double* ex,
                        double* ey, double* lam) {
  if (!c || n < 0 || (n > 0 && (!x || !y || !z || !ex || !ey || !lam)))
    return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_fields: bad argument");
  if (n == 0) return ORBIT_OK;
  if (c->used) ORBIT_CUDA(cudaEventSynchronize(c->done));
  double* d = nullptr;
  ORBIT_CUDA(cudaMalloc(&d, sizeof(double) * 6 * (size_t)n));
  cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, y, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + 2 * (size_t)n, z, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_fields<<<(n + 255) / 256, 256>>>(c->d_st, c->d_phi, c->d_lam, c->nx, c->ny, c->nz, n, d, d + n,
                                        d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n, d + 5 * (size_t)n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(ex, d + 3 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ey, d + 4 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(lam, d + 5 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_error(e, "orbit_sc2p5d_fields");
  return ORBIT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------
// No-allocation variant of trackBunch.
//
// Some callers cannot allocate device memory: code that runs inside another
// framework's memory pool or arena (where a cudaMalloc would bypass its
// accounting or fail under a fixed budget), real-time or embedded loops
// that must not allocate after start-up, and hosts that forbid the implicit
// device synchronisation a cudaMalloc/cudaFree can cause.  For them
// orbit_sc2p5d_track_static runs one kick of a freshly constructed plain
// FP64 calculator with every scratch buffer (solver state, fixed-point
// grids, potential, FFT spectra, Green function, twiddles, status word)
// carved from one file-scope __device__ array of kStaticScratchBytes.
// ---------------------------------------------------------------------
namespace orbit {

static const int kStaticMaxNxy = 128;  // nx, ny <= 128
static const int kStaticMaxNz = 256;   // nz <= 256

static constexpr size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }
static constexpr size_t kStaticScratchBytes =
    al256(sizeof(ScState)) + al256(sizeof(unsigned)) +                              // state, status
    al256(8ull * kStaticMaxNxy * kStaticMaxNxy) + al256(8ull * kStaticMaxNz) +       // fixed-point grids
    2 * al256(8ull * kStaticMaxNxy * kStaticMaxNxy) + al256(8ull * kStaticMaxNz) +   // rho, phi, lambda
    2 * al256(16ull * 2 * kStaticMaxNxy * (kStaticMaxNxy + 1)) +                     // spectrum, Green spectrum
    al256(8ull * 4 * kStaticMaxNxy * kStaticMaxNxy) +                                // Green function
    2 * al256(16ull * 2 * kStaticMaxNxy) +                                           // twiddles x, y
    al256(8ull * kStaticMaxNxy * kStaticMaxNxy) + al256(8ull * kStaticMaxNz);       // fixed-point phi, lambda

// Held by every GPU that loads the library, until the process exits
// (about 2.1 MB).  Shared by all calls: calls that overlap on the GPU race.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of the array in the current context, looked up on every
// call (a runtime table lookup): nothing is cached, so a new primary
// context after a device reset is seen and host threads share no state.
static int static_scratch_ptr(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess) return cuda_error(e, "orbit_sc2p5d_track_static: cudaGetSymbolAddress");
  *out = (unsigned char*)p;
  return ORBIT_OK;
}

}  // namespace orbit

extern "C" int orbit_sc2p5d_track_static(double* dev_coords, int n, int stride, int nx, int ny, int nz,
                                         double xy_ratio, double length, const orbit_sync_t* sync, void* stream) {
  using namespace orbit;
  if (!sync || n < 0 || (n > 0 && (!dev_coords || stride < n)))
    return set_error(ORBIT_ERR_ARG, "orbit_sc2p5d_track_static: bad argument");
  if (nx < 3 || ny < 3) return set_error(ORBIT_ERR_GRID, "Grid2D: the grid size too small (should be more than 3)");
  if (nz < 1) return set_error(ORBIT_ERR_GRID, "Grid1D: the grid size is too small (should be more than 0)");
  if (nx > kStaticMaxNxy || ny > kStaticMaxNxy || nz > kStaticMaxNz)
    return set_error(ORBIT_ERR_UNSUPPORTED,
                     "orbit_sc2p5d_track_static: grid above the static scratch limit (nx, ny <= 128, nz <= 256)");
  orbit_sc2p5d_t c;
  c.fused_conv = false;  // the separate solve kernels: no Green scratch is carved here
  c.nx = nx; c.ny = ny; c.nz = nz; c.form = ORBIT_FORM_PLAIN;
  c.nx2 = 2 * nx; c.ny2 = 2 * ny; c.H = ny + 1;
  c.xy_ratio0 = xy_ratio > 0. ? xy_ratio : 1.0;
  if (!make_fft_plan(c.nx2, c.plan_x) || !make_fft_plan(c.ny2, c.plan_y))
    return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_sc2p5d_track_static: grid sizes must have no prime factor above 13");
  if (n < 2) return ORBIT_OK;  // SpaceChargeCalc2p5D.cc:79-80
  unsigned char* base = nullptr;
  int rc = static_scratch_ptr(&base);
  if (rc) return rc;
  // carve the buffers
  size_t off = 0;
  auto take = [&](size_t bytes) { unsigned char* p = base + off; off += al256(bytes); return (void*)p; };
  size_t ng = (size_t)nx * ny, nhat = (size_t)c.nx2 * c.H;
  c.d_st = (ScState*)take(sizeof(ScState));
  unsigned* d_status = (unsigned*)take(sizeof(unsigned));
  c.d_rho_q = (unsigned long long*)take(8 * ng);
  c.d_z_q = (unsigned long long*)take(8 * (size_t)nz);
  c.d_rho = (double*)take(8 * ng);
  c.d_phi = (double*)take(8 * ng);
  c.d_lam = (double*)take(8 * (size_t)nz);
  c.d_hat = take(16 * nhat);
  c.d_green = take(16 * nhat);
  c.d_gbuf = (double*)take(8 * (size_t)c.nx2 * c.ny2);
  c.d_tw_x = take(16 * (size_t)c.nx2);
  c.d_tw_y = take(16 * (size_t)c.ny2);
  c.d_phi_fix = (long long*)take(8 * ng);
  c.d_lam_fix = (long long*)take(8 * (size_t)nz);
  if (off > kStaticScratchBytes) return set_error(ORBIT_ERR_DEVICE, "orbit_sc2p5d_track_static: scratch layout");
  cudaStream_t s = (cudaStream_t)stream;
  // state of a freshly constructed calculator (SpaceChargeCalc2p5D.cc:25-43);
  // everything else is fully written by the kernels before it is read
  ScState h;
  std::memset(&h, 0, sizeof(h));
  double r = c.xy_ratio0;
  h.xy_ratio = r;
  h.sxmin = -r; h.sxmax = r; h.symin = -1.0; h.symax = 1.0;
  h.sdx = (r - (-r)) / (nx - 1);
  h.sdy = (1.0 - (-1.0)) / (ny - 1);
  h.xmin = -1.0; h.xmax = 1.0; h.ymin = -1.0; h.ymax = 1.0;
  h.dx = 2.0 / (nx - 1); h.dy = 2.0 / (ny - 1); h.inv_dx = 1.0 / h.dx; h.inv_dy = 1.0 / h.dy;
  h.zmin = -0.5; h.zmax = 0.5; h.dz = 1.0 / nz; h.inv_dz = 1.0 / h.dz;
  h.green_dirty = 1;
  for (int k = 0; k < 3; ++k) { h.key[2 * k] = ~0ull; h.key[2 * k + 1] = 0ull; }
  double2 twx[2 * kStaticMaxNxy], twy[2 * kStaticMaxNxy];
  fill_twiddles_host<double>(c.nx2, twx);
  fill_twiddles_host<double>(c.ny2, twy);
  ORBIT_CUDA(cudaMemcpyAsync(c.d_st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  ORBIT_CUDA(cudaMemsetAsync(d_status, 0, sizeof(unsigned), s));
  // the deposit grids start at zero (a kick leaves them cleared, an
  // interrupted one might not)
  ORBIT_CUDA(cudaMemsetAsync(c.d_rho_q, 0, 8 * ng, s));
  ORBIT_CUDA(cudaMemsetAsync(c.d_z_q, 0, 8 * (size_t)nz, s));
  ORBIT_CUDA(cudaMemcpyAsync(c.d_tw_x, twx, sizeof(double2) * c.nx2, cudaMemcpyHostToDevice, s));
  ORBIT_CUDA(cudaMemcpyAsync(c.d_tw_y, twy, sizeof(double2) * c.ny2, cudaMemcpyHostToDevice, s));
  rc = init_attrs(&c);
  if (rc) return rc;
  orbit_bunch_t b;
  b.n = n;
  b.cap = stride;
  b.d_coords = dev_coords;
  b.d_status = d_status;
  b.stream = s;
  b.sync = *sync;
  b.has_msize = 0;
  rc = sc_enqueue_kick(&c, &b, length, s, true, true, nullptr);
  b.d_coords = nullptr;  // the caller owns the coordinates
  b.d_status = nullptr;
  b.stream = nullptr;
  if (rc) return rc;
  unsigned st = 0;
  ORBIT_CUDA(cudaMemcpyAsync(&st, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  ORBIT_CUDA(cudaStreamSynchronize(s));
  if (st & ST_NAN) return set_error(ORBIT_ERR_NAN, "non-finite particle coordinate found by the extrema scan");
  if (st & ST_EXTENT)
    return set_error(ORBIT_ERR_EXTENT,
                     "SpaceChargeCalc2p5D: the bunch min and max sizes are wrong (zero extent); kick skipped");
  if (st) return set_error(ORBIT_ERR_DEVICE, "device-side range check failed");
  return ORBIT_OK;
}
