// Block-cooperative mixed-radix Stockham FFT in shared memory.
//
// Used for the Hockney open-boundary convolution of the 2D Poisson solve
// (the role FFTW plays in src/spacecharge/PoissonSolverFFT2D.cc:57-59, 162,
// 228, 245).  One thread block transforms one length-N sequence held in
// shared memory; stage s with radix p maps
//   b[k*L*p + j + r*L] = sum_q (a[k*L + j + q*N/p] * W_{Lp}^{j q}) W_p^{q r}
// (L = product of the radices before s), so the result is in natural order
// after the last stage.  Twiddles come from a table W_N^e = exp(-2 pi i e/N)
// computed on the host and staged in shared memory; supported radices are
// 2, 3, 4, 5 and any prime up to 13, with fixed-radix butterflies in
// registers for power-of-two lengths.
#pragma once

#include "common.cuh"
#include "sc2p5d.cuh"

namespace orbit {

template <typename T> struct CT;
template <> struct CT<double> { typedef double2 t; };
template <> struct CT<float> { typedef float2 t; };

// Complex product with explicit roundings (the same bits in every kernel
// that inlines it): re = fma(a.x, b.x, -(a.y b.y)), im = fma(a.x, b.y, a.y b.x).
__device__ __forceinline__ double2 c_mul(double2 a, double2 b) {
  double2 r;
  r.x = __fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y));
  r.y = __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x));
  return r;
}
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  float2 r;
  r.x = __fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y));
  r.y = __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x));
  return r;
}
template <typename C>
__device__ __forceinline__ C c_add(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }

// Radix-2 butterfly with a twiddle, o0 = x0 + w x1, o1 = x0 - w x1, in six
// fused multiply-adds instead of a product and four additions:
// o0 = fma(x1.x, w.x, fma(-x1.y, w.y, x0.x)) (and the imaginary part
// likewise), o1 = fma(2, x0, -o0) = 2 x0 - o0, one rounding each.  The FP64
// pipe bounds the transforms on GB300.
__device__ __forceinline__ void bfly2_tw(double2 x0, double2 x1, double2 w, double2& o0, double2& o1) {
  o0.x = __fma_rn(x1.x, w.x, __fma_rn(-x1.y, w.y, x0.x));
  o0.y = __fma_rn(x1.x, w.y, __fma_rn(x1.y, w.x, x0.y));
  o1.x = __fma_rn(2.0, x0.x, -o0.x);
  o1.y = __fma_rn(2.0, x0.y, -o0.y);
}
__device__ __forceinline__ void bfly2_tw(float2 x0, float2 x1, float2 w, float2& o0, float2& o1) {
  o0.x = __fmaf_rn(x1.x, w.x, __fmaf_rn(-x1.y, w.y, x0.x));
  o0.y = __fmaf_rn(x1.x, w.y, __fmaf_rn(x1.y, w.x, x0.y));
  o1.x = __fmaf_rn(2.0f, x0.x, -o0.x);
  o1.y = __fmaf_rn(2.0f, x0.y, -o0.y);
}
template <typename C>
__device__ __forceinline__ C c_sub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C>
__device__ __forceinline__ C c_conj(C a) { a.y = -a.y; return a; }

// Radix-P stage of a power-of-two length (P = 2 or 4) with compile-time
// butterflies: t = k*L + j, inputs a[t + q*N/P], outputs b[k*L*P + j + r*L],
// twiddles W_{LP}^{jq} = tw[(j*q) << lgtw] read from shared memory.
template <typename T, int P, bool INV>
__device__ __forceinline__ void fft_stage_pow2(const typename CT<T>::t* __restrict__ a,
                                               typename CT<T>::t* __restrict__ b, int N, int L, int lgL,
                                               int lgtw, const typename CT<T>::t* __restrict__ tw) {
  typedef typename CT<T>::t C;
  const int Np = N / P;
  for (int t = threadIdx.x; t < Np; t += blockDim.x) {
    const int j = t & (L - 1);
    C x[P];
#pragma unroll
    for (int q = 0; q < P; ++q) x[q] = a[t + q * Np];
    if (P == 2 && L > 1) {
      C w = tw[j << lgtw];
      if (INV) w.y = -w.y;
      C* out = b + ((t - j) * 2) + j;
      bfly2_tw(x[0], x[1], w, out[0], out[L]);
      continue;
    }
    if (L > 1) {  // the first stage has only W^0 = 1
#pragma unroll
      for (int q = 1; q < P; ++q) {
        C w = tw[(j * q) << lgtw];
        if (INV) w.y = -w.y;
        x[q] = c_mul(x[q], w);
      }
    }
    C* out = b + ((t - j) * P) + j;
    if (P == 2) {
      out[0] = c_add(x[0], x[1]);
      out[L] = c_sub(x[0], x[1]);
    } else {
      C a0 = c_add(x[0], x[2]), a1 = c_sub(x[0], x[2]);
      C b0 = c_add(x[1], x[3]), b1 = c_sub(x[1], x[3]);
      C c;  // (-i or +i) * b1
      if (INV) { c.x = -b1.y; c.y = b1.x; } else { c.x = b1.y; c.y = -b1.x; }
      out[0] = c_add(a0, b0);
      out[L] = c_add(a1, c);
      out[2 * L] = c_sub(a0, b0);
      out[3 * L] = c_sub(a1, c);
    }
  }
}

// lg0 > 0: the first lg0 radix-2 stages are done (the caller staged their
// result in a); only with N/2 threads or more (all stages radix 2).
template <typename T, bool INV>
__device__ typename CT<T>::t* block_fft_pow2(typename CT<T>::t* a, typename CT<T>::t* b, const FftPlan& pl,
                                             const typename CT<T>::t* __restrict__ tw, int lg0 = 0) {
  typedef typename CT<T>::t C;
  // FP64 runs at a fraction of a lane per cycle per SM sub-partition, so the
  // transform is bound by how many warps share it: with N/2 threads every
  // stage is radix 2 (one butterfly per thread); with fewer, radix 4 while
  // possible, then one radix 2.
  const int N = pl.n;
  const int lgN = 31 - __clz(N);
  const bool wide = (int)blockDim.x >= N / 2;
  int L = 1 << lg0, lgL = lg0;
  while (lgL < lgN) {
    if (!wide && lgL + 2 <= lgN) {
      fft_stage_pow2<T, 4, INV>(a, b, N, L, lgL, lgN - lgL - 2, tw);
      L *= 4; lgL += 2;
    } else {
      fft_stage_pow2<T, 2, INV>(a, b, N, L, lgL, lgN - lgL - 1, tw);
      L *= 2; lgL += 1;
    }
    __syncthreads();
    C* tmp = a;
    a = b;
    b = tmp;
  }
  return a;
}

// Power-of-two length N = 2^LOGN fixed at compile time, one radix-2
// butterfly per thread (threads >= N/2; the others only synchronise):
// unrolled stages with constant strides, each thread's twiddle of every
// stage read once into registers (W_{2L}^j = tw[j << (LOGN-1-s)], j = t mod
// L), stages from lg0 on (lg0 = 1 when the caller staged the half-zero
// input as for block_fft_pow2).  The same butterflies as
// fft_stage_pow2<T, 2, INV> (bfly2_tw), so the same results.
template <typename T, bool INV, int LOGN>
__device__ __forceinline__ typename CT<T>::t* block_fft_fixed(typename CT<T>::t* a, typename CT<T>::t* b,
                                                              const typename CT<T>::t* __restrict__ tw, int lg0) {
  typedef typename CT<T>::t C;
  constexpr int N = 1 << LOGN, H2 = N / 2;
  const int t = threadIdx.x;
  C w[LOGN];
#pragma unroll
  for (int s = 1; s < LOGN; ++s) {
    w[s] = tw[(t & ((1 << s) - 1)) << (LOGN - 1 - s)];
    if (INV) w[s].y = -w[s].y;
  }
#pragma unroll
  for (int s = 0; s < LOGN; ++s) {
    if (s >= lg0) {
      if (t < H2) {
        const int L = 1 << s;
        const int j = t & (L - 1);
        C x0 = a[t], x1 = a[t + H2];
        C* out = b + ((t - j) << 1) + j;
        if (s > 0) {
          bfly2_tw(x0, x1, w[s], out[0], out[L]);
        } else {
          out[0] = c_add(x0, x1);
          out[L] = c_sub(x0, x1);
        }
      }
      __syncthreads();
      C* tmp = a;
      a = b;
      b = tmp;
    }
  }
  return a;
}

// a: input buffer, b: scratch, tw: the W_N table (shared memory); returns
// the buffer holding the result.  `inv` selects the backward (+i)
// transform; unnormalised.
template <typename T>
__device__ typename CT<T>::t* block_fft(typename CT<T>::t* a, typename CT<T>::t* b, const FftPlan& pl,
                                        const typename CT<T>::t* __restrict__ tw, bool inv) {
  typedef typename CT<T>::t C;
  if (pl.pow2) return inv ? block_fft_pow2<T, true>(a, b, pl, tw) : block_fft_pow2<T, false>(a, b, pl, tw);
  const int N = pl.n;
  int L = 1;
  for (int s = 0; s < pl.nst; ++s) {
    const int p = pl.rad[s];
    const int Np = N / p;
    const int Lp = L * p;
    const int tws = N / Lp;
    for (int t = threadIdx.x; t < Np; t += blockDim.x) {
      const int j = t % L;
      const int k = t / L;
      C x[13];
#pragma unroll 4
      for (int q = 0; q < p; ++q) x[q] = a[k * L + j + q * Np];
      if (j != 0) {
        for (int q = 1; q < p; ++q) {
          C w = tw[j * q * tws];
          if (inv) w.y = -w.y;
          x[q] = c_mul(x[q], w);
        }
      }
      C* out = b + k * Lp + j;
      if (p == 2) {
        out[0] = c_add(x[0], x[1]);
        out[L] = c_sub(x[0], x[1]);
      } else if (p == 4) {
        C a0 = c_add(x[0], x[2]), a1 = c_sub(x[0], x[2]);
        C b0 = c_add(x[1], x[3]), b1 = c_sub(x[1], x[3]);
        C c;  // (-i or +i) * b1
        if (inv) { c.x = -b1.y; c.y = b1.x; } else { c.x = b1.y; c.y = -b1.x; }
        out[0] = c_add(a0, b0);
        out[L] = c_add(a1, c);
        out[2 * L] = c_sub(a0, b0);
        out[3 * L] = c_sub(a1, c);
      } else {
        const int twp = N / p;  // W_p^e = tw[e * twp]
        for (int r = 0; r < p; ++r) {
          C acc = x[0];
          for (int q = 1; q < p; ++q) {
            C w = tw[((q * r) % p) * twp];
            if (inv) w.y = -w.y;
            C m = c_mul(x[q], w);
            acc = c_add(acc, m);
          }
          out[r * L] = acc;
        }
      }
    }
    __syncthreads();
    C* tmp = a;
    a = b;
    b = tmp;
    L = Lp;
  }
  return a;
}

// Forward transform of a power-of-two sequence whose second half is zero
// (the zero-padded half of the Hockney grid), with N/2 threads or more: the
// first radix-2 Stockham stage maps a[t], 0 to b[2t] = b[2t+1] = a[t], so
// the caller stages its input that way into `a` (see fft_halfzero_ok) and
// the transform starts at the second stage.
template <typename T>
__device__ __forceinline__ bool fft_halfzero_ok(const FftPlan& pl, int nin) {
  return pl.pow2 && (int)blockDim.x >= pl.n / 2 && nin <= pl.n / 2;
}

// Copies the W_N twiddle table to shared memory (the caller synchronises).
template <typename C>
__device__ __forceinline__ void load_twiddles(C* s_tw, const C* __restrict__ tw, int N) {
  for (int e = threadIdx.x; e < N; e += blockDim.x) s_tw[e] = tw[e];
}

// Host: factor N into supported radices (4s first, then 2, 3, 5, 7, 11, 13).
bool make_fft_plan(int n, FftPlan& pl);

}  // namespace orbit
