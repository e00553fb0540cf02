// Learned denoising closure of the 2.5D space-charge kick: a 4-level
// convolutional encoder-decoder that maps the charge density deposited by
// few macroparticles to the density many more macroparticles of the same
// beam give on the same grid; the plain FFT Poisson solve turns it into the
// potential.  No counterpart in the reference (a form of this library).
//
// Network (H x W input, H and W multiples of 8; channels in brackets):
//   x0[1] -> conv a1[16] -> conv s1[16] -> pool -> conv a2[32] -> conv s2[32]
//   -> pool -> conv a3[64] -> conv s3[64] -> pool -> conv a4[64] -> conv b4[64]
//   -> up + s3 [128] -> conv d3a[64] -> conv d3[64] -> up + s2 [96]
//   -> conv d2a[32] -> conv d2[32] -> up + s1 [48] -> conv d1a[16]
//   -> conv d1[16] -> 1x1 conv [1] + x0
// Every 3x3 convolution (zero padding) is followed by a ReLU; pooling is a
// 2x2 average, "up" a 2x nearest-neighbour upsample concatenated with the
// skip tensor.  302,561 parameters.  Convolution weights are BF16 (an FP32
// master copy is what Adam updates), biases FP32; activations and all
// accumulation FP32.  Training: mean squared error, Adam, on CUDA-core
// layers.  Single-image inference (the kick's closure) runs the 3x3 layers
// on the tensor cores (k_conv3_tc: tcgen05.mma kind::tf32 into TMEM).
//
// Tensors are NCHW FP32 in device memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace orbit {

// ---------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------
static const int kT = 16;   // output tile edge
static const int kCo = 16;  // output channels per block
static const int kCi = 8;   // input channels per shared-memory chunk

// 3x3 convolution, zero padding, one TT x TT tile of CO output channels per
// block (one thread per pixel): out[n][o][y][x] = b[o] + sum_i sum_k
// in[n][i][y+ky-1][x+kx-1] Wt(o,i,k).  TRANS (data gradient): Wt(o,i,k) =
// W[i][o][8-k] with W stored for the forward layer ([cin][cout][9] here),
// no bias, no ReLU.  Training batches fill the GPU with 16 x 16 tiles of 16
// channels; a single image takes smaller blocks (more of them).
// SPLIT: blockIdx.z = image * splits + part, the block sums input channels
// [part * ci_per, (part + 1) * ci_per) and writes its partial sums to part
// `part` of `out` (parts of N * cout * H * W each; k_split_reduce adds them
// in order with the bias and the ReLU).
template <bool TRANS, bool BIAS_RELU, int TT = kT, int CO = kCo, bool SPLIT = false>
__global__ void __launch_bounds__(256) k_conv3(const float* __restrict__ in, int cin,
                                               const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                               float* __restrict__ out, int cout, int H, int W, int splits = 1,
                                               int ci_per = 1 << 30) {
  static_assert(CO % 4 == 0, "output channels per block: a multiple of 4");
  __shared__ float s_in[kCi][TT + 2][TT + 2];
  // weights as [input channel][tap][output channel]: four output channels
  // per 128-bit shared load
  __shared__ __align__(16) float s_w[kCi][9][CO];
  const int tiles_x = (W + TT - 1) / TT;
  const int tx0 = (blockIdx.x % tiles_x) * TT, ty0 = (blockIdx.x / tiles_x) * TT;
  const int co0 = blockIdx.y * CO;
  const int n = SPLIT ? (int)blockIdx.z / splits : (int)blockIdx.z;
  const int ci_lo = SPLIT ? ((int)blockIdx.z % splits) * ci_per : 0;
  const int ci_hi = SPLIT ? min(cin, ci_lo + ci_per) : cin;
  const int tx = threadIdx.x % TT, ty = threadIdx.x / TT;
  float acc[CO];
#pragma unroll
  for (int o = 0; o < CO; ++o) acc[o] = 0.f;
  for (int ci0 = ci_lo; ci0 < ci_hi; ci0 += kCi) {
    for (int idx = threadIdx.x; idx < kCi * (TT + 2) * (TT + 2); idx += blockDim.x) {
      int c = idx / ((TT + 2) * (TT + 2)), r = idx % ((TT + 2) * (TT + 2));
      int yy = r / (TT + 2), xx = r % (TT + 2);
      int gy = ty0 + yy - 1, gx = tx0 + xx - 1, ci = ci0 + c;
      float v = 0.f;
      if (ci < ci_hi && gy >= 0 && gy < H && gx >= 0 && gx < W) v = in[(((size_t)n * cin + ci) * H + gy) * W + gx];
      s_in[c][yy][xx] = v;
    }
    for (int idx = threadIdx.x; idx < CO * kCi * 9; idx += blockDim.x) {
      int o = idx / (kCi * 9), r = idx % (kCi * 9);
      int c = r / 9, k = r % 9;
      int co = co0 + o, ci = ci0 + c;
      float v = 0.f;
      if (co < cout && ci < ci_hi)
        v = TRANS ? __bfloat162float(w[((size_t)ci * cout + co) * 9 + (8 - k)])
                  : __bfloat162float(w[((size_t)co * cin + ci) * 9 + k]);
      s_w[c][k][o] = v;
    }
    __syncthreads();
#pragma unroll 2
    for (int c = 0; c < kCi; ++c) {
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        float v = s_in[c][ty + k / 3][tx + k % 3];
        const float4* wk = reinterpret_cast<const float4*>(&s_w[c][k][0]);
#pragma unroll
        for (int q = 0; q < CO / 4; ++q) {
          float4 w4 = wk[q];
          acc[4 * q] = fmaf(v, w4.x, acc[4 * q]);
          acc[4 * q + 1] = fmaf(v, w4.y, acc[4 * q + 1]);
          acc[4 * q + 2] = fmaf(v, w4.z, acc[4 * q + 2]);
          acc[4 * q + 3] = fmaf(v, w4.w, acc[4 * q + 3]);
        }
      }
    }
    __syncthreads();
  }
  const int y = ty0 + ty, x = tx0 + tx;
  if (y < H && x < W) {
#pragma unroll
    for (int o = 0; o < CO; ++o) {
      int co = co0 + o;
      if (co < cout) {
        float v = acc[o];
        if (SPLIT) {
          const size_t part = (size_t)((int)blockIdx.z % splits);
          const size_t nimg = gridDim.z / splits;
          out[part * nimg * cout * H * W + (((size_t)n * cout + co) * H + y) * W + x] = v;
        } else {
          if (BIAS_RELU) v = fmaxf(v + bias[co], 0.f);
          out[(((size_t)n * cout + co) * H + y) * W + x] = v;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------
// Tensor-core (tcgen05) forward convolution, the inference path.
//
// One 3x3 layer as an implicit GEMM: D[p][o] = sum_k A[p][k] B[o][k] with p
// a pixel, o an output channel, k = tap * cin + ci (tap = ky * 3 + kx), A
// the zero-padded neighbourhoods of the input (im2col, built in shared
// memory) and B the BF16 weights W[o][ci][tap], exact in TF32.  Each CTA
// computes 128 pixels x N = cout channels (M = 128, N = 16, 32 or 64) in
// TMEM with tcgen05.mma kind::tf32 (FP32 accumulation) over one K stage of
// 32 (four MMAs of K = 8) staged in shared memory, the input rounded to
// TF32 (cvt.rna) as it is staged.  Layers of more than one stage run one
// stage per block (blockIdx.y) and write partial sums, which k_split_reduce
// adds in order (deterministic) with the bias and the ReLU; single-stage
// layers add those directly.
//
// Shared-memory operand layout (K-major, no swizzle): 8-row x 16-byte core
// matrices; element (r, k) of a stage at (r / 8) * 1024 + (k / 4) * 128 +
// (r % 8) * 16 + (k % 4) * 4 bytes, so the MMA over K columns 8j..8j+7
// starts at byte 256 j with LBO = 128 (next core matrix along K) and SBO =
// 1024 (next 8 rows).  Weights are packed into that image once per
// parameter change (k_pack_tc) and copied to shared memory as they are.
// ---------------------------------------------------------------------
static const int kTcM = 128;         // pixels per CTA (MMA M)
static const int kTcKC = 32;         // K per stage
static const int kTcStageA = kTcM * kTcKC * 4;   // 16 KB
static const int kTcStageB = 64 * kTcKC * 4;     // 8 KB (N <= 64)
static const int kTcSmem = kTcStageA + kTcStageB + 1024;  // one stage + alignment slack
static const long long kTcWaitCycles = 2000000000ll;  // ~1 s at 2 GHz: a wait that long has failed

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;    // LBO: next core matrix along K
  d |= (uint64_t)(1024u >> 4) << 32;   // SBO: next 8 rows
  d |= (uint64_t)1 << 46;              // descriptor version of the tcgen05 family
  return d;                            // base offset 0, no swizzle
}

// kind::tf32, D F32, A and B TF32, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ float to_tf32(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the barrier for at most `limit` clock cycles;
// false when it did not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit) {
  long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

// A stage's 32 inputs of this thread's pixel (k = 32 s .. 32 s + 31, k =
// tap * cin + ci): base pointer and bounds test change only with the tap.
__device__ __forceinline__ void tc_load_a(const float* __restrict__ in, int cin, int H, int W, int HW, int K,
                                          bool pin, int py, int px, int s, float v[kTcKC]) {
  int k = s * kTcKC;
  int tap = k / cin, ci = k - tap * cin;
  const float* src = nullptr;
  bool inb = false;
  int cur_tap = -1;
#pragma unroll
  for (int e = 0; e < kTcKC; ++e) {
    if (tap != cur_tap) {
      cur_tap = tap;
      const int yy = py + tap / 3 - 1, xx = px + tap % 3 - 1;
      inb = pin && tap < 9 && yy >= 0 && yy < H && xx >= 0 && xx < W;
      src = in + (inb ? yy * W + xx : 0);
    }
    v[e] = (inb && k + e < K) ? __ldg(src + (size_t)ci * HW) : 0.f;
    if (++ci == cin) {
      ci = 0;
      ++tap;
    }
  }
}

// The bounded waits of a tensor-core layer: `cycles` per wait; `withhold`
// (test only) issues no MMA, so that the wait runs out with nothing in
// flight and the failure path can be exercised.
struct TcWait {
  long long cycles;
  int withhold;
};

// Error flag bits: 1 = a wait gave up; 2 = the MMA had still not completed
// after a second wait of the same length, and its TMEM was released all the
// same (the results and the state of that SM's tensor memory are then not
// to be trusted: the network must not run on the tensor cores again in
// this process).
template <int N, bool SPLIT>
__global__ void __launch_bounds__(128) k_conv3_tc(const float* __restrict__ in, int cin, int H, int W,
                                                  const float* __restrict__ wpk, const float* __restrict__ bias,
                                                  float* __restrict__ out, float* __restrict__ part, int* err,
                                                  TcWait tw) {
  constexpr int BV = N * kTcKC / 4 / 128;  // float4 of the B stage per thread (1, 2 or 4)
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t raw = smem_u32(tc_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u, sB = sA + kTcStageA;
  unsigned char* gA = tc_raw + (sA - raw);
  const int HW = H * W;
  const int stage = SPLIT ? (int)blockIdx.y : 0;
  const int p = blockIdx.x * kTcM + tid;
  const bool pin = p < HW;
  const int py = pin ? p / W : 0, px = pin ? p % W : 0;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&s_tmem)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // the TMEM allocation and the barrier come before the global loads (loads
  // issued first measured slower: 258 against 224 us per 128 x 128 forward)
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  float va[kTcKC];
  float4 vb[BV];
  tc_load_a(in, cin, H, W, HW, cin * 9, pin, py, px, stage, va);
  const float4* srcB = reinterpret_cast<const float4*>(wpk + (size_t)stage * N * kTcKC);
#pragma unroll
  for (int i = 0; i < BV; ++i) vb[i] = __ldg(srcB + tid + 128 * i);
  // A: row tid; B: the packed stage image, copied as it is
  unsigned char* a_row = gA + (tid >> 3) * 1024 + (tid & 7) * 16;
#pragma unroll
  for (int q = 0; q < kTcKC / 4; ++q)
    *reinterpret_cast<float4*>(a_row + q * 128) =
        make_float4(to_tf32(va[4 * q]), to_tf32(va[4 * q + 1]), to_tf32(va[4 * q + 2]), to_tf32(va[4 * q + 3]));
  float4* dstB = reinterpret_cast<float4*>(gA + kTcStageA);
#pragma unroll
  for (int i = 0; i < BV; ++i) dstB[tid + 128 * i] = vb[i];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  if (tid == 0 && !tw.withhold) {
#pragma unroll
    for (int j = 0; j < kTcKC / 8; ++j) {
      const uint64_t ad = tc_desc(sA + 256u * j), bd = tc_desc(sB + 256u * j);
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
          "l"(ad), "l"(bd), "r"(tc_idesc(N)), "r"(j > 0 ? 1u : 0u));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(&s_bar))
                 : "memory");
  }
  // a wait that gives up does so for the whole block
  const bool ok = __syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), 0, tw.cycles));
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    // an MMA that was issued may still write the accumulators and arrive on
    // the barrier: wait once more before the TMEM is released
    if (!tw.withhold && !__syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), 0, tw.cycles)) && tid == 0)
      atomicOr(err, 2);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  float acc[N];
#pragma unroll
  for (int o = 0; o < N; ++o) acc[o] = 0.f;
  if (ok) {
    // row tid of D: TMEM lane 32 * warp + lane, columns 0..N-1
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[c0 + j] = __uint_as_float(r[j]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
  }
  if (!pin) return;
  if (SPLIT) {  // part blockIdx.y of the layer's output, summed by k_split_reduce
#pragma unroll
    for (int o = 0; o < N; ++o) part[((size_t)blockIdx.y * N + o) * HW + p] = acc[o];
  } else {
#pragma unroll
    for (int o = 0; o < N; ++o) out[(size_t)o * HW + p] = fmaxf(acc[o] + bias[o], 0.f);
  }
}

// Batched 3x3 layer on the tensor cores (training and batched forwards):
// a CTA computes 128 consecutive pixels of the nb images (pixel p of image
// p / HW) x N output channels and loops over every K stage of 32 (k = tap
// * cin + ci) with the accumulators in TMEM: per stage the im2col rows and
// the packed weight stage are staged in shared memory (the single-image
// layout), one thread issues four MMAs, and the block waits on their
// commit (phase s of the barrier) before the next stage reuses the buffers.
// MODE 0: out = max(acc + bias, 0) (forward); MODE 1: out = acc (the data
// gradient: `in` is the output gradient, the weights packed flipped and
// transposed by k_pack_tc_t).  The waits are bounded as in k_conv3_tc; a
// block whose wait gives up writes nothing.
static const int kTcbSmem = kTcStageA + 128 * kTcKC * 4 + 1024;  // N <= 128

template <int N, int MODE>
__global__ void __launch_bounds__(128) k_conv3_tcb(const float* __restrict__ in, int cin, int H, int W, int nb,
                                                   const float* __restrict__ wpk, int nst,
                                                   const float* __restrict__ bias, float* __restrict__ out,
                                                   int* err, TcWait tw) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 128, "MMA N");
  constexpr int BV = N * kTcKC / 4 / 128;                          // float4 of a B stage per thread
  constexpr uint32_t COLS = N <= 32 ? 32u : (N <= 64 ? 64u : 128u);  // TMEM columns (a power of two)
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t raw = smem_u32(tc_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u, sB = sA + kTcStageA;
  unsigned char* gA = tc_raw + (sA - raw);
  const int HW = H * W;
  const long long P = (long long)nb * HW;
  const long long p = (long long)blockIdx.x * kTcM + tid;
  const bool pin = p < P;
  const int img = pin ? (int)(p / HW) : 0;
  const int q = pin ? (int)(p % HW) : 0;
  const int py = q / W, px = q % W;
  const float* src = in + (size_t)img * cin * HW;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  unsigned char* a_row = gA + (tid >> 3) * 1024 + (tid & 7) * 16;
  float4* dstB = reinterpret_cast<float4*>(gA + kTcStageA);
  bool ok = true;
  int s = 0;
  // the next stage's global loads are issued before the wait on this
  // stage's MMAs, so their latency overlaps the tensor-core work
  float va[kTcKC];
  float4 vb[BV];
  auto load_stage = [&](int st) {
    tc_load_a(src, cin, H, W, HW, cin * 9, pin, py, px, st, va);
    const float4* srcB = reinterpret_cast<const float4*>(wpk + (size_t)st * N * kTcKC);
#pragma unroll
    for (int i = 0; i < BV; ++i) vb[i] = __ldg(srcB + tid + 128 * i);
  };
  load_stage(0);
  for (; s < nst; ++s) {
#pragma unroll
    for (int u = 0; u < kTcKC / 4; ++u)
      *reinterpret_cast<float4*>(a_row + u * 128) =
          make_float4(to_tf32(va[4 * u]), to_tf32(va[4 * u + 1]), to_tf32(va[4 * u + 2]), to_tf32(va[4 * u + 3]));
#pragma unroll
    for (int i = 0; i < BV; ++i) dstB[tid + 128 * i] = vb[i];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && !tw.withhold) {
#pragma unroll
      for (int j = 0; j < kTcKC / 8; ++j) {
        const uint64_t ad = tc_desc(sA + 256u * j), bd = tc_desc(sB + 256u * j);
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc_idesc(N)), "r"((s > 0 || j > 0) ? 1u : 0u));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&s_bar))
                   : "memory");
    }
    if (s + 1 < nst) load_stage(s + 1);
    // the MMAs of this stage read the buffers the next stage overwrites
    ok = __syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), (uint32_t)(s & 1), tw.cycles));
    if (!ok) break;
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    if (!tw.withhold &&
        !__syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), (uint32_t)(s & 1), tw.cycles)) && tid == 0)
      atomicOr(err, 2);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    // row tid of D: TMEM lane 32 * warp + lane, columns 0..N-1
    float* dst = out + (size_t)img * N * HW + q;
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (pin) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float v = __uint_as_float(r[j]);
          dst[(size_t)(c0 + j) * HW] = MODE == 0 ? fmaxf(v + bias[c0 + j], 0.f) : v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS));
  }
}

// Weight and bias gradients of a 3x3 layer on the tensor cores:
// dW[o][k] = sum_p dy[o][p] X[k][p] over the batch's pixels p (X the im2col
// of the layer's input, k = tap * cin + ci): an M = 128 (rows o < cout, the
// rest zero) x N = 64 (a chunk of k) product whose K runs over a slice of
// 32-pixel stages, accumulated in TMEM; the next stage's loads overlap the
// MMAs.  CTA (chunk, slice) adds its sums to dW with atomics, and the CTAs
// of chunk 0 also the bias gradient sum_p dy[o][p].  TF32 operands, FP32
// accumulation; bounded waits as in k_conv3_tc (a CTA whose wait gives up
// adds nothing).
static const int kWgNC = 64;  // columns of k per CTA

__global__ void __launch_bounds__(128) k_conv3_wgrad_tc(const float* __restrict__ x, int cin,
                                                        const float* __restrict__ dy, int cout, int H, int W,
                                                        int nb, int spc, float* __restrict__ dw,
                                                        float* __restrict__ db, int* err, TcWait tw) {
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t raw = smem_u32(tc_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u, sB = sA + kTcStageA;
  unsigned char* gA = tc_raw + (sA - raw);
  const int HW = H * W, P = nb * HW, K9 = 9 * cin;
  const int k0 = blockIdx.x * kWgNC;
  const int p_begin = blockIdx.y * spc * kTcKC;
  const int nst = min(spc, (P - p_begin + kTcKC - 1) / kTcKC);
  // B row of this thread: k = k0 + (tid >> 1), pixels 16 (tid & 1) .. + 15
  const int kb = k0 + (tid >> 1), half = tid & 1;
  const bool kvalid = kb < K9;
  const int tap = kvalid ? kb / cin : 0, ci = kvalid ? kb % cin : 0;
  const int ky = tap / 3 - 1, kx = tap % 3 - 1;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"((uint32_t)kWgNC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  float va[kTcKC], vb[16];
  float bsum = 0.f;
  auto load_stage = [&](int st) {
    const int p0 = p_begin + st * kTcKC;
    if (tid < cout) {  // A row o = tid: dy[o] at the stage's 32 pixels
      int p = p0, img = p0 / HW, q = p0 - img * HW;
#pragma unroll
      for (int e = 0; e < kTcKC; ++e) {
        va[e] = p < P ? __ldg(dy + ((size_t)img * cout + tid) * HW + q) : 0.f;
        ++p;
        if (++q == HW) {
          q = 0;
          ++img;
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < kTcKC; ++e) va[e] = 0.f;
    }
    int p = p0 + 16 * half, img = p / HW, q = p - img * HW, py = q / W, px = q - py * W;
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const int yy = py + ky, xx = px + kx;
      const bool inb = kvalid && p < P && yy >= 0 && yy < H && xx >= 0 && xx < W;
      vb[e] = inb ? __ldg(x + ((size_t)img * cin + ci) * HW + yy * W + xx) : 0.f;
      ++p;
      if (++px == W) {
        px = 0;
        if (++py == H) {
          py = 0;
          ++img;
        }
      }
    }
  };
  unsigned char* a_row = gA + (tid >> 3) * 1024 + (tid & 7) * 16;
  const int rb = tid >> 1;
  unsigned char* b_row = gA + kTcStageA + (rb >> 3) * 1024 + (rb & 7) * 16 + half * 4 * 128;
  bool ok = true;
  int s = 0;
  load_stage(0);
  for (; s < nst; ++s) {
    if (blockIdx.x == 0 && tid < cout) {
#pragma unroll
      for (int e = 0; e < kTcKC; ++e) bsum += va[e];
    }
#pragma unroll
    for (int u = 0; u < kTcKC / 4; ++u)
      *reinterpret_cast<float4*>(a_row + u * 128) =
          make_float4(to_tf32(va[4 * u]), to_tf32(va[4 * u + 1]), to_tf32(va[4 * u + 2]), to_tf32(va[4 * u + 3]));
#pragma unroll
    for (int u = 0; u < 4; ++u)
      *reinterpret_cast<float4*>(b_row + u * 128) =
          make_float4(to_tf32(vb[4 * u]), to_tf32(vb[4 * u + 1]), to_tf32(vb[4 * u + 2]), to_tf32(vb[4 * u + 3]));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && !tw.withhold) {
#pragma unroll
      for (int j = 0; j < kTcKC / 8; ++j) {
        const uint64_t ad = tc_desc(sA + 256u * j), bd = tc_desc(sB + 256u * j);
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(tc_idesc(kWgNC)), "r"((s > 0 || j > 0) ? 1u : 0u));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&s_bar))
                   : "memory");
    }
    if (s + 1 < nst) load_stage(s + 1);
    ok = __syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), (uint32_t)(s & 1), tw.cycles));
    if (!ok) break;
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    if (!tw.withhold &&
        !__syncthreads_and(mbar_wait_bounded(smem_u32(&s_bar), (uint32_t)(s & 1), tw.cycles)) && tid == 0)
      atomicOr(err, 2);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    // row o = tid of D: TMEM lane 32 * warp + lane, columns 0..63 = k0..k0+63
#pragma unroll
    for (int c0 = 0; c0 < kWgNC; c0 += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (tid < cout) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int k = k0 + c0 + j;
          if (k < K9) atomicAdd(dw + ((size_t)tid * cin + k % cin) * 9 + k / cin, __uint_as_float(r[j]));
        }
      }
    }
    if (blockIdx.x == 0 && tid < cout) atomicAdd(db + tid, bsum);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kWgNC));
  }
}

// The data-gradient weights of one layer (cout x cin x 3 x 3, BF16) packed
// for k_conv3_tcb<cin, 1>: output row ci, K column k = tap' * cout + o with
// the flipped tap (weight W[o][ci][8 - tap']), stages of 32 in the layout of
// k_pack_tc; zero for k >= 9 cout.
__global__ void k_pack_tc_t(const __nv_bfloat16* __restrict__ w, int cout, int cin, int nst, float* __restrict__ out) {
  const int total = nst * cin * kTcKC;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int st = i / (cin * kTcKC), r = i % (cin * kTcKC);
    const int ci = r / kTcKC, kk = r % kTcKC;
    const int k = st * kTcKC + kk;
    float v = 0.f;
    if (k < 9 * cout) {
      const int tap = k / cout, o = k % cout;
      v = __bfloat162float(w[((size_t)o * cin + ci) * 9 + (8 - tap)]);
    }
    out[(size_t)st * cin * kTcKC + (ci >> 3) * 256 + (kk >> 2) * 32 + (ci & 7) * 4 + (kk & 3)] = v;
  }
}

// Packs the BF16 weights of one layer into the per-stage shared-memory
// image of k_conv3_tc: row o, K column k = tap * cin + ci (weight
// W[o][ci][tap]) of stage s = k / 32 at float index s * N * 32 + (o / 8) *
// 256 + (kk / 4) * 32 + (o % 8) * 4 + kk % 4 (kk = k % 32); zero for
// k >= 9 cin.
__global__ void k_pack_tc(const __nv_bfloat16* __restrict__ w, int cin, int n, int nst, float* __restrict__ out) {
  const int total = nst * n * kTcKC;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int s = i / (n * kTcKC), r = i % (n * kTcKC);
    const int o = r / kTcKC, kk = r % kTcKC;
    const int k = s * kTcKC + kk;
    float v = 0.f;
    if (k < 9 * cin) {
      const int tap = k / cin, ci = k % cin;
      v = __bfloat162float(w[((size_t)o * cin + ci) * 9 + tap]);
    }
    out[(size_t)s * n * kTcKC + (o >> 3) * 256 + (kk >> 2) * 32 + (o & 7) * 4 + (kk & 3)] = v;
  }
}

// out = max(b + sum of the split convolution's parts (in order), 0).
__global__ void k_split_reduce(const float* __restrict__ part, int splits, const float* __restrict__ b,
                               float* __restrict__ out, int C, int HW, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v = b[(i / HW) % C];
    // eight parts' loads in flight at a time; the additions keep the order
    // q = 0, 1, ... (the same sums)
    int q = 0;
    for (; q + 8 <= splits; q += 8) {
      float t[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) t[u] = __ldg(part + (size_t)(q + u) * n + i);
#pragma unroll
      for (int u = 0; u < 8; ++u) v += t[u];
    }
    for (; q < splits; ++q) v += __ldg(part + (size_t)q * n + i);
    out[i] = fmaxf(v, 0.f);
  }
}

// The sum of k_split_reduce for a layer whose output also feeds a 2x2
// average pooling and the skip half of a concatenation, or a 2x upsample
// into the first half of one: those copies are written here instead of by
// k_pool and k_upcat, with the same arithmetic (the same values).  One
// thread per 2x2 quad of one channel; cat / pool / up may be null.
__global__ void k_split_reduce_quad(const float* __restrict__ part, int splits, const float* __restrict__ b,
                                    float* __restrict__ out, int C, int H, int W, float* __restrict__ pool,
                                    float* __restrict__ cat, int cat_off, float* __restrict__ up) {
  const int h2 = H / 2, w2 = W / 2;
  const size_t n = (size_t)C * H * W;
  const size_t tot = (size_t)C * h2 * w2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const int x2 = (int)(i % w2), y2 = (int)((i / w2) % h2), c = (int)(i / ((size_t)w2 * h2));
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int y = 2 * y2 + (k >> 1), x = 2 * x2 + (k & 1);
      const size_t e = ((size_t)c * H + y) * W + x;
      float sum = b[c];
      int q = 0;
      for (; q + 8 <= splits; q += 8) {
        float t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) t[u] = __ldg(part + (size_t)(q + u) * n + e);
#pragma unroll
        for (int u = 0; u < 8; ++u) sum += t[u];
      }
      for (; q < splits; ++q) sum += __ldg(part + (size_t)q * n + e);
      v[k] = fmaxf(sum, 0.f);
      out[e] = v[k];
      if (cat) cat[((size_t)(cat_off + c) * H + y) * W + x] = v[k];
      if (up) {
        float* u0 = up + ((size_t)c * 2 * H + 2 * y) * 2 * W + 2 * x;
        u0[0] = v[k];
        u0[1] = v[k];
        u0[2 * W] = v[k];
        u0[2 * W + 1] = v[k];
      }
    }
    if (pool) pool[((size_t)c * h2 + y2) * w2 + x2] = 0.25f * (v[0] + v[1] + v[2] + v[3]);
  }
}

// Weight and bias gradients of a 3x3 convolution:
// dW[o][i][k] += sum_{n,y,x} dy[n][o][y][x] x[n][i][y+ky-1][x+kx-1],
// db[o] += sum dy[n][o].  Block: 16 output x 8 input channels, the 16x16
// tiles t = blockIdx.y, blockIdx.y + gridDim.y, ... of all images.
__global__ void __launch_bounds__(256) k_conv3_wgrad(const float* __restrict__ x, int cin,
                                                     const float* __restrict__ dy, int cout, int H, int W, int N,
                                                     float* __restrict__ dw, float* __restrict__ db) {
  __shared__ float s_dy[kCo][kT * kT];
  __shared__ float s_x[kCi][kT + 2][kT + 2];
  const int itiles = (cin + kCi - 1) / kCi;
  const int co0 = (blockIdx.x / itiles) * kCo, ci0 = (blockIdx.x % itiles) * kCi;
  const int tiles_x = (W + kT - 1) / kT, tiles_y = (H + kT - 1) / kT;
  const int T = N * tiles_x * tiles_y;
  const int nel = kCo * kCi * 9;  // 1152 weights per block
  float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float bacc = 0.f;
  for (int t = blockIdx.y; t < T; t += gridDim.y) {
    const int n = t / (tiles_x * tiles_y), r = t % (tiles_x * tiles_y);
    const int tx0 = (r % tiles_x) * kT, ty0 = (r / tiles_x) * kT;
    for (int idx = threadIdx.x; idx < kCo * kT * kT; idx += blockDim.x) {
      int o = idx / (kT * kT), p = idx % (kT * kT);
      int yy = ty0 + p / kT, xx = tx0 + p % kT, co = co0 + o;
      float v = 0.f;
      if (co < cout && yy < H && xx < W) v = dy[(((size_t)n * cout + co) * H + yy) * W + xx];
      s_dy[o][p] = v;
    }
    for (int idx = threadIdx.x; idx < kCi * (kT + 2) * (kT + 2); idx += blockDim.x) {
      int c = idx / ((kT + 2) * (kT + 2)), rr = idx % ((kT + 2) * (kT + 2));
      int yy = rr / (kT + 2), xx = rr % (kT + 2);
      int gy = ty0 + yy - 1, gx = tx0 + xx - 1, ci = ci0 + c;
      float v = 0.f;
      if (ci < cin && gy >= 0 && gy < H && gx >= 0 && gx < W) v = x[(((size_t)n * cin + ci) * H + gy) * W + gx];
      s_x[c][yy][xx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      int e = threadIdx.x + q * blockDim.x;
      if (e < nel) {
        int o = e / (kCi * 9), rr = e % (kCi * 9);
        int c = rr / 9, k = rr % 9, ky = k / 3, kx = k % 3;
        float s = 0.f;
        for (int p = 0; p < kT * kT; ++p) s = fmaf(s_dy[o][p], s_x[c][p / kT + ky][p % kT + kx], s);
        acc[q] += s;
      }
    }
    if (ci0 == 0 && threadIdx.x < kCo)
      for (int p = 0; p < kT * kT; ++p) bacc += s_dy[threadIdx.x][p];
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    int e = threadIdx.x + q * blockDim.x;
    if (e < nel) {
      int o = e / (kCi * 9), rr = e % (kCi * 9);
      int c = rr / 9, k = rr % 9;
      int co = co0 + o, ci = ci0 + c;
      if (co < cout && ci < cin) atomicAdd(dw + ((size_t)co * cin + ci) * 9 + k, acc[q]);
    }
  }
  if (ci0 == 0 && threadIdx.x < kCo && co0 + (int)threadIdx.x < cout) atomicAdd(db + co0 + threadIdx.x, bacc);
}

// dy *= (y > 0): the gradient through the ReLU that produced y.
__global__ void k_relu_bwd(float* __restrict__ dy, const float* __restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!(y[i] > 0.f)) dy[i] = 0.f;
}

// 2x2 average pooling of [N*C][H][W] into [N*C][H/2][W/2].
__global__ void k_pool(const float* __restrict__ in, float* __restrict__ out, int NC, int H, int W) {
  const int h = H / 2, w = W / 2;
  size_t tot = (size_t)NC * h * w;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % w), y = (int)((i / w) % h);
    size_t nc = i / ((size_t)w * h);
    const float* p = in + (nc * H + 2 * y) * W + 2 * x;
    out[i] = 0.25f * (p[0] + p[1] + p[W] + p[W + 1]);
  }
}

// din[n][c][y][x] += dout[n][c][y/2][x/2] / 4.
__global__ void k_pool_bwd(const float* __restrict__ dout, float* __restrict__ din, int NC, int H, int W) {
  const int h = H / 2, w = W / 2;
  size_t tot = (size_t)NC * H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % W), y = (int)((i / W) % H);
    size_t nc = i / ((size_t)W * H);
    din[i] += 0.25f * dout[(nc * h + y / 2) * w + x / 2];
  }
}

// out = [up2(a) (ca channels at H/2 x W/2), b (cb channels)] at H x W.
__global__ void k_upcat(const float* __restrict__ a, int ca, const float* __restrict__ b, int cb,
                        float* __restrict__ out, int N, int H, int W) {
  const int C = ca + cb;
  size_t tot = (size_t)N * C * H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % W), y = (int)((i / W) % H);
    int c = (int)((i / ((size_t)W * H)) % C);
    size_t n = i / ((size_t)W * H * C);
    out[i] = c < ca ? a[((n * ca + c) * (H / 2) + y / 2) * (W / 2) + x / 2]
                    : b[((n * cb + (c - ca)) * H + y) * W + x];
  }
}

// Gradients of k_upcat: da = 2x2 sums of dout's first ca channels (written),
// db += dout's last cb channels.
__global__ void k_upcat_bwd(const float* __restrict__ dout, int ca, float* __restrict__ da, int cb,
                            float* __restrict__ db, int N, int H, int W) {
  const int C = ca + cb, h = H / 2, w = W / 2;
  size_t ta = (size_t)N * ca * h * w, tb = (size_t)N * cb * H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ta + tb; i += (size_t)gridDim.x * blockDim.x) {
    if (i < ta) {
      int x = (int)(i % w), y = (int)((i / w) % h);
      int c = (int)((i / ((size_t)w * h)) % ca);
      size_t n = i / ((size_t)w * h * ca);
      const float* p = dout + ((n * C + c) * H + 2 * y) * W + 2 * x;
      da[i] = p[0] + p[1] + p[W] + p[W + 1];
    } else {
      size_t j = i - ta;
      int x = (int)(j % W), y = (int)((j / W) % H);
      int c = (int)((j / ((size_t)W * H)) % cb);
      size_t n = j / ((size_t)W * H * cb);
      db[j] += dout[((n * C + ca + c) * H + y) * W + x];
    }
  }
}

// y[n][0] = x0[n][0] + b + sum_c w[c] h[n][c] (1x1 output convolution plus
// the input: the network predicts the correction to the noisy density).
// With `parts`, block k also writes the sum of its outputs clamped at zero
// to parts[k] (a fixed order within the block: the learned closure sums
// the parts in block order, so its charge scale is the same on every run).
__global__ void k_out(const float* __restrict__ h, int C, const float* __restrict__ w, const float* __restrict__ b,
                      const float* __restrict__ x0, float* __restrict__ y, int N, int HW,
                      double* __restrict__ parts) {
  size_t tot = (size_t)N * HW;
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    size_t n = i / HW, p = i % HW;
    float s = x0[i] + b[0];
    for (int c = 0; c < C; ++c) s = fmaf(w[c], h[(n * C + c) * HW + p], s);
    y[i] = s;
    acc += fmaxf(s, 0.f);
  }
  if (!parts) return;
  __shared__ double s_part[32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += s_part[q];
    parts[blockIdx.x] = t;
  }
}

// Gradients of k_out: dh[n][c] = dy w[c]; dw[c] += sum dy h[c]; db += sum dy
// (block partial sums, one atomic per block and channel).
__global__ void k_out_bwd(const float* __restrict__ dy, const float* __restrict__ h, int C,
                          const float* __restrict__ w, float* __restrict__ dh, float* __restrict__ dw,
                          float* __restrict__ db, int N, int HW) {
  __shared__ float s_red[32][17];
  float pw[16], pb = 0.f;
  for (int c = 0; c < 16; ++c) pw[c] = 0.f;
  size_t tot = (size_t)N * HW;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    size_t n = i / HW, p = i % HW;
    float g = dy[i];
    pb += g;
    for (int c = 0; c < C && c < 16; ++c) {
      dh[(n * C + c) * HW + p] = g * w[c];
      pw[c] = fmaf(g, h[(n * C + c) * HW + p], pw[c]);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    pb += __shfl_xor_sync(0xffffffffu, pb, off);
    for (int c = 0; c < 16; ++c) pw[c] += __shfl_xor_sync(0xffffffffu, pw[c], off);
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    for (int c = 0; c < 16; ++c) s_red[wid][c] = pw[c];
    s_red[wid][16] = pb;
  }
  __syncthreads();
  if (threadIdx.x < 17) {
    float s = 0.f;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += s_red[q][threadIdx.x];
    if (threadIdx.x < 16) {
      if ((int)threadIdx.x < C) atomicAdd(dw + threadIdx.x, s);
    } else {
      atomicAdd(db, s);
    }
  }
}

// Mean squared error: loss += sum (y - t)^2 / n, dy = 2 (y - t) / n.
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy, size_t n,
                      float* __restrict__ loss) {
  float s = 0.f;
  const float inv = 1.0f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float d = y[i] - t[i];
    s = fmaf(d, d, s);
    dy[i] = 2.f * d * inv;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// Weighted squared error of one level of the multi-scale loss: loss += w
// mean((y - t)^2), dy (=, or += with acc) 2 w (y - t) / n.
__global__ void k_mse_w(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy, size_t n,
                        float* __restrict__ loss, float w, int acc) {
  float s = 0.f;
  const float inv = 1.0f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float d = y[i] - t[i];
    s = fmaf(d, d, s);
    const float g = 2.f * w * d * inv;
    dy[i] = acc ? dy[i] + g : g;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, w * s * inv);
}

// Adam (Kingma & Ba, 2015) on the FP32 master parameters, then the BF16
// copies of the convolution weights; the gradients are cleared.
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ pb, const unsigned char* __restrict__ is_w, size_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float w = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = w;
    if (is_w[i]) pb[i] = __float2bfloat16_rn(w);
    g[i] = 0.f;
  }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb,
                          const unsigned char* __restrict__ is_w, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    pb[i] = is_w[i] ? __float2bfloat16_rn(p[i]) : __float2bfloat16_rn(0.f);
}

// ---------------------------------------------------------------------
// training beams: transverse positions of Gaussian, KV and waterbag
// beams from a counter-based generator (SplitMix64 of seed and particle
// index), so any particle can be drawn by any thread
// ---------------------------------------------------------------------
__device__ __forceinline__ unsigned long long sm64(unsigned long long& s) {
  unsigned long long z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(unsigned long long& s) {  // (0, 1)
  return ((double)(sm64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// kind 0: Gaussian (rms sx, sy); 1: KV projection, uniform in the ellipse of
// semi-axes 2 sx, 2 sy; 2: waterbag projection, the 2D shadow of a uniform
// 4D ball (density ~ 1 - r^2 inside semi-axes sqrt(6) sx, sqrt(6) sy).
__device__ __forceinline__ void beam_xy(int kind, double sx, double sy, unsigned long long seed, long long i,
                                        double& x, double& y) {
  unsigned long long s = seed ^ ((unsigned long long)i * 0xd1b54a32d192ed03ull);
  if (kind == 0) {
    double r = sqrt(-2.0 * log(u01(s))), t = 6.283185307179586 * u01(s);
    x = sx * r * cos(t);
    y = sy * r * sin(t);
  } else if (kind == 1) {
    double r = sqrt(u01(s)), t = 6.283185307179586 * u01(s);
    x = 2.0 * sx * r * cos(t);
    y = 2.0 * sy * r * sin(t);
  } else {
    // a uniform point of the 4D unit ball: four normals scaled to radius u^(1/4)
    double r1 = sqrt(-2.0 * log(u01(s))), t1 = 6.283185307179586 * u01(s);
    double r2 = sqrt(-2.0 * log(u01(s))), t2 = 6.283185307179586 * u01(s);
    double g0 = r1 * cos(t1), g1 = r1 * sin(t1), g2 = r2 * cos(t2), g3 = r2 * sin(t2);
    double nrm = sqrt(g0 * g0 + g1 * g1 + g2 * g2 + g3 * g3);
    double rad = sqrt(sqrt(u01(s))) / nrm;
    x = 2.449489742783178 * sx * g0 * rad;
    y = 2.449489742783178 * sy * g1 * rad;
  }
}

__global__ void k_beam_sample(double* __restrict__ x, double* __restrict__ y, int n, int kind, double sx, double sy,
                              unsigned long long seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) beam_xy(kind, sx, sy, seed, i, x[i], y[i]);
}

// 9-point deposit (Grid2D weights, Grid2D.cc:141-166) of n beam particles
// with unit weight on the node grid xmin..xmax x ymin..ymax (nx x ny),
// FP32 shared-memory accumulation; particles outside the grid are dropped.
__global__ void k_beam_deposit(float* __restrict__ grid, int nx, int ny, double xmin, double ymin, double inv_dx,
                               double inv_dy, double xmax, double ymax, long long n, int kind, double sx, double sy,
                               unsigned long long seed) {
  extern __shared__ float s_g[];
  for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) s_g[i] = 0.f;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double x, y;
    beam_xy(kind, sx, sy, seed, i, x, y);
    if (x < xmin || x > xmax || y < ymin || y > ymax) continue;
    double tx = (x - xmin) * inv_dx, ty = (y - ymin) * inv_dy;
    int ix = (int)(tx + 0.5), iy = (int)(ty + 0.5);
    ix = ix < 1 ? 1 : (ix > nx - 2 ? nx - 2 : ix);
    iy = iy < 1 ? 1 : (iy > ny - 2 ? ny - 2 : iy);
    float fx = (float)(tx - ix), fy = (float)(ty - iy);
    float wx[3] = {0.5f * (0.25f - fx + fx * fx), 0.75f - fx * fx, 0.5f * (0.25f + fx + fx * fx)};
    float wy[3] = {0.5f * (0.25f - fy + fy * fy), 0.75f - fy * fy, 0.5f * (0.25f + fy + fy * fy)};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) atomicAdd(&s_g[(ix - 1 + a) * ny + (iy - 1 + b)], wx[a] * wy[b]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) {
    float v = s_g[i];
    if (v != 0.f) atomicAdd(grid + i, v);
  }
}

// The same deposit for given positions (a tracked bunch).
__global__ void k_grid_deposit(float* __restrict__ grid, int nx, int ny, double xmin, double ymin, double inv_dx,
                               double inv_dy, double xmax, double ymax, const double* __restrict__ px,
                               const double* __restrict__ py, long long n) {
  extern __shared__ float s_g[];
  for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) s_g[i] = 0.f;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double x = px[i], y = py[i];
    if (!(x >= xmin && x <= xmax && y >= ymin && y <= ymax)) continue;
    double tx = (x - xmin) * inv_dx, ty = (y - ymin) * inv_dy;
    int ix = (int)(tx + 0.5), iy = (int)(ty + 0.5);
    ix = ix < 1 ? 1 : (ix > nx - 2 ? nx - 2 : ix);
    iy = iy < 1 ? 1 : (iy > ny - 2 ? ny - 2 : iy);
    float fx = (float)(tx - ix), fy = (float)(ty - iy);
    float wx[3] = {0.5f * (0.25f - fx + fx * fx), 0.75f - fx * fx, 0.5f * (0.25f + fx + fx * fx)};
    float wy[3] = {0.5f * (0.25f - fy + fy * fy), 0.75f - fy * fy, 0.5f * (0.25f + fy + fy * fy)};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) atomicAdd(&s_g[(ix - 1 + a) * ny + (iy - 1 + b)], wx[a] * wy[b]);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) {
    float v = s_g[i];
    if (v != 0.f) atomicAdd(grid + i, v);
  }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
static int grid_1d(size_t n) {
  size_t b = (n + 255) / 256;
  size_t cap = (size_t)num_sms() * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

struct Conv {
  int cin, cout;
  size_t w_off, b_off;  // offsets in the parameter array
};

}  // namespace orbit

using namespace orbit;

struct orbit_denoiser {
  int H = 0, W = 0, maxb = 0;
  std::vector<Conv> conv;   // 14 3x3 convolutions in network order
  size_t out_w = 0, out_b = 0, nparam = 0;
  float* d_p = nullptr;     // FP32 master parameters
  __nv_bfloat16* d_pb = nullptr;  // BF16 copies (convolution weights; biases unused)
  float* d_g = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  unsigned char* d_isw = nullptr;
  long long step = 0;
  // activations (maxb images) and their gradients
  std::vector<float*> act, grad;
  float* d_loss = nullptr;
  float* d_scratch = nullptr;  // data gradient of the widest convolution input
  cudaStream_t stream = nullptr;
  // tensor-core inference path (single images): packed weights per layer,
  // repacked after any parameter change; error flag of its bounded waits
  bool tc = true;
  bool tc_stale = true;
  unsigned long long version = 1;  // bumped by every parameter change
  float* d_wtc = nullptr;
  std::vector<size_t> tc_off;
  int* d_err = nullptr;
  // batches (training and batched forwards) on the tensor cores: forward
  // layers from d_wtc, data gradients from the flipped, transposed packing
  bool tcb = false;
  bool tct_stale = true;
  float* d_wtct = nullptr;
  std::vector<size_t> tct_off;
  // training loss: 0 levels = mean squared error; L levels = the
  // multi-scale loss sum_s w_s mean((P^s y - P^s t)^2), P = 2x2 average
  // pooling, with its pooled outputs, targets and gradients per level
  int loss_levels = 0;
  float loss_w[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  std::vector<float*> ms_y, ms_t, ms_g;
  long long tc_wait_cycles = kTcWaitCycles;
  int tc_withhold = 0;
  bool tc_failed = false;  // a tensor-core layer reported a failed wait
};

namespace orbit {

int* dn_error_flag(orbit_denoiser_t* d) { return d->d_err; }

// activation indices
enum {
  X0, A1, S1, P1, A2, S2, P2, A3, S3, P3, A4, B4, C3, D3A, D3, C2, D2A, D2, C1, D1A, D1, Y, NACT
};

static void act_shape(const orbit_denoiser_t* d, int a, int* c, int* h, int* w) {
  const int H = d->H, W = d->W;
  static const int ch[NACT] = {1, 16, 16, 16, 32, 32, 32, 64, 64, 64, 64, 64, 128, 64, 64, 96, 32, 32, 48, 16, 16, 1};
  static const int lv[NACT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 2, 1, 1, 1, 0, 0, 0, 0};
  *c = ch[a];
  *h = H >> lv[a];
  *w = W >> lv[a];
}

// The 3x3 layers: (input activation, output activation, conv index).
struct Step3 {
  int in, out, ci;
};
static const Step3 kSteps[14] = {{X0, A1, 0},   {A1, S1, 1},   {P1, A2, 2},   {A2, S2, 3},   {P2, A3, 4},
                                 {A3, S3, 5},   {P3, A4, 6},   {A4, B4, 7},   {C3, D3A, 8},  {D3A, D3, 9},
                                 {C2, D2A, 10}, {D2A, D2, 11}, {C1, D1A, 12}, {D1A, D1, 13}};

static size_t act_size(const orbit_denoiser_t* d, int a, int nb) {
  int c, h, w;
  act_shape(d, a, &c, &h, &w);
  return (size_t)nb * c * h * w;
}

// Forward launch plan: 16x16 tiles of 16 output channels; when that makes
// fewer than two blocks per SM (a single image), the input channels are
// split over enough blocks to fill the GPU, each writing partial sums to the
// scratch, summed in order by k_split_reduce.
static void split_plan(const Conv& cv, int h, int w, int nb, int* splits, int* ci_per) {
  const long long base = (long long)((w + 15) / 16) * ((h + 15) / 16) * ((cv.cout + 15) / 16) * nb;
  const int chunks = (cv.cin + kCi - 1) / kCi;
  int sp = (int)((2LL * num_sms() + base - 1) / base);
  sp = sp < 1 ? 1 : (sp > chunks ? chunks : sp);
  *ci_per = ((chunks + sp - 1) / sp) * kCi;
  *splits = (cv.cin + *ci_per - 1) / *ci_per;
}

static int conv_fwd_cc(orbit_denoiser_t* d, const Step3& s, int nb, cudaStream_t st) {
  const Conv& cv = d->conv[s.ci];
  int c, h, w;
  act_shape(d, s.out, &c, &h, &w);
  const __nv_bfloat16* W = d->d_pb + cv.w_off;
  const float* B = d->d_p + cv.b_off;
  int splits, ci_per;
  split_plan(cv, h, w, nb, &splits, &ci_per);
  dim3 g(((w + 15) / 16) * ((h + 15) / 16), (cv.cout + 15) / 16, nb * splits);
  if (splits == 1) {
    k_conv3<false, true, 16, 16><<<g, 256, 0, st>>>(d->act[s.in], cv.cin, W, B, d->act[s.out], cv.cout, h, w);
  } else {
    const size_t n_out = act_size(d, s.out, nb);
    k_conv3<false, true, 16, 16, true><<<g, 256, 0, st>>>(d->act[s.in], cv.cin, W, B, d->d_scratch, cv.cout, h, w,
                                                          splits, ci_per);
    k_split_reduce<<<grid_1d(n_out), 256, 0, st>>>(d->d_scratch, splits, B, d->act[s.out], cv.cout, h * w, n_out);
  }
  ORBIT_LAUNCH_CHECK("denoiser conv");
  return ORBIT_OK;
}

// Tensor-core plan of one layer: 128-pixel tiles, the K stages split over
// blocks so that the layer fills about one block per SM.
// One K stage per block (one MMA group of 32), parts summed in order by
// k_split_reduce: a single image's layers are short chains of latency, and
// running them side by side beats longer chains per block.  Measured per
// 128 x 128 forward on GB300: 224 us, against 242 us with a few splits per
// pixel tile summed by the tile's last block and 297 us on the CUDA-core
// layers.
static void tc_plan(const Conv& cv, int h, int w, int* tiles, int* nst) {
  *tiles = (h * w + kTcM - 1) / kTcM;
  *nst = (cv.cin * 9 + kTcKC - 1) / kTcKC;
}

static int tc_pack(orbit_denoiser_t* d, cudaStream_t st) {
  for (size_t l = 0; l < d->conv.size(); ++l) {
    const Conv& cv = d->conv[l];
    const int nst = (cv.cin * 9 + kTcKC - 1) / kTcKC;
    k_pack_tc<<<grid_1d((size_t)nst * cv.cout * kTcKC), 256, 0, st>>>(d->d_pb + cv.w_off, cv.cin, cv.cout, nst,
                                                                      d->d_wtc + d->tc_off[l]);
  }
  ORBIT_LAUNCH_CHECK("denoiser tensor-core weight packing");
  d->tc_stale = false;
  return ORBIT_OK;
}

static int tc_pack_t(orbit_denoiser_t* d, cudaStream_t st) {
  for (size_t l = 0; l < d->conv.size(); ++l) {
    const Conv& cv = d->conv[l];
    if (cv.cin < 16) continue;  // the first layer's input gets no gradient
    const int nst = (cv.cout * 9 + kTcKC - 1) / kTcKC;
    k_pack_tc_t<<<grid_1d((size_t)nst * cv.cin * kTcKC), 256, 0, st>>>(d->d_pb + cv.w_off, cv.cout, cv.cin, nst,
                                                                        d->d_wtct + d->tct_off[l]);
  }
  ORBIT_LAUNCH_CHECK("denoiser tensor-core data-gradient weight packing");
  d->tct_stale = false;
  return ORBIT_OK;
}

template <int N, int MODE>
static void launch_tcb(const orbit_denoiser_t* d, cudaStream_t st, const float* in, int cin, int h, int w, int nb,
                       const float* wp, int nst, const float* bias, float* out) {
  const long long P = (long long)nb * h * w;
  const int blocks = (int)((P + kTcM - 1) / kTcM);
  const TcWait tw = {d->tc_wait_cycles, d->tc_withhold};
  k_conv3_tcb<N, MODE><<<blocks, 128, kTcbSmem, st>>>(in, cin, h, w, nb, wp, nst, bias, out, d->d_err, tw);
}

// Forward of one 3x3 layer for nb images on the tensor cores.
static int conv_fwd_tcb(orbit_denoiser_t* d, const Step3& s, int nb, cudaStream_t st) {
  const Conv& cv = d->conv[s.ci];
  int c, h, w;
  act_shape(d, s.out, &c, &h, &w);
  const int nst = (cv.cin * 9 + kTcKC - 1) / kTcKC;
  const float* wp = d->d_wtc + d->tc_off[s.ci];
  const float* B = d->d_p + cv.b_off;
  switch (cv.cout) {
    case 16: launch_tcb<16, 0>(d, st, d->act[s.in], cv.cin, h, w, nb, wp, nst, B, d->act[s.out]); break;
    case 32: launch_tcb<32, 0>(d, st, d->act[s.in], cv.cin, h, w, nb, wp, nst, B, d->act[s.out]); break;
    case 64: launch_tcb<64, 0>(d, st, d->act[s.in], cv.cin, h, w, nb, wp, nst, B, d->act[s.out]); break;
    default: return set_error(ORBIT_ERR_ARG, "denoiser: tensor-core layer width not supported");
  }
  ORBIT_LAUNCH_CHECK("denoiser tensor-core batched conv");
  return ORBIT_OK;
}

// Data gradient of one 3x3 layer for nb images on the tensor cores:
// grad[in] = grad[out] convolved with the flipped, transposed kernel.
static int conv_dgrad_tcb(orbit_denoiser_t* d, const Step3& s, int nb, cudaStream_t st) {
  const Conv& cv = d->conv[s.ci];
  int c, h, w;
  act_shape(d, s.out, &c, &h, &w);
  const int nst = (cv.cout * 9 + kTcKC - 1) / kTcKC;
  const float* wp = d->d_wtct + d->tct_off[s.ci];
  const float* gi = d->grad[s.out];
  float* go = d->grad[s.in];
  switch (cv.cin) {
    case 16: launch_tcb<16, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    case 32: launch_tcb<32, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    case 48: launch_tcb<48, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    case 64: launch_tcb<64, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    case 96: launch_tcb<96, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    case 128: launch_tcb<128, 1>(d, st, gi, cv.cout, h, w, nb, wp, nst, nullptr, go); break;
    default: return set_error(ORBIT_ERR_ARG, "denoiser: tensor-core data-gradient width not supported");
  }
  ORBIT_LAUNCH_CHECK("denoiser tensor-core data gradient");
  return ORBIT_OK;
}

template <int N>
static void launch_conv_tc(dim3 g, cudaStream_t st, bool split, const float* in, int cin, int h, int w,
                           const float* wp, const float* bias, float* out, float* part, int nst, int* err,
                           TcWait tw) {
  if (split)
    k_conv3_tc<N, true><<<g, 128, kTcSmem, st>>>(in, cin, h, w, wp, bias, out, part, err, tw);
  else
    k_conv3_tc<N, false><<<g, 128, kTcSmem, st>>>(in, cin, h, w, wp, bias, out, part, err, tw);
}

// What a tensor-core layer's reduction also writes (see k_split_reduce_quad).
struct TcEpi {
  int pool = -1;     // activation receiving the 2x2 average
  int cat = -1;      // concatenation receiving a copy at channel cat_off
  int cat_off = 0;
  int up = -1;       // concatenation receiving the 2x upsample (channels 0..C-1)
};

static int conv_fwd_tc(orbit_denoiser_t* d, const Step3& s, cudaStream_t st, const TcEpi& ep = TcEpi()) {
  const Conv& cv = d->conv[s.ci];
  int c, h, w, tiles, nst;
  act_shape(d, s.out, &c, &h, &w);
  tc_plan(cv, h, w, &tiles, &nst);
  const float* wp = d->d_wtc + d->tc_off[s.ci];
  const float* B = d->d_p + cv.b_off;
  const bool split = nst > 1;
  dim3 g(tiles, nst);
  float* o = d->act[s.out];
  float* part = d->d_scratch;
  const TcWait tw = {d->tc_wait_cycles, d->tc_withhold};
  switch (cv.cout) {
    case 16: launch_conv_tc<16>(g, st, split, d->act[s.in], cv.cin, h, w, wp, B, o, part, nst, d->d_err, tw); break;
    case 32: launch_conv_tc<32>(g, st, split, d->act[s.in], cv.cin, h, w, wp, B, o, part, nst, d->d_err, tw); break;
    case 64: launch_conv_tc<64>(g, st, split, d->act[s.in], cv.cin, h, w, wp, B, o, part, nst, d->d_err, tw); break;
    default: return set_error(ORBIT_ERR_ARG, "denoiser: tensor-core layer width not supported");
  }
  ORBIT_LAUNCH_CHECK("denoiser tensor-core conv");
  const bool epi = ep.pool >= 0 || ep.cat >= 0 || ep.up >= 0;
  const size_t n_out = (size_t)cv.cout * h * w;
  if (split && epi) {
    k_split_reduce_quad<<<grid_1d(n_out / 4), 256, 0, st>>>(
        part, nst, B, o, cv.cout, h, w, ep.pool >= 0 ? d->act[ep.pool] : nullptr, ep.cat >= 0 ? d->act[ep.cat] : nullptr,
        ep.cat_off, ep.up >= 0 ? d->act[ep.up] : nullptr);
    ORBIT_LAUNCH_CHECK("denoiser split reduce");
    return ORBIT_OK;
  }
  if (split) {
    k_split_reduce<<<grid_1d(n_out), 256, 0, st>>>(part, nst, B, o, cv.cout, h * w, n_out);
    ORBIT_LAUNCH_CHECK("denoiser split reduce");
  }
  if (!epi) return ORBIT_OK;
  // an unsplit layer with consumers: the separate kernels
  if (ep.pool >= 0) k_pool<<<grid_1d(n_out / 4), 256, 0, st>>>(o, d->act[ep.pool], cv.cout, h, w);
  if (ep.cat >= 0) {
    int cc, hh, ww;
    act_shape(d, ep.cat, &cc, &hh, &ww);
    ORBIT_CUDA(cudaMemcpyAsync(d->act[ep.cat] + (size_t)ep.cat_off * h * w, o, sizeof(float) * n_out,
                               cudaMemcpyDeviceToDevice, st));
  }
  if (ep.up >= 0) {
    int cc, hh, ww;
    act_shape(d, ep.up, &cc, &hh, &ww);
    k_upcat<<<grid_1d((size_t)cv.cout * hh * ww), 256, 0, st>>>(o, cv.cout, nullptr, 0, d->act[ep.up], 1, hh, ww);
  }
  ORBIT_LAUNCH_CHECK("denoiser epilogue");
  return ORBIT_OK;
}

// infer: a single image goes through the tensor-core layers (when on);
// training keeps the CUDA-core layers, whose activations the backward
// pass reads and whose gradients are checked against the oracle.
// Set when a tensor-core layer reported an MMA that had not completed after
// two bounded waits (error bit 2): that SM's tensor memory may still have
// been written after its release, so no network of this process uses the
// tensor-core layers again.
static bool g_tc_untrusted = false;

static bool use_tcb(const orbit_denoiser_t* d) { return d->tcb && !d->tc_failed && !g_tc_untrusted; }

static int forward(orbit_denoiser_t* d, int nb, cudaStream_t st, bool infer = false, double* parts = nullptr) {
  const bool tc = infer && d->tc && !d->tc_failed && !g_tc_untrusted && nb == 1;
  const bool tcb = !tc && use_tcb(d);
  if ((tc || tcb) && d->tc_stale) {
    // a packing captured into a graph would run only where that graph is
    // replayed: captures find the weights packed (dn_prepare_capture)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ORBIT_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return set_error(ORBIT_ERR_UNSUPPORTED, "denoiser: parameters changed without dn_prepare_capture before a capture");
    int rc = tc_pack(d, st);
    if (rc) return rc;
  }
  auto conv_fwd = [&](orbit_denoiser_t* dd, const Step3& stp, int n, cudaStream_t ss) -> int {
    return tcb ? conv_fwd_tcb(dd, stp, n, ss) : conv_fwd_cc(dd, stp, n, ss);
  };
  auto pool = [&](int a, int b) -> int {
    int c, h, w;
    act_shape(d, a, &c, &h, &w);
    k_pool<<<grid_1d(act_size(d, b, nb)), 256, 0, st>>>(d->act[a], d->act[b], nb * c, h, w);
    ORBIT_LAUNCH_CHECK("denoiser pool");
    return ORBIT_OK;
  };
  auto upcat = [&](int a, int b, int out) -> int {
    int ca, cb, h, w, t;
    act_shape(d, a, &ca, &t, &t);
    act_shape(d, b, &cb, &h, &w);
    k_upcat<<<grid_1d(act_size(d, out, nb)), 256, 0, st>>>(d->act[a], ca, d->act[b], cb, d->act[out], nb, h, w);
    ORBIT_LAUNCH_CHECK("denoiser upcat");
    return ORBIT_OK;
  };
  int rc = 0;
  if (tc) {
    // the layers' reductions also write the poolings and concatenations
    TcEpi e1, e3, e5, e7, e9, e11;
    e1.pool = P1; e1.cat = C1; e1.cat_off = 32;  // c1 = [up(d2) 32, s1 16]
    e3.pool = P2; e3.cat = C2; e3.cat_off = 64;  // c2 = [up(d3) 64, s2 32]
    e5.pool = P3; e5.cat = C3; e5.cat_off = 64;  // c3 = [up(b4) 64, s3 64]
    e7.up = C3;
    e9.up = C2;
    e11.up = C1;
    const TcEpi none;
    const TcEpi* eps[14] = {&none, &e1, &none, &e3, &none, &e5, &none, &e7, &none, &e9, &none, &e11, &none, &none};
    for (int k = 0; k < 14 && !rc; ++k) rc = conv_fwd_tc(d, kSteps[k], st, *eps[k]);
  } else {
    rc = rc ? rc : conv_fwd(d, kSteps[0], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[1], nb, st);
    rc = rc ? rc : pool(S1, P1);
    rc = rc ? rc : conv_fwd(d, kSteps[2], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[3], nb, st);
    rc = rc ? rc : pool(S2, P2);
    rc = rc ? rc : conv_fwd(d, kSteps[4], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[5], nb, st);
    rc = rc ? rc : pool(S3, P3);
    rc = rc ? rc : conv_fwd(d, kSteps[6], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[7], nb, st);
    rc = rc ? rc : upcat(B4, S3, C3);
    rc = rc ? rc : conv_fwd(d, kSteps[8], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[9], nb, st);
    rc = rc ? rc : upcat(D3, S2, C2);
    rc = rc ? rc : conv_fwd(d, kSteps[10], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[11], nb, st);
    rc = rc ? rc : upcat(D2, S1, C1);
    rc = rc ? rc : conv_fwd(d, kSteps[12], nb, st);
    rc = rc ? rc : conv_fwd(d, kSteps[13], nb, st);
  }
  if (rc) return rc;
  const size_t hw = (size_t)d->H * d->W;
  k_out<<<grid_1d(nb * hw), 256, 0, st>>>(d->act[D1], 16, d->d_p + d->out_w, d->d_p + d->out_b, d->act[X0],
                                          d->act[Y], nb, (int)hw, parts);
  ORBIT_LAUNCH_CHECK("denoiser out");
  return ORBIT_OK;
}

// Backward of one 3x3 layer: grad[out] holds dL/d(output after ReLU); it
// becomes dL/d(pre-activation), the weight and bias gradients accumulate,
// and the data gradient is written to grad[in] (no 3x3 layer's input has a
// second consumer; the input image gets none).
static int conv_bwd(orbit_denoiser_t* d, const Step3& s, int nb, cudaStream_t st) {
  const Conv& cv = d->conv[s.ci];
  int c, h, w;
  act_shape(d, s.out, &c, &h, &w);
  size_t n_out = act_size(d, s.out, nb);
  k_relu_bwd<<<grid_1d(n_out), 256, 0, st>>>(d->grad[s.out], d->act[s.out], n_out);
  const int tiles = ((w + kT - 1) / kT) * ((h + kT - 1) / kT);
  if (use_tcb(d)) {
    // chunks of 64 weight columns x slices of the batch's pixels, about
    // four CTAs per SM in all
    const int chunks = (cv.cin * 9 + kWgNC - 1) / kWgNC;
    const int stages = (int)(((long long)nb * h * w + kTcKC - 1) / kTcKC);
    int want = 4 * num_sms() / chunks;
    want = want < 1 ? 1 : want;
    const int spc = (stages + want - 1) / want;
    const int slices = (stages + spc - 1) / spc;
    const TcWait tw = {d->tc_wait_cycles, d->tc_withhold};
    k_conv3_wgrad_tc<<<dim3(chunks, slices), 128, kTcSmem, st>>>(d->act[s.in], cv.cin, d->grad[s.out], cv.cout, h,
                                                                w, nb, spc, d->d_g + cv.w_off, d->d_g + cv.b_off,
                                                                d->d_err, tw);
  } else {
    const int ttot = tiles * nb;
    const int split = ttot < 64 ? ttot : 64;
    dim3 gw(((cv.cout + kCo - 1) / kCo) * ((cv.cin + kCi - 1) / kCi), split);
    k_conv3_wgrad<<<gw, 256, 0, st>>>(d->act[s.in], cv.cin, d->grad[s.out], cv.cout, h, w, nb, d->d_g + cv.w_off,
                                      d->d_g + cv.b_off);
  }
  if (s.in != X0) {
    // data gradient: dy convolved with the flipped, transposed kernel
    if (use_tcb(d)) {
      if (d->tct_stale) {
        int rc = tc_pack_t(d, st);
        if (rc) return rc;
      }
      int rc = conv_dgrad_tcb(d, s, nb, st);
      if (rc) return rc;
    } else {
      dim3 gd(tiles, (cv.cin + kCo - 1) / kCo, nb);
      k_conv3<true, false><<<gd, 256, 0, st>>>(d->grad[s.out], cv.cout, d->d_pb + cv.w_off, nullptr,
                                               d->grad[s.in], cv.cin, h, w);
    }
  }
  ORBIT_LAUNCH_CHECK("denoiser conv backward");
  return ORBIT_OK;
}

// grad[Y] holds dL/dy; every parameter gradient is accumulated into d_g.
static int backward(orbit_denoiser_t* d, int nb, cudaStream_t st) {
  const size_t hw = (size_t)d->H * d->W;
  // the skip tensors collect gradients from the pooling and the decoder
  for (int a : {S1, S2, S3}) ORBIT_CUDA(cudaMemsetAsync(d->grad[a], 0, sizeof(float) * act_size(d, a, nb), st));
  k_out_bwd<<<grid_1d(nb * hw), 256, 0, st>>>(d->grad[Y], d->act[D1], 16, d->d_p + d->out_w, d->grad[D1],
                                              d->d_g + d->out_w, d->d_g + d->out_b, nb, (int)hw);
  ORBIT_LAUNCH_CHECK("denoiser out backward");
  auto upcat_bwd = [&](int out, int a, int b) -> int {
    int ca, cb, h, w, t;
    act_shape(d, a, &ca, &t, &t);
    act_shape(d, b, &cb, &h, &w);
    k_upcat_bwd<<<grid_1d(act_size(d, out, nb)), 256, 0, st>>>(d->grad[out], ca, d->grad[a], cb, d->grad[b], nb, h,
                                                                 w);
    ORBIT_LAUNCH_CHECK("denoiser upcat backward");
    return ORBIT_OK;
  };
  auto pool_bwd = [&](int pooled, int full) -> int {
    int c, h, w;
    act_shape(d, full, &c, &h, &w);
    k_pool_bwd<<<grid_1d(act_size(d, full, nb)), 256, 0, st>>>(d->grad[pooled], d->grad[full], nb * c, h, w);
    ORBIT_LAUNCH_CHECK("denoiser pool backward");
    return ORBIT_OK;
  };
  int rc = 0;
  rc = rc ? rc : conv_bwd(d, kSteps[13], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[12], nb, st);
  rc = rc ? rc : upcat_bwd(C1, D2, S1);
  rc = rc ? rc : conv_bwd(d, kSteps[11], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[10], nb, st);
  rc = rc ? rc : upcat_bwd(C2, D3, S2);
  rc = rc ? rc : conv_bwd(d, kSteps[9], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[8], nb, st);
  rc = rc ? rc : upcat_bwd(C3, B4, S3);
  rc = rc ? rc : conv_bwd(d, kSteps[7], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[6], nb, st);
  rc = rc ? rc : pool_bwd(P3, S3);
  rc = rc ? rc : conv_bwd(d, kSteps[5], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[4], nb, st);
  rc = rc ? rc : pool_bwd(P2, S2);
  rc = rc ? rc : conv_bwd(d, kSteps[3], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[2], nb, st);
  rc = rc ? rc : pool_bwd(P1, S1);
  rc = rc ? rc : conv_bwd(d, kSteps[1], nb, st);
  rc = rc ? rc : conv_bwd(d, kSteps[0], nb, st);
  return rc;
}

// Forward, loss and backward of nb pairs already in act[X0] and `target`.
static int loss_and_grads(orbit_denoiser_t* d, const float* target, int nb, cudaStream_t st) {
  int rc = forward(d, nb, st);
  if (rc) return rc;
  ORBIT_CUDA(cudaMemsetAsync(d->d_loss, 0, sizeof(float), st));
  size_t n = (size_t)nb * d->H * d->W;
  if (d->loss_levels == 0) {
    k_mse<<<grid_1d(n), 256, 0, st>>>(d->act[Y], target, d->grad[Y], n, d->d_loss);
    ORBIT_LAUNCH_CHECK("denoiser loss");
    return backward(d, nb, st);
  }
  // multi-scale loss: the squared error of the output, then of its 2x2
  // poolings level by level (each level weighted); the gradients of the
  // pooled levels flow back through the pooling to the output
  const int L = d->loss_levels;
  k_mse_w<<<grid_1d(n), 256, 0, st>>>(d->act[Y], target, d->grad[Y], n, d->d_loss, d->loss_w[0], 0);
  const float* yp = d->act[Y];
  const float* tp = target;
  for (int s = 1; s <= L; ++s) {
    const int H = d->H >> (s - 1), W = d->W >> (s - 1);
    const size_t ns = (size_t)nb * (H / 2) * (W / 2);
    k_pool<<<grid_1d(ns), 256, 0, st>>>(yp, d->ms_y[s], nb, H, W);
    k_pool<<<grid_1d(ns), 256, 0, st>>>(tp, d->ms_t[s], nb, H, W);
    k_mse_w<<<grid_1d(ns), 256, 0, st>>>(d->ms_y[s], d->ms_t[s], d->ms_g[s], ns, d->d_loss, d->loss_w[s], 0);
    yp = d->ms_y[s];
    tp = d->ms_t[s];
  }
  for (int s = L; s >= 1; --s) {
    float* din = s > 1 ? d->ms_g[s - 1] : d->grad[Y];
    const int H = d->H >> (s - 1), W = d->W >> (s - 1);
    k_pool_bwd<<<grid_1d((size_t)nb * H * W), 256, 0, st>>>(d->ms_g[s], din, nb, H, W);
  }
  ORBIT_LAUNCH_CHECK("denoiser multi-scale loss");
  return backward(d, nb, st);
}

// SplitMix64 (Steele, Lea, Flood 2014) and Box-Muller normals for the
// initial weights.
static uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unit_open(uint64_t& s) { return ((splitmix64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
static double normal(uint64_t& s) {
  double u = unit_open(s), v = unit_open(s);
  return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
}

static cudaStream_t stream_of(orbit_denoiser_t* d, void* s) { return s ? (cudaStream_t)s : d->stream; }

static int check_batch(const orbit_denoiser_t* d, int nb) {
  if (nb < 1 || nb > d->maxb) return set_error(ORBIT_ERR_ARG, "orbit_denoiser: batch size outside 1..max_batch");
  return ORBIT_OK;
}

// After a synchronised batched step on the tensor cores: a bounded wait
// that gave up (error bits set) makes the network run on the CUDA cores
// from now on, and the step reports the error.
static int tcb_status(orbit_denoiser_t* d) {
  if (!d->tcb || d->tc_failed) return ORBIT_OK;
  int err = 0;
  ORBIT_CUDA(cudaMemcpy(&err, d->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!err) return ORBIT_OK;
  ORBIT_CUDA(cudaMemset(d->d_err, 0, sizeof(int)));
  d->tc_failed = true;
  if (err & 2) g_tc_untrusted = true;
  return set_error(ORBIT_ERR_DEVICE, "denoiser: a tensor-core wait gave up; the network now runs on the CUDA cores");
}

unsigned long long dn_version(const orbit_denoiser_t* d) { return d ? d->version : 0ull; }

int dn_prepare_capture(orbit_denoiser_t* d) {
  if (!d || !d->tc_stale) return ORBIT_OK;
  // forwards in flight may still read the packed weights
  ORBIT_CUDA(cudaDeviceSynchronize());
  int rc = tc_pack(d, d->stream);
  if (rc) return rc;
  ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  return ORBIT_OK;
}

int dn_closure_io(orbit_denoiser_t* d, float** in, const float** out, int* nparts) {
  if (!d) return set_error(ORBIT_ERR_ARG, "dn_closure_io: null network");
  *in = d->act[X0];
  *out = d->act[Y];
  *nparts = grid_1d((size_t)d->H * d->W);
  return ORBIT_OK;
}

int dn_forward_inplace(orbit_denoiser_t* d, cudaStream_t st, double* parts) {
  if (!d) return set_error(ORBIT_ERR_ARG, "dn_forward_inplace: null network");
  return forward(d, 1, st, true, parts);
}

}  // namespace orbit

extern "C" {

int orbit_beam_sample(double* dev_x, double* dev_y, int n, int kind, double sx, double sy, unsigned long long seed) {
  if (!dev_x || !dev_y || n < 0 || kind < 0 || kind > 2 || !(sx > 0) || !(sy > 0))
    return set_error(ORBIT_ERR_ARG, "orbit_beam_sample: bad argument");
  if (n == 0) return ORBIT_OK;
  k_beam_sample<<<grid_1d(n), 256>>>(dev_x, dev_y, n, kind, sx, sy, seed);
  ORBIT_LAUNCH_CHECK("orbit_beam_sample");
  ORBIT_CUDA(cudaDeviceSynchronize());
  return ORBIT_OK;
}

int orbit_beam_deposit(float* dev_grid, int nx, int ny, const double* lim, long long n, int kind, double sx,
                       double sy, unsigned long long seed) {
  if (!dev_grid || !lim || nx < 3 || ny < 3 || n < 0 || kind < 0 || kind > 2 || !(sx > 0) || !(sy > 0) ||
      !(lim[1] > lim[0]) || !(lim[3] > lim[2]))
    return set_error(ORBIT_ERR_ARG, "orbit_beam_deposit: bad argument");
  size_t sm = sizeof(float) * (size_t)nx * ny;
  if (sm > 200 * 1024) return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_beam_deposit: grid above 200 KB of shared memory");
  static bool attr = false;
  if (!attr) {
    ORBIT_CUDA(cudaFuncSetAttribute(k_beam_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  ORBIT_CUDA(cudaMemset(dev_grid, 0, sm));
  double dx = (lim[1] - lim[0]) / (nx - 1), dy = (lim[3] - lim[2]) / (ny - 1);
  long long blocks = (n + 8191) / 8192;
  long long cap = (long long)num_sms() * 2;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_beam_deposit<<<(int)blocks, 512, sm>>>(dev_grid, nx, ny, lim[0], lim[2], 1.0 / dx, 1.0 / dy, lim[1], lim[3], n,
                                           kind, sx, sy, seed);
  ORBIT_LAUNCH_CHECK("orbit_beam_deposit");
  ORBIT_CUDA(cudaDeviceSynchronize());
  return ORBIT_OK;
}

int orbit_grid_deposit(float* dev_grid, int nx, int ny, const double* lim, const double* dev_x, const double* dev_y,
                       long long n) {
  if (!dev_grid || !lim || !dev_x || !dev_y || nx < 3 || ny < 3 || n < 0 || !(lim[1] > lim[0]) ||
      !(lim[3] > lim[2]))
    return set_error(ORBIT_ERR_ARG, "orbit_grid_deposit: bad argument");
  size_t sm = sizeof(float) * (size_t)nx * ny;
  if (sm > 200 * 1024) return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_grid_deposit: grid above 200 KB of shared memory");
  static bool attr = false;
  if (!attr) {
    ORBIT_CUDA(cudaFuncSetAttribute(k_grid_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  ORBIT_CUDA(cudaMemset(dev_grid, 0, sm));
  double dx = (lim[1] - lim[0]) / (nx - 1), dy = (lim[3] - lim[2]) / (ny - 1);
  long long blocks = (n + 8191) / 8192;
  long long cap = (long long)num_sms() * 2;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_grid_deposit<<<(int)blocks, 512, sm>>>(dev_grid, nx, ny, lim[0], lim[2], 1.0 / dx, 1.0 / dy, lim[1], lim[3],
                                           dev_x, dev_y, n);
  ORBIT_LAUNCH_CHECK("orbit_grid_deposit");
  ORBIT_CUDA(cudaDeviceSynchronize());
  return ORBIT_OK;
}

int orbit_denoiser_create(orbit_denoiser_t** out, int max_batch, int h, int w, unsigned long long seed) {
  if (!out || max_batch < 1 || h < 8 || w < 8 || h % 8 || w % 8)
    return set_error(ORBIT_ERR_ARG, "orbit_denoiser_create: sizes must be multiples of 8 (three 2x2 poolings)");
  orbit_denoiser_t* d = new orbit_denoiser_t();
  d->H = h;
  d->W = w;
  d->maxb = max_batch;
  static const int cin[14] = {1, 16, 16, 32, 32, 64, 64, 64, 128, 64, 96, 32, 48, 16};
  static const int cout[14] = {16, 16, 32, 32, 64, 64, 64, 64, 64, 64, 32, 32, 16, 16};
  size_t off = 0;
  for (int k = 0; k < 14; ++k) {
    Conv c;
    c.cin = cin[k];
    c.cout = cout[k];
    c.w_off = off;
    off += (size_t)cin[k] * cout[k] * 9;
    c.b_off = off;
    off += cout[k];
    d->conv.push_back(c);
  }
  d->out_w = off;
  off += 16;
  d->out_b = off;
  off += 1;
  d->nparam = off;
  // initial parameters: He normal for the 3x3 weights, zero biases, small
  // output weights (the network starts near the identity)
  std::vector<float> p(off, 0.f);
  std::vector<unsigned char> isw(off, 0);
  uint64_t rs = seed ^ 0x6a09e667f3bcc909ull;
  for (auto& c : d->conv) {
    double sd = std::sqrt(2.0 / (9.0 * c.cin));
    for (size_t i = 0; i < (size_t)c.cin * c.cout * 9; ++i) {
      p[c.w_off + i] = (float)(sd * normal(rs));
      isw[c.w_off + i] = 1;
    }
  }
  for (int c = 0; c < 16; ++c) p[d->out_w + c] = (float)(0.01 * normal(rs));
  auto fail = [&](int code) {
    orbit_denoiser_destroy(d);
    return code;
  };
  // a blocking stream: work of the legacy default stream (where callers such
  // as PyTorch usually prepare the images) is ordered before it
  cudaError_t e = cudaStreamCreateWithFlags(&d->stream, cudaStreamDefault);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_p, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_pb, sizeof(__nv_bfloat16) * off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_g, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_m, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_v, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_isw, off);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(d->d_p, p.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d->d_isw, isw.data(), off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d->d_g, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(d->d_m, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(d->d_v, 0, sizeof(float) * off);
  d->act.assign(NACT, nullptr);
  d->grad.assign(NACT, nullptr);
  size_t widest = 0;
  for (int a = 0; a < NACT && e == cudaSuccess; ++a) {
    size_t n = act_size(d, a, max_batch);
    widest = n > widest ? n : widest;
    e = cudaMalloc(&d->act[a], sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d->grad[a], sizeof(float) * n);
  }
  if (e != cudaSuccess) return fail(cuda_error(e, "orbit_denoiser_create"));
  // scratch of the split convolutions: the largest splits x output
  size_t scratch = 1;
  for (int nb = 1; nb <= max_batch; ++nb)
    for (const Step3& stp : kSteps) {
      int c, hh, ww, sp, cp;
      act_shape(d, stp.out, &c, &hh, &ww);
      split_plan(d->conv[stp.ci], hh, ww, nb, &sp, &cp);
      if (sp > 1) scratch = std::max(scratch, (size_t)sp * act_size(d, stp.out, nb));
    }
  size_t wtc = 0, wtct = 0;
  for (size_t l = 0; l < d->conv.size(); ++l) {
    const Conv& cv = d->conv[l];
    d->tc_off.push_back(wtc);
    wtc += (size_t)((cv.cin * 9 + kTcKC - 1) / kTcKC) * cv.cout * kTcKC;
    d->tct_off.push_back(wtct);
    if (cv.cin >= 16) wtct += (size_t)((cv.cout * 9 + kTcKC - 1) / kTcKC) * cv.cin * kTcKC;
  }
  for (const Step3& stp : kSteps) {
    int c, hh, ww, tiles, nst;
    act_shape(d, stp.out, &c, &hh, &ww);
    tc_plan(d->conv[stp.ci], hh, ww, &tiles, &nst);
    if (nst > 1) scratch = std::max(scratch, (size_t)nst * d->conv[stp.ci].cout * hh * ww);
  }
  e = cudaMalloc(&d->d_scratch, sizeof(float) * scratch);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_wtc, sizeof(float) * wtc);
  if (e == cudaSuccess) e = cudaMalloc(&d->d_wtct, sizeof(float) * (wtct ? wtct : 1));
  if (e == cudaSuccess) e = cudaMalloc(&d->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d->d_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv3_tc<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return fail(cuda_error(e, "orbit_denoiser_create"));
  k_to_bf16<<<grid_1d(off), 256, 0, d->stream>>>(d->d_p, d->d_pb, d->d_isw, off);
  e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return fail(cuda_error(e, "orbit_denoiser_create"));
  *out = d;
  return ORBIT_OK;
}

int orbit_denoiser_destroy(orbit_denoiser_t* d) {
  if (!d) return ORBIT_OK;
  if (d->stream) cudaStreamSynchronize(d->stream);
  for (float* p : d->act) if (p) cudaFree(p);
  for (float* p : d->grad) if (p) cudaFree(p);
  for (auto v : {&d->ms_y, &d->ms_t, &d->ms_g})
    for (float* p : *v)
      if (p) cudaFree(p);
  void* bufs[] = {d->d_p,       d->d_pb,  d->d_g,    d->d_m,  d->d_v, d->d_isw,
                  d->d_loss,    d->d_scratch, d->d_wtc, d->d_wtct, d->d_err};
  for (void* b : bufs) if (b) cudaFree(b);
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
  return ORBIT_OK;
}

int orbit_denoiser_info(const orbit_denoiser_t* d, int* nparam, int* h, int* w, int* max_batch) {
  if (!d) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_info: bad argument");
  if (nparam) *nparam = (int)d->nparam;
  if (h) *h = d->H;
  if (w) *w = d->W;
  if (max_batch) *max_batch = d->maxb;
  return ORBIT_OK;
}

int orbit_denoiser_get_params(orbit_denoiser_t* d, float* host) {
  if (!d || !host) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_get_params: bad argument");
  ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  ORBIT_CUDA(cudaMemcpy(host, d->d_p, sizeof(float) * d->nparam, cudaMemcpyDeviceToHost));
  return ORBIT_OK;
}

int orbit_denoiser_set_params(orbit_denoiser_t* d, const float* host) {
  if (!d || !host) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_params: bad argument");
  ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  ORBIT_CUDA(cudaMemcpy(d->d_p, host, sizeof(float) * d->nparam, cudaMemcpyHostToDevice));
  ORBIT_CUDA(cudaMemset(d->d_m, 0, sizeof(float) * d->nparam));
  ORBIT_CUDA(cudaMemset(d->d_v, 0, sizeof(float) * d->nparam));
  d->step = 0;
  k_to_bf16<<<grid_1d(d->nparam), 256, 0, d->stream>>>(d->d_p, d->d_pb, d->d_isw, d->nparam);
  ORBIT_LAUNCH_CHECK("orbit_denoiser_set_params");
  d->tc_stale = true;
  d->tct_stale = true;
  ++d->version;
  ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  return ORBIT_OK;
}

int orbit_denoiser_forward(orbit_denoiser_t* d, const float* dev_in, float* dev_out, int nb, void* stream) {
  if (!d || !dev_in || !dev_out) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_forward: bad argument");
  int rc = check_batch(d, nb);
  if (rc) return rc;
  cudaStream_t st = stream_of(d, stream);
  const size_t n = (size_t)nb * d->H * d->W;
  ORBIT_CUDA(cudaMemcpyAsync(d->act[X0], dev_in, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  rc = forward(d, nb, st, true);
  if (rc) return rc;
  ORBIT_CUDA(cudaMemcpyAsync(dev_out, d->act[Y], sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  return ORBIT_OK;
}

int orbit_denoiser_set_batch_tensor_cores(orbit_denoiser_t* d, int on) {
  if (!d) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_batch_tensor_cores: bad argument");
  if (d->stream) ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  d->tcb = on != 0;
  return ORBIT_OK;
}

int orbit_denoiser_set_tensor_cores(orbit_denoiser_t* d, int on) {
  if (!d) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_tensor_cores: bad argument");
  d->tc = on != 0;
  return ORBIT_OK;
}

int orbit_denoiser_tensor_status(orbit_denoiser_t* d, int* on, int* err) {
  if (!d) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_tensor_status: bad argument");
  ORBIT_CUDA(cudaStreamSynchronize(d->stream));
  ORBIT_CUDA(cudaDeviceSynchronize());
  if (on) *on = (d->tc && !d->tc_failed && !g_tc_untrusted) ? 1 : 0;
  if (err) {
    ORBIT_CUDA(cudaMemcpy(err, d->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    ORBIT_CUDA(cudaMemset(d->d_err, 0, sizeof(int)));
    // after a failed wait this network runs its single-image forwards on
    // the CUDA-core layers; after an MMA that never completed no network does
    if (*err) d->tc_failed = true;
    if (*err & 2) g_tc_untrusted = true;
  }
  return ORBIT_OK;
}

int orbit_denoiser_set_loss(orbit_denoiser_t* d, int levels, const float* weights) {
  if (!d || levels < 0 || levels > 7 || (levels > 0 && !weights))
    return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_loss: bad argument");
  if (levels > 0 && ((d->H >> levels) < 1 || (d->W >> levels) < 1 || (d->H % (1 << levels)) || (d->W % (1 << levels))))
    return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_loss: the image does not halve that many times");
  ORBIT_CUDA(cudaDeviceSynchronize());  // training work in flight may use the level buffers
  for (auto v : {&d->ms_y, &d->ms_t, &d->ms_g}) {
    for (float* p : *v)
      if (p) cudaFree(p);
    v->assign(levels + 1, nullptr);
  }
  for (int s = 1; s <= levels; ++s) {
    const size_t bytes = sizeof(float) * (size_t)d->maxb * (d->H >> s) * (d->W >> s);
    ORBIT_CUDA(cudaMalloc(&d->ms_y[s], bytes));
    ORBIT_CUDA(cudaMalloc(&d->ms_t[s], bytes));
    ORBIT_CUDA(cudaMalloc(&d->ms_g[s], bytes));
  }
  d->loss_levels = levels;
  for (int s = 0; s < 8; ++s) d->loss_w[s] = s <= levels ? (levels ? weights[s] : 1.f) : 0.f;
  return ORBIT_OK;
}

int orbit_denoiser_set_wait_limit(orbit_denoiser_t* d, long long cycles, int withhold_mma) {
  if (!d || cycles <= 0) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_set_wait_limit: bad argument");
  d->tc_wait_cycles = cycles;
  d->tc_withhold = withhold_mma != 0;
  return ORBIT_OK;
}

int orbit_denoiser_train_step(orbit_denoiser_t* d, const float* dev_in, const float* dev_target, int nb, float lr,
                              float* loss, void* stream) {
  if (!d || !dev_in || !dev_target) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_train_step: bad argument");
  int rc = check_batch(d, nb);
  if (rc) return rc;
  cudaStream_t st = stream_of(d, stream);
  const size_t n = (size_t)nb * d->H * d->W;
  ORBIT_CUDA(cudaMemcpyAsync(d->act[X0], dev_in, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  rc = loss_and_grads(d, dev_target, nb, st);
  if (rc) return rc;
  d->step += 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)d->step)));
  float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)d->step)));
  k_adam<<<grid_1d(d->nparam), 256, 0, st>>>(d->d_p, d->d_g, d->d_m, d->d_v, d->d_pb, d->d_isw, d->nparam, lr, b1,
                                              b2, eps, c1, c2);
  ORBIT_LAUNCH_CHECK("denoiser adam");
  d->tc_stale = true;
  d->tct_stale = true;
  ++d->version;
  if (loss) {
    ORBIT_CUDA(cudaMemcpyAsync(loss, d->d_loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    ORBIT_CUDA(cudaStreamSynchronize(st));
    return tcb_status(d);
  }
  return ORBIT_OK;
}

int orbit_denoiser_gradients(orbit_denoiser_t* d, const float* dev_in, const float* dev_target, int nb, float* grads,
                             float* loss, float* dev_out, void* stream) {
  if (!d || !dev_in || !dev_target || !grads) return set_error(ORBIT_ERR_ARG, "orbit_denoiser_gradients: bad argument");
  int rc = check_batch(d, nb);
  if (rc) return rc;
  cudaStream_t st = stream_of(d, stream);
  const size_t n = (size_t)nb * d->H * d->W;
  ORBIT_CUDA(cudaMemsetAsync(d->d_g, 0, sizeof(float) * d->nparam, st));
  ORBIT_CUDA(cudaMemcpyAsync(d->act[X0], dev_in, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  rc = loss_and_grads(d, dev_target, nb, st);
  if (rc) return rc;
  ORBIT_CUDA(cudaMemcpyAsync(grads, d->d_g, sizeof(float) * d->nparam, cudaMemcpyDeviceToHost, st));
  if (loss) ORBIT_CUDA(cudaMemcpyAsync(loss, d->d_loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  if (dev_out) ORBIT_CUDA(cudaMemcpyAsync(dev_out, d->act[Y], sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
  ORBIT_CUDA(cudaMemsetAsync(d->d_g, 0, sizeof(float) * d->nparam, st));
  ORBIT_CUDA(cudaStreamSynchronize(st));
  return tcb_status(d);
}

}  // extern "C"
