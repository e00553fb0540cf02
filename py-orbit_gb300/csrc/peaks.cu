// Device roofs measured in-process for the benchmark's roofline report:
// FP64 fused multiply-add throughput (independent DFMA chains on every SM)
// and streaming copy bandwidth.  No counterpart in the reference.
#include <cstring>

#include "common.cuh"
#include "softf64.cuh"

namespace orbit {

__global__ void k_dfma_chain(double* out, int iters, double a, double b) {
  double r[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) r[k] = threadIdx.x + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = fma(r[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += r[k];
  if (s == 123456.789) out[0] = s;  // keeps the chains alive
}

// HW chains of hardware binary64 multiplies and SW chains of integer-pipe
// ones (sf::mul), all independent, per thread.
template <int HW, int SW>
__global__ void k_dmul_chains(double* out, int iters, double a) {
  double r[HW + SW + 1];
#pragma unroll
  for (int q = 0; q < HW + SW; ++q) r[q] = 1.0 + threadIdx.x * 1e-9 + q * 1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < HW; ++q) r[q] = __dmul_rn(r[q], a);
#pragma unroll
    for (int q = HW; q < HW + SW; ++q) r[q] = sf::mul(r[q], a);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < HW + SW; ++q) s += r[q];
  if (s == 123456.789) out[0] = s;  // keeps the chains alive
}

template <int HW, int SW>
static double dmul_rate(double* out, cudaEvent_t e0, cudaEvent_t e1) {
  const int blocks = num_sms() * 2, threads = 512, iters = 1000;
  k_dmul_chains<HW, SW><<<blocks, threads>>>(out, 10, 1.0000001);
  if (cudaDeviceSynchronize() != cudaSuccess) return -1.0;
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dmul_chains<HW, SW><<<blocks, threads>>>(out, iters, 1.0000001);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  return (double)blocks * threads * iters * (HW + SW) / (best * 1e-3) / 1e9;
}

// Operand classes of the device check of sf::mul / add / fma / scale2,
// drawn from a counter hash (splitmix64) of the case index.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double normal_operand(uint64_t r, uint64_t r2, int spread) {
  const int e = (int)(r2 % (uint64_t)(2 * spread + 1)) - spread;
  const double x = sf::from_bits((r >> 12) | ((uint64_t)(1023 + e) << 52));
  return (r2 >> 63) ? -x : x;
}

// One case per thread and loop step; counts[0..5] = mismatches of mul, add,
// fma, scale2, to_float and from_float against the hardware instructions
// (__dmul_rn, __dadd_rn, __fma_rn, a multiply by the power of two,
// __double2float_rn, the float-to-double conversion), NaN matching any NaN.
__global__ void k_softf64_check(long long n, uint64_t seed, unsigned long long* counts) {
  unsigned long long bad[6] = {0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const uint64_t h = mix64(seed ^ (uint64_t)i);
    uint64_t r[6];
    for (int q = 0; q < 6; ++q) r[q] = mix64(h + (uint64_t)q);
    const int cls = (int)(i % 10), sp = (int)((i / 10) % 4);
    const int spread = sp == 0 ? 1000 : (sp == 1 ? 60 : (sp == 2 ? 5 : 0));
    double a = normal_operand(r[0], r[1], spread), b = normal_operand(r[2], r[3], spread),
           c = normal_operand(r[4], r[5], spread);
    switch (cls) {
      case 1: c = -__dmul_rn(a, b); break;                                               // total cancellation
      case 2: c = sf::from_bits(sf::bits(-__dmul_rn(a, b)) ^ (r[5] & 0xFF)); break;     // near cancellation
      case 3: b = sf::from_bits(sf::bits(-a) ^ (r[3] & 0xFFF)); break;                   // add cancellation
      case 4: b = sf::from_bits(sf::bits(a) ^ (r[3] & 0xF)); break;                      // close significands
      case 5: a = sf::from_bits(r[0] | (1ull << 52)); b = sf::from_bits((r[2] & 0x3FFFFFF000ull) | 0x3FF0000000000000ull); break;  // short b: ties
      case 6: b = sf::from_bits(sf::bits(b) & ~((1ull << ((r[3] >> 58) % 52)) - 1)); break;
      case 7: c = __dmul_rn(__dmul_rn(a, b), 0x1p-53) * ((r[5] & 1) ? 1.5 : 0.5); break;  // fma ties
      case 8: a = sf::from_bits(r[0]); b = sf::from_bits(r[2]); c = sf::from_bits(r[4]); break;
      case 9: a = (r[0] & 1) ? 0.0 : -0.0; break;
      default: break;
    }
    const double m1 = __dmul_rn(a, b), m2 = sf::mul(a, b);
    const double s1 = __dadd_rn(a, b), s2 = sf::add(a, b);
    const double f1 = __fma_rn(a, b, c), f2 = sf::fma(a, b, c);
    const int k = (r[5] & 2) ? 1 : -1;
    const double k1 = __dmul_rn(a, k > 0 ? 2.0 : 0.5), k2 = sf::scale2(a, k);
    bad[0] += !(sf::bits(m1) == sf::bits(m2) || (m1 != m1 && m2 != m2));
    bad[1] += !(sf::bits(s1) == sf::bits(s2) || (s1 != s1 && s2 != s2));
    bad[2] += !(sf::bits(f1) == sf::bits(f2) || (f1 != f1 && f2 != f2));
    bad[3] += !(sf::bits(k1) == sf::bits(k2) || (k1 != k1 && k2 != k2));
    // conversions: a over the float range (and exact ties), a random float
    double t = (cls & 1) ? a : __dmul_rn(a, __longlong_as_double((long long)((uint64_t)(1023 + (int)(r[1] % 300) - 150) << 52)));
    if (cls == 5) t = sf::from_bits((sf::bits(t) & ~((1ull << 29) - 1)) | (1ull << 28));
    const float c1 = __double2float_rn(t), c2 = sf::to_float(t);
    bad[4] += !(sf::fbits(c1) == sf::fbits(c2) || (c1 != c1 && c2 != c2));
    const float rf = sf::from_fbits((uint32_t)r[4]);
    const double e1 = (double)rf, e2 = sf::from_float(rf);
    bad[5] += !(sf::bits(e1) == sf::bits(e2) || (e1 != e1 && e2 != e2));
  }
  for (int q = 0; q < 6; ++q)
    if (bad[q]) atomicAdd(counts + q, bad[q]);
}

__global__ void k_copy(const double2* __restrict__ a, double2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

}  // namespace orbit

using namespace orbit;

extern "C" int orbit_device_peaks(double* fp64_tflops, double* copy_gbs) {
  if (!fp64_tflops || !copy_gbs) return set_error(ORBIT_ERR_ARG, "orbit_device_peaks: bad argument");
  cudaEvent_t e0, e1;
  ORBIT_CUDA(cudaEventCreate(&e0));
  ORBIT_CUDA(cudaEventCreate(&e1));
  double* out = nullptr;
  ORBIT_CUDA(cudaMalloc(&out, sizeof(double)));
  int blocks = num_sms() * 8, threads = 256, iters = 4000;
  k_dfma_chain<<<blocks, threads>>>(out, 10, 1.0000001, 1e-9);
  ORBIT_CUDA(cudaDeviceSynchronize());
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dfma_chain<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    ORBIT_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  *fp64_tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (best * 1e-3) / 1e12;
  cudaFree(out);
  size_t n = (size_t)1 << 26;  // 64 Mi double2 = 1 GiB per buffer
  double2 *a = nullptr, *b = nullptr;
  cudaError_t e = cudaMalloc(&a, n * sizeof(double2));
  if (e == cudaSuccess) e = cudaMalloc(&b, n * sizeof(double2));
  if (e == cudaSuccess) e = cudaMemset(a, 0, n * sizeof(double2));
  if (e != cudaSuccess) {
    if (a) cudaFree(a);
    if (b) cudaFree(b);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cuda_error(e, "orbit_device_peaks");
  }
  best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_copy<<<num_sms() * 4, 1024>>>(a, b, n);
    cudaEventRecord(e1);
    ORBIT_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  *copy_gbs = 2.0 * n * sizeof(double2) / (best * 1e-3) / 1e9;
  cudaFree(a);
  cudaFree(b);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ORBIT_OK;
}

// Binary64 multiply rates (G multiplies/s, correctly rounded, all SMs): on
// the FP64 pipe alone, on the integer pipes alone (sf::mul) and half on
// each, which run at the same time.
extern "C" int orbit_device_mul_rates(double* fp64_gmul, double* int_gmul, double* mixed_gmul) {
  if (!fp64_gmul || !int_gmul || !mixed_gmul) return set_error(ORBIT_ERR_ARG, "orbit_device_mul_rates: bad argument");
  cudaEvent_t e0, e1;
  ORBIT_CUDA(cudaEventCreate(&e0));
  ORBIT_CUDA(cudaEventCreate(&e1));
  double* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double));
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cuda_error(e, "orbit_device_mul_rates");
  }
  *fp64_gmul = dmul_rate<12, 0>(out, e0, e1);
  *int_gmul = dmul_rate<0, 12>(out, e0, e1);
  *mixed_gmul = dmul_rate<6, 6>(out, e0, e1);
  cudaFree(out);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (*fp64_gmul < 0 || *int_gmul < 0 || *mixed_gmul < 0)
    return set_error(ORBIT_ERR_CUDA, "orbit_device_mul_rates: kernel failed");
  return ORBIT_OK;
}

// Device check of the integer-pipe binary64 routines against the FP64
// instructions on n generated cases (operand classes in k_softf64_check).
extern "C" int orbit_softf64_check(long long n, unsigned long long seed, long long* mismatches) {
  if (n < 0 || !mismatches) return set_error(ORBIT_ERR_ARG, "orbit_softf64_check: bad argument");
  unsigned long long* d = nullptr;
  ORBIT_CUDA(cudaMalloc(&d, 6 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 6 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_softf64_check<<<num_sms() * 4, 256>>>(n, (uint64_t)seed, d);
    e = cudaGetLastError();
  }
  unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_error(e, "orbit_softf64_check");
  for (int q = 0; q < 6; ++q) mismatches[q] = (long long)h[q];
  return ORBIT_OK;
}
