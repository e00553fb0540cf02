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
