// Device roofs measured in-process for the benchmark's roofline report:
// FP64 fused multiply-add throughput (independent DFMA chains on every SM)
// and streaming copy bandwidth.  No counterpart in the reference.
#include <cstring>

#include "common.cuh"

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
