// Shared declarations of the orbit_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdint>
#include <string>

#include "../../include/orbit_gb300.h"

namespace orbit {

// ---------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------
int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* where);

#define ORBIT_CUDA(expr)                                   \
  do {                                                     \
    cudaError_t _e = (expr);                               \
    if (_e != cudaSuccess) return ::orbit::cuda_error(_e, #expr); \
  } while (0)

#define ORBIT_LAUNCH_CHECK(where)                          \
  do {                                                     \
    cudaError_t _e = cudaGetLastError();                   \
    if (_e != cudaSuccess) return ::orbit::cuda_error(_e, where); \
  } while (0)

// device status word bits (per bunch)
enum : unsigned {
  ST_EXTENT = 1u,   // zero beam extent at an SC kick
  ST_NAN = 2u,      // non-finite coordinate
  ST_RANGE = 4u,    // grid index out of range (should not happen)
  ST_SYNC = 8u,     // a grid-wide barrier of the fused convolution ran out of its wait limit
};

int num_sms();

// Optional per-launch timing (orbit_program_profile): when a profiler is
// installed on the calling thread, every launch site brackets its kernel
// with a pair of CUDA events on the launching stream.
struct Profiler;
extern thread_local Profiler* g_prof;
void prof_begin(const char* tag, cudaStream_t s);
void prof_end(cudaStream_t s);
Profiler* prof_install();
int prof_collect(Profiler* p, int max_kinds, char* names, double* total_ms, int* launches, int* nkinds);
// Host-side NVTX range around one reference-level call (a teapot_base map,
// an SC kick, the turns of a lattice program or of a batch), so that
// Nsight Systems timelines and ncu's --nvtx filters show the node structure.
// nvtx3 is header-only: without an attached tool a range costs a branch.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define ORBIT_NVTX(name) ::orbit::NvtxRange orbit_nvtx_range_(name)

#define ORBIT_PB(tag, s) do { if (::orbit::g_prof) ::orbit::prof_begin(tag, s); } while (0)
#define ORBIT_PE(s) do { if (::orbit::g_prof) ::orbit::prof_end(s); } while (0)

// ---------------------------------------------------------------------
// device-side helpers
// ---------------------------------------------------------------------
// Order-preserving map of a finite double's bits onto uint64 so that
// integer min/max equals double min/max; runs on the integer pipe.
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}
__device__ __forceinline__ bool dfinite_bits(double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return ((u >> 52) & 0x7ff) != 0x7ff;
}

}  // namespace orbit

// ---------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------
struct orbit_bunch {
  int n = 0;
  int cap = 0;            // elements per coordinate array
  double* d_coords = nullptr;   // 6 * cap
  double* d_msize = nullptr;    // optional per-particle macrosize
  int has_msize = 0;
  double msize_abs_sum = 0.0;   // sum |m_i| of the per-particle macrosizes
  unsigned* d_status = nullptr; // device status word
  unsigned* h_status = nullptr; // pinned mirror
  cudaStream_t stream = nullptr;
  orbit_sync_t sync{};
  // diagnostics: per-particle phase attributes (6 rows of phase_cap) and the
  // reduction scratch of the moments
  double* d_phase = nullptr;
  int phase_cap = 0;
  double* d_diag = nullptr;
  double* coord(int c) const { return d_coords + (size_t)c * cap; }
};
