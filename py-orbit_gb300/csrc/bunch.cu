// Bunch handles (device SoA storage), error reporting and device queries.
// Replaces the reference's AoS Bunch storage (src/orbit/Bunch.cc:52-56,
// 445-455): six contiguous FP64 arrays resident in HBM.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace orbit {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_error(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return (e == cudaErrorMemoryAllocation) ? ORBIT_ERR_NOMEM : ORBIT_ERR_CUDA;
}

struct Profiler {
  struct Rec {
    const char* tag;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
};
thread_local Profiler* g_prof = nullptr;

void prof_begin(const char* tag, cudaStream_t s) {
  Profiler::Rec r;
  r.tag = tag;
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, s);
  g_prof->recs.push_back(r);
}

// The host waits for each timed launch, so that every bracket times its own
// launch alone: without the wait, the brackets of the large ring's eager
// turn (1.6e7 particles, launches of milliseconds) each read about one kick
// longer than the launch they enclose, their sum six times the turn.
void prof_end(cudaStream_t s) {
  if (g_prof->recs.empty()) return;
  cudaEventRecord(g_prof->recs.back().b, s);
  cudaEventSynchronize(g_prof->recs.back().b);
}

Profiler* prof_install() {
  g_prof = new Profiler();
  return g_prof;
}

// Sums the elapsed time per tag (in first-seen order) and removes the profiler.
int prof_collect(Profiler* p, int max_kinds, char* names, double* total_ms, int* launches, int* nkinds) {
  g_prof = nullptr;
  std::vector<std::string> tags;
  std::vector<double> ms;
  std::vector<int> cnt;
  cudaError_t err = cudaSuccess;
  for (auto& r : p->recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaError_t e = cudaEventElapsedTime(&t, r.a, r.b);
    if (e != cudaSuccess) err = e;
    size_t k = 0;
    while (k < tags.size() && tags[k] != r.tag) ++k;
    if (k == tags.size()) {
      tags.push_back(r.tag);
      ms.push_back(0.0);
      cnt.push_back(0);
    }
    ms[k] += t;
    cnt[k] += 1;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  delete p;
  if (err != cudaSuccess) return cuda_error(err, "prof_collect");
  int nk = (int)tags.size() < max_kinds ? (int)tags.size() : max_kinds;
  for (int k = 0; k < nk; ++k) {
    std::memset(names + 32 * k, 0, 32);
    std::strncpy(names + 32 * k, tags[k].c_str(), 31);
    total_ms[k] = ms[k];
    launches[k] = cnt[k];
  }
  *nkinds = nk;
  return ORBIT_OK;
}

int num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

static int reserve(orbit_bunch_t* b, int n) {
  if (n <= b->cap) return ORBIT_OK;
  int cap = (n + 255) & ~255;
  double* d = nullptr;
  ORBIT_CUDA(cudaMalloc(&d, sizeof(double) * 6 * (size_t)cap));
  if (b->d_coords) {
    // keep existing particles
    for (int c = 0; c < 6; ++c)
      ORBIT_CUDA(cudaMemcpyAsync(d + (size_t)c * cap, b->coord(c), sizeof(double) * b->n,
                                 cudaMemcpyDeviceToDevice, b->stream));
    ORBIT_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(b->d_coords);
  }
  if (b->d_msize) {
    double* m = nullptr;
    ORBIT_CUDA(cudaMalloc(&m, sizeof(double) * (size_t)cap));
    ORBIT_CUDA(cudaMemcpyAsync(m, b->d_msize, sizeof(double) * b->n, cudaMemcpyDeviceToDevice, b->stream));
    ORBIT_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(b->d_msize);
    b->d_msize = m;
  }
  b->d_coords = d;
  b->cap = cap;
  return ORBIT_OK;
}

int check_status(orbit_bunch_t* b) {
  ORBIT_CUDA(cudaMemcpyAsync(b->h_status, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  unsigned st = *b->h_status;
  if (st == 0) return ORBIT_OK;
  ORBIT_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), b->stream));
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  if (st & ST_NAN) return set_error(ORBIT_ERR_NAN, "non-finite particle coordinate found by the extrema scan");
  if (st & ST_SYNC)
    return set_error(ORBIT_ERR_DEVICE,
                     "fused convolution: a grid-wide barrier ran out of its wait limit; the kick's potential is invalid");
  if (st & ST_EXTENT)
    return set_error(ORBIT_ERR_EXTENT,
                     "SpaceChargeCalc2p5D: the bunch min and max sizes are wrong (zero extent); kick skipped");
  return set_error(ORBIT_ERR_DEVICE, "device-side range check failed");
}

}  // namespace orbit

using namespace orbit;

extern "C" {

int orbit_last_error(char* buf, int len) {
  int n = (int)g_last_error.size();
  if (buf && len > 0) {
    int m = n < len - 1 ? n : len - 1;
    std::memcpy(buf, g_last_error.data(), (size_t)m);
    buf[m] = 0;
  }
  return n;
}

const char* orbit_version(void) { return "orbit_gb300 0.1 sm_103a"; }

int orbit_bunch_create(orbit_bunch_t** out, int capacity) {
  if (!out || capacity < 0) return set_error(ORBIT_ERR_ARG, "orbit_bunch_create: bad argument");
  orbit_bunch_t* b = new orbit_bunch_t();
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete b; return cuda_error(e, "cudaStreamCreate"); }
  e = cudaMalloc(&b->d_status, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_status, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), b->stream);
  if (e != cudaSuccess) { orbit_bunch_destroy(b); return cuda_error(e, "orbit_bunch_create"); }
  b->sync.beta = 0; b->sync.gamma = 1; b->sync.momentum = 0; b->sync.mass = 0.938272013;
  b->sync.charge = 1.0; b->sync.classical_radius = 1.534698e-18; b->sync.macrosize = 0.0;
  if (capacity > 0) {
    int rc = reserve(b, capacity);
    if (rc != ORBIT_OK) { orbit_bunch_destroy(b); return rc; }
  }
  *out = b;
  return ORBIT_OK;
}

int orbit_bunch_destroy(orbit_bunch_t* b) {
  if (!b) return ORBIT_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->d_coords) cudaFree(b->d_coords);
  if (b->d_msize) cudaFree(b->d_msize);
  if (b->d_phase) cudaFree(b->d_phase);
  if (b->d_diag) cudaFree(b->d_diag);
  if (b->d_status) cudaFree(b->d_status);
  if (b->h_status) cudaFreeHost(b->h_status);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return ORBIT_OK;
}

int orbit_bunch_upload(orbit_bunch_t* b, const double* const* soa, int n) {
  if (!b || n < 0 || (n > 0 && !soa)) return set_error(ORBIT_ERR_ARG, "orbit_bunch_upload: bad argument");
  int rc = reserve(b, n);
  if (rc) return rc;
  for (int c = 0; c < 6 && n > 0; ++c) {
    if (!soa[c]) return set_error(ORBIT_ERR_ARG, "orbit_bunch_upload: null coordinate array");
    ORBIT_CUDA(cudaMemcpyAsync(b->coord(c), soa[c], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
  }
  b->n = n;
  return ORBIT_OK;
}

int orbit_bunch_upload_device(orbit_bunch_t* b, const double* const* soa, int n) {
  if (!b || n < 0 || (n > 0 && !soa)) return set_error(ORBIT_ERR_ARG, "orbit_bunch_upload_device: bad argument");
  int rc = reserve(b, n);
  if (rc) return rc;
  for (int c = 0; c < 6 && n > 0; ++c)
    ORBIT_CUDA(cudaMemcpyAsync(b->coord(c), soa[c], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, b->stream));
  b->n = n;
  return ORBIT_OK;
}

int orbit_bunch_download(orbit_bunch_t* b, double* const* soa) {
  if (!b || (b->n > 0 && !soa)) return set_error(ORBIT_ERR_ARG, "orbit_bunch_download: bad argument");
  for (int c = 0; c < 6 && b->n > 0; ++c)
    ORBIT_CUDA(cudaMemcpyAsync(soa[c], b->coord(c), sizeof(double) * (size_t)b->n, cudaMemcpyDeviceToHost, b->stream));
  return check_status(b);
}

int orbit_bunch_size(const orbit_bunch_t* b, int* n) {
  if (!b || !n) return set_error(ORBIT_ERR_ARG, "orbit_bunch_size: bad argument");
  *n = b->n;
  return ORBIT_OK;
}

int orbit_bunch_set_sync(orbit_bunch_t* b, const orbit_sync_t* s) {
  if (!b || !s) return set_error(ORBIT_ERR_ARG, "orbit_bunch_set_sync: bad argument");
  b->sync = *s;
  return ORBIT_OK;
}

int orbit_bunch_get_sync(const orbit_bunch_t* b, orbit_sync_t* s) {
  if (!b || !s) return set_error(ORBIT_ERR_ARG, "orbit_bunch_get_sync: bad argument");
  *s = b->sync;
  return ORBIT_OK;
}

int orbit_bunch_set_macrosizes(orbit_bunch_t* b, const double* m, int n) {
  if (!b) return set_error(ORBIT_ERR_ARG, "orbit_bunch_set_macrosizes: null bunch");
  if (!m) {
    b->has_msize = 0;
    return ORBIT_OK;
  }
  if (n != b->n) return set_error(ORBIT_ERR_ARG, "orbit_bunch_set_macrosizes: size differs from the bunch size");
  if (!b->d_msize) ORBIT_CUDA(cudaMalloc(&b->d_msize, sizeof(double) * (size_t)(b->cap > 0 ? b->cap : 1)));
  if (n > 0) ORBIT_CUDA(cudaMemcpyAsync(b->d_msize, m, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
  double acc = 0.0;
  for (int i = 0; i < n; ++i) acc += m[i] < 0 ? -m[i] : m[i];
  b->msize_abs_sum = acc;
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  b->has_msize = 1;
  return ORBIT_OK;
}

int orbit_bunch_device_coords(orbit_bunch_t* b, double** dev_soa) {
  if (!b || !dev_soa) return set_error(ORBIT_ERR_ARG, "orbit_bunch_device_coords: bad argument");
  for (int c = 0; c < 6; ++c) dev_soa[c] = b->d_coords ? b->coord(c) : nullptr;
  return ORBIT_OK;
}

int orbit_bunch_sync(orbit_bunch_t* b) {
  if (!b) return set_error(ORBIT_ERR_ARG, "orbit_bunch_sync: null bunch");
  return check_status(b);
}

int orbit_bunch_stream(orbit_bunch_t* b, void** stream) {
  if (!b || !stream) return set_error(ORBIT_ERR_ARG, "orbit_bunch_stream: bad argument");
  *stream = (void*)b->stream;
  return ORBIT_OK;
}

}  // extern "C"

// NVTX ranges opened and closed by the host layer (the lattice walk names
// each node); no counterpart in the reference.
extern "C" int orbit_nvtx_push(const char* name) {
  nvtxRangePushA(name ? name : "");
  return ORBIT_OK;
}

extern "C" int orbit_nvtx_pop(void) {
  nvtxRangePop();
  return ORBIT_OK;
}
