// Bunch diagnostics on the device (src/orbit/BunchDiagnostics): the first and
// second moments of BunchTwissAnalysis::analyzeBunch as a deterministic
// two-level reduction, and BunchTuneAnalysis::analyzeBunch per particle
// with its attributes kept on the device.  No coordinate leaves the GPU.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "sc2p5d.cuh"
#include "sc_device.cuh"

namespace orbit {

static const int kMomThreads = 256;
static const int kNMom = 28;  // total macrosize, 6 first moments, 21 second moments (i >= j)

// Per-block sums of m, m c_i, m c_i c_j (i >= j), summed in a fixed order:
// the block results go to part[block], the last block adds them up in block
// order into out[28].
template <bool MS>
__global__ void __launch_bounds__(kMomThreads) k_moments(const double* __restrict__ coords, int cap, int n,
                                                         const double* __restrict__ msize, double* part,
                                                         unsigned* counter, double* out) {
  double s[kNMom];
#pragma unroll
  for (int k = 0; k < kNMom; ++k) s[k] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double c[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) c[q] = coords[(size_t)q * cap + i];
    double m = MS ? msize[i] : 1.0;
    s[0] += m;
    int k = 7;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      double mc = MS ? m * c[q] : c[q];
      s[1 + q] += mc;
#pragma unroll
      for (int r = 0; r <= q; ++r) s[k++] += mc * c[r];
    }
  }
  __shared__ double red[kMomThreads / 32][kNMom];
#pragma unroll
  for (int k = 0; k < kNMom; ++k)
    for (int off = 16; off > 0; off >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], off);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < kNMom; ++k) red[threadIdx.x >> 5][k] = s[k];
  __syncthreads();
  if (threadIdx.x < kNMom) {
    double t = 0.0;
    for (int w = 0; w < kMomThreads / 32; ++w) t += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * kNMom + threadIdx.x] = t;
  }
  if (last_block_done(counter, gridDim.x) && threadIdx.x < kNMom) {
    double t = 0.0;
    for (int bk = 0; bk < (int)gridDim.x; ++bk) t += __ldcg(part + (size_t)bk * kNMom + threadIdx.x);
    out[threadIdx.x] = t;
  }
}

// BunchTwissAnalysis::computeBunchMoments (BunchTwissAnalysis.cc:146-340):
// per block sums, for the cell (i, j) = cells[blockIdx.y], of the
// reference's per-particle term with its recurrences and operation order:
// momX[k+1] = momX[k] (* m) * ((x - dispterm) - xAvg), momY likewise from
// y - yAvg; the term ((momX[i] / xb^i) momY[j]) / yb^j, plus momX[i] momY[j]
// with per-particle macrosizes; cell index -1: the product
// momX[2] momY[order] that the reference's uniform-macrosize loop adds once
// per particle after its loops.  p = {D, E_kin + m, beta^2, xAvg, yAvg};
// pw[k] = xb^k, pw[17 + k] = yb^k (the host's pow).
__global__ void k_xy_moments(const double* __restrict__ coords, int cap, int n, const double* __restrict__ msize,
                             const int2* __restrict__ cells, int order, const double* __restrict__ p,
                             const double* __restrict__ pw, double* __restrict__ part) {
  const int2 cell = cells[blockIdx.y];
  const bool stray = cell.x < 0;
  const int ci = stray ? 2 : cell.x, cj = stray ? order : cell.y;
  const double D = p[0], ekm = p[1], b2 = p[2], xa = p[3], ya = p[4];
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double x = coords[k], y = coords[(size_t)2 * cap + k], de = coords[(size_t)5 * cap + k];
    const double disp = D != 0.0 ? __ddiv_rn(__ddiv_rn(__dmul_rn(D, de), ekm), b2) : 0.0;
    const double dx = __dsub_rn(__dsub_rn(x, disp), xa), dy = __dsub_rn(y, ya);
    const double m = msize ? msize[k] : 1.0;
    double mx = 1.0, my = 1.0;
    for (int q = 0; q < ci; ++q) mx = msize ? __dmul_rn(__dmul_rn(mx, m), dx) : __dmul_rn(mx, dx);
    for (int q = 0; q < cj; ++q) my = msize ? __dmul_rn(__dmul_rn(my, m), dy) : __dmul_rn(my, dy);
    if (stray) {
      s = __dadd_rn(s, __dmul_rn(mx, my));
    } else {
      s = __dadd_rn(s, __ddiv_rn(__dmul_rn(__ddiv_rn(mx, pw[ci]), my), pw[17 + cj]));
      if (msize) s = __dadd_rn(s, __dmul_rn(mx, my));
    }
  }
  __shared__ double red[8];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
}

struct TuneArgs {
  double betax, alphax, etax, etapx, betay, alphay;
  double beta, etot;
};

// BunchTuneAnalysis::analyzeBunch (BunchTuneAnalysis.cc:36-108): normalised
// phases, the phase advance since the last call and the actions; ph holds
// six rows {xLastPhase, yLastPhase, xLastTune, yLastTune, xAction, yAction}.
__global__ void k_tune(const double* __restrict__ coords, int cap, int n, TuneArgs a, double* ph, int pcap) {
  const double twopi = 2.0 * 3.14159265358979323846;  // 2 OrbitConst::PI
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double x = coords[i], xp = coords[(size_t)cap + i];
    double y = coords[2 * (size_t)cap + i], yp = coords[3 * (size_t)cap + i];
    double dE = coords[5 * (size_t)cap + i];
    double dpp = 1 / (a.beta * a.beta) * dE / a.etot;
    double sbx = sqrt(a.betax), sby = sqrt(a.betay);
    double xval = (x - a.etax * dpp) / sbx;
    double xpval = (xp - a.etapx * dpp) * sbx + xval * a.alphax;
    double yval = y / sby;
    double ypval = (yp + y * a.alphay / a.betay) * sby;
    double ang = atan2(xpval, xval);
    if (ang < 0.) ang += twopi;
    double xt = (ph[i] - ang) / twopi;
    if (xt < 0.) xt += 1.;
    ph[i] = ang;
    ph[2 * (size_t)pcap + i] = xt;
    ang = atan2(ypval, yval);
    if (ang < 0.) ang += twopi;
    double yt = (ph[(size_t)pcap + i] - ang) / twopi;
    if (yt < 0.) yt += 1.;
    ph[(size_t)pcap + i] = ang;
    ph[3 * (size_t)pcap + i] = yt;
    double xc = x - a.etax * dpp, yc = y;
    double pxc = (xp - a.etapx * dpp) + xc * (a.alphax / a.betax);
    double pyc = yp + yc * (a.alphay / a.betay);
    ph[4 * (size_t)pcap + i] = xc * xc / a.betax + pxc * pxc * a.betax;
    ph[5 * (size_t)pcap + i] = yc * yc / a.betay + pyc * pyc * a.betay;
  }
}

static int moment_blocks() { return num_sms() * 2; }

// Phase rows of capacity >= n, zero for particles without a value yet.
static int ensure_phase(orbit_bunch_t* b) {
  if (b->d_phase && b->phase_cap >= b->n) return ORBIT_OK;
  int cap = b->cap > b->n ? b->cap : b->n;
  if (cap < 1) cap = 1;
  double* d = nullptr;
  ORBIT_CUDA(cudaMalloc(&d, sizeof(double) * 6 * (size_t)cap));
  ORBIT_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * 6 * (size_t)cap, b->stream));
  if (b->d_phase) {
    int keep = b->phase_cap < b->n ? b->phase_cap : b->n;
    for (int r = 0; r < 6; ++r)
      ORBIT_CUDA(cudaMemcpyAsync(d + (size_t)r * cap, b->d_phase + (size_t)r * b->phase_cap, sizeof(double) * keep,
                                 cudaMemcpyDeviceToDevice, b->stream));
    ORBIT_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(b->d_phase);
  }
  b->d_phase = d;
  b->phase_cap = cap;
  return ORBIT_OK;
}

}  // namespace orbit

using namespace orbit;

extern "C" {

int orbit_bunch_moments(orbit_bunch_t* b, double* out) {
  if (!b || !out) return set_error(ORBIT_ERR_ARG, "orbit_bunch_moments: bad argument");
  const int nb = moment_blocks();
  if (!b->d_diag) {
    // partials, 28 results, then the block counter
    ORBIT_CUDA(cudaMalloc(&b->d_diag, sizeof(double) * ((size_t)nb * kNMom + kNMom + 1)));
    ORBIT_CUDA(cudaMemsetAsync(b->d_diag, 0, sizeof(double) * ((size_t)nb * kNMom + kNMom + 1), b->stream));
  }
  double* part = b->d_diag;
  double* res = part + (size_t)nb * kNMom;
  unsigned* counter = reinterpret_cast<unsigned*>(res + kNMom);
  double h[kNMom];
  if (b->n > 0) {
    if (b->has_msize)
      k_moments<true><<<nb, kMomThreads, 0, b->stream>>>(b->d_coords, b->cap, b->n, b->d_msize, part, counter, res);
    else
      k_moments<false><<<nb, kMomThreads, 0, b->stream>>>(b->d_coords, b->cap, b->n, nullptr, part, counter, res);
    ORBIT_LAUNCH_CHECK("moments");
    ORBIT_CUDA(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, b->stream));
    ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  } else {
    for (int k = 0; k < kNMom; ++k) h[k] = 0.0;
  }
  // BunchTwissAnalysis.cc:95-140: averages and correlations over the total macrosize
  const double total = h[0];
  out[0] = b->n;
  out[1] = total;
  for (int k = 1; k < kNMom; ++k) out[k + 1] = std::fabs(total) > 0. ? h[k] / total : 0.0;
  return ORBIT_OK;
}

int orbit_bunch_xy_moments(orbit_bunch_t* b, int order, const double* params, double* out) {
  if (!b || !params || !out || order < 2 || order > 16)
    return set_error(ORBIT_ERR_ARG, "orbit_bunch_xy_moments: bad argument (2 <= order <= 16)");
  // the cells the reference accumulates (j < order, i <= order - j), and its stray cell
  std::vector<int2> cells;
  for (int j = 0; j < order; ++j)
    for (int i = 0; i < order + 1 - j; ++i) cells.push_back(make_int2(i, j));
  const bool uniform = !b->has_msize;
  if (uniform) cells.push_back(make_int2(-1, -1));
  const int nc = (int)cells.size(), nb = moment_blocks();
  double hp[5] = {params[0], params[1], params[2], params[3], params[4]};
  double hpw[34];
  for (int k = 0; k <= 16; ++k) {
    hpw[k] = std::pow(params[5], (double)k);  // pow(xbetaterm, double(i)) (BunchTwissAnalysis.cc:249)
    hpw[17 + k] = std::pow(params[6], (double)k);
  }
  int2* d_cells = nullptr;
  double *d_p = nullptr, *d_part = nullptr;
  std::vector<double> part((size_t)nc * nb, 0.0);
  auto release = [&]() {
    if (d_cells) cudaFree(d_cells);
    if (d_p) cudaFree(d_p);
    if (d_part) cudaFree(d_part);
  };
  cudaError_t e = cudaMalloc(&d_cells, sizeof(int2) * nc);
  if (e == cudaSuccess) e = cudaMalloc(&d_p, sizeof(double) * 39);
  if (e == cudaSuccess) e = cudaMalloc(&d_part, sizeof(double) * part.size());
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_cells, cells.data(), sizeof(int2) * nc, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_p, hp, sizeof(hp), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_p + 5, hpw, sizeof(hpw), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess && b->n > 0) {
    k_xy_moments<<<dim3(nb, nc), kMomThreads, 0, b->stream>>>(b->d_coords, b->cap, b->n,
                                                               uniform ? nullptr : b->d_msize, d_cells, order, d_p,
                                                               d_p + 5, d_part);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, b->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  release();
  if (e != cudaSuccess) return cuda_error(e, "orbit_bunch_xy_moments");
  // block partials in block order; total macrosize: n for a uniform macrosize
  // (the reference's m_size = 1 there), else the sum of the macrosizes
  double total = (double)b->n;
  if (!uniform) {
    double mom[29];
    int rc = orbit_bunch_moments(b, mom);
    if (rc) return rc;
    total = mom[1];
  }
  const int w = order + 1;
  for (int k = 0; k < w * w; ++k) out[k] = 0.0;
  for (int c = 0; c < nc; ++c) {
    double t = 0.0;
    for (int bk = 0; bk < nb; ++bk) t += part[(size_t)c * nb + bk];
    const int i = cells[c].x < 0 ? 2 : cells[c].x, j = cells[c].x < 0 ? order : cells[c].y;
    out[i * w + j] += t;
  }
  // BunchTwissAnalysis.cc:325-336: divided for i + j <= order (the stray
  // cell [2][order] is not), then the three fixed cells
  if (std::fabs(total) > 0.)
    for (int i = 0; i < w; ++i)
      for (int j = 0; j < w - i; ++j) out[i * w + j] /= total;
  out[0] = 1.0;
  out[1 * w + 0] = params[3];
  out[0 * w + 1] = params[4];
  return ORBIT_OK;
}

int orbit_bunch_tune_analysis(orbit_bunch_t* b, const double* twiss, double etot) {
  if (!b || !twiss) return set_error(ORBIT_ERR_ARG, "orbit_bunch_tune_analysis: bad argument");
  int rc = ensure_phase(b);
  if (rc) return rc;
  if (b->n == 0) return ORBIT_OK;
  TuneArgs a;
  a.betax = twiss[0]; a.alphax = twiss[1]; a.etax = twiss[2]; a.etapx = twiss[3];
  a.betay = twiss[4]; a.alphay = twiss[5];
  a.beta = b->sync.beta;
  a.etot = etot;
  int blocks = (b->n + 255) / 256;
  if (blocks > num_sms() * 8) blocks = num_sms() * 8;
  k_tune<<<blocks, 256, 0, b->stream>>>(b->d_coords, b->cap, b->n, a, b->d_phase, b->phase_cap);
  ORBIT_LAUNCH_CHECK("tune analysis");
  return ORBIT_OK;
}

int orbit_bunch_phase_get(orbit_bunch_t* b, double* host) {
  if (!b || (!host && b->n > 0)) return set_error(ORBIT_ERR_ARG, "orbit_bunch_phase_get: bad argument");
  if (!b->d_phase) return set_error(ORBIT_ERR_ARG, "orbit_bunch_phase_get: no tune analysis has run");
  for (int r = 0; r < 6; ++r)
    ORBIT_CUDA(cudaMemcpyAsync(host + (size_t)r * b->n, b->d_phase + (size_t)r * b->phase_cap,
                               sizeof(double) * b->n, cudaMemcpyDeviceToHost, b->stream));
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  return ORBIT_OK;
}

int orbit_bunch_phase_set(orbit_bunch_t* b, const double* host) {
  if (!b || (!host && b->n > 0)) return set_error(ORBIT_ERR_ARG, "orbit_bunch_phase_set: bad argument");
  int rc = ensure_phase(b);
  if (rc) return rc;
  for (int r = 0; r < 6; ++r)
    ORBIT_CUDA(cudaMemcpyAsync(b->d_phase + (size_t)r * b->phase_cap, host + (size_t)r * b->n,
                               sizeof(double) * b->n, cudaMemcpyHostToDevice, b->stream));
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  return ORBIT_OK;
}

}  // extern "C"
