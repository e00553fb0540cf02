// Per-particle device routines of the 2.5D space-charge kick, shared by the
// stand-alone kernels (sc2p5d.cu) and the fused lattice passes (program.cu).
#pragma once

#include "common.cuh"
#include "sc2p5d.cuh"

namespace orbit {

// ---------------------------------------------------------------------
// extrema (BunchExtremaCalculator::getExtremaXYZ, src/utils/bunch/
// BunchExtremaCalculator.cc:37-83) on order-preserving integer keys
// ---------------------------------------------------------------------
struct ExtAcc {
  unsigned long long mn[3], mx[3];
  bool bad;
  __device__ __forceinline__ void init() {
    for (int c = 0; c < 3; ++c) { mn[c] = ~0ull; mx[c] = 0ull; }
    bad = false;
  }
  __device__ __forceinline__ void add(double x, double y, double z) {
    double v[3] = {x, y, z};
    for (int c = 0; c < 3; ++c) {
      if (!dfinite_bits(v[c])) { bad = true; continue; }
      unsigned long long k = dkey(v[c]);
      mn[c] = k < mn[c] ? k : mn[c];
      mx[c] = k > mx[c] ? k : mx[c];
    }
  }
};

// Block-wide reduction, then one atomic per key per block.
__device__ __forceinline__ void ext_block_commit(ExtAcc& a, ScState* st, unsigned* status) {
  __shared__ unsigned long long s_k[32][6];
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  for (int c = 0; c < 3; ++c) {
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long o1 = __shfl_xor_sync(0xffffffffu, a.mn[c], off);
      unsigned long long o2 = __shfl_xor_sync(0xffffffffu, a.mx[c], off);
      a.mn[c] = o1 < a.mn[c] ? o1 : a.mn[c];
      a.mx[c] = o2 > a.mx[c] ? o2 : a.mx[c];
    }
  }
  __syncthreads();
  if (a.bad) s_bad = 1;
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int c = 0; c < 3; ++c) { s_k[w][2 * c] = a.mn[c]; s_k[w][2 * c + 1] = a.mx[c]; }
  __syncthreads();
  if (threadIdx.x < 6) {
    int nw = (blockDim.x + 31) >> 5;
    unsigned long long v = s_k[0][threadIdx.x];
    bool is_min = (threadIdx.x & 1) == 0;
    for (int q = 1; q < nw; ++q) {
      unsigned long long u = s_k[q][threadIdx.x];
      v = is_min ? (u < v ? u : v) : (u > v ? u : v);
    }
    if (is_min) atomicMin(&st->key[threadIdx.x], v);
    else atomicMax(&st->key[threadIdx.x], v);
  }
  if (threadIdx.x == 0 && s_bad) atomicOr(status, (unsigned)ST_NAN);
}

// ---------------------------------------------------------------------
// 9-point TSC weights (Grid2D.cc:147-156, 220-233)
// ---------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void tsc_index(T t, int n, int& ind, T& frac) {
  // ind = int(t + 0.5) clamped to [1, n-2]; frac = t - ind  (Grid2D.cc:337-349)
  int i = (int)(t + (T)0.5);
  i = i < 1 ? 1 : i;
  i = i > n - 2 ? n - 2 : i;
  ind = i;
  frac = t - (T)i;
}

template <typename T>
__device__ __forceinline__ void tsc_weights(T f, T& wm, T& w0, T& wp) {
  T f2 = f * f;
  wm = (T)0.5 * ((T)0.25 - f + f2);
  w0 = (T)0.75 - f2;
  wp = (T)0.5 * ((T)0.25 + f + f2);
}

// ---------------------------------------------------------------------
// line density index (Grid1D::getIndAndWZ, Grid1D.cc:568-627)
// ---------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void g1_index(T z, T zmin, T inv_dz, int nz, int& i0, int& ip, T& w0, T& wp) {
  if (nz > 1) {
    T ind_dbl = (z - zmin) * inv_dz - (T)0.5;
    int iz0 = (int)ind_dbl;
    iz0 = iz0 > nz - 1 ? nz - 1 : iz0;
    T zf = ind_dbl - (T)iz0;
    if (iz0 == 0 && zf < (T)0) {
      i0 = nz - 1; ip = 0; w0 = -zf; wp = (T)1 + zf;
      return;
    }
    if (iz0 == nz - 1) {
      if (zf > (T)0) { i0 = iz0; ip = 0; w0 = (T)1 - zf; wp = zf; return; }
      ip = iz0; i0 = nz - 2; w0 = -zf; wp = (T)1 + zf;
      return;
    }
    i0 = iz0; ip = iz0 + 1; w0 = (T)1 - zf; wp = zf;
    return;
  }
  i0 = 0; ip = 0; w0 = (T)1; wp = (T)0;
}

// ---------------------------------------------------------------------
// kick (SpaceChargeCalc2p5D.cc:104-119 with Grid2D::calcGradient and
// Grid1D::getValue)
// ---------------------------------------------------------------------
struct KickConst {
  double xmin, ymin, inv_dx, inv_dy, zmin, zmax, inv_dz, fac;
  int nx, ny, nz;
  int skip;
};

__device__ __forceinline__ void load_kick_const(KickConst& k, const ScState* st, double host_factor,
                                                int nx, int ny, int nz) {
  k.xmin = st->xmin; k.ymin = st->ymin; k.inv_dx = st->inv_dx; k.inv_dy = st->inv_dy;
  k.zmin = st->zmin; k.zmax = st->zmax; k.inv_dz = st->inv_dz;
  // factor = 2 L r_c/(beta^2 gamma^3) / (z_step * totalMacrosize)  (:96-100)
  k.fac = host_factor / (st->dz * st->total_m);
  k.nx = nx; k.ny = ny; k.nz = nz;
  k.skip = st->skip;
}

// FP64 plain form: phi/lam may be in shared or global memory.
__device__ __forceinline__ void kick_plain(const KickConst& k, const double* __restrict__ phi,
                                           const double* __restrict__ lam, double x, double y, double z,
                                           double& xp, double& yp) {
  int ix, iy;
  double fx, fy;
  tsc_index<double>((x - k.xmin) * k.inv_dx, k.nx, ix, fx);
  tsc_index<double>((y - k.ymin) * k.inv_dy, k.ny, iy, fy);
  double wxm, wx0, wxp, wym, wy0, wyp;
  tsc_weights<double>(fx, wxm, wx0, wxp);
  tsc_weights<double>(fy, wym, wy0, wyp);
  // dW = -(0.5 - f), -2f, 0.5 + f  (Grid2D.cc:228-233)
  double dxm = fx - 0.5, dx0 = -2.0 * fx, dxp = 0.5 + fx;
  double dym = fy - 0.5, dy0 = -2.0 * fy, dyp = 0.5 + fy;
  const double* r0 = phi + (ix - 1) * k.ny + (iy - 1);
  const double* r1 = r0 + k.ny;
  const double* r2 = r1 + k.ny;
  double a00 = r0[0], a01 = r0[1], a02 = r0[2];
  double a10 = r1[0], a11 = r1[1], a12 = r1[2];
  double a20 = r2[0], a21 = r2[1], a22 = r2[2];
  // separable sums: rows weighted along y, then along x
  double s0 = wym * a00 + wy0 * a01 + wyp * a02;
  double s1 = wym * a10 + wy0 * a11 + wyp * a12;
  double s2 = wym * a20 + wy0 * a21 + wyp * a22;
  double t0 = dym * a00 + dy0 * a01 + dyp * a02;
  double t1 = dym * a10 + dy0 * a11 + dyp * a12;
  double t2 = dym * a20 + dy0 * a21 + dyp * a22;
  double gx = dxm * s0 + dx0 * s1 + dxp * s2;
  double gy = wxm * t0 + wx0 * t1 + wxp * t2;
  // lambda(z)  (Grid1D.cc:191-209)
  double lv = 0.0;
  if (!(z < k.zmin || z > k.zmax)) {
    int i0, ip;
    double w0, wp;
    g1_index<double>(z, k.zmin, k.inv_dz, k.nz, i0, ip, w0, wp);
    lv = (k.nz > 1) ? (w0 * lam[i0] + wp * lam[ip]) : lam[0];
  }
  double lf = -lv * k.fac;
  xp += gx * k.inv_dx * lf;
  yp += gy * k.inv_dy * lf;
}

// FP32 form: gradient and line density in FP32, accumulation into FP64.
__device__ __forceinline__ void kick_fp32(const KickConst& k, const float* __restrict__ phi,
                                          const float* __restrict__ lam, double x, double y, double z,
                                          double& xp, double& yp) {
  float tx = (float)((x - k.xmin) * k.inv_dx);
  float ty = (float)((y - k.ymin) * k.inv_dy);
  int ix, iy;
  float fx, fy;
  tsc_index<float>(tx, k.nx, ix, fx);
  tsc_index<float>(ty, k.ny, iy, fy);
  float wxm, wx0, wxp, wym, wy0, wyp;
  tsc_weights<float>(fx, wxm, wx0, wxp);
  tsc_weights<float>(fy, wym, wy0, wyp);
  float dxm = fx - 0.5f, dx0 = -2.0f * fx, dxp = 0.5f + fx;
  float dym = fy - 0.5f, dy0 = -2.0f * fy, dyp = 0.5f + fy;
  const float* r0 = phi + (ix - 1) * k.ny + (iy - 1);
  const float* r1 = r0 + k.ny;
  const float* r2 = r1 + k.ny;
  float a00 = r0[0], a01 = r0[1], a02 = r0[2];
  float a10 = r1[0], a11 = r1[1], a12 = r1[2];
  float a20 = r2[0], a21 = r2[1], a22 = r2[2];
  float s0 = wym * a00 + wy0 * a01 + wyp * a02;
  float s1 = wym * a10 + wy0 * a11 + wyp * a12;
  float s2 = wym * a20 + wy0 * a21 + wyp * a22;
  float t0 = dym * a00 + dy0 * a01 + dyp * a02;
  float t1 = dym * a10 + dy0 * a11 + dyp * a12;
  float t2 = dym * a20 + dy0 * a21 + dyp * a22;
  float gx = dxm * s0 + dx0 * s1 + dxp * s2;
  float gy = wxm * t0 + wx0 * t1 + wxp * t2;
  float lv = 0.0f;
  if (!(z < k.zmin || z > k.zmax)) {
    float zt = (float)((z - k.zmin) * k.inv_dz);
    int i0, ip;
    float w0, wp;
    g1_index<float>(zt, 0.0f, 1.0f, k.nz, i0, ip, w0, wp);
    lv = (k.nz > 1) ? (w0 * lam[i0] + wp * lam[ip]) : lam[0];
  }
  float lf = -lv * (float)k.fac;
  xp += (double)(gx * (float)k.inv_dx * lf);
  yp += (double)(gy * (float)k.inv_dy * lf);
}

// ---------------------------------------------------------------------
// deposit (Grid2D::binValue, Grid2D.cc:141-166; Grid1D::binValue,
// Grid1D.cc:422-439)
// ---------------------------------------------------------------------
struct DepConst {
  double xmin, xmax, ymin, ymax, inv_dx, inv_dy, zmin, zmax, inv_dz;
  int nx, ny, nz;
  int skip;
};

__device__ __forceinline__ void load_dep_const(DepConst& d, const ScState* st, int nx, int ny, int nz) {
  d.xmin = st->xmin; d.xmax = st->xmax; d.ymin = st->ymin; d.ymax = st->ymax;
  d.inv_dx = st->inv_dx; d.inv_dy = st->inv_dy;
  d.zmin = st->zmin; d.zmax = st->zmax; d.inv_dz = st->inv_dz;
  d.nx = nx; d.ny = ny; d.nz = nz;
  d.skip = st->skip;
}

// Plain form: contributions are rounded to a fixed-point grid of step 1/S
// (S a power of two with S * total macrosize <= 2^62) and summed as 64-bit
// integers, so the deposit is exact and independent of summation order.
__device__ __forceinline__ void deposit_plain(const DepConst& d, unsigned long long* rho, unsigned long long* zg,
                                              double x, double y, double z, double ms) {
  if (!(x < d.xmin || x > d.xmax || y < d.ymin || y > d.ymax)) {
    int ix, iy;
    double fx, fy;
    tsc_index<double>((x - d.xmin) * d.inv_dx, d.nx, ix, fx);
    tsc_index<double>((y - d.ymin) * d.inv_dy, d.ny, iy, fy);
    double wxm, wx0, wxp, wym, wy0, wyp;
    tsc_weights<double>(fx, wxm, wx0, wxp);
    tsc_weights<double>(fy, wym, wy0, wyp);
    double ax[3] = {wxm * ms, wx0 * ms, wxp * ms};
    double wy[3] = {wym, wy0, wyp};
    unsigned long long* base = rho + (ix - 1) * d.ny + (iy - 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        atomicAdd(base + i * d.ny + j, (unsigned long long)__double2ll_rn(ax[i] * wy[j]));
  }
  if (!(z < d.zmin || z > d.zmax)) {
    int i0, ip;
    double w0, wp;
    g1_index<double>(z, d.zmin, d.inv_dz, d.nz, i0, ip, w0, wp);
    if (d.nz > 1) {
      atomicAdd(zg + i0, (unsigned long long)__double2ll_rn(w0 * ms));
      atomicAdd(zg + ip, (unsigned long long)__double2ll_rn(wp * ms));
    } else {
      atomicAdd(zg, (unsigned long long)__double2ll_rn(ms));
    }
  }
}

__device__ __forceinline__ void deposit_fp32(const DepConst& d, float* rho, float* zg, double x, double y,
                                             double z, float m) {
  if (!(x < d.xmin || x > d.xmax || y < d.ymin || y > d.ymax)) {
    float tx = (float)((x - d.xmin) * d.inv_dx);
    float ty = (float)((y - d.ymin) * d.inv_dy);
    int ix, iy;
    float fx, fy;
    tsc_index<float>(tx, d.nx, ix, fx);
    tsc_index<float>(ty, d.ny, iy, fy);
    float wxm, wx0, wxp, wym, wy0, wyp;
    tsc_weights<float>(fx, wxm, wx0, wxp);
    tsc_weights<float>(fy, wym, wy0, wyp);
    float ax[3] = {wxm * m, wx0 * m, wxp * m};
    float wy[3] = {wym, wy0, wyp};
    float* base = rho + (ix - 1) * d.ny + (iy - 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) atomicAdd(base + i * d.ny + j, ax[i] * wy[j]);
  }
  if (!(z < d.zmin || z > d.zmax)) {
    float zt = (float)((z - d.zmin) * d.inv_dz);
    int i0, ip;
    float w0, wp;
    g1_index<float>(zt, 0.0f, 1.0f, d.nz, i0, ip, w0, wp);
    if (d.nz > 1) {
      atomicAdd(zg + i0, w0 * m);
      atomicAdd(zg + ip, wp * m);
    } else {
      atomicAdd(zg, m);
    }
  }
}

}  // namespace orbit
