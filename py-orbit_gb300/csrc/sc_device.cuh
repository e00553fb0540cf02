// Per-particle device routines of the 2.5D space-charge kick, shared by the
// stand-alone kernels (sc2p5d.cu) and the fused lattice passes (program.cu).
#pragma once

#include "common.cuh"
#include "softf64.cuh"
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
// Grid set-up of bunchAnalysis (SpaceChargeCalc2p5D.cc:126-216), run by
// one thread of the last block of the kernel that scanned the extrema.
// ---------------------------------------------------------------------
// Explicitly rounded operations (no contraction), so that the grid limits
// and the persistent xy_ratio evolve exactly as the reference's.  The keys
// and the status word were written by atomics of other blocks: they are
// read from L2.
static __device__ __noinline__ void sc_setup_scalar(ScState* st, unsigned* status, SetupArgs sa) {
  unsigned long long key[6];
  for (int c = 0; c < 6; ++c) key[c] = __ldcg(&st->key[c]);
  double xMin = dkey_inv(key[0]), xMax = dkey_inv(key[1]);
  double yMin = dkey_inv(key[2]), yMax = dkey_inv(key[3]);
  double zMin = dkey_inv(key[4]), zMax = dkey_inv(key[5]);
  for (int c = 0; c < 3; ++c) { st->key[2 * c] = ~0ull; st->key[2 * c + 1] = 0ull; }
  st->conv_bar[0] = 0u;
  st->conv_bar[1] = 0u;
  if (sa.bnd) {
    // a boundary fixes the transverse grid to its extents; only z comes
    // from the bunch (SpaceChargeCalc2p5D.cc:174-196)
    xMin = sa.bxmin; xMax = sa.bxmax; yMin = sa.bymin; yMax = sa.bymax;
  }
  int skip = 0;
  if (__ldcg(status) & ST_NAN) {
    // a non-finite coordinate was met by the extrema scan: no kick
    skip = 1;
  } else if (!(xMin < xMax) || !(yMin < yMax) || !(zMin < zMax)) {  // :131 (also catches an empty scan)
    skip = 1;
    atomicOr(status, (unsigned)ST_EXTENT);
  } else {
    double xy = st->xy_ratio;
    double ratio_beam = __ddiv_rn(__dsub_rn(xMax, xMin), __dsub_rn(yMax, yMin));
    int set_solver = 0;
    if (sa.bnd) {
      xy = ratio_beam;  // :180
    } else if (sa.rb) {
      // SpaceChargeCalc2p5Drb::bunchAnalysis (SpaceChargeCalc2p5Drb.cc:188-203):
      // always stretched to the calculator's own ratio, which never changes
      double width, center;
      if (ratio_beam > xy) {
        center = __ddiv_rn(__dadd_rn(yMax, yMin), 2.0);
        width = __ddiv_rn(__dmul_rn(__dsub_rn(yMax, yMin), __ddiv_rn(ratio_beam, xy)), 2.0);
        yMin = __dsub_rn(center, width);
        yMax = __dadd_rn(center, width);
      } else {
        center = __ddiv_rn(__dadd_rn(xMax, xMin), 2.0);
        width = __ddiv_rn(__ddiv_rn(__dsub_rn(xMax, xMin), __ddiv_rn(ratio_beam, xy)), 2.0);
        xMin = __dsub_rn(center, width);
        xMax = __dadd_rn(center, width);
      }
    } else if (fabs(__dsub_rn(ratio_beam, xy)) < __dmul_rn(0.25, xy)) {  // :152-168
      double width, center;
      if (ratio_beam > xy) {
        center = __ddiv_rn(__dadd_rn(yMax, yMin), 2.0);
        width = __ddiv_rn(__dmul_rn(__dsub_rn(yMax, yMin), __ddiv_rn(ratio_beam, xy)), 2.0);
        yMin = __dsub_rn(center, width);
        yMax = __dadd_rn(center, width);
      } else {
        center = __ddiv_rn(__dadd_rn(xMax, xMin), 2.0);
        width = __ddiv_rn(__ddiv_rn(__dsub_rn(xMax, xMin), __ddiv_rn(ratio_beam, xy)), 2.0);
        xMin = __dsub_rn(center, width);
        xMax = __dadd_rn(center, width);
      }
      xy = __ddiv_rn(__dsub_rn(xMax, xMin), __dsub_rn(yMax, yMin));
    } else {  // :169-173
      xy = ratio_beam;
      set_solver = 1;
    }
    // Grid2D::setGridX/Y (Grid2D.cc:422-433), Grid1D::setGridZ (Grid1D.cc:89-94)
    double dx = __ddiv_rn(__dsub_rn(xMax, xMin), (double)(sa.nx - 1));
    double dy = __ddiv_rn(__dsub_rn(yMax, yMin), (double)(sa.ny - 1));
    double dz = __ddiv_rn(__dsub_rn(zMax, zMin), (double)sa.nz);
    st->xmin = xMin; st->xmax = xMax; st->ymin = yMin; st->ymax = yMax;
    st->dx = dx; st->dy = dy; st->inv_dx = __drcp_rn(dx); st->inv_dy = __drcp_rn(dy);
    st->zmin = zMin; st->zmax = zMax; st->dz = dz; st->inv_dz = __drcp_rn(dz);
    if (!sa.rb) st->xy_ratio = xy;
    // solver-shape check (SpaceChargeCalc2p5D.cc:208-216); the 2.5Drb
    // calculator keeps its solver grid
    if (!set_solver && !sa.rb) {
      double sr = __ddiv_rn(__dsub_rn(st->sxmax, st->sxmin), __dsub_rn(st->symax, st->symin));
      if (fabs(__dsub_rn(sr, xy)) > 0.00000001) set_solver = 1;
    }
    if (set_solver) {  // PoissonSolverFFT2D::setGridXY (PoissonSolverFFT2D.cc:103-111)
      st->sxmin = xMin; st->sxmax = xMax; st->symin = yMin; st->symax = yMax;
      st->sdx = dx; st->sdy = dy;
      st->green_dirty = 1;
    }
    st->scale = log(__ddiv_rn(st->sdx, dx));  // PoissonSolverFFT2D.cc:213
    st->inv_qscale = sa.inv_qscale;
    st->phi_absmax = 0ull;
    st->lam_absmax = 0ull;
    if (sa.cond) cudaGraphSetConditional(sa.cond, st->green_dirty ? 1u : 0u);
  }
  st->skip = skip;
}

// True in exactly one of the nblk blocks that share `counter` (all blocks
// of the grid, or of one bunch of a batched launch): the last to call it.
// Every thread's earlier global writes and atomics are fenced before the
// block is counted; `counter` is left at zero for the next launch.
__device__ __forceinline__ bool last_block_done(unsigned* counter, unsigned nblk) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned prev = atomicAdd(counter, 1u);
    s_last = prev == nblk - 1;
    if (s_last) {
      *counter = 0u;
      __threadfence();
    }
  }
  __syncthreads();
  return s_last != 0;
}

// Extrema commit followed, in the last of the nblk blocks scanning this
// bunch, by the grid set-up.
__device__ __forceinline__ void ext_commit_and_setup(ExtAcc& a, ScState* st, unsigned* status,
                                                     const SetupArgs& sa, unsigned nblk) {
  ext_block_commit(a, st, status);
  if (last_block_done(&st->ext_count, nblk) && threadIdx.x == 0) sc_setup_scalar(st, status, sa);
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
  // FP32 form: grid coordinates t = x inv_dx + c; the z range test on
  // order-preserving integer keys; the float constants.  f32: the grid
  // origin lies within four grid extents of the coordinate origin, so t is
  // formed in float from the coordinate converted on the integer pipes:
  // t = fma(xf, ih, ch) + fma(xf, il, cl), 1/dx = ih + il and c = ch + cl
  // as float pairs, so that no rounding of a per-kick constant shifts or
  // stretches the whole grid (the kick would then sample the field away
  // from where the deposit put the charge); what is left are the unbiased
  // roundings of x and of the two operations, a few 2^-24 x n cells.
  // Otherwise one FP64 FMA and a conversion per coordinate.
  double cx, cy, cz;
  unsigned long long kzmin, kzmax;
  float inv_dx_f, inv_dy_f, fac_f;
  float ihx, ilx, chx, clx, ihy, ily, chy, cly, ihz, ilz, chz, clz;
  int f32;
  int nx, ny, nz;
  int skip;
};

// v as a float pair hi + lo (hi = float(v), lo = float(v - hi)).
__device__ __forceinline__ void split_f(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Grid coordinate of the FP32 form from a float coordinate and the float
// pairs of 1/dx and the offset.
__device__ __forceinline__ float grid_t_f32(float xf, float ih, float il, float ch, float cl) {
  return fmaf(xf, ih, ch) + fmaf(xf, il, cl);
}

// Whether the FP32 form's grid coordinates can be formed in float (see
// KickConst::f32).
__device__ __forceinline__ int grid_f32_ok(double cx, double cy, double cz, int nx, int ny, int nz) {
  return fabs(cx) <= 4.0 * nx && fabs(cy) <= 4.0 * ny && fabs(cz) <= 4.0 * nz + 4.0;
}

// f32: also the FP32 form's constants (a dozen FP64 operations the plain
// form does not need; one thread computes them while the block waits).
__device__ __forceinline__ void load_kick_const(KickConst& k, const ScState* st, double host_factor,
                                                int nx, int ny, int nz, bool f32 = true) {
  k.xmin = st->xmin; k.ymin = st->ymin; k.inv_dx = st->inv_dx; k.inv_dy = st->inv_dy;
  k.zmin = st->zmin; k.zmax = st->zmax; k.inv_dz = st->inv_dz;
  // factor = 2 L r_c/(beta^2 gamma^3) / (z_step * totalMacrosize)  (:96-100)
  k.fac = host_factor / (st->dz * st->total_m);
  k.nx = nx; k.ny = ny; k.nz = nz;
  k.skip = st->skip;
  if (!f32) return;
  k.cx = -k.xmin * k.inv_dx;
  k.cy = -k.ymin * k.inv_dy;
  k.cz = -k.zmin * k.inv_dz;
  k.kzmin = dkey(k.zmin);
  k.kzmax = dkey(k.zmax);
  k.inv_dx_f = (float)k.inv_dx;
  k.inv_dy_f = (float)k.inv_dy;
  k.fac_f = (float)k.fac;
  split_f(k.inv_dx, k.ihx, k.ilx);
  split_f(k.cx, k.chx, k.clx);
  split_f(k.inv_dy, k.ihy, k.ily);
  split_f(k.cy, k.chy, k.cly);
  split_f(k.inv_dz, k.ihz, k.ilz);
  split_f(k.cz, k.chz, k.clz);
  k.f32 = grid_f32_ok(k.cx, k.cy, k.cz, nx, ny, nz);
}

// 2.5Drb longitudinal kick (SpaceChargeCalc2p5Drb.cc:132-154):
// dE += ez(z) * lsf * coeff(r^2), ez the smoothed derivative of the line
// density (Grid1D::getValue), r measured from the beam centre, coeff =
// 1 + 2 ln(R/a) - r^2/a^2 inside a = a_bunch, 2 ln R - ln r^2 outside.
struct RbConst {
  double xc, yc, a2, lin, lout, lsf;
};

__device__ __forceinline__ void load_rb_const(RbConst& r, const ScState* st, double lsf) {
  r.xc = st->rb_xc; r.yc = st->rb_yc; r.a2 = st->rb_a2;
  r.lin = st->rb_lin; r.lout = st->rb_lout; r.lsf = lsf;
}

__device__ __forceinline__ void kick_rb_long(const KickConst& k, const RbConst& r, const double* __restrict__ lamd,
                                             double x, double y, double z, double& dE) {
  double ez = 0.0;
  if (!(z < k.zmin || z > k.zmax)) {
    int i0, ip;
    double w0, wp;
    g1_index<double>(z, k.zmin, k.inv_dz, k.nz, i0, ip, w0, wp);
    ez = (k.nz > 1) ? (w0 * lamd[i0] + wp * lamd[ip]) : lamd[0];
  }
  double ddx = x - r.xc, ddy = y - r.yc;
  double r2 = ddx * ddx + ddy * ddy;
  double coeff = (r2 <= r.a2) ? r.lin - r2 / r.a2 : r.lout - log(r2);
  dE += ez * r.lsf * coeff;
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
  // the FP64 pipe bounds the pass: the coordinates converted to float on
  // the integer pipes (or one FMA and a conversion each, far from the
  // origin), the z range test on integer keys
  float tx, ty;
  if (k.f32) {
    tx = grid_t_f32(sf::to_float(x), k.ihx, k.ilx, k.chx, k.clx);
    ty = grid_t_f32(sf::to_float(y), k.ihy, k.ily, k.chy, k.cly);
  } else {
    tx = (float)fma(x, k.inv_dx, k.cx);
    ty = (float)fma(y, k.inv_dy, k.cy);
  }
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
  const unsigned long long kz = dkey(z);
  if (kz >= k.kzmin && kz <= k.kzmax) {
    float zt = k.f32 ? grid_t_f32(sf::to_float(z), k.ihz, k.ilz, k.chz, k.clz) : (float)fma(z, k.inv_dz, k.cz);
    int i0, ip;
    float w0, wp;
    g1_index<float>(zt, 0.0f, 1.0f, k.nz, i0, ip, w0, wp);
    lv = (k.nz > 1) ? (w0 * lam[i0] + wp * lam[ip]) : lam[0];
  }
  float lf = -lv * k.fac_f;
  xp += sf::from_float(gx * k.inv_dx_f * lf);
  yp += sf::from_float(gy * k.inv_dy_f * lf);
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

// 64-bit accumulation grids.  Global: native 64-bit atomics.  Shared: each
// cell is a low and a high 32-bit word in two separate arrays (so that
// random cells spread over all 32 banks), added with native 32-bit atomics:
// the low word wraps modulo 2^32 and the add that wraps carries 1 into the
// high word, so hi * 2^32 + lo, read once all adds are done, is the exact
// sum modulo 2^64.
template <bool SHARED> struct GridAcc;

template <> struct GridAcc<false> {
  unsigned long long* p;
  __device__ __forceinline__ void add(int i, unsigned long long v) const { atomicAdd(p + i, v); }
  // every particle is deposited by the block that reads it
  __device__ __forceinline__ bool owns(int) const { return true; }
  __device__ __forceinline__ bool owns_outside() const { return true; }
};

template <> struct GridAcc<true> {
  unsigned* lo;  // low words; the high words are at lo + hi_off
  int hi_off;
  __device__ __forceinline__ void add(int i, unsigned long long v) const {
    unsigned l = (unsigned)v, h = (unsigned)(v >> 32);
    unsigned old = atomicAdd(lo + i, l);
    h += (old + l < old) ? 1u : 0u;
    if (h) atomicAdd(lo + hi_off + i, h);
  }
  __device__ __forceinline__ unsigned long long get(int i) const {
    return ((unsigned long long)lo[hi_off + i] << 32) | lo[i];
  }
  __device__ __forceinline__ bool owns(int) const { return true; }
  __device__ __forceinline__ bool owns_outside() const { return true; }
};

// Rows r0..r1-1 of a grid too large for one block's shared memory, plus
// one halo row on each side (the 9-point stencil of a particle whose
// centre row is owned).  A particle is deposited by the block that owns its
// centre row, whole (its line-density contribution included); particles
// outside the transverse grid belong to the first band.  Cell i of the
// grid is local cell i - base, base = first local row * ny.
struct BandAcc {
  unsigned* lo;  // low words; the high words at lo + hi_off
  int hi_off;
  int base;
  int r0, r1;
  bool first;
  __device__ __forceinline__ void add(int i, unsigned long long v) const {
    i -= base;
    unsigned l = (unsigned)v, h = (unsigned)(v >> 32);
    unsigned old = atomicAdd(lo + i, l);
    h += (old + l < old) ? 1u : 0u;
    if (h) atomicAdd(lo + hi_off + i, h);
  }
  __device__ __forceinline__ unsigned long long get(int i) const {
    return ((unsigned long long)lo[hi_off + i] << 32) | lo[i];
  }
  __device__ __forceinline__ bool owns(int ix) const { return ix >= r0 && ix < r1; }
  __device__ __forceinline__ bool owns_outside() const { return first; }
};

// Plain form: contributions are rounded to a fixed-point grid of step 1/S
// (S a power of two with S * total macrosize <= 2^62) and summed as 64-bit
// integers, so the deposit is exact and independent of summation order.
template <class RA, class ZA>
__device__ __forceinline__ void deposit_plain(const DepConst& d, const RA& rho, const ZA& zg, double x, double y,
                                              double z, double ms) {
  const bool in2 = !(x < d.xmin || x > d.xmax || y < d.ymin || y > d.ymax);
  int ix = 0, iy;
  double fx, fy;
  if (in2) tsc_index<double>((x - d.xmin) * d.inv_dx, d.nx, ix, fx);
  if (in2 ? !rho.owns(ix) : !rho.owns_outside()) return;  // another block's particle
  if (in2) {
    tsc_index<double>((y - d.ymin) * d.inv_dy, d.ny, iy, fy);
    double wxm, wx0, wxp, wym, wy0, wyp;
    tsc_weights<double>(fx, wxm, wx0, wxp);
    tsc_weights<double>(fy, wym, wy0, wyp);
    double ax[3] = {wxm * ms, wx0 * ms, wxp * ms};
    double wy[3] = {wym, wy0, wyp};
    const int base = (ix - 1) * d.ny + (iy - 1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) rho.add(base + i * d.ny + j, (unsigned long long)__double2ll_rn(ax[i] * wy[j]));
  }
  if (!(z < d.zmin || z > d.zmax)) {
    int i0, ip;
    double w0, wp;
    g1_index<double>(z, d.zmin, d.inv_dz, d.nz, i0, ip, w0, wp);
    if (d.nz > 1) {
      zg.add(i0, (unsigned long long)__double2ll_rn(w0 * ms));
      zg.add(ip, (unsigned long long)__double2ll_rn(wp * ms));
    } else {
      zg.add(0, (unsigned long long)__double2ll_rn(ms));
    }
  }
}

// ---------------------------------------------------------------------
// Exact fixed-point arithmetic on the integer pipe (plain form).
//
// After one FP64 fused multiply-add per coordinate, v = t + 0.5 with
// t = (x - xmin)/dx in cell units, the index, the fraction and the 9-point
// weights are computed as 64-bit fixed-point integers: the fraction
// f = t - ind exactly as rounded into v (Q56), the weights W = (f -+ 0.5)^2/2
// and 0.75 - f^2 in Q58 (absolute error below 2^-58), the derivative
// weights exactly.  GB300 issues two FP64 FMAs per SM per cycle but dozens
// of integer operations, so this keeps the FP64 pipe for the coordinates.
// ---------------------------------------------------------------------

// v * 2^F truncated toward zero; false when |v| * 2^F could reach 2^63 or v
// is not finite.
__device__ __forceinline__ bool fix_of(double v, int F, long long& out) {
  long long u = __double_as_longlong(v);
  int e = (int)((u >> 52) & 0x7ff);
  long long m = (u & 0x000FFFFFFFFFFFFFll) | 0x0010000000000000ll;
  int sh = e - 1075 + F;
  long long r;
  if (e == 0) {
    r = 0;
  } else if (sh >= 0) {
    if (sh > 10) return false;
    r = m << sh;
  } else {
    r = (sh > -63) ? (m >> (-sh)) : 0;
  }
  out = (u < 0) ? -r : r;
  return true;
}

// Fraction bits F for values below n + 1 (n >= 2): v * 2^F < 2^63.
__host__ __device__ __forceinline__ int fix_bits(int n) {
  int b = 0;
  while ((1 << b) < n + 2) ++b;
  int F = 63 - b;
  return F > 60 ? 60 : F;
}

// g in Q56 with |g| <= 2^57: g^2 in Q58.
__device__ __forceinline__ long long sq_q58(long long g) {
  unsigned long long a = (unsigned long long)(g < 0 ? -g : g) << 5;
  return (long long)__umul64hi(a, a);
}

// Grid2D::getIndAndFracX/Y on v = t + 0.5: ind = floor(v) clamped to
// [1, n-2], f = t - ind in Q56.  False outside 0 <= floor(v) <= n-1.
__device__ __forceinline__ bool tsc_fixed(double v, int n, int F, int& ind, long long& f56) {
  long long V;
  // |f| <= 1.25 keeps every product below 2^63; particles inside the grid
  // limits have 0.5 <= v <= n - 0.5
  if (!fix_of(v, F, V) || V < (1ll << (F - 2)) || V > ((long long)n << F) - (1ll << (F - 2))) return false;
  long long i = V >> F;
  long long fr = V - (i << F) - (1ll << (F - 1));
  long long f = (F <= 56) ? (fr << (56 - F)) : (fr >> (F - 56));
  if (i < 1) { f -= (1ll << 56); i = 1; }
  if (i > n - 2) { f += (1ll << 56); i = n - 2; }
  ind = (int)i;
  f56 = f;
  return true;
}

// 9-point weights Wm, W0, Wp (Q58) and derivative weights (Q58).
__device__ __forceinline__ void tsc_w_fixed(long long f, long long w[3]) {
  w[0] = sq_q58(f - (1ll << 55)) >> 1;
  w[1] = (3ll << 56) - sq_q58(f);
  w[2] = sq_q58(f + (1ll << 55)) >> 1;
}
__device__ __forceinline__ void tsc_dw_fixed(long long f, long long dw[3]) {
  dw[0] = (f - (1ll << 55)) << 2;  // f - 1/2
  dw[1] = -(f << 3);               // -2 f
  dw[2] = (f + (1ll << 55)) << 2;  // f + 1/2
}

// Grid1D index on u = (z - zmin)/dz + 0.5 (nz > 1): floor semantics with
// periodic neighbours reproduce every wrap rule of Grid1D::getIndAndWZ;
// wp (weight of ip) in Q56.
__device__ __forceinline__ bool g1_fixed(double u, int nz, int F, int& i0, int& ip, long long& wp56) {
  long long V;
  if (!fix_of(u, F, V) || V < 0) return false;
  long long i = V >> F;
  if (i > nz) return false;
  long long fr = V - (i << F);
  wp56 = (F <= 56) ? (fr << (56 - F)) : (fr >> (F - 56));
  int a = (int)i - 1;
  i0 = a < 0 ? nz - 1 : a;
  ip = (int)i >= nz ? 0 : (int)i;
  return true;
}

struct DepFix {
  unsigned long long kxmin, kxmax, kymin, kymax, kzmin, kzmax;  // ordered keys of the limits
  double ax, cx, ay, cy, az, cz;   // v = x * ax + cx etc.
  int nx, ny, nz, Fx, Fy, Fz, K;
  int skip;
};

__device__ __forceinline__ void load_dep_fix(DepFix& d, const ScState* st, int nx, int ny, int nz, int K) {
  d.kxmin = dkey(st->xmin); d.kxmax = dkey(st->xmax);
  d.kymin = dkey(st->ymin); d.kymax = dkey(st->ymax);
  d.kzmin = dkey(st->zmin); d.kzmax = dkey(st->zmax);
  d.ax = st->inv_dx; d.cx = 0.5 - st->xmin * st->inv_dx;
  d.ay = st->inv_dy; d.cy = 0.5 - st->ymin * st->inv_dy;
  d.az = st->inv_dz; d.cz = 0.5 - st->zmin * st->inv_dz;
  d.nx = nx; d.ny = ny; d.nz = nz;
  d.Fx = fix_bits(nx); d.Fy = fix_bits(ny); d.Fz = fix_bits(nz);
  d.K = K;
  d.skip = st->skip;
}

// Integer deposit of one particle with unit weight scaled by 2^K (the
// macrosize multiplies the grid afterwards).  Returns false when the
// particle needs the FP64 path (never for finite coordinates in range).
// SHARED: the grids are block-private shared memory.
template <class RA, class ZA>
__device__ __forceinline__ bool deposit_fixed(const DepFix& d, const RA& rho, const ZA& zg, double x, double y,
                                              double z) {
  unsigned long long kx = dkey(x), ky = dkey(y), kz = dkey(z);
  bool in2 = kx >= d.kxmin && kx <= d.kxmax && ky >= d.kymin && ky <= d.kymax;
  bool in1 = kz >= d.kzmin && kz <= d.kzmax;
  int ix = 0, iy = 0, i0 = 0, ip = 0;
  long long fx = 0, fy = 0, wp = 0;
  if (in2) {
    if (!tsc_fixed(fma(x, d.ax, d.cx), d.nx, d.Fx, ix, fx)) return false;
    if (!tsc_fixed(fma(y, d.ay, d.cy), d.ny, d.Fy, iy, fy)) return false;
  }
  if (in1 && d.nz > 1) {
    if (!g1_fixed(fma(z, d.az, d.cz), d.nz, d.Fz, i0, ip, wp)) return false;
  }
  if (in2 ? !rho.owns(ix) : !rho.owns_outside()) return true;  // another block's particle
  if (in2) {
    long long wx[3], wy[3];
    tsc_w_fixed(fx, wx);
    tsc_w_fixed(fy, wy);
    const int sh = 60 - d.K;
    const long long half = 1ll << (sh - 1);
    const int base = (ix - 1) * d.ny + (iy - 1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      long long a = wx[i] << 4;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        long long p = __mul64hi(a, wy[j] << 4);  // Wx Wy in Q60
        rho.add(base + i * d.ny + j, (unsigned long long)((p + half) >> sh));
      }
    }
  }
  if (in1) {
    const int sh = 56 - d.K;
    const long long half = 1ll << (sh - 1);
    if (d.nz > 1) {
      zg.add(i0, (unsigned long long)((((1ll << 56) - wp) + half) >> sh));
      zg.add(ip, (unsigned long long)((wp + half) >> sh));
    } else {
      zg.add(0, (unsigned long long)(1ll << d.K));
    }
  }
  return true;
}

// Fixed-point kick: phi and lambda as 64-bit integers with per-kick scales
// (phi * 2^sphi, lambda * 2^slam, both below 2^61).
struct KickFix {
  double ax, cx, ay, cy, az, cz;
  unsigned long long kzmin, kzmax;
  double gxs, gys;   // inv_dx * 2^-(sphi-5), inv_dy * 2^-(sphi-5)
  double lfs;        // -factor * 2^-(slam-2)
  int nx, ny, nz, Fx, Fy, Fz;
  int sphi, slam;
  int skip;
};

__device__ __forceinline__ int scale_bits(unsigned long long absmax_bits) {
  int e = (int)((absmax_bits >> 52) & 0x7ff);
  return absmax_bits == 0 ? 0 : 1083 - e;  // max * 2^s < 2^61
}

// fac: the kick factor of load_kick_const (the same division).
__device__ __forceinline__ void load_kick_fix(KickFix& k, const ScState* st, double fac, int nx, int ny, int nz) {
  k.ax = st->inv_dx; k.cx = 0.5 - st->xmin * st->inv_dx;
  k.ay = st->inv_dy; k.cy = 0.5 - st->ymin * st->inv_dy;
  k.az = st->inv_dz; k.cz = 0.5 - st->zmin * st->inv_dz;
  k.kzmin = dkey(st->zmin); k.kzmax = dkey(st->zmax);
  k.sphi = scale_bits(st->phi_absmax);
  k.slam = scale_bits(st->lam_absmax);
  k.gxs = ldexp(st->inv_dx, 5 - k.sphi);
  k.gys = ldexp(st->inv_dy, 5 - k.sphi);
  k.lfs = ldexp(-fac, 2 - k.slam);
  k.nx = nx; k.ny = ny; k.nz = nz;
  k.Fx = fix_bits(nx); k.Fy = fix_bits(ny); k.Fz = fix_bits(nz);
  k.skip = st->skip;
}

// The kick constants computed once per block (thread 0) and copied to every
// thread: a thread of a 512-thread block handles only ~13 particles of a
// 1e6-particle bunch, and the set-up holds two FP64 divisions, which on
// GB300 occupy the FP64 pipe that bounds the fused pass.  (Reading the
// constants from shared memory inside the particle loop instead spills
// registers there and is slower.)  Every thread of the block must call it.
__device__ __forceinline__ void load_kick_block(KickConst& k, KickFix* kf, const ScState* st, double host_factor,
                                                int nx, int ny, int nz) {
  __shared__ KickConst s_k;
  __shared__ KickFix s_kf;
  if (threadIdx.x == 0) {
    load_kick_const(s_k, st, host_factor, nx, ny, nz);
    if (kf) load_kick_fix(s_kf, st, s_k.fac, nx, ny, nz);
  }
  __syncthreads();
  k = s_k;
  if (kf) *kf = s_kf;
}

__device__ __forceinline__ long long phi_fixed(double v, int s) {
  long long r;
  return fix_of(v, s, r) ? r : 0;
}

// Returns false when the particle needs the FP64 path.
__device__ __forceinline__ bool kick_fixed(const KickFix& k, const long long* __restrict__ P,
                                           const long long* __restrict__ Lm, double x, double y, double z,
                                           double& xp, double& yp) {
  int ix, iy;
  long long fx, fy;
  if (!tsc_fixed(fma(x, k.ax, k.cx), k.nx, k.Fx, ix, fx)) return false;
  if (!tsc_fixed(fma(y, k.ay, k.cy), k.ny, k.Fy, iy, fy)) return false;
  long long lv = 0;
  unsigned long long kz = dkey(z);
  if (kz >= k.kzmin && kz <= k.kzmax) {
    if (k.nz > 1) {
      int i0, ip;
      long long wp;
      if (!g1_fixed(fma(z, k.az, k.cz), k.nz, k.Fz, i0, ip, wp)) return false;
      lv = __mul64hi(((1ll << 56) - wp) << 6, Lm[i0]) + __mul64hi(wp << 6, Lm[ip]);  // Q(slam-2)
    } else {
      lv = Lm[0] >> 2;
    }
  }
  long long wx[3], wy[3], dwx[3], dwy[3];
  tsc_w_fixed(fx, wx);
  tsc_w_fixed(fy, wy);
  tsc_dw_fixed(fx, dwx);
  tsc_dw_fixed(fy, dwy);
  long long gx = 0, gy = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const long long* r = P + (ix - 1 + i) * k.ny + (iy - 1);
    long long a0 = r[0], a1 = r[1], a2 = r[2];
    long long s = __mul64hi(wy[0] << 4, a0) + __mul64hi(wy[1] << 4, a1) + __mul64hi(wy[2] << 4, a2);     // Q(sphi-2)
    long long t = __mul64hi(dwy[0] << 3, a0) + __mul64hi(dwy[1] << 3, a1) + __mul64hi(dwy[2] << 3, a2);  // Q(sphi-3)
    gx += __mul64hi(dwx[i] << 3, s);  // Q(sphi-5)
    gy += __mul64hi(wx[i] << 4, t);   // Q(sphi-5)
  }
  const double lf = dmul<(ORBIT_SOFT_MUL >> 4) & 1>((double)lv, k.lfs);  // -lambda(z) * factor
  xp = fma((double)gx, dmul<(ORBIT_SOFT_MUL >> 4) & 1>(k.gxs, lf), xp);
  yp = fma((double)gy, dmul<(ORBIT_SOFT_MUL >> 4) & 1>(k.gys, lf), yp);
  return true;
}

}  // namespace orbit
