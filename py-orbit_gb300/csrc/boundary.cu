// Conducting boundaries for the 2.5D solver (BaseBoundary2D,
// ShapedBoundary2D; src/spacecharge/BaseBoundary2D.cc, ShapedBoundary2D.cc).
//
// Set-up runs once on the host: boundary points, extents, the normalising
// radius and the least-squares matrix L = (F^T F)^-1 F^T of the free-space
// modes F.  Per kick the device fits the modes to phi on the boundary
// points (coef = L phi_b) and subtracts the fitted field from every grid
// node; the kick skips particles outside the boundary.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "sc2p5d.cuh"
#include "sc_device.cuh"

struct orbit_boundary {
  int np = 0, nm = 0, shape = -1;  // shape: -1 points given by the caller, 1 circle, 2 ellipse, 3 rectangle
  double r_circle = 0, a_ell = 0, b_ell = 0, a_rect = 0, b_rect = 0;
  double xmin = DBL_MAX, xmax = -DBL_MAX, ymin = DBL_MAX, ymax = -DBL_MAX, rnorm = DBL_MAX;
  bool initialized = false;
  std::vector<double> bx, by, lsq;  // lsq: (2 nm + 1) x np, row-major
  double* d_bx = nullptr;           // device copies, written by initialize
  double* d_by = nullptr;
  double* d_lsq = nullptr;
  double* d_coef = nullptr;         // 2 nm + 1 fitted coefficients of the last kick
};

namespace orbit {

static const double kPi = 3.14159265358979323846;  // OrbitConst::PI

// The 2 nm + 1 free-space modes 1, (r/R)^j cos(j f), (r/R)^j sin(j f) at one
// point (BaseBoundary2D::lsq_fuctions, BaseBoundary2D.cc:321-348).
__host__ __device__ inline void bnd_modes(int nm, double rnorm, double x, double y, double* f) {
  double r2 = x * x + y * y;
  if (r2 == 0.) {
    f[0] = 1.0;
    for (int i = 1; i < 2 * nm + 1; ++i) f[i] = 0.0;
    return;
  }
  double r = sqrt(r2);
  double s = y / r, c = x / r, s0 = s, c0 = c;
  double rfac = r / rnorm, rj = 1.0;
  f[0] = 1.;
  for (int i = 0; i < nm; ++i) {
    rj *= rfac;
    f[2 * i + 1] = rj * c0;
    f[2 * i + 2] = rj * s0;
    double s1 = s * c0 + c * s0;
    double c1 = c * c0 - s * s0;
    s0 = s1;
    c0 = c1;
  }
}

// In-place inverse by Gauss-Jordan elimination with full pivoting, the
// method BaseBoundary2D::_gaussjinv uses (BaseBoundary2D.cc:238-317).
static bool gauss_jordan_inverse(std::vector<double>& a, int n) {
  std::vector<int> col_of(n), row_of(n), used(n, 0);
  auto A = [&](int r, int c) -> double& { return a[(size_t)r * n + c]; };
  for (int step = 0; step < n; ++step) {
    double big = 0.0;
    int prow = 0, pcol = 0;
    for (int j = 0; j < n; ++j) {
      if (used[j] == 1) continue;
      for (int k = 0; k < n; ++k) {
        if (used[k] == 0) {
          if (std::fabs(A(j, k)) >= big) {
            big = std::fabs(A(j, k));
            prow = j;
            pcol = k;
          }
        } else if (used[k] > 1) {
          return false;
        }
      }
    }
    ++used[pcol];
    if (prow != pcol)
      for (int l = 0; l < n; ++l) std::swap(A(prow, l), A(pcol, l));
    row_of[step] = prow;
    col_of[step] = pcol;
    if (A(pcol, pcol) == 0.0) return false;
    double inv = 1.0 / A(pcol, pcol);
    A(pcol, pcol) = 1.0;
    for (int l = 0; l < n; ++l) A(pcol, l) *= inv;
    for (int r = 0; r < n; ++r) {
      if (r == pcol) continue;
      double m = A(r, pcol);
      A(r, pcol) = 0.0;
      for (int l = 0; l < n; ++l) A(r, l) -= A(pcol, l) * m;
    }
  }
  for (int l = n - 1; l >= 0; --l)
    if (row_of[l] != col_of[l])
      for (int k = 0; k < n; ++k) std::swap(A(k, row_of[l]), A(k, col_of[l]));
  return true;
}

// Grid2D::getValue (Grid2D.cc:82-108): the 9-point quadratic interpolation.
__device__ double grid_value(const double* __restrict__ arr, int nx, int ny, double xmin, double ymin, double dx,
                             double dy, double x, double y) {
  int ix, iy;
  double fx, fy;
  tsc_index<double>((x - xmin) / dx, nx, ix, fx);
  tsc_index<double>((y - ymin) / dy, ny, iy, fy);
  double wx[3], wy[3];
  tsc_weights<double>(fx, wx[0], wx[1], wx[2]);
  tsc_weights<double>(fy, wy[0], wy[1], wy[2]);
  double v = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v += wx[i] * wy[j] * arr[(size_t)(ix - 1 + i) * ny + (iy - 1 + j)];
  return v;
}

// Fit of the free-space modes to phi on the boundary points (one block):
// coef = L phi_b (BaseBoundary2D.cc:431-441); max |phi| is reset for the
// corrected grid.
__global__ void k_bnd_fit(ScState* st, const double* __restrict__ phi, const double* __restrict__ bx,
                          const double* __restrict__ by, const double* __restrict__ lsq, double* coef, int np,
                          int nf, int nx, int ny) {
  if (st->skip) return;
  extern __shared__ double s_bphi[];
  const double xmin = st->xmin, ymin = st->ymin, dx = st->dx, dy = st->dy;
  for (int j = threadIdx.x; j < np; j += blockDim.x)
    s_bphi[j] = grid_value(phi, nx, ny, xmin, ymin, dx, dy, bx[j], by[j]);
  __syncthreads();
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    double c = 0.0;
    for (int j = 0; j < np; ++j) c += lsq[(size_t)i * np + j] * s_bphi[j];
    coef[i] = c;
  }
  if (threadIdx.x == 0) st->phi_absmax = 0ull;
}

// sum_k coef_k F_k(x, y), the modes generated in order as bnd_modes does
// and summed in that order.
__device__ __forceinline__ double bnd_field(const double* coef, int nm, double rnorm, double x, double y) {
  double r2 = x * x + y * y;
  double p = 0.;
  if (r2 == 0.) return p + coef[0] * 1.0;
  double r = sqrt(r2);
  double s = y / r, c = x / r, s0 = s, c0 = c;
  double rfac = r / rnorm, rj = 1.0;
  p += coef[0] * 1.;
  for (int i = 0; i < nm; ++i) {
    rj *= rfac;
    p += coef[2 * i + 1] * (rj * c0);
    p += coef[2 * i + 2] * (rj * s0);
    double s1 = s * c0 + c * s0;
    double c1 = c * c0 - s * s0;
    s0 = s1;
    c0 = c1;
  }
  return p;
}

// phi -= sum_k coef_k F_k at every grid node (BaseBoundary2D.cc:443-459),
// then max |phi| of the corrected grid.
__global__ void k_bnd_apply(ScState* st, double* __restrict__ phi, float* __restrict__ phi_f,
                            const double* __restrict__ coef, int nm, double rnorm, int nx, int ny) {
  if (st->skip) return;
  __shared__ double s_coef[128];
  const int nf = 2 * nm + 1;
  for (int k = threadIdx.x; k < nf; k += blockDim.x) s_coef[k] = coef[k];
  __syncthreads();
  const double xmin = st->xmin, ymin = st->ymin, dx = st->dx, dy = st->dy;
  unsigned long long amax = 0ull;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nx * ny; idx += gridDim.x * blockDim.x) {
    int i = idx / ny, j = idx - i * ny;
    double p = bnd_field(s_coef, nm, rnorm, xmin + i * dx, ymin + j * dy);
    double v = phi[idx] - p;
    phi[idx] = v;
    if (phi_f) phi_f[idx] = (float)v;
    unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v));
    amax = b > amax ? b : amax;
  }
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, amax, off);
    amax = o > amax ? o : amax;
  }
  if ((threadIdx.x & 31) == 0 && amax) atomicMax(&st->phi_absmax, amax);
}

BndShape bnd_shape_of(const orbit_boundary* b) {
  BndShape s;
  s.type = -1;
  s.p0 = s.p1 = s.p2 = s.p3 = 0.0;
  if (!b) return s;
  if (b->shape == 1) { s.type = 1; s.p0 = b->r_circle; }
  else if (b->shape == 2) { s.type = 2; s.p0 = b->a_ell; s.p1 = b->b_ell; }
  else if (b->shape == 3) { s.type = 3; s.p0 = b->a_rect; s.p1 = b->b_rect; }
  else { s.type = 0; s.p0 = b->xmin; s.p1 = b->xmax; s.p2 = b->ymin; s.p3 = b->ymax; }
  return s;
}

int bnd_enqueue_potential(const orbit_boundary* b, orbit_sc2p5d_t* c, cudaStream_t s, int* launches) {
  const int nf = 2 * b->nm + 1;
  size_t sm = sizeof(double) * (size_t)b->np;
  ORBIT_PB("boundary", s);
  k_bnd_fit<<<1, 256, sm, s>>>(c->d_st, c->d_phi, b->d_bx, b->d_by, b->d_lsq, b->d_coef, b->np, nf, c->nx, c->ny);
  int ng = c->nx * c->ny;
  int blocks = (ng + 255) / 256;
  k_bnd_apply<<<blocks, 256, 0, s>>>(c->d_st, c->d_phi, c->d_phi_f, b->d_coef, b->nm, b->rnorm, c->nx, c->ny);
  ORBIT_PE(s);
  if (launches) *launches += 2;
  ORBIT_LAUNCH_CHECK("boundary potential");
  return ORBIT_OK;
}

}  // namespace orbit

using namespace orbit;

// The kernels hold the modes in per-thread arrays of 128 and the boundary
// values in shared memory.
static const int kMaxModes = 63;
static const int kMaxPoints = 4096;

static void free_device(orbit_boundary_t* b) {
  void* ptrs[] = {b->d_bx, b->d_by, b->d_lsq, b->d_coef};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  b->d_bx = b->d_by = b->d_lsq = b->d_coef = nullptr;
}

namespace orbit {

// Device copies of the points and the least-squares matrix, made on first
// use (the set-up itself needs no GPU).
int bnd_ensure_device(orbit_boundary_t* b) {
  if (b->d_bx) return ORBIT_OK;
  const int np = b->np, nf = 2 * b->nm + 1;
  cudaError_t e = cudaMalloc(&b->d_bx, sizeof(double) * np);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_by, sizeof(double) * np);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_lsq, sizeof(double) * b->lsq.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_coef, sizeof(double) * nf);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_bx, b->bx.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_by, b->by.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_lsq, b->lsq.data(), sizeof(double) * b->lsq.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_device(b);
    return cuda_error(e, "boundary upload");
  }
  return ORBIT_OK;
}

}  // namespace orbit

extern "C" {

int orbit_boundary_create(orbit_boundary_t** out, int n_points, int n_modes) {
  if (!out) return set_error(ORBIT_ERR_ARG, "orbit_boundary_create: null output");
  if (n_modes < 0 || 2 * n_modes + 1 >= n_points)  // BaseBoundary2D.cc:55-68
    return set_error(ORBIT_ERR_ARG, "Boundary2D: 2*nModes+1 must be below the number of points");
  if (n_modes > kMaxModes || n_points > kMaxPoints)
    return set_error(ORBIT_ERR_UNSUPPORTED, "Boundary2D: at most 63 modes and 4096 points");
  orbit_boundary_t* b = new orbit_boundary_t();
  b->np = n_points;
  b->nm = n_modes;
  b->bx.assign(n_points, DBL_MAX);
  b->by.assign(n_points, DBL_MAX);
  b->lsq.assign((size_t)(2 * n_modes + 1) * n_points, 0.0);
  *out = b;
  return ORBIT_OK;
}

int orbit_boundary_set_point(orbit_boundary_t* b, int i, double x, double y) {
  if (!b) return set_error(ORBIT_ERR_ARG, "orbit_boundary_set_point: null handle");
  if (b->shape > 0)
    return set_error(ORBIT_ERR_ARG, "Boundary2D.setBoundaryPoint: the shape has been defined already");
  if (i >= 0 && i < b->np) {
    b->bx[i] = x;
    b->by[i] = y;
  }
  b->initialized = false;
  return ORBIT_OK;
}

// BaseBoundary2D::initializeBPs (BaseBoundary2D.cc:190-229)
int orbit_boundary_initialize(orbit_boundary_t* b) {
  if (!b) return set_error(ORBIT_ERR_ARG, "orbit_boundary_initialize: null handle");
  const int np = b->np, nf = 2 * b->nm + 1;
  b->xmin = DBL_MAX; b->xmax = -DBL_MAX; b->ymin = DBL_MAX; b->ymax = -DBL_MAX;
  for (int i = 0; i < np; ++i) {
    if (b->xmin > b->bx[i]) b->xmin = b->bx[i];
    if (b->xmax < b->bx[i]) b->xmax = b->bx[i];
    if (b->ymin > b->by[i]) b->ymin = b->by[i];
    if (b->ymax < b->by[i]) b->ymax = b->by[i];
  }
  double ex = b->xmin - b->xmax, ey = b->ymin - b->ymax;
  b->rnorm = std::sqrt(ex * ex + ey * ey);
  std::vector<double> ftf((size_t)nf * nf, 0.0), f(nf);
  for (int p = 0; p < np; ++p) {
    bnd_modes(b->nm, b->rnorm, b->bx[p], b->by[p], f.data());
    for (int i = 0; i < nf; ++i)
      for (int j = 0; j < nf; ++j) ftf[(size_t)i * nf + j] += f[i] * f[j];
  }
  if (!gauss_jordan_inverse(ftf, nf)) return set_error(ORBIT_ERR_ARG, "Boundary2D: matrix A^(-1) does not exist");
  for (int i = 0; i < nf; ++i)
    for (int j = 0; j < np; ++j) {
      bnd_modes(b->nm, b->rnorm, b->bx[j], b->by[j], f.data());
      double v = 0.0;
      for (int k = 0; k < nf; ++k) v += ftf[(size_t)i * nf + k] * f[k];
      b->lsq[(size_t)i * np + j] = v;
    }
  free_device(b);  // uploaded again before the next kick that uses it
  b->initialized = true;
  return ORBIT_OK;
}

// ShapedBoundary2D::ShapedBoundary2D (ShapedBoundary2D.cc:18-145)
int orbit_boundary_create_shape(orbit_boundary_t** out, int n_points, int n_modes, int shape, double xdim,
                                double ydim) {
  if (!out) return set_error(ORBIT_ERR_ARG, "orbit_boundary_create_shape: null output");
  if (shape < 1 || shape > 3)
    return set_error(ORBIT_ERR_ARG, "Boundary2D: the shape should be Circle, Ellipse or Rectangle");
  if (shape == 1 && xdim != ydim)
    return set_error(ORBIT_ERR_ARG, "Boundary2D: the Circle should have the same x and y sizes");
  const int np = 4 * (n_points / 4);
  int rc = orbit_boundary_create(out, np, n_modes);
  if (rc) return rc;
  orbit_boundary_t* b = *out;
  if (shape == 1) {
    b->r_circle = xdim / 2;
    for (int i = 0; i < np; ++i) {
      b->bx[i] = b->r_circle * std::sin(2 * i * kPi / np);
      b->by[i] = b->r_circle * std::cos(2 * i * kPi / np);
    }
  } else if (shape == 2) {
    // points at equal arc length, found by iterating on the quarter ellipse
    const double a = xdim / 2, bb = ydim / 2;
    b->a_ell = a;
    b->b_ell = bb;
    double ds = 2 * kPi * std::sqrt(a * bb) / np, resid = 1.0;
    std::vector<double> th(np + 1, 0.0);
    while (resid > 1.0e-08 || resid < -1.0e-08) {
      double denom = bb;
      double dtheta = ds / denom;
      double t = dtheta / 2.;
      th[0] = 0.;
      for (int i = 0; i < np / 4; ++i) {
        denom = bb * bb + (a * a - bb * bb) * std::sin(t) * std::sin(t);
        denom = std::sqrt(denom);
        dtheta = ds / denom;
        th[i + 1] = th[i] + dtheta;
        t += dtheta;
      }
      resid = th[np / 4] - kPi / 2.;
      ds *= kPi / (2. * th[np / 4]);
    }
    for (int i = 0; i < np / 4; ++i) th[np / 2 - i] = kPi - th[i];
    for (int i = 0; i < np / 2; ++i) th[np / 2 + i] = kPi + th[i];
    for (int i = 0; i < np; ++i) {
      b->bx[i] = a * std::cos(th[i]);
      b->by[i] = bb * std::sin(th[i]);
    }
  } else {
    const double a = xdim, bb = ydim;
    b->a_rect = a;
    b->b_rect = bb;
    const double dx = a / (np / 4), dy = bb / (np / 4);
    int c = 0;
    for (int i = 0; i < np / 4; ++i, ++c) { b->bx[c] = (-a / 2.0) + i * dx; b->by[c] = bb / 2.0; }
    for (int i = 0; i < np / 4; ++i, ++c) { b->bx[c] = a / 2.0; b->by[c] = bb / 2.0 - i * dy; }
    for (int i = 0; i < np / 4; ++i, ++c) { b->bx[c] = a / 2.0 - i * dx; b->by[c] = -bb / 2.0; }
    for (int i = 0; i < np / 4; ++i, ++c) { b->bx[c] = -a / 2.0; b->by[c] = (-bb / 2.0) + i * dy; }
  }
  b->shape = shape;
  rc = orbit_boundary_initialize(b);
  if (rc) {
    delete b;
    *out = nullptr;
  }
  return rc;
}

int orbit_boundary_destroy(orbit_boundary_t* b) {
  if (!b) return ORBIT_OK;
  free_device(b);
  delete b;
  return ORBIT_OK;
}

int orbit_boundary_info(const orbit_boundary_t* b, int* n_points, int* n_modes, int* shape, double* lim,
                        int* initialized) {
  if (!b) return set_error(ORBIT_ERR_ARG, "orbit_boundary_info: null handle");
  if (n_points) *n_points = b->np;
  if (n_modes) *n_modes = b->nm;
  if (shape) *shape = b->shape < 0 ? 0 : b->shape;
  if (lim) { lim[0] = b->xmin; lim[1] = b->xmax; lim[2] = b->ymin; lim[3] = b->ymax; }
  if (initialized) *initialized = b->initialized ? 1 : 0;
  return ORBIT_OK;
}

int orbit_boundary_get_point(const orbit_boundary_t* b, int i, double* x, double* y) {
  if (!b || !x || !y) return set_error(ORBIT_ERR_ARG, "orbit_boundary_get_point: bad argument");
  bool ok = i >= 0 && i < b->np;
  *x = ok ? b->bx[i] : DBL_MAX;  // BaseBoundary2D.cc:154-164
  *y = ok ? b->by[i] : DBL_MAX;
  return ORBIT_OK;
}

int orbit_boundary_is_inside(const orbit_boundary_t* b, double x, double y) {
  if (!b) return 0;
  return bnd_inside(bnd_shape_of(b), x, y) ? 1 : -1;
}

int orbit_boundary_lsq(const orbit_boundary_t* b, double* out) {
  if (!b || !out) return set_error(ORBIT_ERR_ARG, "orbit_boundary_lsq: bad argument");
  if (!b->initialized) return set_error(ORBIT_ERR_ARG, "Boundary2D: the boundary was not initialized");
  std::memcpy(out, b->lsq.data(), sizeof(double) * b->lsq.size());
  return ORBIT_OK;
}

int orbit_boundary_rnorm(const orbit_boundary_t* b, double* rnorm) {
  if (!b || !rnorm) return set_error(ORBIT_ERR_ARG, "orbit_boundary_rnorm: bad argument");
  *rnorm = b->rnorm;
  return ORBIT_OK;
}

}  // extern "C"
