/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- see orbit_oracle.h.
 *
 * A plain-C restatement of the reference algorithms, written to follow the
 * reference's arithmetic order so that with one thread it reproduces the
 * compiled reference bit for bit (checked by tests/test_oracle_vs_reference.py
 * and the committed golden vectors).  Build with -ffp-contract=off so that no
 * compiler fuses multiply-adds (the reference's x86-64 build has no FMA).
 */
#include "orbit_oracle.h"
#include "fft.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Grids                                                              */
/* ------------------------------------------------------------------ */

/* Grid2D: node-centred, dx = (xMax-xMin)/(nx-1) (src/spacecharge/Grid2D.cc:53-54,422-433) */
typedef struct {
  int nx, ny;
  double xmin, xmax, ymin, ymax, dx, dy;
} grid2d_t;

static void g2_setx(grid2d_t* g, double a, double b) { g->xmin = a; g->xmax = b; g->dx = (b - a) / (g->nx - 1); }
static void g2_sety(grid2d_t* g, double a, double b) { g->ymin = a; g->ymax = b; g->dy = (b - a) / (g->ny - 1); }

/* Grid2D::getIndAndFracX/Y (Grid2D.cc:337-349) */
static void g2_indx(const grid2d_t* g, double x, int* ind, double* frac) {
  int i = (int)((x - g->xmin) / g->dx + 0.5);
  if (i < 1) i = 1;
  if (i > g->nx - 2) i = g->nx - 2;
  *ind = i;
  *frac = (x - (g->xmin + i * g->dx)) / g->dx;
}
static void g2_indy(const grid2d_t* g, double y, int* ind, double* frac) {
  int i = (int)((y - g->ymin) / g->dy + 0.5);
  if (i < 1) i = 1;
  if (i > g->ny - 2) i = g->ny - 2;
  *ind = i;
  *frac = (y - (g->ymin + i * g->dy)) / g->dy;
}

/* Grid2D::binValue, 9-point quadratic weights (Grid2D.cc:141-166) */
static void g2_bin(const grid2d_t* g, double* arr, double value, double x, double y) {
  if (x < g->xmin || x > g->xmax || y < g->ymin || y > g->ymax) return;
  int iX, iY;
  double xf, yf;
  g2_indx(g, x, &iX, &xf);
  g2_indy(g, y, &iY, &yf);
  double xf2 = xf * xf, yf2 = yf * yf;
  double Wxm = 0.5 * (0.25 - xf + xf2), Wx0 = 0.75 - xf2, Wxp = 0.5 * (0.25 + xf + xf2);
  double Wym = 0.5 * (0.25 - yf + yf2), Wy0 = 0.75 - yf2, Wyp = 0.5 * (0.25 + yf + yf2);
  int ny = g->ny;
  double* r0 = arr + (size_t)(iX - 1) * ny;
  double* r1 = arr + (size_t)iX * ny;
  double* r2 = arr + (size_t)(iX + 1) * ny;
  r0[iY - 1] += Wxm * Wym * value;
  r0[iY] += Wxm * Wy0 * value;
  r0[iY + 1] += Wxm * Wyp * value;
  r1[iY - 1] += Wx0 * Wym * value;
  r1[iY] += Wx0 * Wy0 * value;
  r1[iY + 1] += Wx0 * Wyp * value;
  r2[iY - 1] += Wxp * Wym * value;
  r2[iY] += Wxp * Wy0 * value;
  r2[iY + 1] += Wxp * Wyp * value;
}

/* Grid2D::calcGradient(x,y,ex,ey) (Grid2D.cc:212-256) */
static void g2_grad(const grid2d_t* g, const double* arr, double x, double y, double* ex, double* ey) {
  int iX, iY;
  double xf, yf;
  g2_indx(g, x, &iX, &xf);
  g2_indy(g, y, &iY, &yf);
  double xf2 = xf * xf, yf2 = yf * yf;
  double Wxm = 0.5 * (0.25 - xf + xf2), Wx0 = 0.75 - xf2, Wxp = 0.5 * (0.25 + xf + xf2);
  double Wym = 0.5 * (0.25 - yf + yf2), Wy0 = 0.75 - yf2, Wyp = 0.5 * (0.25 + yf + yf2);
  double dWxm = (-1.0) * (0.5 - xf), dWx0 = (-1.0) * (+2.) * xf, dWxp = (-1.0) * (-(0.5 + xf));
  double dWym = (-1.0) * (0.5 - yf), dWy0 = (-1.0) * (+2.) * yf, dWyp = (-1.0) * (-(0.5 + yf));
  int ny = g->ny;
  const double* a0 = arr + (size_t)(iX - 1) * ny;
  const double* a1 = arr + (size_t)iX * ny;
  const double* a2 = arr + (size_t)(iX + 1) * ny;
  double gx = dWxm * Wym * a0[iY - 1] + dWxm * Wy0 * a0[iY] + dWxm * Wyp * a0[iY + 1] +
              dWx0 * Wym * a1[iY - 1] + dWx0 * Wy0 * a1[iY] + dWx0 * Wyp * a1[iY + 1] +
              dWxp * Wym * a2[iY - 1] + dWxp * Wy0 * a2[iY] + dWxp * Wyp * a2[iY + 1];
  *ex = gx / g->dx;
  double gy = Wxm * dWym * a0[iY - 1] + Wxm * dWy0 * a0[iY] + Wxm * dWyp * a0[iY + 1] +
              Wx0 * dWym * a1[iY - 1] + Wx0 * dWy0 * a1[iY] + Wx0 * dWyp * a1[iY + 1] +
              Wxp * dWym * a2[iY - 1] + Wxp * dWy0 * a2[iY] + Wxp * dWyp * a2[iY + 1];
  *ey = gy / g->dy;
}

/* Grid1D: periodic, cell-centred, dz = (zMax-zMin)/nz (src/spacecharge/Grid1D.cc:83-94,131-135) */
typedef struct {
  int nz;
  double zmin, zmax, dz;
} grid1d_t;

static void g1_set(grid1d_t* g, double a, double b) { g->zmin = a; g->zmax = b; g->dz = (b - a) / g->nz; }
static double g1_gridz(const grid1d_t* g, int i) { return g->zmin + (i + 0.5) * g->dz; }

/* Grid1D::getIndAndWZ (Grid1D.cc:568-627) */
static void g1_ind(const grid1d_t* g, double z, int* i0, int* ip, double* w0, double* wp) {
  int nz = g->nz;
  if (nz > 1) {
    double ind_dbl = ((z - g->zmin) / g->dz) - 0.5;
    int iZ0 = (int)ind_dbl;
    double zFrac = (z - g1_gridz(g, iZ0)) / g->dz;
    if (iZ0 == 0 && zFrac < 0.) {
      *i0 = nz - 1; *ip = 0; *w0 = -zFrac; *wp = 1.0 + zFrac;
      return;
    }
    if (iZ0 == nz - 1) {
      if (zFrac > 0.) {
        *i0 = iZ0; *ip = 0; *w0 = 1.0 - zFrac; *wp = zFrac;
        return;
      }
      *ip = iZ0; *i0 = nz - 2; *w0 = -zFrac; *wp = 1.0 + zFrac;
      return;
    }
    *i0 = iZ0; *ip = iZ0 + 1; *w0 = 1.0 - zFrac; *wp = zFrac;
    return;
  }
  *i0 = 0; *ip = 0; *w0 = 1.0; *wp = 0.0;
}

/* Grid1D::binValue (Grid1D.cc:422-439) */
static void g1_bin(const grid1d_t* g, double* arr, double value, double z) {
  if (z < g->zmin || z > g->zmax) return;
  int i0, ip;
  double w0, wp;
  g1_ind(g, z, &i0, &ip, &w0, &wp);
  if (g->nz > 1) {
    arr[i0] += w0 * value;
    arr[ip] += wp * value;
  } else {
    arr[i0] += value;
  }
}

/* Grid1D::getValue (Grid1D.cc:191-209) */
static double g1_value(const grid1d_t* g, const double* arr, double z) {
  if (z < g->zmin || z > g->zmax) return 0.;
  int i0, ip;
  double w0, wp;
  g1_ind(g, z, &i0, &ip, &w0, &wp);
  if (g->nz > 1) return w0 * arr[i0] + wp * arr[ip];
  return arr[0];
}

/* ------------------------------------------------------------------ */
/* Poisson solver (src/spacecharge/PoissonSolverFFT2D.cc)             */
/* ------------------------------------------------------------------ */

struct oracle_sc {
  int nx, ny, nz;
  double xy_ratio;
  /* solver grid (PoissonSolver2D.cc:21-33) */
  double sxmin, sxmax, symin, symax, sdx, sdy;
  int nx2, ny2;        /* doubled grid */
  double* green_hat;   /* nx2 * (ny2/2+1) complex */
  double re00;
  double* work_in;     /* nx2 * ny2 */
  double* work_hat;    /* nx2 * (ny2/2+1) complex */
  grid2d_t grho;       /* rho and phi grids share limits */
  grid1d_t gz;
  double* rho;
  double* phi;
  double* zarr;
  double total_macrosize;
  /* SpaceChargeCalc2p5Drb only (SpaceChargeCalc2p5Drb.cc:31-60) */
  int rb;
  int n_long_avg;
  double* zderiv;
  double a_bunch, x_c, y_c;
};

/* _defineGreenF (PoissonSolverFFT2D.cc:115-172) */
static void define_green(oracle_sc_t* s) {
  int nx2 = s->nx2, ny2 = s->ny2;
  double* G = s->work_in;
  for (int iY = 0; iY <= ny2 / 2; iY++) {
    double rY = iY * s->sdy;
    for (int iX = 0; iX <= nx2 / 2; iX++) {
      double rX = iX * s->sdx;
      double r2 = rX * rX + rY * rY;
      G[(size_t)iX * ny2 + iY] = (iX != 0 || iY != 0) ? -log(r2) / 2 : 0.0;
    }
    for (int iX = nx2 / 2 + 1; iX < nx2; iX++) G[(size_t)iX * ny2 + iY] = G[(size_t)(nx2 - iX) * ny2 + iY];
  }
  for (int iY = ny2 / 2 + 1; iY < ny2; iY++)
    for (int iX = 0; iX < nx2; iX++) G[(size_t)iX * ny2 + iY] = G[(size_t)iX * ny2 + (ny2 - iY)];
  oracle_fft_r2c_2d(nx2, ny2, G, s->green_hat);
  s->re00 = s->green_hat[0];
  memset(s->work_in, 0, sizeof(double) * (size_t)nx2 * ny2);
}

/* setGridXY (PoissonSolverFFT2D.cc:103-111) */
static void solver_set_xy(oracle_sc_t* s, double xmin, double xmax, double ymin, double ymax) {
  s->sxmin = xmin; s->sxmax = xmax; s->sdx = (xmax - xmin) / (s->nx - 1);
  s->symin = ymin; s->symax = ymax; s->sdy = (ymax - ymin) / (s->ny - 1);
  define_green(s);
}

/* findPotential (PoissonSolverFFT2D.cc:174-256), shape check omitted
 * because the calculator always passes conforming grids. */
static void find_potential(oracle_sc_t* s) {
  int nx2 = s->nx2, ny2 = s->ny2, h = ny2 / 2 + 1;
  double scale = log(s->sdx / s->grho.dx);
  s->green_hat[0] = s->re00 + scale * (nx2 * ny2);
  for (int i = 0; i < s->nx; i++)
    for (int j = 0; j < s->ny; j++) s->work_in[(size_t)i * ny2 + j] = s->rho[(size_t)i * s->ny + j];
  oracle_fft_r2c_2d(nx2, ny2, s->work_in, s->work_hat);
  for (size_t idx = 0; idx < (size_t)nx2 * h; idx++) {
    double gr = s->green_hat[2 * idx] - scale, gi = s->green_hat[2 * idx + 1];
    double ore = s->work_hat[2 * idx], oim = s->work_hat[2 * idx + 1];
    s->work_hat[2 * idx] = ore * gr - oim * gi;
    s->work_hat[2 * idx + 1] = ore * gi + oim * gr;
  }
  double* res = (double*)malloc(sizeof(double) * (size_t)nx2 * ny2);
  oracle_fft_c2r_2d(nx2, ny2, s->work_hat, res);
  s->green_hat[0] = s->re00;
  double denom = 1.0 / (nx2 * ny2);
  for (int i = 0; i < s->nx; i++)
    for (int j = 0; j < s->ny; j++) s->phi[(size_t)i * s->ny + j] = denom * res[(size_t)i * ny2 + j];
  free(res);
}

oracle_sc_t* oracle_sc_new(int nx, int ny, int nz, double xy_ratio) {
  if (nx < 3 || ny < 3 || nz < 1) return NULL;
  oracle_sc_t* s = (oracle_sc_t*)calloc(1, sizeof(oracle_sc_t));
  s->nx = nx; s->ny = ny; s->nz = nz;
  s->xy_ratio = (xy_ratio > 0.) ? xy_ratio : 1.0;
  s->nx2 = 2 * nx; s->ny2 = 2 * ny;
  size_t h = (size_t)s->ny2 / 2 + 1;
  s->green_hat = (double*)calloc(2 * (size_t)s->nx2 * h, sizeof(double));
  s->work_hat = (double*)calloc(2 * (size_t)s->nx2 * h, sizeof(double));
  s->work_in = (double*)calloc((size_t)s->nx2 * s->ny2, sizeof(double));
  s->rho = (double*)calloc((size_t)nx * ny, sizeof(double));
  s->phi = (double*)calloc((size_t)nx * ny, sizeof(double));
  s->zarr = (double*)calloc((size_t)nz, sizeof(double));
  /* SpaceChargeCalc2p5D constructors (SpaceChargeCalc2p5D.cc:25-43):
   * solver on (-r, r, -1, 1); grids on (-1,1)x(-1,1) and (-0.5,0.5). */
  solver_set_xy(s, -s->xy_ratio, s->xy_ratio, -1.0, 1.0);
  s->grho.nx = nx; s->grho.ny = ny;
  g2_setx(&s->grho, -1.0, 1.0);
  g2_sety(&s->grho, -1.0, 1.0);
  s->gz.nz = nz;
  g1_set(&s->gz, -0.5, 0.5);
  return s;
}

void oracle_sc_free(oracle_sc_t* s) {
  if (!s) return;
  free(s->green_hat); free(s->work_hat); free(s->work_in);
  free(s->rho); free(s->phi); free(s->zarr); free(s->zderiv);
  free(s);
}

/* SpaceChargeCalc2p5Drb constructors (SpaceChargeCalc2p5Drb.cc:31-60): the
 * same solver and grids as the 2.5D calculator plus the derivative grid;
 * three smoothing points. */
oracle_sc_t* oracle_scrb_new(int nx, int ny, int nz, double xy_ratio) {
  oracle_sc_t* s = oracle_sc_new(nx, ny, nz, xy_ratio);
  if (!s) return NULL;
  s->rb = 1;
  s->n_long_avg = 3;
  s->zderiv = (double*)calloc((size_t)nz, sizeof(double));
  return s;
}

void oracle_scrb_set_long_avg(oracle_sc_t* s, int n) { s->n_long_avg = n; }

/* ------------------------------------------------------------------ */
/* trackBunch                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
  const oracle_sc_t* s;
  double* soa;
  const double* msize;
  double m0;
  int n, i0, i1;
  double lim[6];
  double* rho;
  double* zarr;
  double factor;
  int phase;
  /* 2.5Drb longitudinal kick */
  double lsf, lsf_in, lsf_out, a2, xc, yc;
} slice_t;

/* BunchExtremaCalculator::getExtremaXYZ loop (BunchExtremaCalculator.cc:47-62) */
static void slice_extrema(slice_t* t) {
  double* lim = t->lim;
  lim[0] = DBL_MAX; lim[1] = -DBL_MAX; lim[2] = DBL_MAX; lim[3] = -DBL_MAX; lim[4] = DBL_MAX; lim[5] = -DBL_MAX;
  const double* x = t->soa;
  const double* y = t->soa + 2 * (size_t)t->n;
  const double* z = t->soa + 4 * (size_t)t->n;
  for (int i = t->i0; i < t->i1; i++) {
    if (x[i] < lim[0]) lim[0] = x[i];
    if (x[i] > lim[1]) lim[1] = x[i];
    if (y[i] < lim[2]) lim[2] = y[i];
    if (y[i] > lim[3]) lim[3] = y[i];
    if (z[i] < lim[4]) lim[4] = z[i];
    if (z[i] > lim[5]) lim[5] = z[i];
  }
}

/* Grid2D::binBunch + Grid1D::binBunch on one slice (Grid2D.cc:120-138, Grid1D.cc:241-275) */
static void slice_bin(slice_t* t) {
  const oracle_sc_t* s = t->s;
  const double* x = t->soa;
  const double* y = t->soa + 2 * (size_t)t->n;
  const double* z = t->soa + 4 * (size_t)t->n;
  for (int i = t->i0; i < t->i1; i++) {
    double m = t->msize ? t->msize[i] : t->m0;
    g2_bin(&s->grho, t->rho, m, x[i], y[i]);
  }
  for (int i = t->i0; i < t->i1; i++) {
    double m = t->msize ? t->msize[i] : t->m0;
    g1_bin(&s->gz, t->zarr, m, z[i]);
  }
}

/* kick loop (SpaceChargeCalc2p5D.cc:104-119) */
static void slice_kick(slice_t* t) {
  const oracle_sc_t* s = t->s;
  double* x = t->soa;
  double* xp = t->soa + (size_t)t->n;
  double* y = t->soa + 2 * (size_t)t->n;
  double* yp = t->soa + 3 * (size_t)t->n;
  double* z = t->soa + 4 * (size_t)t->n;
  for (int i = t->i0; i < t->i1; i++) {
    double ex, ey;
    g2_grad(&s->grho, s->phi, x[i], y[i], &ex, &ey);
    double Lfactor = -g1_value(&s->gz, s->zarr, z[i]) * t->factor;
    xp[i] += ex * Lfactor;
    yp[i] += ey * Lfactor;
  }
}

/* kick loop of SpaceChargeCalc2p5Drb::trackBunch (SpaceChargeCalc2p5Drb.cc:132-154) */
static void slice_kick_rb(slice_t* t) {
  const oracle_sc_t* s = t->s;
  double* x = t->soa;
  double* xp = t->soa + (size_t)t->n;
  double* y = t->soa + 2 * (size_t)t->n;
  double* yp = t->soa + 3 * (size_t)t->n;
  double* z = t->soa + 4 * (size_t)t->n;
  double* dE = t->soa + 5 * (size_t)t->n;
  for (int i = t->i0; i < t->i1; i++) {
    double r2 = (x[i] - t->xc) * (x[i] - t->xc) + (y[i] - t->yc) * (y[i] - t->yc);
    double ex, ey;
    g2_grad(&s->grho, s->phi, x[i], y[i], &ex, &ey);
    double ez = g1_value(&s->gz, s->zderiv, z[i]);
    double Lfactor = -g1_value(&s->gz, s->zarr, z[i]) * t->factor;
    xp[i] += ex * Lfactor;
    yp[i] += ey * Lfactor;
    double coeff = (r2 <= t->a2) ? t->lsf_in - r2 / t->a2 : t->lsf_out - log(r2);
    dE[i] += ez * t->lsf * coeff;
  }
}

static void* slice_worker(void* arg) {
  slice_t* t = (slice_t*)arg;
  if (t->phase == 0) slice_extrema(t);
  else if (t->phase == 1) slice_bin(t);
  else if (t->phase == 2) slice_kick(t);
  else slice_kick_rb(t);
  return NULL;
}

static void run_phase(slice_t* sl, int nt, int phase) {
  for (int k = 0; k < nt; k++) sl[k].phase = phase;
  if (nt == 1) { slice_worker(&sl[0]); return; }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
  for (int k = 1; k < nt; k++) pthread_create(&th[k], NULL, slice_worker, &sl[k]);
  slice_worker(&sl[0]);
  for (int k = 1; k < nt; k++) pthread_join(th[k], NULL);
  free(th);
}

int oracle_sc_track(oracle_sc_t* s, double* soa, int n, const double* msize,
                    const oracle_sync_t* sync, double length, int nthreads) {
  if (n < 2) return 0; /* SpaceChargeCalc2p5D.cc:79-80 */
  int nt = nthreads < 1 ? 1 : nthreads;
  if (nt > n) nt = n;
  slice_t* sl = (slice_t*)calloc((size_t)nt, sizeof(slice_t));
  for (int k = 0; k < nt; k++) {
    sl[k].s = s; sl[k].soa = soa; sl[k].msize = msize; sl[k].m0 = sync->macrosize; sl[k].n = n;
    sl[k].i0 = (int)((long)n * k / nt);
    sl[k].i1 = (int)((long)n * (k + 1) / nt);
  }
  /* extrema, then the MAX "allreduce" */
  run_phase(sl, nt, 0);
  double xMin = sl[0].lim[0], xMax = sl[0].lim[1], yMin = sl[0].lim[2], yMax = sl[0].lim[3],
         zMin = sl[0].lim[4], zMax = sl[0].lim[5];
  for (int k = 1; k < nt; k++) {
    if (sl[k].lim[0] < xMin) xMin = sl[k].lim[0];
    if (sl[k].lim[1] > xMax) xMax = sl[k].lim[1];
    if (sl[k].lim[2] < yMin) yMin = sl[k].lim[2];
    if (sl[k].lim[3] > yMax) yMax = sl[k].lim[3];
    if (sl[k].lim[4] < zMin) zMin = sl[k].lim[4];
    if (sl[k].lim[5] > zMax) zMax = sl[k].lim[5];
  }
  /* bunchAnalysis (SpaceChargeCalc2p5D.cc:122-234) */
  if (xMin >= xMax || yMin >= yMax || zMin >= zMax) { free(sl); return -2; }
  double xy_ratio_beam = (xMax - xMin) / (yMax - yMin);
  if (fabs(xy_ratio_beam - s->xy_ratio) < 0.25 * s->xy_ratio) {
    double width, center;
    if (xy_ratio_beam > s->xy_ratio) {
      center = (yMax + yMin) / 2.0;
      width = ((yMax - yMin) * (xy_ratio_beam / s->xy_ratio)) / 2.0;
      yMin = center - width;
      yMax = center + width;
    } else {
      center = (xMax + xMin) / 2.0;
      width = ((xMax - xMin) / (xy_ratio_beam / s->xy_ratio)) / 2.0;
      xMin = center - width;
      xMax = center + width;
    }
    s->xy_ratio = (xMax - xMin) / (yMax - yMin);
  } else {
    s->xy_ratio = xy_ratio_beam;
    solver_set_xy(s, xMin, xMax, yMin, yMax);
  }
  g2_setx(&s->grho, xMin, xMax);
  g2_sety(&s->grho, yMin, yMax);
  g1_set(&s->gz, zMin, zMax);
  if (fabs((s->sxmax - s->sxmin) / (s->symax - s->symin) - s->xy_ratio) > 0.00000001)
    solver_set_xy(s, xMin, xMax, yMin, yMax);
  /* private grids per slice, then the SUM "allreduce" */
  size_t ng = (size_t)s->nx * s->ny;
  for (int k = 0; k < nt; k++) {
    sl[k].rho = (k == 0) ? s->rho : (double*)calloc(ng, sizeof(double));
    sl[k].zarr = (k == 0) ? s->zarr : (double*)calloc((size_t)s->nz, sizeof(double));
  }
  memset(s->rho, 0, sizeof(double) * ng);
  memset(s->zarr, 0, sizeof(double) * (size_t)s->nz);
  run_phase(sl, nt, 1);
  for (int k = 1; k < nt; k++) {
    for (size_t q = 0; q < ng; q++) s->rho[q] += sl[k].rho[q];
    for (int q = 0; q < s->nz; q++) s->zarr[q] += sl[k].zarr[q];
    free(sl[k].rho);
    free(sl[k].zarr);
  }
  double total = 0.;
  for (int iz = 0; iz < s->nz; iz++) total += s->zarr[iz];
  s->total_macrosize = total;
  double z_step = s->gz.dz;
  find_potential(s);
  double factor = 2 * length * sync->classical_radius / (pow(sync->beta, 2) * pow(sync->gamma, 3));
  factor = factor / (z_step * total);
  for (int k = 0; k < nt; k++) sl[k].factor = factor;
  run_phase(sl, nt, 2);
  free(sl);
  return 0;
}

/* SpaceChargeCalc2p5Drb::calculateLongDerivative
 * (SpaceChargeCalc2p5Drb.cc:257-306): quadratic least-squares fit over
 * n_long_avg neighbouring cells, derivative at the cell centre. */
static void rb_long_derivative(oracle_sc_t* s) {
  const int nZ = s->nz;
  const double z_step = s->gz.dz;
  if (nZ == 1) {
    s->zderiv[0] = 0.;
    return;
  }
  if (nZ == 2) {
    /* Grid1D::calcGradient at the midpoint (Grid1D.cc:520-534) */
    double zm = (g1_gridz(&s->gz, 0) + g1_gridz(&s->gz, 1)) * 0.5;
    double d = 0.;
    if (!(zm < s->gz.zmin || zm > s->gz.zmax)) {
      int i0, ip;
      double w0, wp;
      g1_ind(&s->gz, zm, &i0, &ip, &w0, &wp);
      d = (s->zarr[ip] - s->zarr[i0]) / s->gz.dz;
    }
    s->zderiv[0] = d / z_step;
    s->zderiv[1] = d / z_step;
    return;
  }
  int nAvg = s->n_long_avg;
  if (nZ < nAvg) nAvg = nZ;
  for (int iz = 0; iz < nZ; iz++) {
    double zc = g1_gridz(&s->gz, iz);
    int i0 = iz - nAvg / 2;
    if (i0 < 0) i0 = 0;
    if (i0 + nAvg >= nZ) i0 = nZ - nAvg;
    /* power sums: m[j] = sum t^j, q[j] = sum t^j y, t = 1..nAvg */
    double m[5], q[5];
    for (int j = 0; j < 5; j++) {
      m[j] = 0.;
      q[j] = 0.;
      for (int i = i0; i < i0 + nAvg; i++) {
        double t = 1.0 * (i - i0 + 1), y = s->zarr[i];
        m[j] += pow(t, j) * pow(y, 0);
        q[j] += pow(t, j) * pow(y, 1);
      }
    }
    /* normal equations of y = a t^2 + b t + c by Cramer's rule */
    double det = (m[0] * m[2] * m[4] - m[1] * m[1] * m[4] - m[0] * m[3] * m[3] + 2 * m[1] * m[2] * m[3] -
                  m[2] * m[2] * m[2]);
    double a = (q[0] * m[1] * m[3] - q[1] * m[0] * m[3] - q[0] * m[2] * m[2] + q[1] * m[1] * m[2] +
                q[2] * m[0] * m[2] - q[2] * m[1] * m[1]) / det;
    double b = (q[1] * m[0] * m[4] - q[0] * m[1] * m[4] + q[0] * m[2] * m[3] - q[2] * m[0] * m[3] -
                q[1] * m[2] * m[2] + q[2] * m[1] * m[2]) / det;
    double dy = 2 * a * (zc - g1_gridz(&s->gz, i0) + z_step) / z_step + b;
    dy = dy / z_step;
    s->zderiv[iz] = dy / z_step;
  }
}

/* SpaceChargeCalc2p5Drb::trackBunch + bunchAnalysis
 * (SpaceChargeCalc2p5Drb.cc:107-255). */
int oracle_scrb_track(oracle_sc_t* s, double* soa, int n, const double* msize, const oracle_sync_t* sync,
                      double length, double pipe_radius, int nthreads) {
  if (n < 2) return 0; /* SpaceChargeCalc2p5Drb.cc:109-110 */
  int nt = nthreads < 1 ? 1 : nthreads;
  if (nt > n) nt = n;
  slice_t* sl = (slice_t*)calloc((size_t)nt, sizeof(slice_t));
  for (int k = 0; k < nt; k++) {
    sl[k].s = s; sl[k].soa = soa; sl[k].msize = msize; sl[k].m0 = sync->macrosize; sl[k].n = n;
    sl[k].i0 = (int)((long)n * k / nt);
    sl[k].i1 = (int)((long)n * (k + 1) / nt);
  }
  run_phase(sl, nt, 0);
  double xMin = sl[0].lim[0], xMax = sl[0].lim[1], yMin = sl[0].lim[2], yMax = sl[0].lim[3],
         zMin = sl[0].lim[4], zMax = sl[0].lim[5];
  for (int k = 1; k < nt; k++) {
    if (sl[k].lim[0] < xMin) xMin = sl[k].lim[0];
    if (sl[k].lim[1] > xMax) xMax = sl[k].lim[1];
    if (sl[k].lim[2] < yMin) yMin = sl[k].lim[2];
    if (sl[k].lim[3] > yMax) yMax = sl[k].lim[3];
    if (sl[k].lim[4] < zMin) zMin = sl[k].lim[4];
    if (sl[k].lim[5] > zMax) zMax = sl[k].lim[5];
  }
  if (xMin >= xMax || yMin >= yMax || zMin >= zMax) { free(sl); return -2; } /* :172-186 */
  /* always stretched to the calculator's fixed ratio (:188-203) */
  double xy_ratio_beam = (xMax - xMin) / (yMax - yMin);
  double width, center;
  if (xy_ratio_beam > s->xy_ratio) {
    center = (yMax + yMin) / 2.0;
    width = ((yMax - yMin) * (xy_ratio_beam / s->xy_ratio)) / 2.0;
    yMin = center - width;
    yMax = center + width;
  } else {
    center = (xMax + xMin) / 2.0;
    width = ((xMax - xMin) / (xy_ratio_beam / s->xy_ratio)) / 2.0;
    xMin = center - width;
    xMax = center + width;
  }
  g2_setx(&s->grho, xMin, xMax);
  g2_sety(&s->grho, yMin, yMax);
  g1_set(&s->gz, zMin, zMax);
  size_t ng = (size_t)s->nx * s->ny;
  for (int k = 0; k < nt; k++) {
    sl[k].rho = (k == 0) ? s->rho : (double*)calloc(ng, sizeof(double));
    sl[k].zarr = (k == 0) ? s->zarr : (double*)calloc((size_t)s->nz, sizeof(double));
  }
  memset(s->rho, 0, sizeof(double) * ng);
  memset(s->zarr, 0, sizeof(double) * (size_t)s->nz);
  memset(s->zderiv, 0, sizeof(double) * (size_t)s->nz);
  run_phase(sl, nt, 1);
  for (int k = 1; k < nt; k++) {
    for (size_t q = 0; q < ng; q++) s->rho[q] += sl[k].rho[q];
    for (int q = 0; q < s->nz; q++) s->zarr[q] += sl[k].zarr[q];
    free(sl[k].rho);
    free(sl[k].zarr);
  }
  rb_long_derivative(s);
  /* moments of the rho grid (:226-254); the reference takes y from the
   * x grid (getGridX(iy)), kept for identical results */
  double x_avg = 0., x2_avg = 0., y_avg = 0., y2_avg = 0., total = 0.;
  for (int ix = 0; ix < s->nx; ix++) {
    for (int iy = 0; iy < s->ny; iy++) {
      double val = s->rho[(size_t)ix * s->ny + iy];
      double x = s->grho.xmin + ix * s->grho.dx;
      double y = s->grho.xmin + iy * s->grho.dx;
      total += val;
      x_avg += x * val;
      x2_avg += x * x * val;
      y_avg += y * val;
      y2_avg += y * y * val;
    }
  }
  x_avg /= total;
  x2_avg /= total;
  y_avg /= total;
  y2_avg /= total;
  s->x_c = x_avg;
  s->y_c = y_avg;
  x2_avg = fabs(x2_avg - x_avg * x_avg);
  y2_avg = fabs(y2_avg - y_avg * y_avg);
  s->a_bunch = sqrt(2 * (x2_avg + y2_avg));
  s->total_macrosize = total;
  double z_step = s->gz.dz;
  find_potential(s);
  double factor = 2 * length * sync->classical_radius / (pow(sync->beta, 2) * pow(sync->gamma, 3));
  factor = factor / (z_step * total);
  double a2 = s->a_bunch * s->a_bunch;
  for (int k = 0; k < nt; k++) {
    sl[k].factor = factor;
    sl[k].lsf_in = 1.0 + 2 * log(pipe_radius / s->a_bunch);
    sl[k].lsf_out = 2 * log(pipe_radius);
    sl[k].a2 = a2;
    sl[k].lsf = -length * sync->classical_radius * sync->mass / (pow(sync->gamma, 2));
    sl[k].xc = s->x_c;
    sl[k].yc = s->y_c;
  }
  run_phase(sl, nt, 3);
  free(sl);
  return 0;
}

void oracle_scrb_extra(const oracle_sc_t* s, double* zderiv, double* abx) {
  if (zderiv && s->zderiv) memcpy(zderiv, s->zderiv, sizeof(double) * (size_t)s->nz);
  if (abx) {
    abx[0] = s->a_bunch;
    abx[1] = s->x_c;
    abx[2] = s->y_c;
  }
}

/* ------------------------------------------------------------------ */
/* Conducting boundary (src/spacecharge/BaseBoundary2D.cc,            */
/* ShapedBoundary2D.cc) and SpaceChargeCalc2p5D with a boundary       */
/* ------------------------------------------------------------------ */

struct oracle_bnd {
  int np, nm, shape; /* shape: -1 points given by the caller, 1 circle, 2 ellipse, 3 rectangle */
  double r_circle, a_ell, b_ell, a_rect, b_rect;
  double xmin, xmax, ymin, ymax, rnorm;
  int initialized;
  double* bx;
  double* by;
  double* lsq;  /* (2 nm + 1) x np */
  double* fv;   /* 2 nm + 1 */
};

static const double ORACLE_PI = 3.14159265358979323846; /* OrbitConst::PI */

/* BaseBoundary2D::lsq_fuctions (BaseBoundary2D.cc:321-348): the free-space
 * modes 1, (r/R)^j cos(j f), (r/R)^j sin(j f) at one point. */
static void bnd_funcs(oracle_bnd_t* b, double x, double y) {
  int nf = 2 * b->nm + 1;
  double r2 = x * x + y * y;
  if (r2 == 0.) {
    b->fv[0] = 1.0;
    for (int i = 1; i < nf; i++) b->fv[i] = 0.0;
    return;
  }
  double r = sqrt(r2);
  double sin_f = y / r, cos_f = x / r;
  double sin_f0 = sin_f, cos_f0 = cos_f;
  double rfac = r / b->rnorm, rj = 1.0;
  b->fv[0] = 1.;
  for (int i = 0; i < b->nm; i++) {
    rj *= rfac;
    b->fv[2 * i + 1] = rj * cos_f0;
    b->fv[2 * i + 2] = rj * sin_f0;
    double sin_f1 = sin_f * cos_f0 + cos_f * sin_f0;
    double cos_f1 = cos_f * cos_f0 - sin_f * sin_f0;
    sin_f0 = sin_f1;
    cos_f0 = cos_f1;
  }
}

/* BaseBoundary2D::_gaussjinv (BaseBoundary2D.cc:238-317): Gauss-Jordan
 * inversion in place with full pivoting. Returns -1 for a singular matrix
 * (the reference stops). */
static int bnd_gaussj(double* a, int n) {
  int* indxc = (int*)calloc((size_t)n, sizeof(int));
  int* indxr = (int*)calloc((size_t)n, sizeof(int));
  int* ipiv = (int*)calloc((size_t)n, sizeof(int));
  int irow = 0, icol = 0, rc = 0;
#define A(r, c) a[(size_t)(r) * n + (c)]
  for (int i = 0; i < n && rc == 0; i++) {
    double big = 0.0;
    for (int j = 0; j < n; j++)
      if (ipiv[j] != 1)
        for (int k = 0; k < n; k++) {
          if (ipiv[k] == 0) {
            if (fabs(A(j, k)) >= big) {
              big = fabs(A(j, k));
              irow = j;
              icol = k;
            }
          } else if (ipiv[k] > 1) {
            rc = -1;
          }
        }
    ++(ipiv[icol]);
    if (irow != icol)
      for (int l = 0; l < n; l++) {
        double t = A(irow, l);
        A(irow, l) = A(icol, l);
        A(icol, l) = t;
      }
    indxr[i] = irow;
    indxc[i] = icol;
    if (A(icol, icol) == 0.0) { rc = -1; break; }
    double pivinv = 1.0 / A(icol, icol);
    A(icol, icol) = 1.0;
    for (int l = 0; l < n; l++) A(icol, l) *= pivinv;
    for (int ll = 0; ll < n; ll++)
      if (ll != icol) {
        double dum = A(ll, icol);
        A(ll, icol) = 0.0;
        for (int l = 0; l < n; l++) A(ll, l) -= A(icol, l) * dum;
      }
  }
  if (rc == 0)
    for (int l = n - 1; l >= 0; l--)
      if (indxr[l] != indxc[l])
        for (int k = 0; k < n; k++) {
          double t = A(k, indxr[l]);
          A(k, indxr[l]) = A(k, indxc[l]);
          A(k, indxc[l]) = t;
        }
#undef A
  free(indxc); free(indxr); free(ipiv);
  return rc;
}

/* BaseBoundary2D::BaseBoundary2D (BaseBoundary2D.cc:21-97) */
oracle_bnd_t* oracle_bnd_new(int np, int nm) {
  if (2 * nm + 1 >= np || nm < 0) return NULL;
  oracle_bnd_t* b = (oracle_bnd_t*)calloc(1, sizeof(oracle_bnd_t));
  b->np = np; b->nm = nm; b->shape = -1;
  b->xmin = DBL_MAX; b->xmax = -DBL_MAX; b->ymin = DBL_MAX; b->ymax = -DBL_MAX;
  b->rnorm = DBL_MAX;
  b->bx = (double*)malloc(sizeof(double) * (size_t)np);
  b->by = (double*)malloc(sizeof(double) * (size_t)np);
  for (int i = 0; i < np; i++) { b->bx[i] = DBL_MAX; b->by[i] = DBL_MAX; }
  b->lsq = (double*)calloc((size_t)(2 * nm + 1) * np, sizeof(double));
  b->fv = (double*)calloc((size_t)(2 * nm + 1), sizeof(double));
  return b;
}

void oracle_bnd_free(oracle_bnd_t* b) {
  if (!b) return;
  free(b->bx); free(b->by); free(b->lsq); free(b->fv);
  free(b);
}

void oracle_bnd_set_point(oracle_bnd_t* b, int i, double x, double y) {
  if (i >= 0 && i < b->np) { b->bx[i] = x; b->by[i] = y; }
  b->initialized = 0;
}

/* BaseBoundary2D::initializeBPs (BaseBoundary2D.cc:190-229): extents, the
 * normalising radius and the least-squares matrix (F^T F)^-1 F^T. */
int oracle_bnd_initialize(oracle_bnd_t* b) {
  int nf = 2 * b->nm + 1, np = b->np;
  b->xmin = DBL_MAX; b->xmax = -DBL_MAX; b->ymin = DBL_MAX; b->ymax = -DBL_MAX;
  for (int i = 0; i < np; i++) {
    double x = b->bx[i], y = b->by[i];
    if (b->xmin > x) b->xmin = x;
    if (b->xmax < x) b->xmax = x;
    if (b->ymin > y) b->ymin = y;
    if (b->ymax < y) b->ymax = y;
  }
  b->rnorm = sqrt((b->xmin - b->xmax) * (b->xmin - b->xmax) + (b->ymin - b->ymax) * (b->ymin - b->ymax));
  double* t = (double*)calloc((size_t)nf * nf, sizeof(double));
  for (int p = 0; p < np; p++) {
    bnd_funcs(b, b->bx[p], b->by[p]);
    for (int i = 0; i < nf; i++)
      for (int j = 0; j < nf; j++) t[(size_t)i * nf + j] += b->fv[i] * b->fv[j];
  }
  int rc = bnd_gaussj(t, nf);
  for (int i = 0; i < nf; i++)
    for (int j = 0; j < np; j++) {
      double v = 0.0;
      bnd_funcs(b, b->bx[j], b->by[j]);
      for (int k = 0; k < nf; k++) v += t[(size_t)i * nf + k] * b->fv[k];
      b->lsq[(size_t)i * np + j] = v;
    }
  free(t);
  b->initialized = rc == 0;
  return rc;
}

/* ShapedBoundary2D::ShapedBoundary2D (ShapedBoundary2D.cc:18-145):
 * shape 1 circle (diameter xDim), 2 ellipse (axes xDim, yDim), 3 rectangle
 * (xDim x yDim); the number of points is rounded down to a multiple of 4. */
oracle_bnd_t* oracle_bnd_new_shape(int np, int nm, int shape, double xdim, double ydim) {
  np = 4 * (np / 4);
  oracle_bnd_t* b = oracle_bnd_new(np, nm);
  if (!b) return NULL;
  b->shape = shape;
  if (shape == 1) b->r_circle = xdim / 2;
  else if (shape == 2) { b->a_ell = xdim / 2; b->b_ell = ydim / 2; }
  else if (shape == 3) { b->a_rect = xdim; b->b_rect = ydim; }
  else { oracle_bnd_free(b); return NULL; }
  if (shape == 1 && xdim != ydim) { oracle_bnd_free(b); return NULL; }
  if (shape == 1) {
    for (int i = 0; i < np; i++)
      oracle_bnd_set_point(b, i, b->r_circle * sin(2 * i * ORACLE_PI / np), b->r_circle * cos(2 * i * ORACLE_PI / np));
  } else if (shape == 2) {
    /* equal arc lengths by iteration on the quarter ellipse */
    double a = b->a_ell, bb = b->b_ell;
    double ds = 2 * ORACLE_PI * sqrt(a * bb) / np, resid = 1.0;
    double* th_arr = (double*)calloc((size_t)np + 1, sizeof(double));
    while (resid > 1.0e-08 || resid < -1.0e-08) {
      double denom = bb;
      double dtheta = ds / denom;
      double th = dtheta / 2.;
      th_arr[0] = 0.;
      for (int i = 0; i < np / 4; i++) {
        denom = bb * bb + (a * a - bb * bb) * sin(th) * sin(th);
        denom = sqrt(denom);
        dtheta = ds / denom;
        th_arr[i + 1] = th_arr[i] + dtheta;
        th += dtheta;
      }
      resid = th_arr[np / 4] - ORACLE_PI / 2.;
      ds *= ORACLE_PI / (2. * th_arr[np / 4]);
    }
    for (int i = 0; i < np / 4; i++) th_arr[np / 2 - i] = ORACLE_PI - th_arr[i];
    for (int i = 0; i < np / 2; i++) th_arr[np / 2 + i] = ORACLE_PI + th_arr[i];
    for (int i = 0; i < np; i++) oracle_bnd_set_point(b, i, a * cos(th_arr[i]), bb * sin(th_arr[i]));
    free(th_arr);
  } else {
    double ar = b->a_rect, br = b->b_rect;
    double dx = ar / (np / 4), dy = br / (np / 4);
    int c = 0;
    for (int i = 0; i < np / 4; i++) oracle_bnd_set_point(b, c++, (-ar / 2.0) + i * dx, br / 2.0);
    for (int i = 0; i < np / 4; i++) oracle_bnd_set_point(b, c++, ar / 2.0, br / 2.0 - i * dy);
    for (int i = 0; i < np / 4; i++) oracle_bnd_set_point(b, c++, ar / 2.0 - i * dx, -br / 2.0);
    for (int i = 0; i < np / 4; i++) oracle_bnd_set_point(b, c++, -ar / 2.0, (-br / 2.0) + i * dy);
  }
  oracle_bnd_initialize(b);
  return b;
}

/* isInside: BaseBoundary2D.cc:144-151, ShapedBoundary2D.cc:284-304 */
int oracle_bnd_is_inside(const oracle_bnd_t* b, double x, double y) {
  if (b->shape == 1) return (x * x + y * y < b->r_circle * b->r_circle) ? 1 : -1;
  if (b->shape == 2) {
    double xx = x / b->a_ell, yy = y / b->b_ell;
    return ((xx * xx + yy * yy) < 1.0) ? 1 : -1;
  }
  if (b->shape == 3) return (fabs(x / b->a_rect) < 0.5 && fabs(y / b->b_rect) < 0.5) ? 1 : -1;
  return (x > b->xmin && x < b->xmax && y > b->ymin && y < b->ymax) ? 1 : -1;
}

/* {np, nm, xmin, xmax, ymin, ymax, rnorm} then bx[np], by[np], lsq[(2nm+1) np] */
void oracle_bnd_get(const oracle_bnd_t* b, double* head, double* bx, double* by, double* lsq) {
  if (head) {
    head[0] = b->np; head[1] = b->nm; head[2] = b->xmin; head[3] = b->xmax;
    head[4] = b->ymin; head[5] = b->ymax; head[6] = b->rnorm;
  }
  if (bx) memcpy(bx, b->bx, sizeof(double) * (size_t)b->np);
  if (by) memcpy(by, b->by, sizeof(double) * (size_t)b->np);
  if (lsq) memcpy(lsq, b->lsq, sizeof(double) * (size_t)(2 * b->nm + 1) * b->np);
}

/* Grid2D::getValue (Grid2D.cc:82-108) */
static double g2_value(const grid2d_t* g, const double* arr, double x, double y) {
  int iX, iY;
  double xf, yf;
  g2_indx(g, x, &iX, &xf);
  g2_indy(g, y, &iY, &yf);
  double xf2 = xf * xf, yf2 = yf * yf;
  double Wxm = 0.5 * (0.25 - xf + xf2), Wx0 = 0.75 - xf2, Wxp = 0.5 * (0.25 + xf + xf2);
  double Wym = 0.5 * (0.25 - yf + yf2), Wy0 = 0.75 - yf2, Wyp = 0.5 * (0.25 + yf + yf2);
  int ny = g->ny;
  const double* a0 = arr + (size_t)(iX - 1) * ny;
  const double* a1 = arr + (size_t)iX * ny;
  const double* a2 = arr + (size_t)(iX + 1) * ny;
  return Wxm * Wym * a0[iY - 1] + Wxm * Wy0 * a0[iY] + Wxm * Wyp * a0[iY + 1] + Wx0 * Wym * a1[iY - 1] +
         Wx0 * Wy0 * a1[iY] + Wx0 * Wyp * a1[iY + 1] + Wxp * Wym * a2[iY - 1] + Wxp * Wy0 * a2[iY] +
         Wxp * Wyp * a2[iY + 1];
}

/* BaseBoundary2D::addBoundaryPotential (BaseBoundary2D.cc:352-460): fit the
 * free-space modes to phi on the boundary points and subtract the fit on
 * every grid node. Returns -1 for an uninitialized boundary or points
 * outside the grid (the reference stops). */
static int bnd_add_potential(oracle_bnd_t* b, oracle_sc_t* s) {
  if (!b->initialized) return -1;
  const grid2d_t* g = &s->grho;
  if (g->xmin > b->xmin || g->xmax < b->xmax || g->ymin > b->ymin || g->ymax < b->ymax) return -1;
  int nf = 2 * b->nm + 1, np = b->np;
  double* bphi = (double*)malloc(sizeof(double) * (size_t)np);
  double* coef = (double*)malloc(sizeof(double) * (size_t)nf);
  for (int j = 0; j < np; j++) bphi[j] = g2_value(g, s->phi, b->bx[j], b->by[j]);
  for (int i = 0; i < nf; i++) {
    coef[i] = 0.0;
    for (int j = 0; j < np; j++) coef[i] += b->lsq[(size_t)i * np + j] * bphi[j];
  }
  for (int i = 0; i < s->nx; i++)
    for (int j = 0; j < s->ny; j++) {
      double phi = 0.;
      bnd_funcs(b, g->xmin + i * g->dx, g->ymin + j * g->dy);
      for (int k = 0; k < nf; k++) phi += coef[k] * b->fv[k];
      s->phi[(size_t)i * s->ny + j] -= phi;
    }
  free(bphi);
  free(coef);
  return 0;
}

typedef struct {
  slice_t* t;
  const oracle_bnd_t* b;
} bslice_t;

/* kick loop with the boundary test (SpaceChargeCalc2p5D.cc:104-119) */
static void* bnd_kick_worker(void* arg) {
  bslice_t* w = (bslice_t*)arg;
  slice_t* t = w->t;
  const oracle_sc_t* s = t->s;
  double* x = t->soa;
  double* xp = t->soa + (size_t)t->n;
  double* y = t->soa + 2 * (size_t)t->n;
  double* yp = t->soa + 3 * (size_t)t->n;
  double* z = t->soa + 4 * (size_t)t->n;
  for (int i = t->i0; i < t->i1; i++) {
    if (oracle_bnd_is_inside(w->b, x[i], y[i]) != 1) continue;
    double ex, ey;
    g2_grad(&s->grho, s->phi, x[i], y[i], &ex, &ey);
    double Lfactor = -g1_value(&s->gz, s->zarr, z[i]) * t->factor;
    xp[i] += ex * Lfactor;
    yp[i] += ey * Lfactor;
  }
  return NULL;
}

/* SpaceChargeCalc2p5D::trackBunch(bunch, length, boundary) with
 * bunchAnalysis's boundary branch (SpaceChargeCalc2p5D.cc:77-120, 174-234). */
int oracle_sc_track_bnd(oracle_sc_t* s, double* soa, int n, const double* msize, const oracle_sync_t* sync,
                        double length, oracle_bnd_t* b, int nthreads) {
  if (n < 2) return 0;
  int nt = nthreads < 1 ? 1 : nthreads;
  if (nt > n) nt = n;
  slice_t* sl = (slice_t*)calloc((size_t)nt, sizeof(slice_t));
  for (int k = 0; k < nt; k++) {
    sl[k].s = s; sl[k].soa = soa; sl[k].msize = msize; sl[k].m0 = sync->macrosize; sl[k].n = n;
    sl[k].i0 = (int)((long)n * k / nt);
    sl[k].i1 = (int)((long)n * (k + 1) / nt);
  }
  run_phase(sl, nt, 0);  /* only z is used (getExtremaZ) */
  double zMin = sl[0].lim[4], zMax = sl[0].lim[5];
  for (int k = 1; k < nt; k++) {
    if (sl[k].lim[4] < zMin) zMin = sl[k].lim[4];
    if (sl[k].lim[5] > zMax) zMax = sl[k].lim[5];
  }
  double xMax = b->xmax, xMin = b->xmin, yMax = b->ymax, yMin = b->ymin;
  s->xy_ratio = (xMax - xMin) / (yMax - yMin);
  if (zMin >= zMax) { free(sl); return -2; }
  g2_setx(&s->grho, xMin, xMax);
  g2_sety(&s->grho, yMin, yMax);
  g1_set(&s->gz, zMin, zMax);
  if (fabs((s->sxmax - s->sxmin) / (s->symax - s->symin) - s->xy_ratio) > 0.00000001)
    solver_set_xy(s, xMin, xMax, yMin, yMax);
  size_t ng = (size_t)s->nx * s->ny;
  for (int k = 0; k < nt; k++) {
    sl[k].rho = (k == 0) ? s->rho : (double*)calloc(ng, sizeof(double));
    sl[k].zarr = (k == 0) ? s->zarr : (double*)calloc((size_t)s->nz, sizeof(double));
  }
  memset(s->rho, 0, sizeof(double) * ng);
  memset(s->zarr, 0, sizeof(double) * (size_t)s->nz);
  run_phase(sl, nt, 1);
  for (int k = 1; k < nt; k++) {
    for (size_t q = 0; q < ng; q++) s->rho[q] += sl[k].rho[q];
    for (int q = 0; q < s->nz; q++) s->zarr[q] += sl[k].zarr[q];
    free(sl[k].rho);
    free(sl[k].zarr);
  }
  double total = 0.;
  for (int iz = 0; iz < s->nz; iz++) total += s->zarr[iz];
  s->total_macrosize = total;
  double z_step = s->gz.dz;
  find_potential(s);
  if (bnd_add_potential(b, s)) { free(sl); return -3; }
  double factor = 2 * length * sync->classical_radius / (pow(sync->beta, 2) * pow(sync->gamma, 3));
  factor = factor / (z_step * total);
  bslice_t* w = (bslice_t*)calloc((size_t)nt, sizeof(bslice_t));
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
  for (int k = 0; k < nt; k++) { sl[k].factor = factor; w[k].t = &sl[k]; w[k].b = b; }
  for (int k = 1; k < nt; k++) pthread_create(&th[k], NULL, bnd_kick_worker, &w[k]);
  bnd_kick_worker(&w[0]);
  for (int k = 1; k < nt; k++) pthread_join(th[k], NULL);
  free(th);
  free(w);
  free(sl);
  return 0;
}

void oracle_sc_grids(const oracle_sc_t* s, double* rho, double* phi, double* zg, double* lim) {
  size_t ng = (size_t)s->nx * s->ny;
  if (rho) memcpy(rho, s->rho, sizeof(double) * ng);
  if (phi) memcpy(phi, s->phi, sizeof(double) * ng);
  if (zg) memcpy(zg, s->zarr, sizeof(double) * (size_t)s->nz);
  if (lim) {
    lim[0] = s->grho.xmin; lim[1] = s->grho.xmax; lim[2] = s->grho.ymin; lim[3] = s->grho.ymax;
    lim[4] = s->gz.zmin; lim[5] = s->gz.zmax; lim[6] = s->grho.dx; lim[7] = s->grho.dy;
    lim[8] = s->gz.dz; lim[9] = s->xy_ratio; lim[10] = s->total_macrosize;
  }
}

void oracle_sc_fields(const oracle_sc_t* s, int n, const double* x, const double* y,
                      const double* z, double* ex, double* ey, double* lam) {
  for (int i = 0; i < n; i++) {
    g2_grad(&s->grho, s->phi, x[i], y[i], &ex[i], &ey[i]);
    lam[i] = g1_value(&s->gz, s->zarr, z[i]);
  }
}

/* ------------------------------------------------------------------ */
/* TEAPOT maps (src/teapot/teapotbase.cc)                             */
/* ------------------------------------------------------------------ */

#define X(i) soa[(size_t)(i)]
#define XP(i) soa[(size_t)n + (i)]
#define Y(i) soa[2 * (size_t)n + (i)]
#define YP(i) soa[3 * (size_t)n + (i)]
#define Z(i) soa[4 * (size_t)n + (i)]
#define DE(i) soa[5 * (size_t)n + (i)]

static const double ORBIT_C = 2.99792458e+8; /* OrbitConst.cc:27 */
static double g_fact[50];
static int g_fact_init = 0;
static void init_fact(void) { /* teapotbase.cc:45-57 */
  if (g_fact_init) return;
  g_fact[0] = 1.0;
  for (int i = 1; i < 50; i++) g_fact[i] = i * g_fact[i - 1];
  g_fact_init = 1;
}

/* rotatexy (teapotbase.cc:80-101) */
void oracle_rotatexy(double* soa, int n, double angle) {
  double cs = cos(angle), sn = sin(angle);
  for (int i = 0; i < n; i++) {
    double xt = X(i), pxt = XP(i), yt = Y(i), pyt = YP(i);
    X(i) = cs * xt - sn * yt;
    XP(i) = cs * pxt - sn * pyt;
    Y(i) = sn * xt + cs * yt;
    YP(i) = sn * pxt + cs * pyt;
  }
}

/* drifti body (teapotbase.cc:120-140) */
static void drift_one(double* soa, int n, int i, double gamma2i, double dp_p_coeff, double length) {
  double dp_p = DE(i) * dp_p_coeff;
  double KNL = 1.0 / (1.0 + dp_p);
  X(i) += KNL * length * XP(i);
  Y(i) += KNL * length * YP(i);
  double phifac = (XP(i) * XP(i) + YP(i) * YP(i) + dp_p * dp_p * gamma2i) / 2.0;
  phifac = (phifac * KNL - dp_p * gamma2i) * KNL;
  Z(i) -= length * phifac;
}

/* drift (teapotbase.cc:158-184) */
void oracle_drift(double* soa, int n, oracle_sync_t* s, double length) {
  double v = ORBIT_C * s->beta;
  s->time = s->time + length / v;
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) drift_one(soa, n, i, gamma2i, dp_p_coeff, length);
}

/* wrapbunch (teapotbase.cc:202-212) */
void oracle_wrapbunch(double* soa, int n, double length) {
  for (int i = 0; i < n; i++) {
    if (Z(i) < -length / 2.0) Z(i) += length;
    if (Z(i) > length / 2.0) Z(i) -= length;
  }
}

/* kick (teapotbase.cc:232-258) */
void oracle_kick(double* soa, int n, double kx, double ky, double kE) {
  if (kx != 0.) for (int i = 0; i < n; i++) XP(i) += kx;
  if (ky != 0.) for (int i = 0; i < n; i++) YP(i) += ky;
  if (kE != 0.) for (int i = 0; i < n; i++) DE(i) += kE;
}

/* complex helpers, same operation order as std::complex<double>
 * multiplication in libstdc++ without -ffast-math: (a+ib)(c+id) =
 * (ac - bd) + i(ad + bc) */
typedef struct { double re, im; } cx;
static cx cmul(cx a, cx b) { cx r; r.re = a.re * b.re - a.im * b.im; r.im = a.re * b.im + a.im * b.re; return r; }
static cx cadd(cx a, cx b) { cx r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static cx csub(cx a, cx b) { cx r; r.re = a.re - b.re; r.im = a.im - b.im; return r; }
static cx cneg(cx a) { cx r; r.re = -a.re; r.im = -a.im; return r; }
static cx cmk(double re, double im) { cx r; r.re = re; r.im = im; return r; }

/* multp (teapotbase.cc:336-374) */
void oracle_multp(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew) {
  if (s->charge == 0.) return;
  init_fact();
  double kl1 = kl / g_fact[pole];
  for (int i = 0; i < n; i++) {
    cx z = cmk(X(i), Y(i));
    cx zn = cmk(1.0, 0.0);
    for (int k = 0; k < pole; k++) zn = cmul(zn, z);
    if (skew) {
      XP(i) += kl1 * zn.im;
      YP(i) += kl1 * zn.re;
    } else {
      XP(i) -= kl1 * zn.re;
      YP(i) += kl1 * zn.im;
    }
  }
}

/* multpfringeIN / OUT (teapotbase.cc:395-600); sgn = -1 for IN, +1 for OUT */
static void multpfringe(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew, int sgn) {
  if (s->charge == 0.) return;
  init_fact();
  cx rootm1 = cmk(0.0, 1.0);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  int lm1 = pole, l = pole + 1, lp1 = pole + 2, lp2 = pole + 3;
  cx cxl = cmk(l, 0.0), cxlp2 = cmk(lp2, 0.0);
  double klfactlp1 = kl / (4.0 * g_fact[lp1]);
  cx kterm = skew ? cmk(0.0, klfactlp1) : cmk(klfactlp1, 0.0);
  cx kt = (sgn < 0) ? cneg(kterm) : kterm;
  for (int i = 0; i < n; i++) {
    double x = X(i), y = Y(i);
    cx z = cmk(x, y);
    double px = XP(i), py = YP(i);
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    cx zlm1 = cmk(1., 0.);
    for (int k = 0; k < lm1; k++) zlm1 = cmul(zlm1, z);
    cx zl = cmul(zlm1, z);
    cx fxterm = cmk(l * x, -lp2 * y);
    cx dxfxterm = cmul(cxl, cadd(fxterm, z));
    cx dyfxterm = cmul(rootm1, csub(cmul(cxl, fxterm), cmul(cxlp2, z)));
    cx fyterm = cmk(l * y, lp2 * x);
    cx dxfyterm = cadd(cmul(cxl, fyterm), cmul(cmul(rootm1, cxlp2), z));
    cx dyfyterm = cmul(cxl, cadd(cmul(rootm1, fyterm), z));
    cx fxcx = cmul(cmul(kt, zl), fxterm);
    cx dxfxcx = cmul(cmul(kt, zlm1), dxfxterm);
    cx dyfxcx = cmul(cmul(kt, zlm1), dyfxterm);
    cx fycx = cmul(cmul(kt, zl), fyterm);
    cx dxfycx = cmul(cmul(kt, zlm1), dxfyterm);
    cx dyfycx = cmul(cmul(kt, zlm1), dyfyterm);
    X(i) -= fxcx.re * KNL;
    Y(i) -= fycx.re * KNL;
    double M11 = 1.0 - dxfxcx.re * KNL;
    double M12 = -dxfycx.re * KNL;
    double M21 = -dyfxcx.re * KNL;
    double M22 = 1.0 - dyfycx.re * KNL;
    double detM = M11 * M22 - M12 * M21;
    double pxnew = (M22 * px - M12 * py) / detM;
    double pynew = (-M21 * px + M11 * py) / detM;
    XP(i) = pxnew;
    YP(i) = pynew;
    Z(i) -= (pxnew * fxcx.re + pynew * fycx.re) * KNL * KNL;
  }
}
void oracle_multpfringeIN(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew) {
  multpfringe(soa, n, s, pole, kl, skew, -1);
}
void oracle_multpfringeOUT(double* soa, int n, const oracle_sync_t* s, int pole, double kl, int skew) {
  multpfringe(soa, n, s, pole, kl, skew, +1);
}

/* quad1 (teapotbase.cc:620-701) */
void oracle_quad1(double* soa, int n, oracle_sync_t* s, double length, double kq) {
  if (kq == 0. || s->charge == 0.) { oracle_drift(soa, n, s, length); return; }
  double kqc = kq;
  double sqrt_kq, kqlength, cx_, sx, cy, sy;
  double m11 = 0., m12 = 0., m21 = 0., m22 = 0., m33 = 0., m34 = 0., m43 = 0., m44 = 0.;
  double v = ORBIT_C * s->beta;
  if (length > 0.) s->time = s->time + length / v;
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  if (kqc > 0.) {
    sqrt_kq = pow(kqc, 0.5);
    kqlength = sqrt_kq * length;
    cx_ = cos(kqlength); sx = sin(kqlength); cy = cosh(kqlength); sy = sinh(kqlength);
    m11 = cx_; m12 = sx / sqrt_kq; m21 = -sx * sqrt_kq; m22 = cx_;
    m33 = cy; m34 = sy / sqrt_kq; m43 = sy * sqrt_kq; m44 = cy;
  } else if (kqc < 0.) {
    sqrt_kq = pow(-kqc, 0.5);
    kqlength = sqrt_kq * length;
    cx_ = cosh(kqlength); sx = sinh(kqlength); cy = cos(kqlength); sy = sin(kqlength);
    m11 = cx_; m12 = sx / sqrt_kq; m21 = sx * sqrt_kq; m22 = cx_;
    m33 = cy; m34 = sy / sqrt_kq; m43 = -sy * sqrt_kq; m44 = cy;
  }
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double x0 = X(i), xp0 = XP(i), y0 = Y(i), yp0 = YP(i);
    X(i) = x0 * m11 + xp0 * m12;
    XP(i) = x0 * m21 + xp0 * m22;
    Y(i) = y0 * m33 + yp0 * m34;
    YP(i) = y0 * m43 + yp0 * m44;
    Z(i) += dp_p * gamma2i * length;
  }
}

/* quad2 (teapotbase.cc:719-744); bend2 is the same map (teapotbase.cc:1164-1189) */
void oracle_quad2(double* soa, int n, const oracle_sync_t* s, double length) {
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    X(i) -= KNL * length * dp_p * XP(i);
    Y(i) -= KNL * length * dp_p * YP(i);
    double phifac = (XP(i) * XP(i) + YP(i) * YP(i) + dp_p * dp_p * gamma2i) / 2.0;
    phifac = (phifac * KNL + dp_p * dp_p * gamma2i) * KNL;
    Z(i) -= length * phifac;
  }
}

/* quadfringeIN/OUT (teapotbase.cc:784-904); sgn = +1 IN, -1 OUT */
static void quadfringe(double* soa, int n, const oracle_sync_t* s, double kq, int sgn) {
  if (s->charge == 0.) return;
  double kqc = kq;
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    double x0 = X(i), xp0 = XP(i), y0 = Y(i), yp0 = YP(i);
    double t = (kqc * KNL / 4.) * (x0 * x0 - y0 * y0);
    double detM = 1.0 - pow(t, 2);
    if (sgn > 0) {
      X(i) += (kqc * KNL / 12.) * x0 * (x0 * x0 + 3. * y0 * y0);
      XP(i) -= (kqc * KNL / 4.) * (xp0 * (x0 * x0 + y0 * y0) - 2. * yp0 * x0 * y0);
      XP(i) /= detM;
      Y(i) -= (kqc * KNL / 12.) * y0 * (y0 * y0 + 3. * x0 * x0);
      YP(i) -= (kqc * KNL / 4.) * (-yp0 * (x0 * x0 + y0 * y0) + 2. * xp0 * x0 * y0);
      YP(i) /= detM;
      Z(i) += (kqc * KNL * KNL / 12.) * (xp0 * x0 * (x0 * x0 + 3. * y0 * y0) - yp0 * y0 * (y0 * y0 + 3. * x0 * x0));
    } else {
      X(i) -= (kqc * KNL / 12.) * x0 * (x0 * x0 + 3. * y0 * y0);
      XP(i) += (kqc * KNL / 4.) * (xp0 * (x0 * x0 + y0 * y0) - 2. * yp0 * x0 * y0);
      XP(i) /= detM;
      Y(i) += (kqc * KNL / 12.) * y0 * (y0 * y0 + 3. * x0 * x0);
      YP(i) += (kqc * KNL / 4.) * (-yp0 * (x0 * x0 + y0 * y0) + 2. * xp0 * x0 * y0);
      YP(i) /= detM;
      Z(i) -= (kqc * KNL * KNL / 12.) * (xp0 * x0 * (x0 * x0 + 3. * y0 * y0) - yp0 * y0 * (y0 * y0 + 3. * x0 * x0));
    }
  }
}
void oracle_quadfringeIN(double* soa, int n, const oracle_sync_t* s, double kq) { quadfringe(soa, n, s, kq, +1); }
void oracle_quadfringeOUT(double* soa, int n, const oracle_sync_t* s, double kq) { quadfringe(soa, n, s, kq, -1); }

/* wedgerotate (teapotbase.cc:923-967) */
void oracle_wedgerotate(double* soa, int n, const oracle_sync_t* s, double e, int frinout) {
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  double cs = cos(e), sn = sin(e);
  for (int i = 0; i < n; i++) {
    double dp_p, xp_temp, p0_temp, p0;
    if (frinout == 0) {
      dp_p = DE(i) * dp_p_coeff;
      xp_temp = XP(i);
      p0_temp = 1.0 + dp_p;
      X(i) /= cs;
      XP(i) = xp_temp * cs + p0_temp * sn;
      p0 = -xp_temp * sn + p0_temp * cs;
      dp_p = p0 - 1.0;
      Z(i) = (-X(i) * sn + Z(i)) * cs;
    } else {
      dp_p = DE(i) * dp_p_coeff;
      p0 = 1.0 + dp_p;
      Z(i) = X(i) * sn + Z(i) / cs;
      X(i) *= cs;
      xp_temp = XP(i) * cs - p0 * sn;
      p0_temp = XP(i) * sn + p0 * cs;
      XP(i) = xp_temp;
      dp_p = p0_temp - 1.0;
    }
    DE(i) = dp_p / dp_p_coeff;
  }
}

/* wedgedrift (teapotbase.cc:986-1016) */
void oracle_wedgedrift(double* soa, int n, const oracle_sync_t* s, double e, int inout) {
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  double ct = cos(e) / sin(e);
  for (int i = 0; i < n; i++) {
    double sl;
    if (inout == 0) {
      double dp_p = DE(i) * dp_p_coeff;
      double tn = XP(i) / (1.0 + dp_p);
      sl = X(i) / (ct - tn);
    } else {
      sl = X(i) / ct;
    }
    drift_one(soa, n, i, gamma2i, dp_p_coeff, sl);
  }
}

/* wedgebend (teapotbase.cc:1037-1080) */
void oracle_wedgebend(double* soa, int n, const oracle_sync_t* s, double e, int inout, double rho, int nsteps) {
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  int nst = nsteps / 2;
  if (nst < 1) nst = 1;
  double ct = cos(e) / sin(e);
  for (int i = 0; i < n; i++) {
    double sl;
    if (inout == 0) {
      sl = -X(i) / ct;
    } else {
      double dp_p = DE(i) * dp_p_coeff;
      double tn = XP(i) / (1.0 + dp_p);
      sl = -X(i) / (ct + tn);
    }
    double sm = sl / nst, sm2 = sm / 2.0;
    drift_one(soa, n, i, gamma2i, dp_p_coeff, sm2);
    XP(i) -= sm / rho;
    for (int j = 1; j < nst; j++) {
      drift_one(soa, n, i, gamma2i, dp_p_coeff, sm);
      XP(i) -= sm / rho;
    }
    drift_one(soa, n, i, gamma2i, dp_p_coeff, sm2);
  }
}

/* bend1 (teapotbase.cc:1099-1146) */
void oracle_bend1(double* soa, int n, oracle_sync_t* s, double length, double th) {
  double v = ORBIT_C * s->beta;
  if (length > 0.) s->time = s->time + length / v;
  double betasq = s->beta * s->beta;
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  double rho = length / th;
  double cx_ = cos(th), sx = sin(th);
  double m11 = cx_, m12 = rho * sx, m16 = rho * (1.0 - cx_);
  double m21 = -sx / rho, m22 = cx_, m26 = sx;
  double m51 = -sx, m52 = -rho * (1.0 - cx_), m56 = -betasq * length + rho * sx;
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double x0 = X(i), xp0 = XP(i);
    X(i) = x0 * m11 + xp0 * m12 + dp_p * m16;
    XP(i) = x0 * m21 + xp0 * m22 + dp_p * m26;
    Y(i) += length * YP(i);
    Z(i) += x0 * m51 + xp0 * m52 + dp_p * m56;
  }
}

void oracle_bend2(double* soa, int n, const oracle_sync_t* s, double length) { oracle_quad2(soa, n, s, length); }

/* bend3 (teapotbase.cc:1208-1232) */
void oracle_bend3(double* soa, int n, const oracle_sync_t* s, double th) {
  double gamma2i = 1.0 / (s->gamma * s->gamma);
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    double phifac = (YP(i) * YP(i) + dp_p * dp_p * gamma2i) / 2.0;
    XP(i) -= phifac * KNL * th;
    Y(i) += KNL * YP(i) * X(i) * th;
    phifac = (phifac * KNL - dp_p * gamma2i) * KNL;
    Z(i) -= th * phifac * X(i);
  }
}

/* bend4 (teapotbase.cc:1251-1274) */
void oracle_bend4(double* soa, int n, const oracle_sync_t* s, double th) {
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    double xfac = 1.0 + KNL * XP(i) * th / 2.0;
    double phifac = KNL * KNL * XP(i) * XP(i) / 2.0;
    X(i) *= xfac * xfac;
    XP(i) /= xfac;
    Z(i) -= th * phifac * X(i);
  }
}

/* bendfringeIN/OUT (teapotbase.cc:1292-1348); sgn = +1 IN, -1 OUT */
static void bendfringe(double* soa, int n, const oracle_sync_t* s, double rho, int sgn) {
  double dp_p_coeff = 1.0 / (s->momentum * s->beta);
  for (int i = 0; i < n; i++) {
    double dp_p = DE(i) * dp_p_coeff;
    double KNL = 1.0 / (1.0 + dp_p);
    if (sgn > 0) {
      X(i) += KNL * Y(i) * Y(i) / (2. * rho);
      YP(i) -= KNL * XP(i) * Y(i) / rho;
      Z(i) += KNL * KNL * XP(i) * Y(i) * Y(i) / (2. * rho);
    } else {
      X(i) -= KNL * Y(i) * Y(i) / (2. * rho);
      YP(i) += KNL * XP(i) * Y(i) / rho;
      Z(i) -= KNL * KNL * XP(i) * Y(i) * Y(i) / (2. * rho);
    }
  }
}
void oracle_bendfringeIN(double* soa, int n, const oracle_sync_t* s, double rho) { bendfringe(soa, n, s, rho, +1); }
void oracle_bendfringeOUT(double* soa, int n, const oracle_sync_t* s, double rho) { bendfringe(soa, n, s, rho, -1); }

/* ------------------------------------------------------------------ */
/* programs                                                           */
/* ------------------------------------------------------------------ */

/* op codes: keep in sync with ORBIT_OP_* in include/orbit_gb300.h */
enum {
  OP_DRIFT = 1, OP_QUAD1 = 2, OP_QUAD2 = 3, OP_QFRIN = 4, OP_QFROUT = 5,
  OP_BEND1 = 6, OP_BEND2 = 7, OP_BEND3 = 8, OP_BEND4 = 9, OP_BFRIN = 10, OP_BFROUT = 11,
  OP_MULTP = 12, OP_MPFRIN = 13, OP_MPFROUT = 14, OP_ROTXY = 15, OP_WRAP = 16, OP_KICK = 17,
  OP_WEDGEROT = 18, OP_WEDGEDRIFT = 19, OP_WEDGEBEND = 20, OP_SC = 32
};

int oracle_run_program(const oracle_op_t* ops, int nops, int turns, double* soa, int n,
                       const double* msize, oracle_sync_t* s, oracle_sc_t** calcs, int nthreads) {
  for (int t = 0; t < turns; t++) {
    for (int k = 0; k < nops; k++) {
      const oracle_op_t* o = &ops[k];
      switch (o->code) {
        case OP_DRIFT: oracle_drift(soa, n, s, o->d[0]); break;
        case OP_QUAD1: oracle_quad1(soa, n, s, o->d[0], o->d[1]); break;
        case OP_QUAD2: oracle_quad2(soa, n, s, o->d[0]); break;
        case OP_QFRIN: oracle_quadfringeIN(soa, n, s, o->d[0]); break;
        case OP_QFROUT: oracle_quadfringeOUT(soa, n, s, o->d[0]); break;
        case OP_BEND1: oracle_bend1(soa, n, s, o->d[0], o->d[1]); break;
        case OP_BEND2: oracle_bend2(soa, n, s, o->d[0]); break;
        case OP_BEND3: oracle_bend3(soa, n, s, o->d[0]); break;
        case OP_BEND4: oracle_bend4(soa, n, s, o->d[0]); break;
        case OP_BFRIN: oracle_bendfringeIN(soa, n, s, o->d[0]); break;
        case OP_BFROUT: oracle_bendfringeOUT(soa, n, s, o->d[0]); break;
        case OP_MULTP: oracle_multp(soa, n, s, o->i0, o->d[0], o->i1); break;
        case OP_MPFRIN: oracle_multpfringeIN(soa, n, s, o->i0, o->d[0], o->i1); break;
        case OP_MPFROUT: oracle_multpfringeOUT(soa, n, s, o->i0, o->d[0], o->i1); break;
        case OP_ROTXY: oracle_rotatexy(soa, n, o->d[0]); break;
        case OP_WRAP: oracle_wrapbunch(soa, n, o->d[0]); break;
        case OP_KICK: oracle_kick(soa, n, o->d[0], o->d[1], o->d[2]); break;
        case OP_WEDGEROT: oracle_wedgerotate(soa, n, s, o->d[0], o->i0); break;
        case OP_WEDGEDRIFT: oracle_wedgedrift(soa, n, s, o->d[0], o->i0); break;
        case OP_WEDGEBEND: oracle_wedgebend(soa, n, s, o->d[0], o->i0, o->d[1], o->i1); break;
        case OP_SC: {
          int rc = calcs[o->i0]->rb
                       ? oracle_scrb_track(calcs[o->i0], soa, n, msize, s, o->d[0], o->d[1], nthreads)
                       : oracle_sc_track(calcs[o->i0], soa, n, msize, s, o->d[0], nthreads);
          if (rc != 0) return rc;
          break;
        }
        default: return -1;
      }
    }
  }
  return 0;
}

/* BunchTwissAnalysis::analyzeBunch + getEmittance for planes 0,1
 * (BunchTwissAnalysis.cc:49-140, 372-390), equal macrosizes. */
/* BunchTwissAnalysis::analyzeBunch (BunchTwissAnalysis.cc:49-140):
 * out = {count, total macrosize, <c_i> [6], <c_i c_j> for i >= j [21, row i
 * holds j = 0..i]}, macrosize-weighted when msize is given. */
void oracle_twiss_moments(const double* soa, int n, const double* msize, double* out) {
  double avg[6] = {0}, corr[36] = {0}, total = 0.;
  if (msize) {
    for (int ip = 0; ip < n; ip++) {
      double m = msize[ip];
      total += m;
      for (int i = 0; i < 6; i++) avg[i] += m * soa[(size_t)i * n + ip];
      for (int i = 0; i < 6; i++)
        for (int j = 0; j < i + 1; j++) corr[i + 6 * j] += m * soa[(size_t)i * n + ip] * soa[(size_t)j * n + ip];
    }
  } else {
    double m = 1.0;
    for (int ip = 0; ip < n; ip++) {
      for (int i = 0; i < 6; i++) avg[i] += soa[(size_t)i * n + ip];
      for (int i = 0; i < 6; i++)
        for (int j = 0; j < i + 1; j++) corr[i + 6 * j] += soa[(size_t)i * n + ip] * soa[(size_t)j * n + ip];
    }
    total += n * m;
    for (int i = 0; i < 6; i++) avg[i] *= m;
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < i + 1; j++) corr[i + 6 * j] *= m;
  }
  out[0] = n;
  out[1] = total;
  int k = 8;
  for (int i = 0; i < 6; i++) out[2 + i] = fabs(total) > 0. ? avg[i] / total : 0.;
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < i + 1; j++) out[k++] = fabs(total) > 0. ? corr[i + 6 * j] / total : 0.;
}

/* BunchTuneAnalysis::analyzeBunch (BunchTuneAnalysis.cc:36-108): per
 * particle the normalised phases, the phase advance since the last call
 * ("tune") and the actions; ph holds six SoA rows {xLastPhase, yLastPhase,
 * xLastTune, yLastTune, xAction, yAction} of n.  twiss = {betax, alphax,
 * etax, etapx, betay, alphay}; etot = kinetic energy + mass. */
void oracle_tune_analysis(const double* soa, int n, double beta, double etot, const double* twiss, double* ph) {
  const double betax = twiss[0], alphax = twiss[1], etax = twiss[2], etapx = twiss[3];
  const double betay = twiss[4], alphay = twiss[5];
  for (int i = 0; i < n; i++) {
    double x = X(i), xp = XP(i), y = Y(i), yp = YP(i);
    double dpp = 1 / (beta * beta) * DE(i) / etot;
    double xval = (x - etax * dpp) / sqrt(betax);
    double xpval = (xp - etapx * dpp) * sqrt(betax) + xval * alphax;
    double yval = y / sqrt(betay);
    double ypval = (yp + y * alphay / betay) * sqrt(betay);
    double angle = atan2(xpval, xval);
    if (angle < 0.) angle += (2.0 * ORACLE_PI);
    double xPhase = angle;
    double xTune = (ph[(size_t)0 * n + i] - xPhase) / (2.0 * ORACLE_PI);
    if (xTune < 0.) xTune += 1.;
    ph[(size_t)0 * n + i] = xPhase;
    ph[(size_t)2 * n + i] = xTune;
    angle = atan2(ypval, yval);
    if (angle < 0.) angle += (2.0 * ORACLE_PI);
    double yPhase = angle;
    double yTune = (ph[(size_t)1 * n + i] - yPhase) / (2.0 * ORACLE_PI);
    if (yTune < 0.) yTune += 1.;
    ph[(size_t)1 * n + i] = yPhase;
    ph[(size_t)3 * n + i] = yTune;
    double xc = x - etax * dpp, yc = y;
    double xpfac = xp - etapx * dpp, ypfac = yp;
    double pxc = xpfac + xc * (alphax / betax);
    double pyc = ypfac + yc * (alphay / betay);
    ph[(size_t)4 * n + i] = xc * xc / betax + pxc * pxc * betax;
    ph[(size_t)5 * n + i] = yc * yc / betay + pyc * pyc * betay;
  }
}

void oracle_rms_emittance(const double* soa, int n, double* ex, double* ey) {
  double avg[6] = {0}, corr[36] = {0};
  for (int ip = 0; ip < n; ip++) {
    double c[6];
    for (int i = 0; i < 6; i++) c[i] = soa[(size_t)i * n + ip];
    for (int i = 0; i < 6; i++) avg[i] += c[i];
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < i + 1; j++) corr[i + 6 * j] += c[i] * c[j];
  }
  double tm = (double)n;
  for (int i = 0; i < 6; i++) avg[i] = avg[i] / tm;
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < i + 1; j++) {
      double v = corr[i + 6 * j] / tm;
      corr[i + 6 * j] = v;
      corr[j + 6 * i] = v;
    }
#define CORR(a, b) (corr[(a) + 6 * (b)] - avg[a] * avg[b])
  double out[2];
  for (int ic = 0; ic < 2; ic++) {
    double x2 = fabs(CORR(2 * ic, 2 * ic)), xp2 = fabs(CORR(2 * ic + 1, 2 * ic + 1));
    double xxp = CORR(2 * ic, 2 * ic + 1), xdE = CORR(2 * ic, 5), xpdE = CORR(2 * ic + 1, 5);
    double dE2 = fabs(CORR(5, 5));
    if (dE2 == 0)
      out[ic] = sqrt(fabs(x2 * xp2 - xxp * xxp));
    else
      out[ic] = sqrt(fabs((x2 - xdE * xdE / dE2) * (xp2 - xpdE * xpdE / dE2) -
                          (xxp - xdE * xpdE / dE2) * (xxp - xdE * xpdE / dE2)));
  }
#undef CORR
  *ex = out[0];
  *ey = out[1];
}
