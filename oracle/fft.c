/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- see fft.h.
 * Mixed-radix decimation-in-time FFT, FP64, with a cached twiddle table per
 * transform length.  Accuracy is that of direct twiddles from libm cos/sin
 * (about 1e-16 relative per twiddle).
 */
#include "fft.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cplx;

#define MAX_TABLES 32
static struct { int n; cplx* tw; } g_tables[MAX_TABLES];
static int g_ntables = 0;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

/* exp(-2 pi i e / n) for e = 0..n-1 */
static const cplx* twiddles(int n) {
  pthread_mutex_lock(&g_lock);
  for (int i = 0; i < g_ntables; ++i) {
    if (g_tables[i].n == n) {
      const cplx* t = g_tables[i].tw;
      pthread_mutex_unlock(&g_lock);
      return t;
    }
  }
  cplx* t = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  for (int e = 0; e < n; ++e) {
    /* reduce to the first octant-free form: angle = 2*pi*e/n */
    double a = 2.0 * M_PI * (double)e / (double)n;
    t[e].re = cos(a);
    t[e].im = -sin(a);
  }
  /* exact values where the angle is a multiple of pi/2 */
  if (n % 4 == 0) {
    t[0].re = 1.0; t[0].im = 0.0;
    t[n / 4].re = 0.0; t[n / 4].im = -1.0;
    t[n / 2].re = -1.0; t[n / 2].im = 0.0;
    t[3 * n / 4].re = 0.0; t[3 * n / 4].im = 1.0;
  } else if (n % 2 == 0) {
    t[n / 2].re = -1.0; t[n / 2].im = 0.0;
  }
  if (g_ntables < MAX_TABLES) {
    g_tables[g_ntables].n = n;
    g_tables[g_ntables].tw = t;
    ++g_ntables;
  }
  pthread_mutex_unlock(&g_lock);
  return t;
}

static int smallest_factor(int n) {
  if (n % 4 == 0) return 4;
  if (n % 2 == 0) return 2;
  for (int p = 3; p * p <= n; p += 2)
    if (n % p == 0) return p;
  return n;
}

/* out[k] (contiguous, length n) = DFT of in[j*istride], j < n.
 * tw is the table for length N; W_n^e = tw[e * (N/n)]. */
static void fft_rec(const cplx* in, int istride, cplx* out, int n, int sign,
                    const cplx* tw, int N) {
  if (n == 1) { out[0] = in[0]; return; }
  int p = smallest_factor(n);
  int m = n / p;
  for (int r = 0; r < p; ++r)
    fft_rec(in + (size_t)r * istride, istride * p, out + (size_t)r * m, m, sign, tw, N);
  int step = N / n; /* W_n^e = tw[e*step] */
  cplx tmp[64];
  cplx* t = (p <= 64) ? tmp : (cplx*)malloc(sizeof(cplx) * (size_t)p);
  for (int k = 0; k < m; ++k) {
    for (int r = 0; r < p; ++r) {
      cplx f = out[(size_t)r * m + k];
      long e = ((long)r * k) % n;
      cplx w = tw[e * step];
      if (sign > 0) w.im = -w.im;
      t[r].re = f.re * w.re - f.im * w.im;
      t[r].im = f.re * w.im + f.im * w.re;
    }
    if (p == 2) {
      out[k].re = t[0].re + t[1].re; out[k].im = t[0].im + t[1].im;
      out[k + m].re = t[0].re - t[1].re; out[k + m].im = t[0].im - t[1].im;
    } else if (p == 4) {
      /* radix-4 butterfly: W_4 = -i (forward) or +i (backward) */
      double a0r = t[0].re + t[2].re, a0i = t[0].im + t[2].im;
      double a1r = t[0].re - t[2].re, a1i = t[0].im - t[2].im;
      double b0r = t[1].re + t[3].re, b0i = t[1].im + t[3].im;
      double b1r = t[1].re - t[3].re, b1i = t[1].im - t[3].im;
      /* multiply b1 by -i*sign' : forward (sign<0) -> -i, backward -> +i */
      double cr, ci;
      if (sign < 0) { cr = b1i; ci = -b1r; } else { cr = -b1i; ci = b1r; }
      out[k].re = a0r + b0r;         out[k].im = a0i + b0i;
      out[k + m].re = a1r + cr;      out[k + m].im = a1i + ci;
      out[k + 2 * m].re = a0r - b0r; out[k + 2 * m].im = a0i - b0i;
      out[k + 3 * m].re = a1r - cr;  out[k + 3 * m].im = a1i - ci;
    } else {
      int stp = N / p; /* W_p^e = tw[e * stp] */
      for (int q = 0; q < p; ++q) {
        double sr = 0.0, si = 0.0;
        for (int r = 0; r < p; ++r) {
          long e = ((long)r * q) % p;
          cplx w = tw[e * stp];
          if (sign > 0) w.im = -w.im;
          sr += t[r].re * w.re - t[r].im * w.im;
          si += t[r].re * w.im + t[r].im * w.re;
        }
        out[k + (size_t)q * m].re = sr;
        out[k + (size_t)q * m].im = si;
      }
    }
  }
  if (t != tmp) free(t);
}

void oracle_fft_c2c(double* data, int n, int stride, int sign) {
  if (n <= 1) return;
  const cplx* tw = twiddles(n);
  cplx* in = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* out = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* d = (cplx*)data;
  for (int j = 0; j < n; ++j) in[j] = d[(size_t)j * stride];
  fft_rec(in, 1, out, n, sign, tw, n);
  for (int j = 0; j < n; ++j) d[(size_t)j * stride] = out[j];
  free(in);
  free(out);
}

void oracle_fft_r2c_2d(int n0, int n1, const double* in, double* out) {
  int h = n1 / 2 + 1;
  double* row = (double*)malloc(sizeof(double) * 2 * (size_t)n1);
  for (int i = 0; i < n0; ++i) {
    for (int j = 0; j < n1; ++j) { row[2 * j] = in[(size_t)i * n1 + j]; row[2 * j + 1] = 0.0; }
    oracle_fft_c2c(row, n1, 1, -1);
    memcpy(out + (size_t)2 * i * h, row, sizeof(double) * 2 * (size_t)h);
  }
  for (int k = 0; k < h; ++k) oracle_fft_c2c(out + 2 * (size_t)k, n0, h, -1);
  free(row);
}

void oracle_fft_c2r_2d(int n0, int n1, const double* in, double* out) {
  int h = n1 / 2 + 1;
  double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n0 * h);
  memcpy(tmp, in, sizeof(double) * 2 * (size_t)n0 * h);
  for (int k = 0; k < h; ++k) oracle_fft_c2c(tmp + 2 * (size_t)k, n0, h, +1);
  double* row = (double*)malloc(sizeof(double) * 2 * (size_t)n1);
  for (int i = 0; i < n0; ++i) {
    const double* src = tmp + (size_t)2 * i * h;
    /* Hermitian extension along the last dimension */
    for (int k = 0; k < h; ++k) { row[2 * k] = src[2 * k]; row[2 * k + 1] = src[2 * k + 1]; }
    row[1] = 0.0;                               /* k1 = 0 is self-conjugate */
    if (n1 % 2 == 0) row[2 * (n1 / 2) + 1] = 0.0; /* k1 = n1/2 likewise */
    for (int k = h; k < n1; ++k) { row[2 * k] = src[2 * (n1 - k)]; row[2 * k + 1] = -src[2 * (n1 - k) + 1]; }
    oracle_fft_c2c(row, n1, 1, +1);
    for (int j = 0; j < n1; ++j) out[(size_t)i * n1 + j] = row[2 * j];
  }
  free(row);
  free(tmp);
}
