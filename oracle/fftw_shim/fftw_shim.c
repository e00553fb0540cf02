/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- FFTW3 stand-in, see fftw3.h.
 * A plan records the arrays and sizes; fftw_execute runs oracle/fft.c.
 */
#include "fftw3.h"
#include "../fft.h"

#include <stdlib.h>

struct oracle_fftw_plan_s {
  int kind; /* 0 = r2c, 1 = c2r */
  int n0, n1;
  void* in;
  void* out;
};

void* fftw_malloc(size_t n) {
  void* p = NULL;
  if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
  return p;
}

void fftw_free(void* p) { free(p); }

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->kind = 0; p->n0 = n0; p->n1 = n1; p->in = in; p->out = out;
  return p;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->kind = 1; p->n0 = n0; p->n1 = n1; p->in = in; p->out = out;
  return p;
}

void fftw_execute(const fftw_plan p) {
  if (p->kind == 0)
    oracle_fft_r2c_2d(p->n0, p->n1, (const double*)p->in, (double*)p->out);
  else
    oracle_fft_c2r_2d(p->n0, p->n1, (const double*)p->in, (double*)p->out);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
