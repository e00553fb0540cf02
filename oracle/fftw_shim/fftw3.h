/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * FFTW3 is not installed in this image.  This header declares the subset of
 * the FFTW3 double-precision API that the reference's PoissonSolverFFT2D
 * calls (src/spacecharge/PoissonSolverFFT2D.hh:18, PoissonSolverFFT2D.cc:49-59,
 * 77-85, 162, 228, 245), with the same names and argument meaning, so that
 * the reference's own source compiles unmodified against it.  The transforms
 * are computed by oracle/fft.c (project code); every parity report that uses
 * the compiled reference states "FFT = project shim (FFTW unavailable)".
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s* fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_ESTIMATE (1U << 6)

void* fftw_malloc(size_t n);
void fftw_free(void* p);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif

#endif
