/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C FP64 mixed-radix FFT used by the CPU oracle and by the FFTW
 * stand-in (fftw_shim/) that lets the reference's PoissonSolverFFT2D be
 * compiled here.  FFTW is not installed in this image; this transform
 * follows the published definitions FFTW documents for the calls the
 * reference makes (src/spacecharge/PoissonSolverFFT2D.cc:57-59,162,228,245):
 *   r2c 2D:  Y[k0][k1] = sum_{j0,j1} x[j0][j1] e^{-2 pi i (j0 k0/n0 + j1 k1/n1)},
 *            k1 = 0..n1/2 (unnormalised, row-major, last dim halved)
 *   c2r 2D:  the unnormalised backward (+i) transform of the Hermitian
 *            extension of the half spectrum; imaginary parts of the
 *            self-conjugate k1 = 0 and k1 = n1/2 columns are ignored.
 * Never linked into the product library.
 */
#ifndef ORACLE_FFT_H
#define ORACLE_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

/* In-place complex FFT of length n on interleaved (re,im) doubles with the
 * given stride (in complex elements).  sign = -1 forward, +1 backward.
 * Unnormalised.  Works for any n >= 1 (mixed radix; prime factors done as
 * direct DFTs). */
void oracle_fft_c2c(double* data, int n, int stride, int sign);

/* 2D real-to-complex, FFTW r2c_2d layout: in n0*n1 reals, out n0*(n1/2+1)
 * complex (interleaved). */
void oracle_fft_r2c_2d(int n0, int n1, const double* in, double* out);

/* 2D complex-to-real, FFTW c2r_2d semantics (unnormalised).  `in` is
 * n0*(n1/2+1) complex and is not modified. */
void oracle_fft_c2r_2d(int n0, int n1, const double* in, double* out);

#ifdef __cplusplus
}
#endif

#endif
