/*
 * Double-precision discrete Fourier transform used by the oracle (test
 * infrastructure only).  Written from the mathematics: iterative radix-2
 * Cooley-Tukey for powers of two, Bluestein's chirp-z algorithm (L. Bluestein,
 * 1970) on top of it for every other length.  Unnormalised, like FFTW:
 *   X[k] = sum_n x[n] exp(sign * 2*pi*i*n*k/N),  sign = -1 forward, +1 backward.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* In-place 1-D transform of n complex values (separate re/im arrays). */
void fft64_c2c(int n, double *re, double *im, int sign);

/* In-place 2-D transform of an n0 x n1 row-major complex array. */
void fft64_c2c_2d(int n0, int n1, double *re, double *im, int sign);

#ifdef __cplusplus
}
#endif
