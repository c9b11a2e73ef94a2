/*
 * FFTW-3 single-precision API stand-in, used ONLY to compile the reference's
 * own AREC3D sources into oracle/_ref (test infrastructure).  FFTW itself is
 * not installed on this machine, so the transforms are computed in double
 * precision by oracle/fft64.c and rounded to float: outputs follow FFTW's
 * definitions (unnormalised, FFTW_FORWARD = -1) but not FFTW's float rounding.
 *
 * Symbols: the ones referenced by AREC3D/AREC3D/{align2dstack,arecImage,
 * imagetools}.cpp (fftwf_plan_dft_{2d,r2c_1d,c2r_1d,r2c_2d,c2r_2d},
 * fftwf_execute, fftwf_destroy_plan, fftwf_malloc, fftwf_free).
 */
#pragma once
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef struct fftwf_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_ESTIMATE (1U << 6)

void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif
