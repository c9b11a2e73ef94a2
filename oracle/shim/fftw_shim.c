/* FFTW-3 single-precision API stand-in over oracle/fft64.c (see fftw3.h).
 * Test infrastructure only. */
#include "fftw3.h"

#include <stdlib.h>
#include <string.h>

#include "../fft64.h"

enum kind { K_C2C, K_R2C, K_C2R };

struct fftwf_plan_s {
    enum kind kind;
    int rank, n0, n1, sign;
    void *in, *out;
};

void *fftwf_malloc(size_t n) { return malloc(n ? n : 1); }
void fftwf_free(void *p) { free(p); }

static fftwf_plan mk(enum kind k, int rank, int n0, int n1, int sign, void *in, void *out) {
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    p->kind = k;
    p->rank = rank;
    p->n0 = n0;
    p->n1 = n1;
    p->sign = sign;
    p->in = in;
    p->out = out;
    return p;
}

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags) {
    (void)flags;
    return mk(K_C2C, 2, n0, n1, sign, in, out);
}
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags) {
    (void)flags;
    return mk(K_C2C, 2, 1, n, sign, in, out);
}
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags) {
    (void)flags;
    return mk(K_R2C, 2, 1, n, -1, in, out);
}
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags) {
    (void)flags;
    return mk(K_C2R, 2, 1, n, +1, in, out);
}
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float *in, fftwf_complex *out, unsigned flags) {
    (void)flags;
    return mk(K_R2C, 2, n0, n1, -1, in, out);
}
fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex *in, float *out, unsigned flags) {
    (void)flags;
    return mk(K_C2R, 2, n0, n1, +1, in, out);
}

void fftwf_execute(const fftwf_plan p) {
    int n0 = p->n0, n1 = p->n1, h = n1 / 2 + 1;
    size_t n = (size_t)n0 * n1;
    double *re = (double *)calloc(n, sizeof(double));
    double *im = (double *)calloc(n, sizeof(double));
    if (p->kind == K_C2C) {
        const float(*in)[2] = (const float(*)[2])p->in;
        for (size_t i = 0; i < n; i++) {
            re[i] = in[i][0];
            im[i] = in[i][1];
        }
        fft64_c2c_2d(n0, n1, re, im, p->sign);
        float(*out)[2] = (float(*)[2])p->out;
        for (size_t i = 0; i < n; i++) {
            out[i][0] = (float)re[i];
            out[i][1] = (float)im[i];
        }
    } else if (p->kind == K_R2C) {
        const float *in = (const float *)p->in;
        for (size_t i = 0; i < n; i++) re[i] = in[i];
        fft64_c2c_2d(n0, n1, re, im, -1);
        float(*out)[2] = (float(*)[2])p->out;
        for (int r = 0; r < n0; r++)
            for (int c = 0; c < h; c++) {
                out[(size_t)r * h + c][0] = (float)re[(size_t)r * n1 + c];
                out[(size_t)r * h + c][1] = (float)im[(size_t)r * n1 + c];
            }
    } else {
        /* complex-to-real: Hermitian extension of the stored half spectrum */
        const float(*in)[2] = (const float(*)[2])p->in;
        for (int r = 0; r < n0; r++)
            for (int c = 0; c < n1; c++) {
                if (c < h) {
                    re[(size_t)r * n1 + c] = in[(size_t)r * h + c][0];
                    im[(size_t)r * n1 + c] = in[(size_t)r * h + c][1];
                } else {
                    int rr = (n0 - r) % n0, cc = n1 - c;
                    re[(size_t)r * n1 + c] = in[(size_t)rr * h + cc][0];
                    im[(size_t)r * n1 + c] = -in[(size_t)rr * h + cc][1];
                }
            }
        fft64_c2c_2d(n0, n1, re, im, +1);
        float *out = (float *)p->out;
        for (size_t i = 0; i < n; i++) out[i] = (float)re[i];
    }
    free(re);
    free(im);
}

void fftwf_destroy_plan(fftwf_plan p) { free(p); }
