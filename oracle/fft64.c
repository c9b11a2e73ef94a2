/* Double-precision FFT for the oracle; see fft64.h.  Test infrastructure only. */
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double TWO_PI = 6.283185307179586476925286766559;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* Radix-2 decimation-in-time on a power-of-two length. */
static void fft_pow2(int n, double *re, double *im, int sign) {
    /* bit reversal permutation */
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i];
            re[i] = re[j];
            re[j] = t;
            t = im[i];
            im[i] = im[j];
            im[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        double ang = sign * TWO_PI / (double)len;
        for (int k = 0; k < half; k++) {
            /* twiddles evaluated directly (no recurrence) for accuracy */
            double wr = cos(ang * k), wi = sin(ang * k);
            for (int s = 0; s < n; s += len) {
                int a = s + k, b = s + k + half;
                double xr = re[b] * wr - im[b] * wi;
                double xi = re[b] * wi + im[b] * wr;
                re[b] = re[a] - xr;
                im[b] = im[a] - xi;
                re[a] += xr;
                im[a] += xi;
            }
        }
    }
}

/* Bluestein: x[n] w[n] convolved with conj chirp, length m >= 2n-1 power of two. */
static void fft_bluestein(int n, double *re, double *im, int sign) {
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    double *ar = (double *)calloc((size_t)m, sizeof(double));
    double *ai = (double *)calloc((size_t)m, sizeof(double));
    double *br = (double *)calloc((size_t)m, sizeof(double));
    double *bi = (double *)calloc((size_t)m, sizeof(double));
    double *cr = (double *)malloc((size_t)n * sizeof(double));
    double *ci = (double *)malloc((size_t)n * sizeof(double));
    for (int k = 0; k < n; k++) {
        /* chirp exp(sign*pi*i*k^2/n); k^2 reduced mod 2n to keep the argument small */
        long long k2 = ((long long)k * k) % (2LL * n);
        double ang = sign * TWO_PI * 0.5 * (double)k2 / (double)n;
        cr[k] = cos(ang);
        ci[k] = sin(ang);
    }
    for (int k = 0; k < n; k++) {
        ar[k] = re[k] * cr[k] - im[k] * ci[k];
        ai[k] = re[k] * ci[k] + im[k] * cr[k];
    }
    br[0] = cr[0];
    bi[0] = -ci[0];
    for (int k = 1; k < n; k++) {
        br[k] = br[m - k] = cr[k];
        bi[k] = bi[m - k] = -ci[k];
    }
    fft_pow2(m, ar, ai, -1);
    fft_pow2(m, br, bi, -1);
    for (int k = 0; k < m; k++) {
        double xr = ar[k] * br[k] - ai[k] * bi[k];
        double xi = ar[k] * bi[k] + ai[k] * br[k];
        ar[k] = xr;
        ai[k] = xi;
    }
    fft_pow2(m, ar, ai, +1);
    for (int k = 0; k < n; k++) {
        double xr = ar[k] / m, xi = ai[k] / m;
        re[k] = xr * cr[k] - xi * ci[k];
        im[k] = xr * ci[k] + xi * cr[k];
    }
    free(ar);
    free(ai);
    free(br);
    free(bi);
    free(cr);
    free(ci);
}

void fft64_c2c(int n, double *re, double *im, int sign) {
    if (n <= 1) return;
    if (is_pow2(n))
        fft_pow2(n, re, im, sign);
    else
        fft_bluestein(n, re, im, sign);
}

void fft64_c2c_2d(int n0, int n1, double *re, double *im, int sign) {
    for (int r = 0; r < n0; r++) fft64_c2c(n1, re + (size_t)r * n1, im + (size_t)r * n1, sign);
    double *tr = (double *)malloc((size_t)n0 * sizeof(double));
    double *ti = (double *)malloc((size_t)n0 * sizeof(double));
    for (int c = 0; c < n1; c++) {
        for (int r = 0; r < n0; r++) {
            tr[r] = re[(size_t)r * n1 + c];
            ti[r] = im[(size_t)r * n1 + c];
        }
        fft64_c2c(n0, tr, ti, sign);
        for (int r = 0; r < n0; r++) {
            re[(size_t)r * n1 + c] = tr[r];
            im[(size_t)r * n1 + c] = ti[r];
        }
    }
    free(tr);
    free(ti);
}
