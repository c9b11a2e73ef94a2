/*
 * ORACLE — CPU restatement of the AREC3D reconstruction path (see
 * arec_oracle.h).  Test infrastructure only; never linked into the product.
 *
 * Build: gcc -O2 -ffp-contract=off (oracle/Makefile).  With contraction off the
 * double/float expression order below is exactly the reference's C++ order, so
 * results agree bit for bit with the reference compiled the same way.
 */
#define _POSIX_C_SOURCE 200809L
#include "arec_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fft64.h"

/* ----------------------------------------------------------------------------
 * Kaiser-Bessel blob table (AREC3D/AREC3D/arecproject.cpp:192-338): the same
 * floats, entries 0..511 (the reachable range).
 */
static const float KB_LUT[512] = {
#include "../arec3d_gb300/csrc/kb_lut_table.inc"
};
/* `float DR = LUT_RANGE / (LUT_SIZE - 1)` (arecproject.cpp:194): 3.0/999 in
 * double, stored as float. */
static float kb_dr(void) { return (float)(3.0 / 999); }

/* interp1_R_MOD (arecproject.cpp:340-346): float argument; the left product is
 * evaluated in double, the right one in float, the sum returned as float. */
static float kb_interp(float x) {
    x = fabsf(x);
    x /= kb_dr();
    int ind = (int)x;
    x -= (float)ind;
    float right = KB_LUT[ind + 1] * x;
    double v = (double)KB_LUT[ind] * (1.0 - (double)x) + (double)right;
    return (float)v;
}

/* ----------------------------------------------------------------------------
 * Square-pixel footprint (AREC3D/AREC3D/arecproject.h:11-47).
 */
typedef struct {
    double a, b, ymax;
} sq_par;

static sq_par sq_points(double angle) {
    double c = cos(angle), s = sin(angle);
    double cms = fabs(0.5 * (c - s));
    double cps = fabs(0.5 * (c + s));
    sq_par p;
    p.a = (cps < cms) ? cps : cms;          /* std::min */
    p.b = ((cms < cps) ? cps : cms) + 1e-6; /* std::max + 1e-6 */
    p.ymax = 1 / (((p.b - p.a) + 2 * p.a));
    return p;
}

/* Piecewise CDF of the footprint; the linear piece is tested first, within
 * a + 1e-3, before the two quadratic pieces (arecproject.h:36-42). */
static double sq_cdf(double x, sq_par p) {
    if (x < -p.b) return 0.0;
    if (x > p.b) return 1.0;
    const double a_eps = p.a + 1e-3;
    if (x > -a_eps && x < a_eps) return 0.5 * p.ymax * (p.b + p.a) + p.ymax * x;
    if (x < -p.a) return 0.5 * p.ymax * (x + p.b) * (x + p.b) / (p.b - p.a);
    if (x > p.a) return 0.5 * p.ymax * (p.b - x) * (p.b - x) / (p.a - p.b) + 1.0;
    return 0.0;
}

/* ----------------------------------------------------------------------------
 * Cylinder support (AREC3D/AREC3D/arecImage.cpp:29-86): the radius-squared and
 * the centred offsets are truncated toward zero by int conversion.
 */
static int cyl_nx(double radius) { return (int)round(2 * radius + 1); }

static int cyl_scan(double radius, int *cord) {
    int nx = cyl_nx(radius);
    int r2 = (int)(radius * radius);
    int n = 0;
    for (int iz = 0; iz < nx; iz++) {
        int zs = (int)(iz - radius);
        int zz = zs * zs;
        for (int ix = 0; ix < nx; ix++) {
            int xs = (int)(ix - radius);
            if (zz + xs * xs <= r2) {
                if (cord) {
                    cord[2 * n] = ix;
                    cord[2 * n + 1] = iz;
                }
                n++;
            }
        }
    }
    return n;
}

int oc_cyl_count(double radius, int *nx_out, int *nrays_out) {
    *nx_out = cyl_nx(radius);
    *nrays_out = cyl_scan(radius, NULL);
    return 0;
}

int oc_cyl_cord(double radius, int *cord) {
    cyl_scan(radius, cord);
    return 0;
}

/* ----------------------------------------------------------------------------
 * Projector pair.  `ny` is the number of slices held (a slab for ranks > 1).
 *
 * Ray positions use `cos(angles[ia])` on a float angle (arecproject.cpp:72,
 * 153, 368, 457, 599, 699): in C++ that resolves to the float overload, so the
 * direction cosines are cosf/sinf widened to double.  The square-pixel
 * footprint instead takes the angle as a double (sqpoints, arecproject.h:11).
 */
typedef struct {
    double radius;
    int nx, nrays;
    int *cord; /* 2*nrays + 3 entries: the tail is zero (see oc_project LIN) */
} geom;

static int geom_init(geom *g, double radius) {
    g->radius = radius;
    g->nx = cyl_nx(radius);
    g->nrays = cyl_scan(radius, NULL);
    g->cord = (int *)calloc((size_t)2 * g->nrays + 3, sizeof(int));
    if (!g->cord) return -1;
    cyl_scan(radius, g->cord);
    return 0;
}

static void geom_free(geom *g) { free(g->cord); }

/* arecProject2D_KB (arecproject.cpp:351-437): weights are the float table
 * interpolant evaluated at float(xb - bin). */
static void kb_weights(double xb, int *iqx_out, double w[3]) {
    int iqx = (int)rint(xb);
    w[0] = (double)kb_interp((float)(xb - (iqx - 1)));
    w[1] = (double)kb_interp((float)(xb - iqx));
    w[2] = (double)kb_interp((float)(xb - (iqx + 1)));
    *iqx_out = iqx;
}

/* arecProject2D (arecproject.cpp:19-99), pmethod=1.  The loop runs i = 1..nrays
 * but reads the 0-based cord table through the 2-argument macro
 * cord(i,j) = cord[2j+i] (arecImage.h:20): ray k = i-1 is placed at
 * (cord[2k+3], cord[2k+4]) = (iz of ray k+1, ix of ray k+2), centred at
 * (int)radius + 1.  The last two rays read past the table; those entries are
 * taken as zero (geom.cord has three zero entries at the end).  xb is stored as
 * float and floored; weights 1-d and d go to bins floor(xb)-1 and floor(xb). */
static void lin_weights(const geom *g, int k, double c, double s, int *b0, float *w0, float *w1) {
    int xcent = (int)g->radius + 1;
    int xc = g->cord[2 * k + 3] - xcent;
    int zc = g->cord[2 * k + 4] - xcent;
    float xb = (float)(xc * c + zc * s + xcent);
    int iqx = (int)floorf(xb);
    float d = xb - (float)iqx;
    *w0 = (float)(1.0 - (double)d);
    *w1 = d;
    *b0 = iqx - 1;
}

/* ----------------------------------------------------------------------------
 * Slab "ranks": nthreads threads each own a contiguous slab of slices, sized as
 * arecReadImageDistbyY does (AREC3D/AREC3D/arecImageIO_mpi.cpp:173-184).  The
 * only cross-rank operation of the solvers is a SUM Allreduce of one double,
 * summed here in rank order.
 */
typedef struct {
    int nranks;
    pthread_barrier_t bar;
    double *slot;
} comm_t;

static double allreduce_sum(comm_t *cm, int rank, double v) {
    if (cm->nranks == 1) return v;
    cm->slot[rank] = v;
    pthread_barrier_wait(&cm->bar);
    double s = 0.0;
    for (int r = 0; r < cm->nranks; r++) s += cm->slot[r];
    pthread_barrier_wait(&cm->bar);
    return s;
}

static void slab_range(int ny, int nranks, int rank, int *y0, int *nyl) {
    int off = 0;
    for (int r = 0; r < nranks; r++) {
        int n = ny / nranks + (r < ny % nranks ? 1 : 0);
        if (r == rank) {
            *y0 = off;
            *nyl = n;
            return;
        }
        off += n;
    }
}

/* Threads per projector call (1 = the reference's single loop); see op_run. */
static int op_threads = 1;

void oc_set_op_threads(int n) { op_threads = n < 1 ? 1 : n; }

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define REAL float
#define FN(n) n
#include "oracle_ops.inc"
#undef REAL
#undef FN
#define REAL double
#define FN(n) CAT(n, 64)
#include "oracle_ops.inc"
#undef REAL
#undef FN

/* ----------------------------------------------------------------------------
 * Cross-correlation shift search.
 */

/* ccorr2d (AREC3D/AREC3D/align2dstack.cpp:480-521): c = IDFT(conj(DFT x) * DFT y),
 * unnormalised.  The DFTs are full complex transforms in double; the reference
 * uses single-precision FFTW r2c/c2r, which compute the same quantity. */
void oc_ccorr2d(int nx, int ny, const float *x, const float *y, float *c) {
    size_t n = (size_t)nx * ny;
    double *xr = (double *)calloc(n, sizeof(double)), *xi = (double *)calloc(n, sizeof(double));
    double *yr = (double *)calloc(n, sizeof(double)), *yi = (double *)calloc(n, sizeof(double));
    for (size_t i = 0; i < n; i++) {
        xr[i] = x[i];
        yr[i] = y[i];
    }
    fft64_c2c_2d(ny, nx, xr, xi, -1);
    fft64_c2c_2d(ny, nx, yr, yi, -1);
    for (size_t i = 0; i < n; i++) {
        double re = xr[i] * yr[i] + xi[i] * yi[i];
        double im = xr[i] * yi[i] - xi[i] * yr[i];
        xr[i] = re;
        xi[i] = im;
    }
    fft64_c2c_2d(ny, nx, xr, xi, +1);
    for (size_t i = 0; i < n; i++) c[i] = (float)xr[i];
    free(xr);
    free(xi);
    free(yr);
    free(yi);
}

/* quad2dfit (align2dstack.cpp:1125-1166): least-squares paraboloid through the
 * 3x3 neighbourhood z (z[(j+1)*3 + (i+1)], i along x, j along y), in double;
 * the shift is clamped to [-1, 1]. */
void oc_quad2dfit(const float *z, float *xsh, float *ysh, float *peakv) {
#define Z(i, j) ((double)z[((j)-1) * 3 + (i)-1])
    double c1 = (26.0 * Z(1, 1) - Z(1, 2) + 2.0 * Z(1, 3) - Z(2, 1) - 19.0 * Z(2, 2) -
                 7.0 * Z(2, 3) + 2.0 * Z(3, 1) - 7.0 * Z(3, 2) + 14.0 * Z(3, 3)) /
                9.0;
    double c2 = (8. * Z(1, 1) - 8. * Z(1, 2) + 5. * Z(2, 1) - 8. * Z(2, 2) + 3. * Z(2, 3) +
                 2. * Z(3, 1) - 8. * Z(3, 2) + 6. * Z(3, 3)) /
                (-6.);
    double c3 = (Z(1, 1) - 2. * Z(1, 2) + Z(1, 3) + Z(2, 1) - 2. * Z(2, 2) + Z(2, 3) + Z(3, 1) -
                 2. * Z(3, 2) + Z(3, 3)) /
                6.0;
    double c4 = (8. * Z(1, 1) + 5. * Z(1, 2) + 2. * Z(1, 3) - 8. * Z(2, 1) - 8. * Z(2, 2) -
                 8. * Z(2, 3) + 3. * Z(3, 2) + 6. * Z(3, 3)) /
                (-6.0);
    double c5 = (Z(1, 1) - Z(1, 3) - Z(3, 1) + Z(3, 3)) / 4.0;
    double c6 = (Z(1, 1) + Z(1, 2) + Z(1, 3) - 2. * Z(2, 1) - 2. * Z(2, 2) - 2. * Z(2, 3) +
                 Z(3, 1) + Z(3, 2) + Z(3, 3)) /
                6.0;
#undef Z
    *ysh = 0.0f;
    *xsh = 0.0f;
    double denom = 4. * c3 * c6 - c5 * c5;
    if (denom != 0.0) {
        *ysh = (float)((c4 * c5 - 2. * c2 * c6) / denom - 2.0);
        *xsh = (float)((c2 * c5 - 2. * c4 * c3) / denom - 2.0);
        double pv = 4. * c1 * c3 * c6 - c1 * c5 * c5 - c2 * c2 * c6 + c2 * c4 * c5 - c4 * c4 * c3;
        *peakv = (float)(pv / denom);
        if (*ysh < -1.0f) *ysh = -1.0f;
        if (*ysh > 1.0f) *ysh = +1.0f;
        if (*xsh < -1.0f) *xsh = -1.0f;
        if (*xsh > 1.0f) *xsh = +1.0f;
    }
}

/* speak (align2dstack.cpp:1059-1105).  The scan runs x outer, y inner
 * (1-based); an element replaces the current peak when |v| > pmax, and pmax then
 * holds the SIGNED v, so after a negative peak every later element replaces
 * it.  The 3x3 window wraps around; the shift is wrapped to (-n/2, n/2].
 * ix0/iy0 (optional) receive the 0-based integer peak position. */
void oc_speak(int nx, int ny, const float *data, float *xt, float *yt, int *ix0, int *iy0) {
    int ix = 1, iy = 1;
    float pmax = 0.0f;
    for (int i = 1; i <= nx; i++)
        for (int j = 1; j <= ny; j++) {
            float v = data[(size_t)(j - 1) * nx + (i - 1)];
            if (fabsf(v) > pmax) {
                ix = i;
                iy = j;
                pmax = v;
            }
        }
    float rsq[9];
    for (int j = -1; j <= 1; j++) {
        int jc = iy + j;
        if (jc < 1) jc += ny;
        if (jc > ny) jc -= ny;
        for (int i = -1; i <= 1; i++) {
            int ir = ix + i;
            if (ir < 1) ir += nx;
            if (ir > nx) ir -= nx;
            rsq[(j + 1) * 3 + (i + 1)] = data[(size_t)(jc - 1) * nx + (ir - 1)];
        }
    }
    float xsh, ysh, pv;
    oc_quad2dfit(rsq, &xsh, &ysh, &pv);
    ix--;
    iy--;
    if (ix0) *ix0 = ix;
    if (iy0) *iy0 = iy;
    *xt = xsh + (float)ix;
    *yt = ysh + (float)iy;
    if (*xt > nx / 2) *xt = *xt - (float)nx;
    if (*yt > ny / 2) *yt = *yt - (float)ny;
}

typedef struct {
    int nx, ny, z0, z1;
    const float *d1, *d2;
    float *sx, *sy;
} cc_arg;

static void *cc_thread(void *p) {
    cc_arg *a = (cc_arg *)p;
    size_t n = (size_t)a->nx * a->ny;
    float *c = (float *)malloc(sizeof(float) * n);
    for (int i = a->z0; i < a->z1; i++) {
        oc_ccorr2d(a->nx, a->ny, a->d1 + n * i, a->d2 + n * i, c);
        oc_speak(a->nx, a->ny, c, &a->sx[i], &a->sy[i], NULL, NULL);
    }
    free(c);
    return NULL;
}

/* arecCCImages (arecImage.cpp:384-434), pairs split over nthreads; the
 * Blackman-Harris filtering there writes buffers nothing reads, so it is omitted. */
int oc_cc_images(int nx, int ny, int nz, const float *d1, const float *d2, float *sx, float *sy,
                 int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nz) nthreads = nz > 0 ? nz : 1;
    cc_arg *args = (cc_arg *)calloc((size_t)nthreads, sizeof(cc_arg));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        args[t].nx = nx;
        args[t].ny = ny;
        args[t].z0 = (int)((long long)nz * t / nthreads);
        args[t].z1 = (int)((long long)nz * (t + 1) / nthreads);
        args[t].d1 = d1;
        args[t].d2 = d2;
        args[t].sx = sx;
        args[t].sy = sy;
    }
    if (nthreads == 1)
        cc_thread(&args[0]);
    else {
        for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, cc_thread, &args[t]);
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    }
    free(args);
    free(th);
    return 0;
}
