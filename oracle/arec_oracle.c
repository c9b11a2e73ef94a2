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

/* arecProject2D_SQ (arecproject.cpp:540-648) */
static void fp_sq(const geom *g, int ny, const float *x, const float *angles, int na, float *q) {
    const int nx = g->nx;
    const double xcent = g->radius, zcent = g->radius;
    memset(q, 0, sizeof(float) * (size_t)nx * ny * na);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        sq_par p = sq_points((double)angles[ia]);
        float *qa = q + (size_t)ia * nx * ny;
        for (int i = 0; i < g->nrays; i++) {
            double xc = g->cord[2 * i] - xcent;
            double zc = g->cord[2 * i + 1] - zcent;
            double xb = xc * c + zc * s + xcent;
            int iqx = (int)rint(xb);
            double xv = iqx - xb;
            double v0 = sq_cdf(xv - 1.5, p), v1 = sq_cdf(xv - 0.5, p);
            double v2 = sq_cdf(xv + 0.5, p), v3 = sq_cdf(xv + 1.5, p);
            double w[3] = {v1 - v0, v2 - v1, v3 - v2};
            const float *xr = x + (size_t)i * ny;
            for (int iy = 0; iy < ny; iy++) {
                float ct = xr[iy];
                float *row = qa + (size_t)iy * nx;
                for (int j = 0; j < 3; j++) {
                    int b = iqx - 1 + j;
                    if (b >= 0 && b < nx) row[b] = (float)((double)row[b] + w[j] * (double)ct);
                }
            }
        }
    }
}

/* arecBackProject2D_SQ (arecproject.cpp:650-765) */
static void bp_sq(const geom *g, int ny, const float *q, const float *angles, int na, float *out) {
    const int nx = g->nx;
    const double xcent = g->radius, zcent = g->radius;
    memset(out, 0, sizeof(float) * (size_t)g->nrays * ny);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        sq_par p = sq_points((double)angles[ia]);
        const float *qa = q + (size_t)ia * nx * ny;
        for (int i = 0; i < g->nrays; i++) {
            double xc = g->cord[2 * i] - xcent;
            double zc = g->cord[2 * i + 1] - zcent;
            double xb = xc * c + zc * s + xcent;
            int iqx = (int)rint(xb);
            double xv = iqx - xb;
            double v0 = sq_cdf(xv - 1.5, p), v1 = sq_cdf(xv - 0.5, p);
            double v2 = sq_cdf(xv + 0.5, p), v3 = sq_cdf(xv + 1.5, p);
            double w[3] = {v1 - v0, v2 - v1, v3 - v2};
            float *o = out + (size_t)i * ny;
            for (int iy = 0; iy < ny; iy++) {
                const float *row = qa + (size_t)iy * nx;
                for (int j = 0; j < 3; j++) {
                    int b = iqx - 1 + j;
                    if (b >= 0 && b < nx) o[iy] = (float)((double)o[iy] + w[j] * (double)row[b]);
                }
            }
        }
    }
}

/* arecProject2D_KB (arecproject.cpp:351-437): weights are the float table
 * interpolant evaluated at float(xb - bin). */
static void kb_weights(double xb, int *iqx_out, double w[3]) {
    int iqx = (int)rint(xb);
    w[0] = (double)kb_interp((float)(xb - (iqx - 1)));
    w[1] = (double)kb_interp((float)(xb - iqx));
    w[2] = (double)kb_interp((float)(xb - (iqx + 1)));
    *iqx_out = iqx;
}

static void fp_kb(const geom *g, int ny, const float *x, const float *angles, int na, float *q) {
    const int nx = g->nx;
    const double xcent = g->radius, zcent = g->radius;
    memset(q, 0, sizeof(float) * (size_t)nx * ny * na);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        float *qa = q + (size_t)ia * nx * ny;
        for (int i = 0; i < g->nrays; i++) {
            double xc = g->cord[2 * i] - xcent;
            double zc = g->cord[2 * i + 1] - zcent;
            double xb = xc * c + zc * s + xcent;
            int iqx;
            double w[3];
            kb_weights(xb, &iqx, w);
            const float *xr = x + (size_t)i * ny;
            for (int iy = 0; iy < ny; iy++) {
                float ct = xr[iy];
                float *row = qa + (size_t)iy * nx;
                for (int j = 0; j < 3; j++) {
                    int b = iqx - 1 + j;
                    if (b >= 0 && b < nx) row[b] = (float)((double)row[b] + w[j] * (double)ct);
                }
            }
        }
    }
}

/* arecBackProject2D_KB (arecproject.cpp:447-535) */
static void bp_kb(const geom *g, int ny, const float *q, const float *angles, int na, float *out) {
    const int nx = g->nx;
    const double xcent = g->radius, zcent = g->radius;
    memset(out, 0, sizeof(float) * (size_t)g->nrays * ny);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        const float *qa = q + (size_t)ia * nx * ny;
        for (int i = 0; i < g->nrays; i++) {
            double xc = g->cord[2 * i] - xcent;
            double zc = g->cord[2 * i + 1] - zcent;
            double xb = xc * c + zc * s + xcent;
            int iqx;
            double w[3];
            kb_weights(xb, &iqx, w);
            float *o = out + (size_t)i * ny;
            for (int iy = 0; iy < ny; iy++) {
                const float *row = qa + (size_t)iy * nx;
                for (int j = 0; j < 3; j++) {
                    int b = iqx - 1 + j;
                    if (b >= 0 && b < nx) o[iy] = (float)((double)o[iy] + w[j] * (double)row[b]);
                }
            }
        }
    }
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

static void fp_lin(const geom *g, int ny, const float *x, const float *angles, int na, float *q) {
    const int nx = g->nx;
    memset(q, 0, sizeof(float) * (size_t)nx * ny * na);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        float *qa = q + (size_t)ia * nx * ny;
        for (int k = 0; k < g->nrays; k++) {
            int b0;
            float w0, w1;
            lin_weights(g, k, c, s, &b0, &w0, &w1);
            const float *xr = x + (size_t)k * ny;
            for (int iy = 0; iy < ny; iy++) {
                float ct = xr[iy];
                float *row = qa + (size_t)iy * nx;
                if (b0 >= 0 && b0 < nx) row[b0] += w0 * ct;
                if (b0 + 1 >= 0 && b0 + 1 < nx) row[b0 + 1] += w1 * ct;
            }
        }
    }
}

/* arecBackProject2D (arecproject.cpp:109-183): the two taps are applied as two
 * passes over the slices, in float. */
static void bp_lin(const geom *g, int ny, const float *q, const float *angles, int na,
                   float *out) {
    const int nx = g->nx;
    memset(out, 0, sizeof(float) * (size_t)g->nrays * ny);
    for (int ia = 0; ia < na; ia++) {
        double c = (double)cosf(angles[ia]), s = (double)sinf(angles[ia]);
        const float *qa = q + (size_t)ia * nx * ny;
        for (int k = 0; k < g->nrays; k++) {
            int b0;
            float w0, w1;
            lin_weights(g, k, c, s, &b0, &w0, &w1);
            float *o = out + (size_t)k * ny;
            if (b0 >= 0 && b0 < nx)
                for (int iy = 0; iy < ny; iy++) o[iy] += w0 * qa[(size_t)iy * nx + b0];
            if (b0 + 1 >= 0 && b0 + 1 < nx)
                for (int iy = 0; iy < ny; iy++) o[iy] += w1 * qa[(size_t)iy * nx + b0 + 1];
        }
    }
}

static void geom_fp(int weighting, const geom *g, int ny, const float *x, const float *angles,
                    int na, float *q) {
    if (weighting == 1)
        fp_lin(g, ny, x, angles, na, q);
    else if (weighting == 2)
        fp_kb(g, ny, x, angles, na, q);
    else
        fp_sq(g, ny, x, angles, na, q);
}

static void geom_bp(int weighting, const geom *g, int ny, const float *q, const float *angles,
                    int na, float *out) {
    if (weighting == 1)
        bp_lin(g, ny, q, angles, na, out);
    else if (weighting == 2)
        bp_kb(g, ny, q, angles, na, out);
    else
        bp_sq(g, ny, q, angles, na, out);
}

int oc_project(int weighting, double radius, int ny, const float *x, const float *angles,
               int nangles, float *q) {
    geom g;
    if (geom_init(&g, radius)) return -1;
    geom_fp(weighting, &g, ny, x, angles, nangles, q);
    geom_free(&g);
    return 0;
}

int oc_backproject(int weighting, double radius, int ny, const float *q, const float *angles,
                   int nangles, float *out) {
    geom g;
    if (geom_init(&g, radius)) return -1;
    geom_bp(weighting, &g, ny, q, angles, nangles, out);
    geom_free(&g);
    return 0;
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

typedef struct {
    int method; /* 0 = SIRT, 1 = CGLS */
    int weighting, nx, ny, na;
    const float *b, *angles;
    float lam, tol;
    int maxit, warm, verbose;
    double rnorm_ref;
    float *x;
    oc_trace *tr;
    comm_t *cm;
    int rank;
    int status;
} solve_arg;

/* cyl_sirt_SQ (AREC3D/AREC3D/arecsirt.cpp:193-373) on one slab.  The
 * squared norm of A^T b is accumulated into a variable that is never reset, so
 * after each restart the denominator grows (arecsirt.cpp:273,285-290). */
static int sirt_slab(solve_arg *a, const geom *g, int nyl, const float *bl, float *xl) {
    const int nx = g->nx, na = a->na, rank = a->rank;
    size_t nnz = (size_t)g->nrays * nyl, nsin = (size_t)nx * nyl * na;
    float *proj = (float *)calloc(nsin ? nsin : 1, sizeof(float));
    float *bvol = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    float *pvol = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    float *grad = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    float lam = a->lam;
    double relnrm0 = 1.00001, bnorm2 = 0.0, bnorm = 0.0;
    int restarts = 0, iter = 1, count = 0;
    memset(xl, 0, sizeof(float) * nnz);
    while (iter <= a->maxit) {
        double relnrm;
        if (iter == 1) {
            if (restarts == 0) geom_bp(a->weighting, g, nyl, bl, a->angles, na, bvol);
            for (size_t j = 0; j < nnz; j++) {
                bnorm2 += (double)(bvol[j] * bvol[j]);
                grad[j] = bvol[j];
            }
            bnorm = sqrt(allreduce_sum(a->cm, rank, bnorm2));
        } else {
            geom_fp(a->weighting, g, nyl, xl, a->angles, na, proj);
            geom_bp(a->weighting, g, nyl, proj, a->angles, na, pvol);
            for (size_t j = 0; j < nnz; j++) {
                grad[j] = bvol[j];
                grad[j] -= pvol[j];
            }
        }
        double rn2 = 0.0;
        for (size_t j = 0; j < nnz; j++) rn2 += grad[j] * (double)grad[j];
        double rnorm = sqrt(allreduce_sum(a->cm, rank, rn2));
        relnrm = rnorm / bnorm;
        if (rank == 0 && a->tr) {
            if (count < OC_MAX_TRACE) {
                a->tr->rel[count] = relnrm;
                a->tr->rnorm[count] = rnorm;
            }
            if (count == 0) a->tr->rnorm0 = rnorm;
        }
        count++;
        if (rank == 0 && a->verbose)
            printf("iter = %3d, rnorm / bnorm = %11.3e, rnorm = %11.3e\n", iter, relnrm, rnorm);
        if (relnrm > relnrm0) {
            if (restarts > 20) {
                if (rank == 0 && a->verbose)
                    printf("Failure to converge, even with lam = %11.3e\n", lam);
                break;
            }
            ++restarts;
            iter = 1;
            lam /= 2.0;
            relnrm0 = 1.0001;
            memset(xl, 0, sizeof(float) * nnz);
            memset(pvol, 0, sizeof(float) * nnz);
            if (rank == 0 && a->verbose) printf("reducing lam to %11.3e, restarting\n", lam);
            continue;
        }
        if (relnrm < a->tol || relnrm > relnrm0) break;
        relnrm0 = relnrm;
        for (size_t j = 0; j < nnz; j++) {
            xl[j] += lam * grad[j];
            pvol[j] = 0.0f;
        }
        ++iter;
    }
    if (rank == 0 && a->tr) {
        a->tr->iterations = count;
        a->tr->restarts = restarts;
        a->tr->lam_final = lam;
    }
    free(proj);
    free(bvol);
    free(pvol);
    free(grad);
    return 0;
}

/* cyl_cgls_SQ (AREC3D/AREC3D/areccgls.cpp:245-478) on one slab.  Scalars are
 * double; vector updates evaluate in double and store float; norms sum float
 * products in double; the best iterate (smallest normal-equation residual) is
 * restored unless it is the iterate maxit-1 (areccgls.cpp:459-463). */
static int cgls_slab(solve_arg *a, const geom *g, int nyl, const float *bl, float *xl) {
    const int nx = g->nx, na = a->na, rank = a->rank;
    size_t nnz = (size_t)g->nrays * nyl, nsin = (size_t)nx * nyl * na;
    float *proj = (float *)calloc(nsin ? nsin : 1, sizeof(float));
    float *sres = (float *)calloc(nsin ? nsin : 1, sizeof(float));
    float *gvol = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    float *pvol = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    float *xsave = (float *)calloc(nnz ? nnz : 1, sizeof(float));
    int iterbest = a->maxit - 1, iter = 1, count = 0;
    double gamma, gamma0 = 0.0, rnorm, rnorm0, relnrm, rnorm_min;
    if (a->warm)
        geom_fp(a->weighting, g, nyl, xl, a->angles, na, proj);
    else
        memset(xl, 0, sizeof(float) * nnz);
    for (size_t i = 0; i < nsin; i++) sres[i] = bl[i] - proj[i];
    geom_bp(a->weighting, g, nyl, sres, a->angles, na, gvol);
    double rn2 = 0.0;
    for (size_t j = 0; j < nnz; j++) rn2 += (double)(gvol[j] * gvol[j]);
    gamma = allreduce_sum(a->cm, rank, rn2);
    rnorm0 = sqrt(gamma);
    double denom = a->rnorm_ref > 0 ? a->rnorm_ref : rnorm0;
    if (rank == 0 && a->verbose) printf("CG iter = 0, resnrm = %11.3e\n", rnorm0);
    if (rank == 0 && a->tr) a->tr->rnorm0 = rnorm0;
    rnorm_min = rnorm0;
    while (iter <= a->maxit) {
        if (iter == 1) {
            memcpy(pvol, gvol, sizeof(float) * nnz);
        } else {
            double beta = gamma / gamma0;
            for (size_t j = 0; j < nnz; j++) pvol[j] = (float)((double)gvol[j] + beta * (double)pvol[j]);
        }
        geom_fp(a->weighting, g, nyl, pvol, a->angles, na, proj);
        double pn2 = 0.0;
        for (size_t j = 0; j < nsin; j++) pn2 += (double)(proj[j] * proj[j]);
        double alpha = gamma / allreduce_sum(a->cm, rank, pn2);
        for (size_t j = 0; j < nnz; j++) xl[j] = (float)((double)xl[j] + alpha * (double)pvol[j]);
        for (size_t j = 0; j < nsin; j++)
            sres[j] = (float)((double)sres[j] - alpha * (double)proj[j]);
        geom_bp(a->weighting, g, nyl, sres, a->angles, na, gvol);
        rn2 = 0.0;
        for (size_t j = 0; j < nnz; j++) rn2 += (double)(gvol[j] * gvol[j]);
        gamma0 = gamma;
        gamma = allreduce_sum(a->cm, rank, rn2);
        rnorm = sqrt(gamma);
        relnrm = rnorm / denom;
        if (rnorm < rnorm_min) {
            rnorm_min = rnorm;
            iterbest = iter;
            memcpy(xsave, xl, sizeof(float) * nnz);
        }
        if (rank == 0 && a->tr && count < OC_MAX_TRACE) {
            a->tr->rel[count] = relnrm;
            a->tr->rnorm[count] = rnorm;
        }
        count++;
        if (rank == 0 && a->verbose)
            printf("CG iter = %3d, rnorm / bnorm = %11.3e, rnorm = %11.3e\n", iter, relnrm, rnorm);
        if (relnrm < a->tol) break;
        ++iter;
    }
    if (iterbest < a->maxit - 1) memcpy(xl, xsave, sizeof(float) * nnz);
    if (rank == 0 && a->tr) {
        a->tr->iterations = count;
        a->tr->iterbest = iterbest;
    }
    free(proj);
    free(sres);
    free(gvol);
    free(pvol);
    free(xsave);
    return 0;
}

static void *solve_thread(void *p) {
    solve_arg *a = (solve_arg *)p;
    geom g;
    if (geom_init(&g, 0.5 * (a->nx - 1))) {
        a->status = -1;
        return NULL;
    }
    int y0 = 0, nyl = 0;
    slab_range(a->ny, a->cm->nranks, a->rank, &y0, &nyl);
    const int nx = a->nx, na = a->na;
    /* gather this slab's slices of b ([na][ny][nx]) and of x ([nrays][ny]) */
    float *bl = (float *)malloc(sizeof(float) * ((size_t)nx * nyl * na + 1));
    float *xl = (float *)malloc(sizeof(float) * ((size_t)g.nrays * nyl + 1));
    for (int ia = 0; ia < na; ia++)
        memcpy(bl + (size_t)ia * nyl * nx, a->b + ((size_t)ia * a->ny + y0) * nx,
               sizeof(float) * (size_t)nyl * nx);
    for (int k = 0; k < g.nrays; k++)
        memcpy(xl + (size_t)k * nyl, a->x + (size_t)k * a->ny + y0, sizeof(float) * nyl);
    a->status = a->method == 0 ? sirt_slab(a, &g, nyl, bl, xl) : cgls_slab(a, &g, nyl, bl, xl);
    for (int k = 0; k < g.nrays; k++)
        memcpy(a->x + (size_t)k * a->ny + y0, xl + (size_t)k * nyl, sizeof(float) * nyl);
    free(bl);
    free(xl);
    geom_free(&g);
    return NULL;
}

static int run_solver(solve_arg *proto, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > proto->ny) nthreads = proto->ny;
    comm_t cm;
    cm.nranks = nthreads;
    cm.slot = (double *)calloc((size_t)nthreads, sizeof(double));
    if (nthreads > 1) pthread_barrier_init(&cm.bar, NULL, (unsigned)nthreads);
    solve_arg *args = (solve_arg *)calloc((size_t)nthreads, sizeof(solve_arg));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int r = 0; r < nthreads; r++) {
        args[r] = *proto;
        args[r].cm = &cm;
        args[r].rank = r;
        if (r > 0) args[r].tr = NULL;
    }
    if (nthreads == 1) {
        solve_thread(&args[0]);
    } else {
        for (int r = 0; r < nthreads; r++) pthread_create(&th[r], NULL, solve_thread, &args[r]);
        for (int r = 0; r < nthreads; r++) pthread_join(th[r], NULL);
        pthread_barrier_destroy(&cm.bar);
    }
    int st = 0;
    for (int r = 0; r < nthreads; r++)
        if (args[r].status) st = args[r].status;
    free(args);
    free(th);
    free(cm.slot);
    return st;
}

int oc_sirt(int weighting, int nx, int ny, int nangles, const float *b, const float *angles,
            float lam, int maxit, float tol, float *x, int nthreads, int verbose, oc_trace *tr) {
    solve_arg a;
    memset(&a, 0, sizeof(a));
    a.method = 0;
    a.weighting = weighting;
    a.nx = nx;
    a.ny = ny;
    a.na = nangles;
    a.b = b;
    a.angles = angles;
    a.lam = lam;
    a.tol = tol;
    a.maxit = maxit;
    a.verbose = verbose;
    a.x = x;
    a.tr = tr;
    return run_solver(&a, nthreads);
}

int oc_cgls(int weighting, int nx, int ny, int nangles, const float *b, const float *angles,
            int maxit, float tol, float *x, int warm, double rnorm_ref, int nthreads, int verbose,
            oc_trace *tr) {
    solve_arg a;
    memset(&a, 0, sizeof(a));
    a.method = 1;
    a.weighting = weighting;
    a.nx = nx;
    a.ny = ny;
    a.na = nangles;
    a.b = b;
    a.angles = angles;
    a.tol = tol;
    a.maxit = maxit;
    a.warm = warm;
    a.rnorm_ref = rnorm_ref;
    a.verbose = verbose;
    a.x = x;
    a.tr = tr;
    return run_solver(&a, nthreads);
}

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
