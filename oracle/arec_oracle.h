/*
 * ORACLE — CPU restatement of the AREC3D reconstruction path.
 *
 * Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may call this; the product library never does.
 *
 * Each function restates the reference algorithm at the cited lines of
 * axarekma/AREC3D (paths relative to that project) with the same precision
 * choices (double weights, float accumulation, double scalar reductions).  It is
 * pinned bit for bit against the reference itself, compiled from its own sources
 * by oracle/build_ref.sh, and against the reference's Catch tests
 * (AREC3D/AREC3D_test/AREC3D_test.cpp); see tests/test_oracle.py.
 *
 * Weightings follow the reference's `pmethod`: 1 = linear (2 taps, with the
 * reference's shifted ray coordinates), 2 = Kaiser-Bessel table, 3 = square
 * pixel footprint ("SQ").
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#define OC_MAX_TRACE 4096

typedef struct {
    int iterations;       /* iterations whose residual was computed */
    int restarts;         /* SIRT step-size restarts */
    int iterbest;         /* CGLS best iterate (reference convention) */
    int status;           /* reference status code */
    float lam_final;      /* SIRT step size after restarts */
    double rnorm0;        /* first residual norm */
    double rel[OC_MAX_TRACE];   /* per-iteration relative residual */
    double rnorm[OC_MAX_TRACE]; /* per-iteration residual norm */
} oc_trace;

/* arecAllocateCylImage (AREC3D/AREC3D/arecImage.cpp:29-86). */
int oc_cyl_count(double radius, int *nx_out, int *nrays_out);
int oc_cyl_cord(double radius, int *cord);

/* Threads used inside each projector call (default 1).  The forward projector
 * splits angles and the back projector rays, so results are bit-identical for
 * any count; this only shortens large oracle runs. */
void oc_set_op_threads(int n);

/* Projector pair (AREC3D/AREC3D/arecproject.cpp:19-183, 351-535, 540-765).
 * x: [nrays][ny]; q: [nangles][ny][nx]; both overwritten (reference `reset`). */
int oc_project(int weighting, double radius, int ny, const float *x, const float *angles,
               int nangles, float *q);
int oc_backproject(int weighting, double radius, int ny, const float *q, const float *angles,
                   int nangles, float *g);

/* cyl_sirt{,_KB,_SQ} (AREC3D/AREC3D/arecsirt.cpp:11-373, arecsirt_KB.cpp:11-191).
 * b: [nangles][ny][nx]; x: [nrays][ny] output; nthreads slabs of slices stand in
 * for the reference's MPI ranks (1 = single rank). */
int oc_sirt(int weighting, int nx, int ny, int nangles, const float *b, const float *angles,
            float lam, int maxit, float tol, float *x, int nthreads, int verbose, oc_trace *tr);

/* cyl_cgls{,_KB,_SQ} (AREC3D/AREC3D/areccgls.cpp:12-478, areccgls_KB.cpp:12-240).
 * warm != 0: x holds the initial guess (reference `xvol->data != NULL`).
 * rnorm_ref > 0 replaces the denominator of the stopping test (the reference
 * uses the initial normal-equation residual); 0 keeps the reference rule. */
int oc_cgls_stat(int weighting, int nx, int ny, int nangles, const float *b,
                 const float *angles, int maxit, float tol, float *x, int warm, int nthreads,
                 int verbose, oc_trace *tr);
int oc_cgls_stat64(int weighting, int nx, int ny, int nangles, const double *b,
                   const float *angles, int maxit, float tol, double *x, int warm, int nthreads,
                   int verbose, oc_trace *tr);
int oc_cgls(int weighting, int nx, int ny, int nangles, const float *b, const float *angles,
            int maxit, float tol, float *x, int warm, double rnorm_ref, int nthreads, int verbose,
            oc_trace *tr);

/* FP64 oracle: the same operators (the reference's weights) applied with
 * every sum, update and vector in double; arrays are double. */
int oc_project64(int weighting, double radius, int ny, const double *x, const float *angles,
                 int nangles, double *q);
int oc_backproject64(int weighting, double radius, int ny, const double *q, const float *angles,
                     int nangles, double *g);
int oc_sirt64(int weighting, int nx, int ny, int nangles, const double *b, const float *angles,
              float lam, int maxit, float tol, double *x, int nthreads, int verbose, oc_trace *tr);
int oc_cgls64(int weighting, int nx, int ny, int nangles, const double *b, const float *angles,
              int maxit, float tol, double *x, int warm, double rnorm_ref, int nthreads,
              int verbose, oc_trace *tr);

/* ccorr2d / speak / quad2dfit / arecCCImages
 * (AREC3D/AREC3D/align2dstack.cpp:480-521, 1059-1166; arecImage.cpp:384-434).
 * Images are [ny][nx] row-major; the FFT is oracle/fft64.c in double. */
void oc_ccorr2d(int nx, int ny, const float *x, const float *y, float *c);
void oc_quad2dfit(const float *z, float *xsh, float *ysh, float *peakv);
void oc_speak(int nx, int ny, const float *data, float *xt, float *yt, int *ix0, int *iy0);
int oc_cc_images(int nx, int ny, int nz, const float *d1, const float *d2, float *sx, float *sy,
                 int nthreads);

#ifdef __cplusplus
}
#endif
