/*
 * Reference-compatible layer of libarec_gb300.
 *
 * The library defines the reference's own C++ entry points with the reference's
 * signatures, so a program built against the reference's headers links against
 * this library unchanged (the translation units it replaces are left out of
 * that program's build):
 *
 *   arecProject2D, arecProject2D_KB, arecProject2D_SQ        AREC3D/AREC3D/arecproject.h:55-62
 *   arecBackProject2D, arecBackProject2D_KB, arecBackProject2D_SQ
 *   cyl_sirt, cyl_sirt_SQ                                    AREC3D/AREC3D/arecsirt.h:6-10
 *   cyl_sirt_KB                                              AREC3D/AREC3D/arecsirt_KB.h:6-7
 *   cyl_cgls, cyl_cgls_SQ                                    AREC3D/AREC3D/areccgls.h:6-10
 *   cyl_cgls_KB                                              AREC3D/AREC3D/areccgls_KB.h:6-7
 *   cyl_cgls_stat, cyl_cgls_KB_stat, cyl_cgls_SQ_stat,
 *   init_weights                                             AREC3D/AREC3D/areccgls_stat.h:6-13
 *   arecCCImages                                             AREC3D/AREC3D/arecImage.h:36
 *   arecRotCCImages                                          AREC3D/AREC3D/arecImage.h:37
 *   arecRotateImages, arecRotateImages_skew,
 *   arecRotateImages_skew_safe                               AREC3D/AREC3D/arecImage.h:46-48
 *   arecImageTakeLog                                         AREC3D/AREC3D/arecImage.h:34
 *   makePeriodicSlice, periodicDecomposition                 AREC3D/AREC3D/imagetools.h:4-5
 *   arecReadImageHeader, arecReadImage, arecWriteImage       AREC3D/AREC3D/arecImageIO.h:65-67
 *   arecReadImageDistbyZ, arecReadImageDistbyY,
 *   arecWriteImageMergeY, arecWriteImageMergeZ               AREC3D/AREC3D/arecImageIO_mpi.h:3-6
 *   ccorr2d, speak, fshift2d                                 AREC3D/AREC3D/align2dstack.h:9,13,25
 *
 * and, for C and FFI callers, the extern "C" aliases declared below (same
 * arguments, `arecgb_` prefix).  Arguments, ownership and status codes are the
 * reference's: input images are passed by value and owned by the caller;
 * projection outputs are caller-allocated and overwritten; a solver allocates
 * *xvol (calloc) when xvol->data == NULL and otherwise warm-starts CGLS from it.
 * CUDA failures return ARECGB_ERR_* codes (arec_gb300.h) where the reference
 * would call MPI_Abort.  The communicator is accepted and ignored: the whole
 * problem runs on the current GPU.
 */
#pragma once

#include "arec_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef MPI_VERSION
/* No <mpi.h> in this translation unit: MPICH's integer communicator handle. */
typedef int MPI_Comm;
#endif

#ifndef ARECGB_IMAGE_DEFINED
#define ARECGB_IMAGE_DEFINED
/* Same layout as the reference's `arecImage` (AREC3D/AREC3D/arecImage.h:5-18). */
typedef struct Image {
    int nx;
    int ny;
    int nz;
    double radius;
    int height;
    int nnz;
    int nrays;
    int *cord;
    int is_cyl;
    float *data;
} arecImage;
#endif

/* Host data model (AREC3D/AREC3D/arecImage.cpp:15-241, 796-826). */
int arecgb_arecAllocateCBImage(arecImage *cbimage, int nx, int ny, int nz);
int arecgb_arecAllocateCylImage(arecImage *cylimage, double radius, int height);
int arecgb_ImageCyl2CB(arecImage cylimage, arecImage cbimage, int nx, int ny, int nz);
int arecgb_ImageCB2Cyl(arecImage cbimage, arecImage cylimage, int xcent, int zcent, double radius,
                       int height);
void arecgb_arecImageFree(arecImage *image);
void arecgb_reset(arecImage *image);
void arecgb_soft_noneg(arecImage *image);

/* Projectors. */
int arecgb_arecProject2D(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecgb_arecProject2D_KB(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecgb_arecProject2D_SQ(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecgb_arecBackProject2D(arecImage images, float *angles, int nangles, arecImage *bvol);
int arecgb_arecBackProject2D_KB(arecImage images, float *angles, int nangles, arecImage *bvol);
int arecgb_arecBackProject2D_SQ(arecImage images, float *angles, int nangles, arecImage *bvol);

/* Solvers. */
int arecgb_cyl_sirt(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                    int maxit, float tol);
int arecgb_cyl_sirt_KB(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                       float lam, int maxit, float tol);
int arecgb_cyl_sirt_SQ(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                       float lam, int maxit, float tol);
int arecgb_cyl_cgls(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                    int maxit, float tol);
int arecgb_cyl_cgls_KB(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                       float lam, int maxit, float tol);
int arecgb_cyl_cgls_SQ(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                       float lam, int maxit, float tol);

/* Statistically weighted CGLS (weights exp(-b) with a Tukey taper along x). */
int arecgb_cyl_cgls_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                         float lam, int maxit, float tol);
int arecgb_cyl_cgls_KB_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                            float lam, int maxit, float tol);
int arecgb_cyl_cgls_SQ_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol,
                            float lam, int maxit, float tol);
int arecgb_init_weights(MPI_Comm comm, arecImage projections, arecImage *weights);

/* Alignment. */
int arecgb_arecCCImages(MPI_Comm comm, arecImage images1, arecImage images2, float *sx,
                        float *sy);
/* ccorr2d and arecCCImages: nx, ny in [2, 4096] with prime factors 2, 3, 5, 7
 * (the reference's FFTW takes any length; other lengths return
 * ARECGB_ERR_ARG from arecCCImages, and ccorr2d leaves c untouched and reports
 * the error on stderr). */
void arecgb_ccorr2d(int nx, int ny, float *x, float *y, float *c);
void arecgb_speak(int nx, int ny, float *data, float *xt, float *yt);
/* Fourier shift of one image (nx 2..4096, ny 2..2048, prime factors 2, 3, 5,
 * 7; otherwise the output is left untouched and the error reported on stderr). */
void arecgb_fshift2d(int nx, int ny, float *imagein, float *imageout, float sx, float sy);
/* Rotation search and rotations (2 <= r2 <= min(2048, nx/2, ny/2)). */
int arecgb_arecRotCCImages(MPI_Comm comm, arecImage images1, arecImage images2, int r2,
                           float *angles);
void arecgb_arecRotateImages(arecImage *images, float *angles);
void arecgb_arecRotateImages_skew(arecImage *images, float *angles);
void arecgb_arecRotateImages_skew_safe(arecImage *images, arecImage *images_ref, float *angles);

/* Preprocessing (in place on host stacks). */
void arecgb_arecImageTakeLog(arecImage image);
void arecgb_periodicDecomposition(arecImage img);
void arecgb_makePeriodicSlice(int nx, int ny, float *data, float *out);

/* MRC files (one rank: the distributed forms read and write the whole stack;
 * failures print and leave image->data NULL where the reference aborts). */
int arecgb_arecReadImageHeader(char *fname, int *nx, int *ny, int *nz);
int arecgb_arecReadImage(char *fname, arecImage *image);
int arecgb_arecWriteImage(char *fname, arecImage image);
void arecgb_arecReadImageDistbyZ(MPI_Comm comm, const char *fname, arecImage *image);
void arecgb_arecReadImageDistbyY(MPI_Comm comm, const char *fname, arecImage *image);
void arecgb_arecWriteImageMergeY(MPI_Comm comm, const char *fname, arecImage image);
void arecgb_arecWriteImageMergeZ(MPI_Comm comm, const char *fname, arecImage image);

/* Residual trace of the last solver call on this thread (relative residuals,
 * oldest first); returns the number of entries written (<= cap). */
int arecgb_last_trace(double *rel, int cap, arecgb_solve_info *info);

#ifdef __cplusplus
}

/* The same entry points under the reference's own C++ names and signatures
 * (C++ linkage), for C++ callers that include this header in place of the
 * reference's arecproject.h, arecsirt.h, arecsirt_KB.h, areccgls.h,
 * areccgls_KB.h, areccgls_stat.h and the alignment declarations of arecImage.h
 * and align2dstack.h. */
int arecProject2D(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecProject2D_KB(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecProject2D_SQ(arecImage cylvol, float *angles, int nangles, arecImage *projstack);
int arecBackProject2D(arecImage images, float *angles, int nangles, arecImage *bvol);
int arecBackProject2D_KB(arecImage images, float *angles, int nangles, arecImage *bvol);
int arecBackProject2D_SQ(arecImage images, float *angles, int nangles, arecImage *bvol);
int cyl_sirt(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam, int maxit,
             float tol);
int cyl_sirt_KB(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                int maxit, float tol);
int cyl_sirt_SQ(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                int maxit, float tol);
int cyl_cgls(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam, int maxit,
             float tol);
int cyl_cgls_KB(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                int maxit, float tol);
int cyl_cgls_SQ(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                int maxit, float tol);
int cyl_cgls_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                  int maxit, float tol);
int cyl_cgls_KB_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                     int maxit, float tol);
int cyl_cgls_SQ_stat(MPI_Comm comm, arecImage images, float *angles, arecImage *xvol, float lam,
                     int maxit, float tol);
int init_weights(MPI_Comm comm, arecImage projections, arecImage *weights);
int arecCCImages(MPI_Comm comm, arecImage images1, arecImage images2, float *sx, float *sy);
int arecRotCCImages(MPI_Comm comm, arecImage images1, arecImage images2, int r2, float *angle);
void arecRotateImages(arecImage *images, float *angles);
void arecRotateImages_skew(arecImage *images, float *angles);
void arecRotateImages_skew_safe(arecImage *images, arecImage *images_ref, float *angles);
void arecImageTakeLog(arecImage image);
void ccorr2d(int nx, int ny, float *x, float *y, float *c);
void speak(int nx, int ny, float *data, float *xt, float *yt);
void fshift2d(int nx, int ny, float *imagein, float *imageout, float sx, float sy);
void makePeriodicSlice(int nx, int ny, float *data, float *out);
void periodicDecomposition(arecImage img);
#endif
