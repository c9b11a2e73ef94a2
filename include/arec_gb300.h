/*
 * libarec_gb300 — C ABI of the GB300 (sm_103a) implementation of the AREC3D
 * reconstruction path.  Plain pointers and sizes only.
 *
 * Two layers:
 *   1. This header: a device-resident core API over an opaque geometry plan.
 *      Arrays are CUDA device memory in the device layouts:
 *        volume    [nrays][ys]         (ys = slice stride, see arecgb_plan_info)
 *        sinogram  [nangles][nx][ys]   (bin before slice; padding slices zero)
 *   2. arec_compat.h: the reference's own entry points (arecProject2D_SQ,
 *      cyl_cgls_SQ, arecCCImages, ...) over host `arecImage` buffers, plus
 *      extern "C" aliases of them for FFI callers.
 *
 * Status codes follow the reference where it defines them (0 = OK; projector
 * 1 = volume not cylindrical / nz != nangles, 2 = shape mismatch, -1 = shape
 * mismatch in back-projection; AREC3D/AREC3D/arecproject.cpp:40-44,63-66,
 * 120-141).  Failures the reference handles with MPI_Abort or does not have
 * return negative codes instead:
 *   ARECGB_ERR_ARG       invalid argument (message in arecgb_last_error())
 *   ARECGB_ERR_NOMEM     device or host allocation failed
 *   ARECGB_ERR_CUDA_BASE - cudaError_t   any other CUDA runtime error
 *
 * The library keeps per-device state between calls (cached plans of the
 * compatible entry points, FFT twiddle tables, the static shift-search
 * scratch, kernel shared-memory limits).  cudaDeviceReset destroys the device
 * memory behind that state without the library knowing: do not call the
 * library on a device after resetting it in the same process.
 */
#pragma once

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Projector weightings, numbered like the reference's `pmethod`
 * (AREC3D/AREC3D/AREC3D.cpp:145-169). */
#define ARECGB_LIN 1 /* 2-tap linear (arecProject2D, arecproject.cpp:19-183) */
#define ARECGB_KB 2  /* Kaiser-Bessel table (arecproject.cpp:192-535) */
#define ARECGB_SQ 3  /* square-pixel footprint (arecproject.cpp:540-765) */

#define ARECGB_OK 0
#define ARECGB_ERR_ARG (-90)
#define ARECGB_ERR_NOMEM (-91)
#define ARECGB_ERR_CUDA_BASE (-100)

typedef struct arecgb_plan arecgb_plan;

typedef struct {
    int iterations; /* iterations whose residual was computed */
    int iterbest;   /* CGLS best iterate, reference convention (areccgls.cpp:423-428) */
    int restarts;   /* SIRT step-size restarts (arecsirt.cpp:318-338) */
    int status;     /* reference-style status of the solve */
    float lam_final;
    double rnorm0;    /* initial residual norm (SIRT: ||A^T b||) */
    double rel_final; /* last relative residual */
} arecgb_solve_info;

/* Last error message of the calling thread ("" if none). */
const char *arecgb_last_error(void);
int arecgb_version(void);

/* Geometry plan for one cylinder: radius (pixels, as arecAllocateCylImage,
 * AREC3D/AREC3D/arecImage.cpp:29), ny slices, nangles float radians (copied).
 * Allocates device tables on the current device. */
int arecgb_plan_create(arecgb_plan **plan, int weighting, double radius, int ny, int nangles,
                       const float *angles);
int arecgb_plan_destroy(arecgb_plan *plan);
/* nx = detector width = round(2r+1), nrays = pixels in the disk, ys = slice stride. */
int arecgb_plan_info(const arecgb_plan *plan, int *nx, int *nrays, int *ys);

/* Device-side consistency flag of the plan's kernels since the last check
 * (0 = none; nonzero means a geometric bound the kernels rely on was violated),
 * cleared by the call.  Synchronises the device. */
int arecgb_plan_check(arecgb_plan *plan);

/* q = A x (replaces arecProject2D[_KB|_SQ], arecproject.cpp:19,351,540).
 * d_norm2 (device, optional) receives sum(q*q) accumulated in double. */
int arecgb_project(arecgb_plan *plan, const float *d_x, float *d_q, double *d_norm2,
                   void *stream);
/* g = A^T s (replaces arecBackProject2D[_KB|_SQ], arecproject.cpp:109,447,650). */
int arecgb_backproject(arecgb_plan *plan, const float *d_s, float *d_g, double *d_norm2,
                       void *stream);

/* Filtered back projection, a cheap first reconstruction (no counterpart in
 * the reference): d_x = (pi / nangles) A^T (h * d_b), with h the discrete
 * Ram-Lak ramp filter along detector bins (h(0) = 1/4, h(d) = -1/(pi d)^2 for
 * odd d, 0 for even d != 0) applied as a linear convolution (bins off the
 * detector are zero).  Device layouts; d_work: a sinogram-sized device buffer
 * that receives the filtered sinogram.  d_atb_norm2 (device, optional):
 * ||A^T d_b||^2 as well, by one more back projection (the cold start's
 * denominator of the CGLS stopping test). */
int arecgb_fbp(arecgb_plan *plan, const float *d_b, float *d_x, float *d_work,
               double *d_atb_norm2, void *stream);
/* The ramp filter alone: d_f = (pi / nangles) h * d_s (sinogram layouts). */
int arecgb_ramp_filter(arecgb_plan *plan, const float *d_s, float *d_f, void *stream);

/* CGLS on device arrays (replaces cyl_cgls[_KB|_SQ], areccgls.cpp:12,245,
 * areccgls_KB.cpp:12).  b: sinogram (device layout); x: volume, used as the
 * initial guess when warm != 0.  rnorm_ref > 0 fixes the denominator of the
 * relative normal-equation residual (0 = the reference's initial residual).
 * rel_history (host, optional, maxit entries) receives the residual trace. */
int arecgb_cgls(arecgb_plan *plan, const float *d_b, float *d_x, int warm, int maxit, float tol,
                double rnorm_ref, double *rel_history, arecgb_solve_info *info, void *stream);

/* SIRT/Landweber with the reference's restart rule (replaces cyl_sirt[_KB|_SQ],
 * arecsirt.cpp:11,193, arecsirt_KB.cpp:11).  x is always started from zero. */
int arecgb_sirt(arecgb_plan *plan, const float *d_b, float *d_x, float lam, int maxit, float tol,
                double *rel_history, arecgb_solve_info *info, void *stream);

/* Layout conversion between the reference's [na][ny][nx] stack and the device
 * sinogram layout [na][nx][ys]. */
int arecgb_sino_from_reference(const float *d_ref, float *d_dev, int na, int ny, int nx, int ys,
                               void *stream);
int arecgb_sino_to_reference(const float *d_dev, float *d_ref, int na, int ny, int nx, int ys,
                             void *stream);

/* Statistically weighted CGLS (replaces cyl_cgls[_KB|_SQ]_stat,
 * AREC3D/AREC3D/areccgls_stat.cpp:49-731): CGLS on the weighted normal
 * equations, weights w = expf(-b) times a Tukey window (alpha 0.5) along the
 * detector (init_weights, :12-46), computed on the device from d_b; stops when
 * ||A^T W r|| / ||A^T W r0|| < tol.  Arguments as arecgb_cgls without rnorm_ref. */
int arecgb_cgls_stat(arecgb_plan *plan, const float *d_b, float *d_x, int warm, int maxit,
                     float tol, double *rel_history, arecgb_solve_info *info, void *stream);

/* CGLS over n independent problems, one plan each (cylinders of uneven radius,
 * slice count and angle set; each plan at most once): the arguments of
 * arecgb_cgls per problem (warm, rnorm_ref: arrays or NULL; info: n entries or
 * NULL).  One iteration of all problems is one CUDA graph launch, the problems
 * being parallel branches; a problem that meets its stopping test stops
 * (its kernels become no-ops).  No counterpart in the reference. */
int arecgb_cgls_batch(arecgb_plan *const *plans, const float *const *d_b, float *const *d_x,
                      const int *warm, int n, int maxit, float tol, const double *rnorm_ref,
                      arecgb_solve_info *info, void *stream);

/* Projector timing for measurement: mode 1 resets and starts recording a
 * CUDA event pair around every forward and back projection of this plan (on
 * the stream it runs on); mode 2 reports the summed device time and call
 * counts so far; mode 0 reports and stops.  Reporting synchronises with the
 * last recorded event.  No counterpart in the reference. */
int arecgb_plan_timing(arecgb_plan *plan, int mode, double *fp_ms, long long *fp_calls,
                       double *bp_ms, long long *bp_calls);

/* Autotuner: times the projectors of this plan for the forward projector's
 * band height (32, 64, 128 lines) and floats per lane (the plan's VEC or half
 * of it) and the back projector's shape (VEC or VEC/2 floats per lane, one or
 * two chunks of 32*VEC slices per block) on the caller's buffers d_x (a volume) and d_q (a sinogram),
 * which it overwrites, and keeps the fastest; reports the band and the chunks
 * (either pointer may be NULL; arecgb_plan_shapes reports all four).  Results
 * do not depend on the choice beyond float summation order across bands.  No
 * counterpart in the reference. */
int arecgb_plan_autotune(arecgb_plan *plan, float *d_x, float *d_q, int *fp_band, int *bp_nsc,
                         void *stream);

/* Set the launch shapes directly (e.g. ones arecgb_plan_autotune chose for
 * another plan of the same geometry): band 32, 64 or 128; vectors the plan's
 * VEC or half of it; chunks 1 or 2.  No counterpart in the reference. */
int arecgb_plan_set_shapes(arecgb_plan *plan, int fp_band, int fp_vec, int bp_vec, int bp_nsc);

/* Device bytes of the plan's projector tables (0: none).  A plan for the
 * square-pixel or Kaiser-Bessel weighting stores the taps of every (ray,
 * angle) and the back projector's per-tile ring plans when they take at most
 * 40 % of the free device memory and the environment variable
 * ARECGB_PLAN_TABLES is not "0" at creation; the projectors compute the same
 * values without them (identical results).  No counterpart in the reference. */
long long arecgb_plan_table_bytes(const arecgb_plan *plan);

/* Launch shapes in use: forward band height and floats per lane,
 * back-projection floats per lane and slice chunks per block (0: chosen by
 * size).  No counterpart in the reference. */
int arecgb_plan_shapes(const arecgb_plan *plan, int *fp_band, int *fp_vec, int *bp_vec,
                       int *bp_nsc);

/* Kernel launches issued by this library so far (all threads, approximate
 * only in that concurrent callers interleave). */
long long arecgb_launch_count(void);

/* Cross-correlation shift search over nz image pairs of ny x nx floats, device
 * memory, reference layout [nz][ny][nx] (replaces the loop of arecCCImages,
 * AREC3D/AREC3D/arecImage.cpp:414-428: ccorr2d + speak per pair).
 * sx, sy (device, nz floats): sub-pixel shifts; ix, iy (device, optional):
 * 0-based integer peak positions.  nx and ny in [2, 4096] whose prime factors
 * are 2, 3, 5 and 7 (powers of two take the fastest transforms); other
 * lengths return ARECGB_ERR_ARG. */
int arecgb_cc_shifts(const float *d_img1, const float *d_img2, int nz, int ny, int nx,
                     float *d_sx, float *d_sy, int *d_ix, int *d_iy, void *stream);

/* Fourier shift of a stack of nz images [nz][ny][nx] (device memory) by
 * (d_sx[i], d_sy[i]) pixels each (replaces the per-image loop over fshift2d,
 * AREC3D/AREC3D/align2dstack.cpp:566-630, used by the alignment driver,
 * AREC3D.cpp:219,230): out = Re(IDFT(DFT(in) exp(-2 pi i (sx kx + sy ky)))) /
 * (nx ny) with the reference's frequencies and float phase.  nx in [2, 4096],
 * ny in [2, 2048], both with prime factors 2, 3, 5 and 7 only.  d_in and d_out
 * may not overlap. */
int arecgb_fshift2d_device(const float *d_in, float *d_out, int nz, int ny, int nx,
                           const float *d_sx, const float *d_sy, void *stream);

/* Rotation search over nz image pairs, device memory [nz][ny][nx] (replaces
 * arecRotCCImages, AREC3D/AREC3D/arecImage.cpp:555-598): per pair, radial
 * profiles over n = (int)(2 pi r2) directions (sum over radii 0..r2-1 of the
 * bilinear sample times the radius, getRadialProfile :534-553), their circular
 * cross-correlation (ccorr1d, align2dstack.cpp:437-476), the 7-point
 * polynomial fit around the first maximum (findPeak1d / PRB1D), converted to
 * degrees in (-180, 180]; |angle| > 45 gives 0.  d_angles: nz floats (device).
 * 2 <= r2 <= min(2048, nx/2, ny/2).  Synchronises `stream` before returning. */
int arecgb_rot_cc_images(const float *d_img1, const float *d_img2, int nz, int ny, int nx, int r2,
                         float *d_angles, void *stream);

/* Bilinear rotation of each image by d_angles[i] degrees about (nx/2, ny/2),
 * zero outside (replaces arecRotateImages, AREC3D/AREC3D/arecImage.cpp:674-690,
 * with rotate2d, align2dstack.cpp:774-816).  In place. */
int arecgb_rotate_images(float *d_img, int nz, int ny, int nx, const float *d_angles,
                         void *stream);

/* Rotation by three circular shears (replaces arecRotateImages_skew,
 * AREC3D/AREC3D/arecImage.cpp:692-738): an angle below -180 / above 180 moves
 * by one turn; |angle| > 45 is set to 0 and leaves the image; 10 < |angle| <= 45
 * rotates bilinearly; otherwise shear x by -tan(-a/2), y by sin(-a), x again
 * (shearX_circ / shearY_circ, imagetools.cpp:244-291: integer circular shift
 * plus a linear sub-pixel tap).  Images and d_angles are updated in place. */
int arecgb_rotate_images_skew(float *d_img, int nz, int ny, int nx, float *d_angles,
                              void *stream);

/* Guarded shear rotation (replaces arecRotateImages_skew_safe,
 * AREC3D/AREC3D/arecImage.cpp:740-790): a slice keeps its rotation only when
 * its Tukey-filtered normalised cross-correlation with d_ref[i] rises by more
 * than 1e-5, and its angle is then halved; otherwise the slice is restored and
 * its angle set to 0.  n_rot and mean_cc (host, optional) receive the number of
 * slices rotated and the mean of the kept correlations.  Synchronises. */
int arecgb_rotate_images_skew_safe(float *d_img, const float *d_ref, int nz, int ny, int nx,
                                   float *d_angles, int *n_rot, double *mean_cc, void *stream);

/* Tukey-window (alpha 0.3) normalised cross-correlation of each image pair,
 * FP64 sums (replaces getNormalizedCrossCorrelationWithFilter,
 * AREC3D/AREC3D/imagetools.cpp:415-446).  d_cc: nz doubles (device). */
int arecgb_ncc_filtered(const float *d_a, const float *d_b, int nz, int ny, int nx, double *d_cc,
                        void *stream);

/* ---- Preprocessing of the image stack (AREC3D/AREC3D/AREC3D.cpp:81,105) ----
 * -log(v) for v > 0, else 0, in place over n floats (replaces arecImageTakeLog,
 * AREC3D/AREC3D/arecImage.cpp:358-381). */
int arecgb_take_log(float *d_data, size_t n, void *stream);

/* Periodic-plus-smooth decomposition of each image of a device stack
 * [nz][ny][nx] (replaces periodicDecomposition, AREC3D/AREC3D/imagetools.cpp:
 * 77-114, with makePeriodicSlice :17-75): S solves the periodic Poisson
 * equation for the boundary jumps (DFT, divide by 2cos + 2cos - 4, zero mean),
 * and the image loses exp(-dist^2/50) S, dist = distance to the border.  Any
 * nx in [2, 65536], ny in [2, 65535].  d_smooth != NULL: write S there instead
 * and leave the images.  Synchronises. */
int arecgb_periodic_decomposition(float *d_images, int nz, int ny, int nx, float *d_smooth,
                                  void *stream);

/* Prealign's vertical alignment of projection profiles (replaces the
 * correlation loops of TubeAlign::profile_gc_img, successive = 0, and
 * TubeAlign::profile_cc_img, successive = 1; Prealign/Prealign/TubeAlign.cpp:
 * 128-223, with ccorr1d and findMaxCC_fit, TubeAlign_utils.cpp:220-253,
 * 465-479).  d_profiles: prof_y profiles of prof_x floats (device).  Each
 * profile's segment [pad, prof_x - pad) is correlated with the mean profile's
 * (global) or with the previous profile's (successive); the fitted peaks are
 * damped (global: |s| > 10 -> s pad / s^2) or summed (successive), and their
 * mean removed: shifts (host, prof_y doubles); spread (host, optional) =
 * max - min before the mean removal.  The caller applies sY[j] -= shifts[j].
 * Synchronises. */
int arecgb_profile_shifts(const float *d_profiles, int prof_y, int prof_x, int pad,
                          int successive, double *shifts, double *spread, void *stream);

/* ---- MRC image stacks (the reference's file format, arecImageIO.h:12-63) ----
 * Header of an MRC file: sizes and mode (1, 6: 16-bit, read as signed; 2:
 * float32).  (Replaces arecReadImageHeader, AREC3D/AREC3D/arecImageIO.cpp:10.) */
int arecgb_mrc_read_header(const char *fname, int *nx, int *ny, int *nz, int *mode);

/* Read one rank's part of an MRC stack straight into device memory
 * [nz_loc][ny_loc][nx] as float: by_y = 0 splits the images (replaces
 * arecReadImageDistbyZ, AREC3D/AREC3D/arecImageIO_mpi.cpp:7-124), by_y = 1 the
 * rows of every image (arecReadImageDistbyY, :126-260), the first n % nranks
 * ranks taking one more; rank 0 of 1 reads the whole stack (arecReadImage,
 * arecImageIO.cpp:31-82).  The file streams through two pinned buffers
 * (read and copy overlap); 16-bit data converts on the device.  d_out NULL:
 * only report the sizes.  cap_floats: capacity of d_out.  Synchronises. */
int arecgb_mrc_read_device(const char *fname, int rank, int nranks, int by_y, float *d_out,
                           size_t cap_floats, int *nx, int *ny_loc, int *nz_loc, void *stream);

/* Write a device stack [nz][ny][nx] as a mode-2 MRC file with the header of
 * arecWriteImage (AREC3D/AREC3D/arecImageIO.cpp:84-173; min, max and FP64 mean
 * computed on the device; the header fields the reference leaves unset are
 * zero).  Copy-back and file writes overlap.  Synchronises. */
int arecgb_mrc_write_device(const char *fname, const float *d_in, int nz, int ny, int nx,
                            void *stream);

/* Shift search that allocates nothing (no counterpart in the reference: its
 * arecCCImages allocates per call).  Same arguments, results and layout as
 * arecgb_cc_shifts, for callers that cannot allocate device memory while they
 * run (an alignment loop beside a solve on another stream, where cudaFree
 * would synchronise the device; memory owned by another allocator).
 * Scratch is one static 3.5 MiB device array per device.  Limit: nx, ny powers
 * of two in [16, 512] and nz * ny * nx <= 262144 (one 512 x 512 pair);
 * larger requests return ARECGB_ERR_ARG.  The first call on a device does the
 * set-up (resolves the scratch address, uploads twiddle tables, synchronously)
 * and should come before any stream capture.  The call is asynchronous on
 * `stream`.  All calls on a device share the scratch: calls that can overlap
 * (other streams, unordered host threads) race.  The kernels' shared-memory
 * limits are process-wide; the library only ever raises them, so a concurrent
 * allocating call on smaller images cannot make this launch fail. */
int arecgb_cc_shifts_static(const float *d_img1, const float *d_img2, int nz, int ny, int nx,
                            float *d_sx, float *d_sy, int *d_ix, int *d_iy, void *stream);

/* Full correlation image (replaces ccorr2d, AREC3D/AREC3D/align2dstack.cpp:480):
 * c = IDFT(conj(DFT x) * DFT y), unnormalised, device memory [ny][nx]. */
int arecgb_ccorr2d_device(const float *d_x, const float *d_y, float *d_c, int ny, int nx,
                          void *stream);

/* ---- Learned warm start (no counterpart in the reference) -------------------
 * A BF16 4-level U-Net (32 base channels, FP32 accumulation and master
 * weights) over square images of height x width (multiples of 8), NHWC with
 * one channel: image stacks are [n][height][width] floats, device memory.
 * Parameters are one flat FP32 vector; per layer the weights [Cout][9][Cin]
 * then the biases (arecgb_unet_layer_offsets gives the 18 layers' offsets and
 * channel counts in network order: c1a c1b c2a c2b c3a c3b c4a c4b u3 d3a d3b
 * u2 d2a d2b u1 d1a d1b out).  train != 0 allocates gradients, AdamW moments
 * and backward scratch. */
typedef struct arecgb_unet arecgb_unet;

/* The network's tensor-core building block, exposed for testing:
 * Y[p][co] = act(bias[co] + sum_{tap,ci} X[p+tap][ci] * Wt[co][tap][ci]),
 * 3x3, zero padding, X [n][H][W][Cin] and Y [n][H][W][Cout] bf16 (raw 16-bit),
 * Wt [Cout][9][Cin] bf16, bias FP32 (optional); Cin a multiple of 32, Cout in
 * {32, 64, 128, 256}; relu != 0 applies ReLU; layout must be 0 (1 exchanges
 * the descriptor's two byte offsets, a wrong layout kept to validate them);
 * *d_err (device int) gets bit 4 if a tensor-core wait timed out. */
int arecgb_conv3x3_bf16(const void *d_x, const void *d_wt, const float *d_bias, void *d_y, int n,
                        int height, int width, int cin, int cout, int relu, int layout,
                        int *d_err, void *stream);

int arecgb_unet_create(arecgb_unet **net, int height, int width, int max_batch, int train,
                       unsigned long long seed);
int arecgb_unet_destroy(arecgb_unet *net);
long long arecgb_unet_num_params(const arecgb_unet *net);
/* fills up to 18 entries of each (any may be NULL); returns the layer count */
int arecgb_unet_layer_offsets(const arecgb_unet *net, long long *w_off, long long *b_off,
                              int *cin, int *cout);
int arecgb_unet_get_params(const arecgb_unet *net, float *d_params, void *stream);
int arecgb_unet_set_params(arecgb_unet *net, const float *d_params, void *stream);
/* out = in + net(in); n_images <= max_batch; synchronises the stream */
int arecgb_unet_forward(arecgb_unet *net, const float *d_in, float *d_out, int n_images,
                        void *stream);
/* gradient of a loss with d(loss)/d(out) = d_dout for the last forward's input
 * (which must still be valid); d_grads (optional) receives the flat gradient */
int arecgb_unet_backward(arecgb_unet *net, const float *d_dout, float *d_grads, void *stream);
/* one AdamW step on the mean squared error against d_target; *loss (optional,
 * synchronises) = that mean before the step */
int arecgb_unet_train_step(arecgb_unet *net, const float *d_in, const float *d_target,
                           int n_images, float lr, float weight_decay, double *loss,
                           void *stream);
/* cylinder volume (device layout [nrays][ys]) slices y0..y0+count <-> images
 * [count][npad][npad] (zero outside the disk), values multiplied by scale */
int arecgb_unet_images_from_volume(const arecgb_plan *plan, const float *d_vol, float *d_img,
                                   int npad, int y0, int count, float scale, void *stream);
int arecgb_unet_images_to_volume(const arecgb_plan *plan, const float *d_img, float *d_vol,
                                 int npad, int y0, int count, float scale, void *stream);
/* x0 = s * net(x_early / s) for every slice, s = RMS of x_early over the
 * cylinder; img_in/img_out: scratch of max_batch * height * width floats each;
 * the net's images must be square with height >= the cylinder's width.
 * x0 may equal x_early.  Follow with arecgb_cgls(..., warm = 1, ...). */
int arecgb_warm_start(const arecgb_plan *plan, arecgb_unet *net, const float *d_x_early,
                      float *d_x0, float *d_img_in, float *d_img_out, void *stream);
/* Training loss of a training net: levels = 0 (default) the mean square error
 * over the images; levels > 0 adds, for s = 1..levels, ratio^s times the mean
 * square of the error averaged over 2^s x 2^s blocks (H and W divisible by
 * 2^levels), so low spatial frequencies weigh more. */
int arecgb_unet_set_loss(arecgb_unet *net, int levels, float ratio);
/* Image size and batch of a network (any pointer may be NULL). */
int arecgb_unet_shape(const arecgb_unet *net, int *height, int *width, int *max_batch);

/* Detector bins nx = round(2 radius + 1), rays and slice stride ys of the
 * reference's cylinder of this radius (arecAllocateCylImage,
 * AREC3D/AREC3D/arecImage.cpp:29-86), without creating a plan: the sizes of
 * the device layouts (volume [nrays][ys], sinogram [nangles][nx][ys]). */
int arecgb_cylinder_info(double radius, int ny, int *nx, int *nrays, int *ys);

/* One problem of an uneven batch: weighting, cylinder radius, slices, angles
 * (host, radians) and its device sinogram (read) and volume (written), in the
 * device layouts (arecgb_cylinder_info gives the sizes; padding slices zero). */
typedef struct arecgb_problem {
    int weighting;
    double radius;
    int ny;
    int nangles;
    const float *angles;
    const float *d_b;
    float *d_x;
} arecgb_problem;

/* Many cylinders of uneven radius, width, slices and angles on one GPU (no
 * counterpart in the reference, which solves one cylinder per run over MPI
 * ranks, AREC3D/AREC3D/AREC3D.cpp:293-315).  Inputs and results stay where
 * the caller put them; the solver workspace of all problems may exceed device
 * memory, so the problems are packed into waves whose workspace fits
 * budget_bytes (first fit, largest first; a problem above the budget runs
 * alone).  Per wave: a plan per problem (without the optional projector
 * tables), with n_nets > 0 the learned warm start per problem (the
 * network's input: SIRT of sirt_iters iterations at step sirt_lam_scale /
 * (nangles nx), or with sirt_iters = 0 the filtered back projection
 * (arecgb_fbp); then the smallest of the networks `nets` whose images hold the
 * problem's width: the same parameters at several image sizes), then one
 * batched CGLS of all the
 * wave's problems, one CUDA graph launch per iteration, each to
 * ||A^T r|| / ||A^T b|| <= tol (max maxit iterations).  info[i] (may be NULL)
 * receives problem i's CGLS summary and wave_of[i] (may be NULL) its wave.
 * Synchronises.  With ARECGB_PROGRESS=1 in the environment one line per wave
 * on stderr (problems, workspace, seconds of plans, warm start and CGLS). */
int arecgb_solve_uneven(const arecgb_problem *probs, int n, size_t budget_bytes,
                        arecgb_unet *const *nets, int n_nets, int sirt_iters,
                        double sirt_lam_scale, int maxit, float tol, arecgb_solve_info *info,
                        int *wave_of, void *stream);

/* One reconstruction end to end over HOST buffers in the reference's layouts
 * (the path a caller without device memory of its own takes; no counterpart
 * in the reference, whose cyl_cgls_SQ is the net == NULL case):
 *   b_host [nangles][ny][nx] float (cyl_cgls_SQ's `images.data`), read;
 *   x_host [nrays][ny] float (its `xvol->data`), written.
 * With net != NULL: the network's input (SIRT from zero, sirt_iters
 * iterations of step sirt_lam, or with sirt_iters = 0 the filtered back
 * projection, arecgb_fbp), the network's warm start, then CGLS to
 * ||A^T r|| / ||A^T b|| <= tol with the denominator ||A^T b|| of the cold
 * start (at most maxit iterations); with net == NULL: CGLS from zero.  The copies are cudaMemcpyAsync on `stream`
 * (full speed from page-locked memory).  Device buffers belong to the plan,
 * allocated on first use and kept; the call returns after x_host is written.
 * info (may be NULL) receives the CGLS summary.  With ARECGB_PROGRESS=1 in
 * the environment the call prints its phases' seconds on stderr (upload,
 * layout change, first reconstruction, network, CGLS, download; each phase
 * then synchronises). */
int arecgb_reconstruct_host(arecgb_plan *plan, const float *b_host, float *x_host,
                            arecgb_unet *net, int sirt_iters, float sirt_lam, int maxit,
                            float tol, arecgb_solve_info *info, void *stream);

#ifdef __cplusplus
}
#endif
