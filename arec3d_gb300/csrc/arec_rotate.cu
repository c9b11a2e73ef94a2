// Rotational alignment of image stacks: the in-plane rotation search and the
// rotations of the projection-matching loop (reference AREC3D/AREC3D):
//
//   rot_cc_angles     arecRotCCImages        arecImage.cpp:555-598
//                       getRadialProfile     arecImage.cpp:534-553 (+ blerp :515-532)
//                       ccorr1d              align2dstack.cpp:437-476
//                       findPeak1d, PRB1D    arecImage.cpp:486-513, align2dstack.cpp:1028-1056
//   rotate_stack      arecRotateImages       arecImage.cpp:674-690 (rotate2d align2dstack.cpp:774-816)
//                     arecRotateImages_skew  arecImage.cpp:692-738
//                     arecRotateImages_skew_safe  arecImage.cpp:740-790
//                       shearX_circ, shearY_circ   imagetools.cpp:171-291
//   ncc_filtered      getNormalizedCrossCorrelationWithFilter  imagetools.cpp:331-366, 415-446
//   profile_shifts    Prealign TubeAlign::profile_gc_img / profile_cc_img
//                       (Prealign/Prealign/TubeAlign.cpp:128-223) with ccorr1d and
//                       findMaxCC_fit (TubeAlign_utils.cpp:220-253, 465-479)
//
// Images are the reference layout [nz][ny][nx] in device memory.  The
// reference's mixed float / double expressions are kept operation for
// operation: float steps use __f*_rn and double steps __d*_rn, so nothing is
// contracted into an FMA that the reference (built without contraction) does
// not form.  Per-angle trigonometry of the radial profile and the Tukey window
// are tables computed on the host with the C library in double, as the
// reference computes them; the per-slice rotation trigonometry runs on the
// device in double (float results: the double value rounded to float).
#include <math.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "arec_internal.cuh"

namespace arecgb {

namespace {

constexpr double kPi = 3.14159265358979323846;  // atan(1) * 4 in double

// ---------------------------------------------------------------------------
// Radial profiles: prof[m][z][i] = sum_{ri < R} blerp(image_m[z], xc + cos(a_i) ri,
// yc + sin(a_i) ri) * ri, accumulated in float in ri order.

__device__ __forceinline__ float blerp_raw(const float *im, int nx, int ny, float x, float y) {
    int xb = (int)x, yb = (int)y;
    double xf = (double)__fsub_rn(x, (float)xb);
    double yf = (double)__fsub_rn(y, (float)yb);
    if (xf < 0.0) xf = 0.0;
    if (yf < 0.0) yf = 0.0;
    // arguments are validated so that 0 <= xb <= nx-2, 0 <= yb <= ny-2; the
    // clamps only keep a stray rounding in bounds
    xb = min(max(xb, 0), nx - 2);
    yb = min(max(yb, 0), ny - 2);
    const float *p = im + (size_t)yb * nx + xb;
    const double ll = p[0], lr = p[1], ul = p[nx], ur = p[nx + 1];
    const double up = __dadd_rn(ul, __dmul_rn(xf, __dsub_rn(ur, ul)));
    const double lo = __dadd_rn(ll, __dmul_rn(xf, __dsub_rn(lr, ll)));
    return (float)__dadd_rn(lo, __dmul_rn(yf, __dsub_rn(up, lo)));
}

__global__ void k_radial_profile(const float *__restrict__ img1, const float *__restrict__ img2,
                                 int nx, int ny, int nz, int n, int R,
                                 const double *__restrict__ cs, float *__restrict__ prof) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y, m = blockIdx.z;
    if (i >= n) return;
    const float *im = (m == 0 ? img1 : img2) + (size_t)z * nx * ny;
    const double c = cs[i], s = cs[n + i];
    const double xc = 0.5 * (nx - 1), yc = 0.5 * (ny - 1);
    float acc = 0.0f;
    for (int ri = 0; ri < R; ri++) {
        const float x = (float)__dadd_rn(xc, __dmul_rn(c, (double)ri));
        const float y = (float)__dadd_rn(yc, __dmul_rn(s, (double)ri));
        acc = __fadd_rn(acc, __fmul_rn(blerp_raw(im, nx, ny, x, y), (float)ri));
    }
    prof[((size_t)m * nz + z) * n + i] = acc;
}

// ---------------------------------------------------------------------------
// Circular cross-correlation of the two profiles of a slice, its peak and the
// 7-point polynomial fit, converted to degrees.  One block per slice.
//   c[k] = sum_i x[i] y[(i + k) mod n]   (ccorr1d's IDFT(conj(X) Y) without the
//   factor n, which neither the arg max nor the fit depends on); FP32 products
//   summed in chunks of 64, chunks accumulated in FP64.

constexpr int kPeakThreads = 512;

// Whole block: c[k] = sum_i x[i] y[(i + k) mod n] for the n values at x and y
// (global memory), through shared memory sh (4n floats); then the first arg
// max of c and the 7-point parabola vertex around it (PRB1D, NPOINT = 7,
// relative to the centre; 0 when the fit is flat).  Thread 0 receives maxind
// and pos.
__device__ void block_ccorr_fit(const float *__restrict__ xg, const float *__restrict__ yg, int n,
                                float *sh, int &maxind, double &pos) {
    __shared__ float bv[kPeakThreads / 32];
    __shared__ int bi[kPeakThreads / 32];
    float *x = sh, *y = sh + n, *c = sh + 3 * n;  // y holds two periods
    const int t = threadIdx.x;
    for (int i = t; i < n; i += blockDim.x) {
        x[i] = xg[i];
        const float v = yg[i];
        y[i] = v;
        y[i + n] = v;
    }
    __syncthreads();
    for (int k = t; k < n; k += blockDim.x) {
        double acc = 0.0;
        for (int i0 = 0; i0 < n; i0 += 64) {
            const int i1 = min(n, i0 + 64);
            float part = 0.0f;
            for (int i = i0; i < i1; i++) part = fmaf(x[i], y[i + k], part);
            acc += (double)part;
        }
        c[k] = (float)acc;
    }
    __syncthreads();
    // arg max, first index on ties (findMaxIndex: strict >)
    float best = -INFINITY;
    int bidx = INT_MAX;
    for (int k = t; k < n; k += blockDim.x) {
        const float v = c[k];
        if (v > best || (v == best && k < bidx)) {
            best = v;
            bidx = k;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
            best = ov;
            bidx = oi;
        }
    }
    if ((t & 31) == 0) {
        bv[t >> 5] = best;
        bi[t >> 5] = bidx;
    }
    __syncthreads();
    if (t == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (bv[w] > best || (bv[w] == best && bi[w] < bidx)) {
                best = bv[w];
                bidx = bi[w];
            }
        // a profile of NaNs leaves no maximum: the reference's scan keeps index 0
        maxind = bidx == INT_MAX ? 0 : bidx;
        double B[7];
        for (int k = -3; k <= 3; k++) B[k + 3] = c[((maxind + k) % n + n) % n];
        // least-squares parabola through 7 points (PRB1D, NPOINT = 7)
        double c2 = __dmul_rn(49.0, B[0]);
        c2 = __dadd_rn(c2, __dmul_rn(6.0, B[1]));
        c2 = __dsub_rn(c2, __dmul_rn(21.0, B[2]));
        c2 = __dsub_rn(c2, __dmul_rn(32.0, B[3]));
        c2 = __dsub_rn(c2, __dmul_rn(27.0, B[4]));
        c2 = __dsub_rn(c2, __dmul_rn(6.0, B[5]));
        c2 = __dadd_rn(c2, __dmul_rn(31.0, B[6]));
        double c3 = __dmul_rn(5.0, B[0]);
        c3 = __dsub_rn(c3, __dmul_rn(3.0, B[2]));
        c3 = __dsub_rn(c3, __dmul_rn(4.0, B[3]));
        c3 = __dsub_rn(c3, __dmul_rn(3.0, B[4]));
        c3 = __dadd_rn(c3, __dmul_rn(5.0, B[6]));
        pos = 0.0;
        if (c3 != 0.0) pos = __dsub_rn(__ddiv_rn(c2, __dmul_rn(2.0, c3)), 4.0);
    }
}

__global__ void __launch_bounds__(kPeakThreads)
    k_rot_peak(const float *__restrict__ prof, int nz, int n, float *__restrict__ angles) {
    extern __shared__ float sh[];
    const int z = blockIdx.x;
    int maxind = 0;
    double pos = 0.0;
    block_ccorr_fit(prof + (size_t)z * n, prof + ((size_t)nz + z) * n, n, sh, maxind, pos);
    if (threadIdx.x == 0) {
        float a = (float)__dadd_rn(pos, (double)maxind);  // findPeak1d
        a = (float)__dmul_rn((double)a, 2.0 * kPi / n);  // index to radians
        if ((double)a > kPi) a = (float)__dsub_rn((double)a, 2.0 * kPi);
        a = (float)__dmul_rn((double)a, 180.0 / kPi);  // to degrees
        if (fabsf(a) > 45.0f) a = 0.0f;                 // "probably bad CC, do nothing"
        angles[z] = a;
    }
}

// ---------------------------------------------------------------------------
// Prealign's vertical profile alignment (TubeAlign.cpp:128-223): per profile j
// the correlation of its segment [pad, pad + L) with the mean profile
// (ref != NULL) or with profile j - 1 (ref == NULL, j >= 1), and
// findMaxCC_fit (TubeAlign_utils.cpp:465-479): the fitted peak, wrapped to
// (-L, L/2].

// mean profile in the reference's order: m[i] += p[j][i] / prof_y (float)
__global__ void k_mean_profile(const float *__restrict__ prof, int prof_y, int prof_x,
                               float *__restrict__ m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= prof_x) return;
    float s = 0.0f;
    for (int j = 0; j < prof_y; j++)
        s = __fadd_rn(s, __fdiv_rn(prof[(size_t)j * prof_x + i], (float)prof_y));
    m[i] = s;
}

__global__ void __launch_bounds__(kPeakThreads)
    k_profile_peak(const float *__restrict__ prof, int prof_x, int pad, int L,
                   const float *__restrict__ ref, double *__restrict__ out) {
    extern __shared__ float sh[];
    const int j = blockIdx.x;
    if (!ref && j == 0) {
        if (threadIdx.x == 0) out[0] = 0.0;
        return;
    }
    const float *x = prof + (size_t)j * prof_x + pad;
    const float *y = ref ? ref + pad : prof + (size_t)(j - 1) * prof_x + pad;
    int maxind = 0;
    double pos = 0.0;
    block_ccorr_fit(x, y, L, sh, maxind, pos);
    if (threadIdx.x == 0) {
        double r = 1.0 * (maxind + pos);
        if (r > L / 2) r -= L;
        out[j] = r;
    }
}

// ---------------------------------------------------------------------------
// Rotations.  Per slice: a mode and the three shears / the bilinear rotation's
// cosine and sine, from the slice's angle in degrees.

enum RotKind { kRotBilinear = 0, kRotSkew = 1, kRotSafe = 2 };
enum RotMode { kModeNone = 0, kModeShear = 1, kModeBilinear = 2 };

struct RotParam {
    float shx, shy;  // shearX: -tan(-a/2), shearY: sin(-a)
    double cod, sid; // rotate2d
    int mode;
};

__device__ __forceinline__ float rad_of_deg(float a) {
    return (float)__ddiv_rn(__dmul_rn((double)a, kPi), 180.0);
}

__global__ void k_rot_params(float *angles, int nz, int kind, RotParam *par) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= nz) return;
    float a = angles[z];
    RotParam p;
    p.shx = p.shy = 0.0f;
    p.cod = 1.0;
    p.sid = 0.0;
    p.mode = kModeNone;
    int mode = kModeShear;
    if (kind == kRotBilinear) {
        mode = kModeBilinear;
    } else if (kind == kRotSkew) {
        // one period fix each way, then the size rules (arecImage.cpp:711-738)
        if (a < -180.0f) a = (float)((double)a + 360.0);
        if (a > 180.0f) a = (float)((double)a - 360.0);
        if (fabsf(a) > 45.0f) {
            a = 0.0f;
            mode = kModeNone;
        } else if (fabsf(a) > 10.0f) {
            mode = kModeBilinear;
        }
        angles[z] = a;
    }
    if (mode == kModeShear) {
        const float r = rad_of_deg(a);
        p.shx = (float)(-tan(__dmul_rn(-0.5, (double)r)));
        p.shy = (float)sin((double)(-r));
    } else if (mode == kModeBilinear) {
        float th = rad_of_deg(a);
        if ((double)th > kPi) th = (float)__dadd_rn(-2.0 * kPi, (double)th);
        if ((double)th < -kPi) th = (float)__dadd_rn(2.0 * kPi, (double)th);
        p.cod = (double)(float)cos((double)th);
        p.sid = (double)(float)sin((double)th);
    }
    p.mode = mode;
    par[z] = p;
}

// Circular shear with linear sub-pixel weights along x (rows), or along y
// (columns): the row (column) is circularly shifted by floor(skew), then
// out[i] = (p[i] - p[i] f) + p[i-1] f with f = skew - floor(skew) and p[-1] =
// p[n-1] (shearX_circ / shearY_circ).  skew = shear * (j - centre) for row
// (column) j.
__device__ __forceinline__ float shear_tap(float a, float b, float f) {
    return __fadd_rn(__fsub_rn(a, __fmul_rn(a, f)), __fmul_rn(b, f));
}

__device__ __forceinline__ void shear_split(float shear, int j, int n_other, int &si, float &f) {
    const double centre = 0.5 * (n_other - 1);
    const float skew = (float)__dmul_rn((double)shear, (double)j - centre);
    si = (int)floorf(skew);
    f = (float)__dsub_rn((double)skew, (double)si);
}

// rotate2d (bilinear, zero outside), output pixel (row i, column k), 0-based.
__device__ __forceinline__ float rotate2d_pixel(const float *im, int nx, int ny, int i, int k,
                                                double cod, double sid) {
    const int kcent = nx / 2 + 1, icent = ny / 2 + 1;
    const double Y = (double)(i + 1 - icent);
    const double ycod = __dadd_rn(__dmul_rn(Y, cod), (double)icent);
    const double ysid = __dadd_rn(__dmul_rn(-Y, sid), (double)kcent);
    const double X = (double)(k + 1 - kcent);
    const double xold = __dadd_rn(__dmul_rn(X, cod), ysid);
    const double yold = __dadd_rn(__dmul_rn(X, sid), ycod);
    const int iy = (int)yold, ix = (int)xold;
    if (iy >= 1 && iy <= ny - 1 && ix >= 1 && ix <= nx - 1) {
        const double ydif = __dsub_rn(yold, (double)iy), yrem = __dsub_rn(1.0, ydif);
        const double xdif = __dsub_rn(xold, (double)ix), xrem = __dsub_rn(1.0, xdif);
        const float *p = im + (size_t)(iy - 1) * nx + (ix - 1);
        const double top = __dadd_rn(__dmul_rn((double)p[nx], xrem), __dmul_rn((double)p[nx + 1], xdif));
        const double bot = __dadd_rn(__dmul_rn((double)p[0], xrem), __dmul_rn((double)p[1], xdif));
        return (float)__dadd_rn(__dmul_rn(ydif, top), __dmul_rn(yrem, bot));
    }
    return 0.0f;
}

// One pass of the three-pass rotation over a batch of slices z0 .. z0+nb-1.
//   pass 0: shear slices: shearX; bilinear slices: rotate2d; others: copy
//   pass 1: shear slices: shearY; others: copy
//   pass 2: shear slices: shearX; others: copy
__global__ void k_rot_pass(const float *__restrict__ in, float *__restrict__ out, int nx, int ny,
                           const RotParam *__restrict__ par, int z0, int pass) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, zb = blockIdx.z;
    if (x >= nx) return;
    const RotParam p = par[z0 + zb];
    const float *im = in + (size_t)zb * nx * ny;
    float v;
    if (p.mode == kModeShear && pass != 1) {
        int si;
        float f;
        shear_split(p.shx, y, ny, si, f);
        int xa = (x - si) % nx;
        if (xa < 0) xa += nx;
        const int xb = xa == 0 ? nx - 1 : xa - 1;
        const float *row = im + (size_t)y * nx;
        v = shear_tap(row[xa], row[xb], f);
    } else if (p.mode == kModeShear) {
        int si;
        float f;
        shear_split(p.shy, x, nx, si, f);
        int ya = (y - si) % ny;
        if (ya < 0) ya += ny;
        const int yb = ya == 0 ? ny - 1 : ya - 1;
        v = shear_tap(im[(size_t)ya * nx + x], im[(size_t)yb * nx + x], f);
    } else if (p.mode == kModeBilinear && pass == 0) {
        v = rotate2d_pixel(im, nx, ny, y, x, p.cod, p.sid);
    } else {
        v = im[(size_t)y * nx + x];
    }
    out[((size_t)zb * ny + y) * nx + x] = v;
}

// ---------------------------------------------------------------------------
// Tukey-filtered normalised cross-correlation, one block per (slice, pair).
// filter = float(hx * hy) (tukey_filter of ones, alpha 0.3); with a = im1 * f
// and b = im2 * f in float, means over nx*ny in double, then
// cov / sqrt(var1 var2) in double.  Pair p of slice z correlates A_p[z] with B.

constexpr int kNccThreads = 1024;

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

__global__ void __launch_bounds__(kNccThreads)
    k_ncc(const float *__restrict__ a0, const float *__restrict__ a1, const float *__restrict__ b,
          int nx, int ny, const double *__restrict__ hx, const double *__restrict__ hy,
          double *__restrict__ cc, int nz_cc) {
    __shared__ double red[33];
    const int z = blockIdx.x, pr = blockIdx.y;
    const size_t np = (size_t)nx * ny, off = (size_t)z * np;
    const float *A = (pr == 0 ? a0 : a1) + off, *Bp = b + off;
    double s1 = 0.0, s2 = 0.0;
    for (size_t i = threadIdx.x; i < np; i += blockDim.x) {
        const int yy = (int)(i / nx), xx = (int)(i - (size_t)yy * nx);
        const float f = (float)__dmul_rn(hx[xx], hy[yy]);
        s1 += (double)__fmul_rn(A[i], f);
        s2 += (double)__fmul_rn(Bp[i], f);
    }
    const double m1 = block_sum(s1, red) / ((double)nx * ny);
    const double m2 = block_sum(s2, red) / ((double)nx * ny);
    double cv = 0.0, v1 = 0.0, v2 = 0.0;
    for (size_t i = threadIdx.x; i < np; i += blockDim.x) {
        const int yy = (int)(i / nx), xx = (int)(i - (size_t)yy * nx);
        const float f = (float)__dmul_rn(hx[xx], hy[yy]);
        const double d1 = __dsub_rn((double)__fmul_rn(A[i], f), m1);
        const double d2 = __dsub_rn((double)__fmul_rn(Bp[i], f), m2);
        cv = __dadd_rn(cv, __dmul_rn(d1, d2));
        v1 = __dadd_rn(v1, __dmul_rn(d1, d1));
        v2 = __dadd_rn(v2, __dmul_rn(d2, d2));
    }
    cv = block_sum(cv, red);
    v1 = block_sum(v1, red);
    v2 = block_sum(v2, red);
    if (threadIdx.x == 0) cc[(size_t)pr * nz_cc + z] = cv / sqrt(__dmul_rn(v1, v2));
}

// skew_safe decision per slice: keep the rotation when cc(rotated) exceeds
// cc(original) + 1e-5, then halve the angle; else keep the original and set
// the angle to 0.  keep[z] records the choice.
__global__ void k_safe_decide(const double *cc, int nb, int z0, float *angles, int *keep,
                              double *ccsel) {
    const int zb = blockIdx.x * blockDim.x + threadIdx.x;
    if (zb >= nb) return;
    const double c1 = cc[zb], c2 = cc[nb + zb];
    const int k = __dadd_rn(c2, 0.00001) < c1;
    const int z = z0 + zb;
    angles[z] = k ? angles[z] * 0.5f : 0.0f;
    keep[z] = k;
    ccsel[z] = k ? c1 : c2;
}

__global__ void k_safe_apply(const float *__restrict__ rot, float *__restrict__ img, int nx, int ny,
                             const int *__restrict__ keep, int z0) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, zb = blockIdx.z;
    if (x >= nx || !keep[z0 + zb]) return;
    const size_t i = ((size_t)zb * ny + y) * nx + x;
    img[i] = rot[i];
}

// mean CC (sum in slice order, as the reference's loop) and slices rotated
__global__ void k_safe_summary(const double *ccsel, const int *keep, int nz, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    int n = 0;
    for (int z = 0; z < nz; z++) {
        s += ccsel[z];
        n += keep[z];
    }
    out[0] = s / nz;
    out[1] = (double)n;
}

void tukey_table(int n, double alpha, std::vector<double> &h) {
    // tukey_filter (imagetools.cpp:331-366) along one axis
    h.resize(n);
    const double a = 0.5 * alpha * (n - 1), b = (1.0 - 0.5 * alpha) * (n - 1);
    const double A = 2.0 * (std::atan(1.0) * 4) / alpha;
    for (int i = 0; i < n; i++) {
        const double va = 0.5 * (1.0 + std::cos(A * (1.0 * i / (n - 1) - alpha / 2)));
        const double vb = 0.5 * (1.0 + std::cos(A * (1.0 * i / (n - 1) - 1.0 + alpha / 2)));
        h[i] = i < a ? va : (i > b ? vb : 1.0);
    }
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

int check_stack(const char *who, int nz, int ny, int nx) {
    if (nz < 0 || nx < 4 || ny < 4 || nx > 65536 || ny > 65535) {
        set_error(std::string(who) + ": image sizes must be 4 <= nx <= 65536, 4 <= ny <= 65535");
        return ARECGB_ERR_ARG;
    }
    return 0;
}

}  // namespace

int ncc_filtered(const float *d_a, const float *d_a2, const float *d_b, int nz, int ny, int nx,
                 double *d_cc, int npairs, cudaStream_t st);

int rot_cc_angles(const float *d1, const float *d2, int nz, int ny, int nx, int r2, float *d_angles,
                  cudaStream_t st) {
    if (int rc = check_stack("rot_cc_images", nz, ny, nx)) return rc;
    if (r2 < 2 || r2 > 2048 || r2 > std::min(nx, ny) / 2) {
        set_error("rot_cc_images: r2 must be in [2, min(2048, nx/2, ny/2)]");
        return ARECGB_ERR_ARG;
    }
    if (nz == 0) return 0;
    const int n = (int)(r2 * 2 * (std::atan(1.0) * 4));  // angular samples
    std::vector<double> cs(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        const double alpha = 2 * (std::atan(1.0) * 4) * i / n;
        cs[i] = std::cos(alpha);
        cs[n + i] = std::sin(alpha);
    }
    const size_t prof_bytes = ((sizeof(float) * 2 * (size_t)nz * n + 255) / 256) * 256;
    DevBuf buf;
    ARECGB_CUDA(cudaMalloc(&buf.p, prof_bytes + sizeof(double) * cs.size()));
    float *prof = (float *)buf.p;                              // [2][nz][n]
    double *d_cs = (double *)((char *)buf.p + prof_bytes);     // cos, sin tables
    ARECGB_CUDA(cudaMemcpyAsync(d_cs, cs.data(), sizeof(double) * cs.size(), cudaMemcpyHostToDevice, st));
    for (int z0 = 0; z0 < nz; z0 += 65535) {
        const int nb = std::min(65535, nz - z0);
        // slices z0.. of both images: profiles written at their own slice rows
        dim3 grid((n + 127) / 128, nb, 2);
        k_radial_profile<<<grid, 128, 0, st>>>(d1 + (size_t)z0 * nx * ny, d2 + (size_t)z0 * nx * ny,
                                               nx, ny, nz, n, r2, d_cs, prof + (size_t)z0 * n);
        count_launches(1);
    }
    ARECGB_CUDA(cudaGetLastError());
    const size_t smem = sizeof(float) * 4 * (size_t)n;
    ARECGB_CUDA(cudaFuncSetAttribute(k_rot_peak, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_rot_peak<<<nz, kPeakThreads, smem, st>>>(prof, nz, n, d_angles);
    count_launches(1);
    ARECGB_CUDA(cudaGetLastError());
    // the scratch is freed after the work that reads it
    ARECGB_CUDA(cudaStreamSynchronize(st));
    return 0;
}

// TubeAlign::profile_gc_img (successive = 0) / profile_cc_img (successive = 1)
// (Prealign/Prealign/TubeAlign.cpp:128-223): the per-profile shifts after the
// reference's damping (global: |s| > 10 -> s * pad / s^2) or integration
// (successive: running sum), with their mean removed, into shifts (host,
// prof_y values); spread = |max - min| before the mean removal.  The caller
// applies sY[j] -= shifts[j] as the reference does.
int profile_shifts(const float *d_prof, int prof_y, int prof_x, int pad, int successive,
                   double *shifts, double *spread, cudaStream_t st) {
    const int L = prof_x - 2 * pad;
    if (prof_y < 1 || pad < 0 || L < 1 || L > 14000) {
        set_error("profile_shifts: need prof_y >= 1, pad >= 0, 1 <= prof_x - 2 pad <= 14000");
        return ARECGB_ERR_ARG;
    }
    DevBuf buf;
    ARECGB_CUDA(cudaMalloc(&buf.p, sizeof(double) * prof_y + sizeof(float) * prof_x));
    double *d_out = (double *)buf.p;
    float *d_mean = (float *)(d_out + prof_y);
    if (!successive) {
        k_mean_profile<<<(prof_x + 127) / 128, 128, 0, st>>>(d_prof, prof_y, prof_x, d_mean);
        count_launches(1);
    }
    const size_t smem = sizeof(float) * 4 * (size_t)L;
    ARECGB_CUDA(cudaFuncSetAttribute(k_profile_peak, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    k_profile_peak<<<prof_y, kPeakThreads, smem, st>>>(d_prof, prof_x, pad, L,
                                                      successive ? nullptr : d_mean, d_out);
    count_launches(1);
    ARECGB_CUDA(cudaGetLastError());
    std::vector<double> s(prof_y);
    ARECGB_CUDA(cudaMemcpyAsync(s.data(), d_out, sizeof(double) * prof_y, cudaMemcpyDeviceToHost,
                                st));
    ARECGB_CUDA(cudaStreamSynchronize(st));
    if (!successive) {
        for (int j = 0; j < prof_y; j++) {
            const double shift = std::fabs(s[j]);
            if (shift > 10.0) {
                s[j] *= pad;
                s[j] /= shift * shift;
            }
        }
    } else {
        for (int j = 1; j < prof_y; j++) s[j] += s[j - 1];
    }
    double mn = s[0], mx = s[0], mean = 0.0;
    for (int j = 0; j < prof_y; j++) {
        if (s[j] < mn) mn = s[j];
        if (s[j] > mx) mx = s[j];
        mean += s[j];
    }
    mean /= prof_y;
    for (int j = 0; j < prof_y; j++) shifts[j] = s[j] - mean;
    if (spread) *spread = std::fabs(mx - mn);
    return 0;
}

int ncc_filtered(const float *d_a, const float *d_a2, const float *d_b, int nz, int ny, int nx,
                 double *d_cc, int npairs, cudaStream_t st) {
    if (int rc = check_stack("ncc_filtered", nz, ny, nx)) return rc;
    if (nz == 0) return 0;
    std::vector<double> h;
    std::vector<double> tab;
    tukey_table(nx, 0.3, h);
    tab = h;
    tukey_table(ny, 0.3, h);
    tab.insert(tab.end(), h.begin(), h.end());
    DevBuf buf;
    ARECGB_CUDA(cudaMalloc(&buf.p, sizeof(double) * tab.size()));
    double *d_h = (double *)buf.p;
    ARECGB_CUDA(cudaMemcpyAsync(d_h, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st));
    for (int z0 = 0; z0 < nz; z0 += 65535) {
        const int nb = std::min(65535, nz - z0);
        const size_t o = (size_t)z0 * nx * ny;
        // results of pair p, slice z at d_cc[p * nz + z]
        k_ncc<<<dim3(nb, npairs), kNccThreads, 0, st>>>(d_a + o, d_a2 ? d_a2 + o : d_a + o, d_b + o,
                                                        nx, ny, d_h, d_h + nx, d_cc + z0, nz);
        count_launches(1);
    }
    ARECGB_CUDA(cudaGetLastError());
    ARECGB_CUDA(cudaStreamSynchronize(st));
    return 0;
}

// kind: 0 bilinear (arecRotateImages), 1 skew (arecRotateImages_skew),
// 2 skew_safe (arecRotateImages_skew_safe, needs d_ref; summary -> host).
int rotate_stack(float *d_img, const float *d_ref, int nz, int ny, int nx, float *d_angles,
                 int kind, int *n_rot, double *mean_cc, cudaStream_t st) {
    if (int rc = check_stack("rotate_images", nz, ny, nx)) return rc;
    if (kind < kRotBilinear || kind > kRotSafe || (kind == kRotSafe && !d_ref)) {
        set_error("rotate_images: bad kind or missing reference stack");
        return ARECGB_ERR_ARG;
    }
    if (nz == 0) {
        if (n_rot) *n_rot = 0;
        if (mean_cc) *mean_cc = 0.0;
        return 0;
    }
    const size_t slice = (size_t)nx * ny;
    // two slice buffers per batch, about 1 GiB together
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(
                                                   std::min<size_t>((size_t)nz, 65535),
                                                   (size_t(1) << 29) / (sizeof(float) * slice)));
    std::vector<double> tab;
    if (kind == kRotSafe) {
        std::vector<double> h;
        tukey_table(nx, 0.3, h);
        tab = h;
        tukey_table(ny, 0.3, h);
        tab.insert(tab.end(), h.begin(), h.end());
    }
    const size_t bytes_t = sizeof(float) * 2 * slice * batch;
    const size_t bytes_p = ((sizeof(RotParam) * nz + 255) / 256) * 256;
    const size_t bytes_s = kind == kRotSafe ? sizeof(double) * (2 * (size_t)batch + nz + 2) +
                                                  sizeof(double) * tab.size() + sizeof(int) * nz
                                            : 0;
    DevBuf buf;
    ARECGB_CUDA(cudaMalloc(&buf.p, bytes_t + bytes_p + bytes_s));
    float *t1 = (float *)buf.p, *t2 = t1 + slice * batch;
    RotParam *par = (RotParam *)((char *)buf.p + bytes_t);
    double *cc = (double *)((char *)buf.p + bytes_t + bytes_p);
    double *ccsel = cc + 2 * (size_t)batch, *summary = ccsel + nz, *d_h = summary + 2;
    int *keep = (int *)(d_h + tab.size());
    if (kind == kRotSafe)
        ARECGB_CUDA(cudaMemcpyAsync(d_h, tab.data(), sizeof(double) * tab.size(),
                                    cudaMemcpyHostToDevice, st));
    k_rot_params<<<(nz + 127) / 128, 128, 0, st>>>(d_angles, nz, kind, par);
    count_launches(1);
    for (int z0 = 0; z0 < nz; z0 += batch) {
        const int nb = std::min(batch, nz - z0);
        float *img = d_img + (size_t)z0 * slice;
        dim3 grid((nx + 127) / 128, ny, nb);
        k_rot_pass<<<grid, 128, 0, st>>>(img, t1, nx, ny, par, z0, 0);
        k_rot_pass<<<grid, 128, 0, st>>>(t1, t2, nx, ny, par, z0, 1);
        if (kind != kRotSafe) {
            k_rot_pass<<<grid, 128, 0, st>>>(t2, img, nx, ny, par, z0, 2);
            count_launches(3);
        } else {
            k_rot_pass<<<grid, 128, 0, st>>>(t2, t1, nx, ny, par, z0, 2);
            // cc[0..nb): rotated vs reference, cc[nb..2nb): original vs reference
            k_ncc<<<dim3(nb, 2), kNccThreads, 0, st>>>(t1, img, d_ref + (size_t)z0 * slice, nx, ny,
                                                       d_h, d_h + nx, cc, nb);
            k_safe_decide<<<(nb + 127) / 128, 128, 0, st>>>(cc, nb, z0, d_angles, keep, ccsel);
            k_safe_apply<<<grid, 128, 0, st>>>(t1, img, nx, ny, keep, z0);
            count_launches(6);
        }
        ARECGB_CUDA(cudaGetLastError());
    }
    double h_sum[2] = {0.0, 0.0};
    if (kind == kRotSafe) {
        k_safe_summary<<<1, 32, 0, st>>>(ccsel, keep, nz, summary);
        count_launches(1);
        ARECGB_CUDA(cudaGetLastError());
        ARECGB_CUDA(cudaMemcpyAsync(h_sum, summary, sizeof(h_sum), cudaMemcpyDeviceToHost, st));
    }
    // the scratch is freed after the work that reads it
    ARECGB_CUDA(cudaStreamSynchronize(st));
    if (mean_cc) *mean_cc = h_sum[0];
    if (n_rot) *n_rot = (int)h_sum[1];
    return 0;
}

}  // namespace arecgb
