// FFT cross-correlation shift search (reference arecCCImages,
// AREC3D/AREC3D/arecImage.cpp:384-434 = ccorr2d + speak per image pair,
// AREC3D/AREC3D/align2dstack.cpp:480-521, 1059-1166).
//
//   c = IDFT2( conj(DFT2 x) * DFT2 y )   (unnormalised, [ny][nx], real)
//   peak = speak(c): |c| argmax with the reference's scan-order rules,
//          3x3 paraboloid fit, wrap to (-n/2, n/2].
//
// Pipeline per batch of image pairs (all FP32, sizes 2..4096 whose prime
// factors are 2, 3, 5 and 7):
//   1. rows:    z = x + i*y, complex FFT of each row (one transform gives the
//               row spectra of both real images), split into the half spectra
//               Xh, Yh [ny][nx/2+1] (Hermitian symmetry).
//   2. columns: column FFTs of Xh and Yh, C = conj(X)*Y, inverse column FFT,
//               written back over Xh (each block owns its columns).
//   3. rows:    Hermitian row -> inverse complex FFT -> c (real part), with
//               per-row peak statistics fused.
//   4. peak:    one block per pair reduces the row statistics exactly in the
//               reference's x-major scan order and fits the paraboloid in FP64.
// FFTs run in shared memory: Stockham passes, twiddles from a per-length table
// computed in double on the host.  Powers of two: radix 16 and one radix-2/4/8
// pass, one radix-16 butterfly per thread per pass held in registers; other
// lengths: radix 16/8/4/2 and then 7/5/3 passes, each thread holding up to 16
// elements' butterflies.
#include <math.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "arec_internal.cuh"

namespace arecgb {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-register radix-R DFT (forward sign) of v[off .. off+R), iterative DIT.
template <int R>
__device__ __forceinline__ void dft_reg(float2 *v) {
    constexpr int LOG = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
    // cos/sin(2*pi*m/16), m = 0..7
    const float C16[8] = {1.0f, 0.92387953251128676f, 0.70710678118654752f,
                          0.38268343236508977f, 0.0f, -0.38268343236508977f,
                          -0.70710678118654752f, -0.92387953251128676f};
    const float S16[8] = {0.0f, 0.38268343236508977f, 0.70710678118654752f,
                          0.92387953251128676f, 1.0f, 0.92387953251128676f,
                          0.70710678118654752f, 0.38268343236508977f};
#pragma unroll
    for (int i = 0; i < R; i++) {
        int j = 0;
#pragma unroll
        for (int bbit = 0; bbit < LOG; bbit++) j |= ((i >> bbit) & 1) << (LOG - 1 - bbit);
        if (i < j) {
            float2 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
#pragma unroll
    for (int len = 2; len <= R; len <<= 1) {
        const int half = len >> 1;
#pragma unroll
        for (int s = 0; s < R; s += len) {
#pragma unroll
            for (int k = 0; k < half; k++) {
                const int m = k * (16 / len);
                const float c = C16[m], sn = S16[m];
                const float2 a = v[s + k], b = v[s + k + half];
                // b * exp(-2*pi*i*k/len)
                const float2 bw = make_float2(b.x * c + b.y * sn, b.y * c - b.x * sn);
                v[s + k] = make_float2(a.x + bw.x, a.y + bw.y);
                v[s + k + half] = make_float2(a.x - bw.x, a.y - bw.y);
            }
        }
    }
}

// Shared-memory lines are padded by one element per 16 (index i at
// pz(i) = i + i/16, line length plen(N)): the Stockham passes write with
// strides of 16 elements, which would otherwise fall in one bank.
__device__ __host__ __forceinline__ int pz(int i) { return i + (i >> 4); }
__device__ __host__ __forceinline__ int plen(int n) { return n + (n >> 4); }

template <int R>
__device__ __forceinline__ void stockham_pass(float2 *L, int N, int Ns, int b, bool active,
                                              const float2 *__restrict__ tw) {
    constexpr int NBT = 16 / R;
    const int NR = N / R;
    float2 v[16];
    if (active) {
#pragma unroll
        for (int i = 0; i < NBT; i++) {
            const int j = b * NBT + i;
            const int k = j % Ns;
            const int step = N / (Ns * R);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float2 x = L[pz(j + r * NR)];
                const float2 w = __ldg(&tw[(r * k * step) & (N - 1)]);
                v[i * R + r] = cmul(x, w);
            }
        }
    }
    __syncthreads();
    if (active) {
#pragma unroll
        for (int i = 0; i < NBT; i++) {
            dft_reg<R>(v + i * R);
            const int j = b * NBT + i;
            const int k = j % Ns;
            const int d = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; r++) L[pz(d + r * Ns)] = v[i * R + r];
        }
    }
    __syncthreads();
}

// Direct DFT (forward sign) of R = 3, 5 or 7 values in registers: the
// butterflies of the lengths with odd prime factors.  cos / sin(2 pi m / R)
// for m <= R / 2 (the other half by symmetry).
template <int R>
__device__ __forceinline__ void dft_odd(float2 *v) {
    static_assert(R == 3 || R == 5 || R == 7, "odd radices 3, 5, 7");
    float C[R], S[R];
    if constexpr (R == 3) {
        C[1] = -0.5f;
        S[1] = 0.86602540378443865f;
    } else if constexpr (R == 5) {
        C[1] = 0.30901699437494742f;
        S[1] = 0.95105651629515357f;
        C[2] = -0.80901699437494742f;
        S[2] = 0.58778525229247313f;
    } else {
        C[1] = 0.62348980185873353f;
        S[1] = 0.78183148246802981f;
        C[2] = -0.22252093395631440f;
        S[2] = 0.97492791218182361f;
        C[3] = -0.90096886790241913f;
        S[3] = 0.43388373911755812f;
    }
    C[0] = 1.0f;
    S[0] = 0.0f;
#pragma unroll
    for (int m = 1; m <= R / 2; m++) {
        C[R - m] = C[m];
        S[R - m] = -S[m];
    }
    float2 out[R];
#pragma unroll
    for (int m = 0; m < R; m++) {
        float re = v[0].x, im = v[0].y;
#pragma unroll
        for (int r = 1; r < R; r++) {
            const int e = (r * m) % R;  // v_r * exp(-2 pi i r m / R)
            re += v[r].x * C[e] + v[r].y * S[e];
            im += v[r].y * C[e] - v[r].x * S[e];
        }
        out[m] = make_float2(re, im);
    }
#pragma unroll
    for (int m = 0; m < R; m++) v[m] = out[m];
}

template <int R>
__device__ __forceinline__ void dft_any(float2 *v) {
    if constexpr (R == 3 || R == 5 || R == 7)
        dft_odd<R>(v);
    else
        dft_reg<R>(v);
}

// Lines of length n per block: G * n <= 4096 elements (16 per thread).
__device__ __host__ __forceinline__ int lines_per_block(int n) { return n >= 4096 ? 1 : 4096 / n; }

// One Stockham pass of radix R over G lines of any length N (N % R == 0,
// G * N <= 4096), every thread of the 256 holding up to ceil(16 / R)
// butterflies: all loads (times twiddles) before a barrier, then the
// butterflies and the stores.  Twiddle index r * k * N / (Ns * R) < N.
template <int R>
__device__ void mixed_pass(float2 *buf, int N, int lstride, int G, int Ns,
                           const float2 *__restrict__ tw) {
    constexpr int NBT = (16 + R - 1) / R;
    const int NR = N / R, B = G * NR, step = N / (Ns * R);
    float2 v[NBT * R];
#pragma unroll
    for (int i = 0; i < NBT; i++) {
        const int t = threadIdx.x + i * 256;
        if (t < B) {
            const int line = t / NR, j = t % NR, k = j % Ns;
            const float2 *L = buf + (size_t)line * lstride;
#pragma unroll
            for (int r = 0; r < R; r++)
                v[i * R + r] = cmul(L[pz(j + r * NR)], __ldg(&tw[r * k * step]));
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NBT; i++) {
        const int t = threadIdx.x + i * 256;
        if (t < B) {
            dft_any<R>(v + i * R);
            const int line = t / NR, j = t % NR, k = j % Ns;
            float2 *L = buf + (size_t)line * lstride;
            const int d = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; r++) L[pz(d + r * Ns)] = v[i * R + r];
        }
    }
    __syncthreads();
}

// Lengths whose prime factors are 2, 3, 5 and 7 (the reference's FFTW takes any
// length; these cover the detector and crop sizes the alignment sees).
static inline bool smooth_length(int n) {
    if (n < 2 || n > 4096) return false;
    const int primes[4] = {2, 3, 5, 7};
    for (int p : primes)
        while (n % p == 0) n /= p;
    return n == 1;
}

// Forward FFT of G lines of a length that is not a power of two: radix 16, 8,
// 4, 2, 7, 5, 3 passes in that order (the product of the radices done is Ns).
__device__ void fft_lines_mixed(float2 *buf, int N, int lstride, int G, const float2 *tw) {
    int rest = N, Ns = 1;
    while (rest > 1) {
        int R;
        if (rest % 16 == 0) R = 16;
        else if (rest % 8 == 0) R = 8;
        else if (rest % 4 == 0) R = 4;
        else if (rest % 2 == 0) R = 2;
        else if (rest % 7 == 0) R = 7;
        else if (rest % 5 == 0) R = 5;
        else R = 3;
        switch (R) {
            case 16: mixed_pass<16>(buf, N, lstride, G, Ns, tw); break;
            case 8: mixed_pass<8>(buf, N, lstride, G, Ns, tw); break;
            case 4: mixed_pass<4>(buf, N, lstride, G, Ns, tw); break;
            case 2: mixed_pass<2>(buf, N, lstride, G, Ns, tw); break;
            case 7: mixed_pass<7>(buf, N, lstride, G, Ns, tw); break;
            case 5: mixed_pass<5>(buf, N, lstride, G, Ns, tw); break;
            default: mixed_pass<3>(buf, N, lstride, G, Ns, tw); break;
        }
        Ns *= R;
        rest /= R;
    }
}

// In-place forward FFT of G lines of length N (power of two, 16..4096; G * N
// <= 4096) held in shared memory at buf + l*lstride (padded lines: element i
// at pz(i)).  N/16 threads per line, one radix-16 butterfly per thread per
// pass; all threads of the block must call it.
__device__ void fft_lines(float2 *buf, int N, int lstride, int G, const float2 *tw) {
    const int tpl = N / 16;
    const int line = threadIdx.x / tpl, b = threadIdx.x % tpl;
    const bool active = line < G;
    float2 *L = buf + (size_t)(active ? line : 0) * lstride;
    for (int Ns = 1; Ns < N;) {
        const int R = min(16, N / Ns);
        if (R == 16) stockham_pass<16>(L, N, Ns, b, active, tw);
        else if (R == 8) stockham_pass<8>(L, N, Ns, b, active, tw);
        else if (R == 4) stockham_pass<4>(L, N, Ns, b, active, tw);
        else stockham_pass<2>(L, N, Ns, b, active, tw);
        Ns *= R;
    }
}

// The kernels below are instantiated twice: MIXED = false for power-of-two
// lengths (fft_lines), true for the other lengths (fft_lines_mixed), so the
// power-of-two kernels keep their own register allocation.
template <bool MIXED>
__device__ __forceinline__ void fft_any(float2 *buf, int N, int lstride, int G, const float2 *tw) {
    if constexpr (MIXED)
        fft_lines_mixed(buf, N, lstride, G, tw);
    else
        fft_lines(buf, N, lstride, G, tw);
}

// ---------------------------------------------------------------------------
struct RowStat {
    float m;   // max |c| over the row
    int xpos;  // first x with c == +m (INT_MAX if none)
    int xneg;  // last x with c == -m (-1 if none)
    int pad;
};

// Global loads per thread issued together before their shared-memory stores
// (a block stages 4096 elements: 16 per thread in one batch).  The three
// passes are capped at 128 registers (two blocks per SM): the radix-16
// butterflies spill a little, which costs less than running one block per SM.
constexpr int kLoadBatch = 16;

// Pass 1: rows of z = x + i*y -> half spectra of x and y.
template <bool MIXED>
__global__ void __launch_bounds__(256, 2) k_cc_rows_fwd(const float *__restrict__ x,
                                                     const float *__restrict__ y,
                                                     float2 *__restrict__ Xh,
                                                     float2 *__restrict__ Yh, int nx, int ny,
                                                     const float2 *__restrict__ tw) {
    extern __shared__ float2 sm[];
    const int G = lines_per_block(nx);
    const int row0 = blockIdx.x * G, pair = blockIdx.y;
    const int H = nx / 2 + 1;
    const size_t img = (size_t)pair * nx * ny;
    // all of a thread's loads issued before any store (G * nx = 4096: 16 each)
    for (int i0 = 0; i0 < G * nx; i0 += kLoadBatch * 256) {
        float2 z[kLoadBatch];
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, l = i / nx, c = i % nx, row = row0 + l;
            z[e] = make_float2(0.f, 0.f);
            if (i < G * nx && row < ny)
                z[e] = make_float2(x[img + (size_t)row * nx + c], y[img + (size_t)row * nx + c]);
        }
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, l = i / nx, c = i % nx;
            if (i < G * nx) sm[l * plen(nx) + pz(c)] = z[e];
        }
    }
    __syncthreads();
    fft_any<MIXED>(sm, nx, plen(nx), G, tw);
    const size_t half = (size_t)pair * ny * H;
    for (int i = threadIdx.x; i < G * H; i += blockDim.x) {
        const int l = i / H, k = i % H, row = row0 + l;
        if (row >= ny) continue;
        const float2 Z = sm[l * plen(nx) + pz(k)], Zm = sm[l * plen(nx) + pz(k ? nx - k : 0)];
        Xh[half + (size_t)row * H + k] = make_float2(0.5f * (Z.x + Zm.x), 0.5f * (Z.y - Zm.y));
        Yh[half + (size_t)row * H + k] = make_float2(0.5f * (Z.y + Zm.y), -0.5f * (Z.x - Zm.x));
    }
}

// Pass 2: columns.  ct columns of Xh and Yh per block (ct = col_tile(ny): the
// two arrays' ct columns stay within 64 KB of shared memory, so several blocks
// share an SM); W = IDFT_col(conj(X)*Y) overwrites Xh.
constexpr int kColTile = 4;
static inline int col_tile(int ny) { return ny <= 1024 ? 4 : (ny <= 2048 ? 2 : 1); }
template <bool MIXED>
__global__ void __launch_bounds__(256, 2) k_cc_cols(float2 *__restrict__ Xh,
                                                 const float2 *__restrict__ Yh, int nx, int ny,
                                                 const float2 *__restrict__ tw, int ct) {
    extern __shared__ float2 sm[];
    const int H = nx / 2 + 1;
    const int c0 = blockIdx.x * ct, pair = blockIdx.y;
    const int nc = min(ct, H - c0);
    const size_t half = (size_t)pair * ny * H;
    const int PN = plen(ny);
    float2 *sx = sm, *sy = sm + ct * PN;
    for (int i0 = 0; i0 < ct * ny; i0 += kLoadBatch * 256) {
        float2 a[kLoadBatch], b[kLoadBatch];
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, row = i / ct, c = i % ct;
            a[e] = b[e] = make_float2(0.f, 0.f);
            if (i < ct * ny && c < nc) {
                a[e] = Xh[half + (size_t)row * H + c0 + c];
                b[e] = Yh[half + (size_t)row * H + c0 + c];
            }
        }
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, row = i / ct, c = i % ct;
            if (i < ct * ny) {
                sx[c * PN + pz(row)] = a[e];
                sy[c * PN + pz(row)] = b[e];
            }
        }
    }
    __syncthreads();
    const int G = lines_per_block(ny);
    for (int l0 = 0; l0 < 2 * ct; l0 += G)
        fft_any<MIXED>(sm + (size_t)l0 * PN, ny, PN, min(G, 2 * ct - l0), tw);
    // conj(X)*Y, conjugated again for the inverse transform (IDFT = conj DFT conj)
    for (int i = threadIdx.x; i < ct * ny; i += blockDim.x) {
        const int c = i / ny, row = i % ny, o = c * PN + pz(row);
        const float2 a = sx[o], b = sy[o];
        const float2 cc = make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
        sx[o] = make_float2(cc.x, -cc.y);
    }
    __syncthreads();
    for (int l0 = 0; l0 < ct; l0 += G)
        fft_any<MIXED>(sm + (size_t)l0 * PN, ny, PN, min(G, ct - l0), tw);
    for (int i = threadIdx.x; i < ct * ny; i += blockDim.x) {
        const int row = i / ct, c = i % ct;
        if (c < nc) {
            const float2 w = sx[c * PN + pz(row)];
            Xh[half + (size_t)row * H + c0 + c] = make_float2(w.x, -w.y);
        }
    }
}

// Combine two row statistics in favour of the reference's scan order.
__device__ __forceinline__ RowStat stat_merge(RowStat a, RowStat b) {
    if (b.m > a.m) return b;
    if (a.m > b.m) return a;
    RowStat r = a;
    r.xpos = min(a.xpos, b.xpos);
    r.xneg = max(a.xneg, b.xneg);
    return r;
}

// Pass 3: inverse row transforms -> c rows, with per-row peak statistics.
template <bool MIXED>
__global__ void __launch_bounds__(256, 2) k_cc_rows_inv(const float2 *__restrict__ Wh,
                                                     float *__restrict__ c, RowStat *stats,
                                                     int nx, int ny,
                                                     const float2 *__restrict__ tw) {
    extern __shared__ float2 sm[];
    const int G = lines_per_block(nx);
    const int row0 = blockIdx.x * G, pair = blockIdx.y;
    const int H = nx / 2 + 1;
    const size_t half = (size_t)pair * ny * H;
    for (int i0 = 0; i0 < G * nx; i0 += kLoadBatch * 256) {
        float2 w[kLoadBatch];
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, l = i / nx, k = i % nx, row = row0 + l;
            w[e] = make_float2(0.f, 0.f);
            if (i < G * nx && row < ny) {
                if (k < H) {
                    w[e] = Wh[half + (size_t)row * H + k];
                    w[e].y = -w[e].y;  // conj for the inverse
                } else {
                    w[e] = Wh[half + (size_t)row * H + (nx - k)];  // conj(conj(W[nx-k]))
                }
            }
        }
#pragma unroll
        for (int e = 0; e < kLoadBatch; e++) {
            const int i = i0 + e * 256 + threadIdx.x, l = i / nx, k = i % nx;
            if (i < G * nx) sm[l * plen(nx) + pz(k)] = w[e];
        }
    }
    __syncthreads();
    fft_any<MIXED>(sm, nx, plen(nx), G, tw);
    // one warp per row for the statistics
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t img = (size_t)pair * nx * ny;
    for (int l = warp; l < G; l += blockDim.x / 32) {
        const int row = row0 + l;
        if (row >= ny) continue;
        RowStat s{-1.0f, INT_MAX, -1, 0};
        for (int i = lane; i < nx; i += 32) {
            const float v = sm[l * plen(nx) + pz(i)].x;
            if (c) c[img + (size_t)row * nx + i] = v;
            const float a = fabsf(v);
            RowStat t{a, v == a && a == a ? i : INT_MAX, v == -a && v != a ? i : -1, 0};
            if (!(a == a)) t = RowStat{-1.0f, INT_MAX, -1, 0};  // NaN never wins
            s = stat_merge(s, t);
        }
        for (int o = 16; o > 0; o >>= 1) {
            RowStat t;
            t.m = __shfl_down_sync(0xffffffffu, s.m, o);
            t.xpos = __shfl_down_sync(0xffffffffu, s.xpos, o);
            t.xneg = __shfl_down_sync(0xffffffffu, s.xneg, o);
            t.pad = 0;
            s = stat_merge(s, t);
        }
        if (lane == 0) stats[(size_t)pair * ny + row] = s;
    }
}

// Row statistics of an existing image (for speak on a given correlation map).
__global__ void __launch_bounds__(256) k_row_stats(const float *__restrict__ c, RowStat *stats,
                                                   int nx, int ny) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * 8 + warp, pair = blockIdx.y;
    if (row >= ny) return;
    const float *cr = c + ((size_t)pair * ny + row) * nx;
    RowStat s{-1.0f, INT_MAX, -1, 0};
    for (int i = lane; i < nx; i += 32) {
        const float v = cr[i];
        const float a = fabsf(v);
        RowStat t{a, v == a ? i : INT_MAX, (v == -a && v != a) ? i : -1, 0};
        if (!(a == a)) t = RowStat{-1.0f, INT_MAX, -1, 0};
        s = stat_merge(s, t);
    }
    for (int o = 16; o > 0; o >>= 1) {
        RowStat t;
        t.m = __shfl_down_sync(0xffffffffu, s.m, o);
        t.xpos = __shfl_down_sync(0xffffffffu, s.xpos, o);
        t.xneg = __shfl_down_sync(0xffffffffu, s.xneg, o);
        t.pad = 0;
        s = stat_merge(s, t);
    }
    if (lane == 0) stats[(size_t)pair * ny + row] = s;
}

// quad2dfit (align2dstack.cpp:1125-1166) in double.
__device__ void quad2dfit_dev(const float *z, float *xsh, float *ysh) {
#define Z(i, j) ((double)z[((j)-1) * 3 + (i)-1])
    const double c2 = (8. * Z(1, 1) - 8. * Z(1, 2) + 5. * Z(2, 1) - 8. * Z(2, 2) + 3. * Z(2, 3) +
                       2. * Z(3, 1) - 8. * Z(3, 2) + 6. * Z(3, 3)) /
                      (-6.);
    const double c3 = (Z(1, 1) - 2. * Z(1, 2) + Z(1, 3) + Z(2, 1) - 2. * Z(2, 2) + Z(2, 3) +
                       Z(3, 1) - 2. * Z(3, 2) + Z(3, 3)) /
                      6.0;
    const double c4 = (8. * Z(1, 1) + 5. * Z(1, 2) + 2. * Z(1, 3) - 8. * Z(2, 1) - 8. * Z(2, 2) -
                       8. * Z(2, 3) + 3. * Z(3, 2) + 6. * Z(3, 3)) /
                      (-6.0);
    const double c5 = (Z(1, 1) - Z(1, 3) - Z(3, 1) + Z(3, 3)) / 4.0;
    const double c6 = (Z(1, 1) + Z(1, 2) + Z(1, 3) - 2. * Z(2, 1) - 2. * Z(2, 2) - 2. * Z(2, 3) +
                       Z(3, 1) + Z(3, 2) + Z(3, 3)) /
                      6.0;
#undef Z
    float ys = 0.0f, xs = 0.0f;
    const double den = 4. * c3 * c6 - c5 * c5;
    if (den != 0.0) {
        ys = (float)((c4 * c5 - 2. * c2 * c6) / den - 2.0);
        xs = (float)((c2 * c5 - 2. * c4 * c3) / den - 2.0);
        if (ys < -1.0f) ys = -1.0f;
        if (ys > 1.0f) ys = 1.0f;
        if (xs < -1.0f) xs = -1.0f;
        if (xs > 1.0f) xs = 1.0f;
    }
    *xsh = xs;
    *ysh = ys;
}

// Pass 4: the reference's peak (speak, align2dstack.cpp:1072-1079) scans x
// outer, y inner, replacing the peak when |v| > pmax and then storing the
// SIGNED v.  Hence: if +M (M = max|v|) occurs, the answer is its first
// occurrence in that order; otherwise the scan passes the last -M and, with
// pmax negative, continues from the next element; that rare case is replayed
// element by element (bounded by the image size).
__global__ void __launch_bounds__(256) k_peak(const float *__restrict__ c,
                                              const RowStat *__restrict__ stats, int nx, int ny,
                                              float *sx, float *sy, int *ixo, int *iyo) {
    __shared__ float sm_m[256];
    __shared__ long long sm_pos[256], sm_neg[256];
    const int pair = blockIdx.x;
    const RowStat *st = stats + (size_t)pair * ny;
    const float *cp = c + (size_t)pair * nx * ny;
    float m = -1.0f;
    for (int r = threadIdx.x; r < ny; r += 256) m = fmaxf(m, st[r].m);
    sm_m[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm_m[threadIdx.x] = fmaxf(sm_m[threadIdx.x], sm_m[threadIdx.x + o]);
        __syncthreads();
    }
    const float M = sm_m[0];
    // order key in x-major scan order: x * ny + y
    long long pos = LLONG_MAX, neg = -1;
    for (int r = threadIdx.x; r < ny; r += 256) {
        const RowStat s = st[r];
        if (s.m == M) {
            if (s.xpos != INT_MAX) pos = min(pos, (long long)s.xpos * ny + r);
            if (s.xneg >= 0) neg = max(neg, (long long)s.xneg * ny + r);
        }
    }
    sm_pos[threadIdx.x] = pos;
    sm_neg[threadIdx.x] = neg;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sm_pos[threadIdx.x] = min(sm_pos[threadIdx.x], sm_pos[threadIdx.x + o]);
            sm_neg[threadIdx.x] = max(sm_neg[threadIdx.x], sm_neg[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    long long t;
    if (!(M > 0.0f)) {
        t = 0;  // nothing exceeds pmax = 0 (the reference leaves the peak undefined)
    } else if (sm_pos[0] != LLONG_MAX) {
        t = sm_pos[0];
    } else {
        // replay the reference's state machine after the last -M
        t = sm_neg[0];
        float pmax = -M;
        const long long n = (long long)nx * ny;
        for (long long u = t + 1; u < n; u++) {
            const int xx = (int)(u / ny), yy = (int)(u % ny);
            const float v = cp[(size_t)yy * nx + xx];
            if (fabsf(v) > pmax) {
                pmax = v;
                t = u;
            }
        }
    }
    const int ix = (int)(t / ny), iy = (int)(t % ny);  // 0-based
    float z[9];
    for (int j = -1; j <= 1; j++)
        for (int i = -1; i <= 1; i++) {
            const int xc = (ix + i + nx) % nx, yc = (iy + j + ny) % ny;
            z[(j + 1) * 3 + (i + 1)] = cp[(size_t)yc * nx + xc];
        }
    float xsh, ysh;
    quad2dfit_dev(z, &xsh, &ysh);
    float xt = xsh + (float)ix, yt = ysh + (float)iy;
    if (xt > (float)(nx / 2)) xt = xt - (float)nx;
    if (yt > (float)(ny / 2)) yt = yt - (float)ny;
    sx[pair] = xt;
    sy[pair] = yt;
    if (ixo) ixo[pair] = ix;
    if (iyo) iyo[pair] = iy;
}

// ---------------------------------------------------------------------------
// Fourier shift (fshift2d, align2dstack.cpp:566-630) of a stack of images:
//   out = Re(IDFT2(DFT2(in) * exp(i * phase))) / (nx * ny),
//   phase = -2 pi (sx kx + sy ky) in the reference's precisions: the frequencies
//   and sx*kx + sy*ky in float, the product with 2 pi in double rounded to a
//   float, then the float cosine and sine (cos/sin of a float resolve to the
//   float overloads) and a float complex product.  Full complex transforms, as
//   the reference's: at the Nyquist frequencies the factor is not conjugate
//   symmetric and only the real part is kept.

// Pass 1: real rows -> complex spectra of the rows.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_fs_rows(const float *__restrict__ in,
                                                 float2 *__restrict__ C, int nx, int ny,
                                                 const float2 *__restrict__ tw) {
    extern __shared__ float2 sm[];
    const int G = lines_per_block(nx);
    const int row0 = blockIdx.x * G;
    const size_t img = (size_t)blockIdx.y * nx * ny;
    for (int i = threadIdx.x; i < G * nx; i += blockDim.x) {
        const int l = i / nx, c = i % nx, row = row0 + l;
        sm[l * plen(nx) + pz(c)] = make_float2(row < ny ? in[img + (size_t)row * nx + c] : 0.f, 0.f);
    }
    __syncthreads();
    fft_any<MIXED>(sm, nx, plen(nx), G, tw);
    for (int i = threadIdx.x; i < G * nx; i += blockDim.x) {
        const int l = i / nx, c = i % nx, row = row0 + l;
        if (row < ny) C[img + (size_t)row * nx + c] = sm[l * plen(nx) + pz(c)];
    }
}

__device__ __forceinline__ float fs_freq(int i, int n) {
    const int h = (n + 1) / 2;  // ceil(n / 2)
    return i < h ? (float)i / (float)n : (float)(i - n) / (float)n;
}

// Pass 2: column transforms, the phase factor, inverse column transforms.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_fs_cols(float2 *__restrict__ C, int nx, int ny,
                                                 const float *__restrict__ sxs,
                                                 const float *__restrict__ sys,
                                                 const float2 *__restrict__ tw) {
    extern __shared__ float2 sm[];
    const int c0 = blockIdx.x * kColTile;
    const size_t img = (size_t)blockIdx.y * nx * ny;
    const float sx = sxs[blockIdx.y], sy = sys[blockIdx.y];
    const double two_pi = 2.0 * 3.14159265358979323846;
    const int PN = plen(ny);
    for (int i = threadIdx.x; i < kColTile * ny; i += blockDim.x) {
        const int row = i / kColTile, c = i % kColTile;
        sm[c * PN + pz(row)] = c0 + c < nx ? C[img + (size_t)row * nx + c0 + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int G = lines_per_block(ny);
    for (int l0 = 0; l0 < kColTile; l0 += G)
        fft_any<MIXED>(sm + (size_t)l0 * PN, ny, PN, min(G, kColTile - l0), tw);
    for (int i = threadIdx.x; i < kColTile * ny; i += blockDim.x) {
        const int c = i / ny, row = i % ny, o = c * PN + pz(row);
        const float t = __fadd_rn(__fmul_rn(sx, fs_freq(c0 + c, nx)), __fmul_rn(sy, fs_freq(row, ny)));
        const float ph = (float)(-two_pi * (double)t);
        float sn, cs;
        sincosf(ph, &sn, &cs);
        const float2 f = sm[o];
        const float re = __fsub_rn(__fmul_rn(f.x, cs), __fmul_rn(f.y, sn));
        const float im = __fadd_rn(__fmul_rn(f.x, sn), __fmul_rn(f.y, cs));
        sm[o] = make_float2(re, -im);  // conjugated: IDFT = conj(DFT(conj))
    }
    __syncthreads();
    for (int l0 = 0; l0 < kColTile; l0 += G)
        fft_any<MIXED>(sm + (size_t)l0 * PN, ny, PN, min(G, kColTile - l0), tw);
    for (int i = threadIdx.x; i < kColTile * ny; i += blockDim.x) {
        const int row = i / kColTile, c = i % kColTile;
        const float2 w = sm[c * PN + pz(row)];
        if (c0 + c < nx) C[img + (size_t)row * nx + c0 + c] = make_float2(w.x, -w.y);
    }
}

// Pass 3: inverse row transforms, real part, divided by nx*ny.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_fs_rows_inv(const float2 *__restrict__ C,
                                                     float *__restrict__ out, int nx, int ny,
                                                     const float2 *__restrict__ tw) {
    extern __shared__ float2 sm[];
    const int G = lines_per_block(nx);
    const int row0 = blockIdx.x * G;
    const size_t img = (size_t)blockIdx.y * nx * ny;
    for (int i = threadIdx.x; i < G * nx; i += blockDim.x) {
        const int l = i / nx, c = i % nx, row = row0 + l;
        float2 z = make_float2(0.f, 0.f);
        if (row < ny) {
            z = C[img + (size_t)row * nx + c];
            z.y = -z.y;
        }
        sm[l * plen(nx) + pz(c)] = z;
    }
    __syncthreads();
    fft_any<MIXED>(sm, nx, plen(nx), G, tw);
    const float scale = (float)(nx * ny);
    for (int i = threadIdx.x; i < G * nx; i += blockDim.x) {
        const int l = i / nx, c = i % nx, row = row0 + l;
        if (row < ny) out[img + (size_t)row * nx + c] = sm[l * plen(nx) + pz(c)].x / scale;
    }
}

// ---------------------------------------------------------------------------
// Host side.

static std::mutex g_tw_mu;
static std::map<std::pair<int, int>, float2 *> g_tw;  // (device, N) -> table

static int twiddles(int N, const float2 **out) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto it = g_tw.find({dev, N});
    if (it != g_tw.end()) {
        *out = it->second;
        return 0;
    }
    std::vector<float2> h(N);
    for (int k = 0; k < N; k++) {
        const double a = 2.0 * M_PI * (double)k / (double)N;
        h[k] = make_float2((float)std::cos(a), (float)-std::sin(a));
    }
    float2 *d = nullptr;
    ARECGB_CUDA(cudaMalloc(&d, sizeof(float2) * N));
    ARECGB_CUDA(cudaMemcpy(d, h.data(), sizeof(float2) * N, cudaMemcpyHostToDevice));
    g_tw[{dev, N}] = d;
    *out = d;
    return 0;
}

static bool pow2_ok(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

static int rows_per_block(int nx) { return lines_per_block(nx); }

static std::mutex g_smem_mu;
static std::map<std::pair<int, const void *>, size_t> g_smem;  // (device, kernel) -> limit set

// Raises a kernel's dynamic shared-memory limit to at least `bytes` and never
// lowers it: the limit is process-wide, so a caller on another host thread
// with smaller images cannot drop it between this caller's set and launch.
static int set_smem(const void *fn, size_t bytes) {
    int dev = 0;
    ARECGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_smem_mu);
    size_t &cur = g_smem[{dev, fn}];
    if (bytes <= cur) return 0;
    ARECGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return 0;
}

// Correlate `np` pairs; optionally keep the correlation images in `c`
// (np*ny*nx floats) and/or reduce them to peaks.
static int correlate_batch(const float *d1, const float *d2, int np, int ny, int nx, float *c,
                           RowStat *stats, float2 *Xh, float2 *Yh, cudaStream_t st) {
    const float2 *twx, *twy;
    int rc = twiddles(nx, &twx);
    if (!rc) rc = twiddles(ny, &twy);
    if (rc) return rc;
    const int G = rows_per_block(nx);
    const int ct = col_tile(ny);
    const size_t row_smem = sizeof(float2) * (size_t)G * plen(nx);
    const size_t col_smem = sizeof(float2) * 2 * ct * (size_t)plen(ny);
    // kernel instantiations for the two lengths (MIXED: not a power of two)
    auto rows_fwd = pow2_ok(nx) ? k_cc_rows_fwd<false> : k_cc_rows_fwd<true>;
    auto rows_inv = pow2_ok(nx) ? k_cc_rows_inv<false> : k_cc_rows_inv<true>;
    auto cols = pow2_ok(ny) ? k_cc_cols<false> : k_cc_cols<true>;
    if ((rc = set_smem((const void *)rows_fwd, row_smem))) return rc;
    if ((rc = set_smem((const void *)rows_inv, row_smem))) return rc;
    if ((rc = set_smem((const void *)cols, col_smem))) return rc;
    const int H = nx / 2 + 1;
    rows_fwd<<<dim3((ny + G - 1) / G, np), 256, row_smem, st>>>(d1, d2, Xh, Yh, nx, ny, twx);
    cols<<<dim3((H + ct - 1) / ct, np), 256, col_smem, st>>>(Xh, Yh, nx, ny, twy, ct);
    rows_inv<<<dim3((ny + G - 1) / G, np), 256, row_smem, st>>>(Xh, c, stats, nx, ny, twx);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

struct CcScratch {
    float2 *Xh = nullptr, *Yh = nullptr;
    float *c = nullptr;
    RowStat *stats = nullptr;
};

static void cc_free(CcScratch &s) {
    cudaFree(s.Xh);
    cudaFree(s.Yh);
    cudaFree(s.c);
    cudaFree(s.stats);
}

static int cc_alloc(CcScratch &s, int np, int ny, int nx, bool need_c) {
    const size_t H = nx / 2 + 1;
    ARECGB_CUDA(cudaMalloc(&s.Xh, sizeof(float2) * H * ny * np));
    ARECGB_CUDA(cudaMalloc(&s.Yh, sizeof(float2) * H * ny * np));
    if (need_c) ARECGB_CUDA(cudaMalloc(&s.c, sizeof(float) * (size_t)nx * ny * np));
    ARECGB_CUDA(cudaMalloc(&s.stats, sizeof(RowStat) * (size_t)ny * np));
    return 0;
}

int cc_shifts(const float *d1, const float *d2, int nz, int ny, int nx, float *sx, float *sy,
              int *ix, int *iy, cudaStream_t st) {
    if (!smooth_length(nx) || !smooth_length(ny) || nz < 0 || !d1 || !d2 || !sx || !sy) {
        set_error("cc_shifts: nx and ny must be in [2, 4096] with prime factors 2, 3, 5, 7 "
                  "(got " + std::to_string(nx) + " x " + std::to_string(ny) + ")");
        return ARECGB_ERR_ARG;
    }
    if (nz == 0) return 0;
    // pairs per batch: keep the scratch near 1 GiB
    const size_t per_pair = (size_t)ny * ((size_t)(nx / 2 + 1) * 16 + (size_t)nx * 4 + 16);
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(nz, (1ull << 30) / per_pair));
    CcScratch s;
    int rc = cc_alloc(s, batch, ny, nx, true);
    for (int p0 = 0; !rc && p0 < nz; p0 += batch) {
        const int np = std::min(batch, nz - p0);
        const size_t off = (size_t)p0 * nx * ny;
        rc = correlate_batch(d1 + off, d2 + off, np, ny, nx, s.c, s.stats, s.Xh, s.Yh, st);
        if (rc) break;
        k_peak<<<np, 256, 0, st>>>(s.c, s.stats, nx, ny, sx + p0, sy + p0, ix ? ix + p0 : nullptr,
                                   iy ? iy + p0 : nullptr);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(std::string("cc_shifts: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    cudaStreamSynchronize(st);
    cc_free(s);
    return rc;
}

int ccorr_image(const float *dx, const float *dy, float *dc, int ny, int nx, cudaStream_t st) {
    if (!smooth_length(nx) || !smooth_length(ny)) {
        set_error("ccorr2d: nx and ny must be in [2, 4096] with prime factors 2, 3, 5, 7 (got " +
                  std::to_string(nx) + " x " + std::to_string(ny) + ")");
        return ARECGB_ERR_ARG;
    }
    CcScratch s;
    int rc = cc_alloc(s, 1, ny, nx, false);
    if (!rc) rc = correlate_batch(dx, dy, 1, ny, nx, dc, s.stats, s.Xh, s.Yh, st);
    cudaStreamSynchronize(st);
    cc_free(s);
    return rc;
}

int fshift_stack(const float *d_in, float *d_out, int nz, int ny, int nx, const float *d_sx,
                 const float *d_sy, cudaStream_t st) {
    if (!smooth_length(nx) || !smooth_length(ny) || ny > 2048 || nz < 0 || !d_in || !d_out ||
        !d_sx || !d_sy) {
        set_error("fshift2d: nx in [2, 4096] and ny in [2, 2048] with prime factors 2, 3, 5, 7 "
                  "(got " + std::to_string(nx) + " x " + std::to_string(ny) + ")");
        return ARECGB_ERR_ARG;
    }
    if (nz == 0) return 0;
    const float2 *twx, *twy;
    int rc = twiddles(nx, &twx);
    if (!rc) rc = twiddles(ny, &twy);
    if (rc) return rc;
    const int G = rows_per_block(nx);
    const size_t row_smem = sizeof(float2) * (size_t)G * plen(nx);
    const size_t col_smem = sizeof(float2) * kColTile * (size_t)plen(ny);
    auto fs_rows = pow2_ok(nx) ? k_fs_rows<false> : k_fs_rows<true>;
    auto fs_rows_inv = pow2_ok(nx) ? k_fs_rows_inv<false> : k_fs_rows_inv<true>;
    auto fs_cols = pow2_ok(ny) ? k_fs_cols<false> : k_fs_cols<true>;
    if ((rc = set_smem((const void *)fs_rows, row_smem))) return rc;
    if ((rc = set_smem((const void *)fs_rows_inv, row_smem))) return rc;
    if ((rc = set_smem((const void *)fs_cols, col_smem))) return rc;
    // images per batch: complex scratch near 1 GiB
    const size_t per = sizeof(float2) * (size_t)nx * ny;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(nz, (1ull << 30) / per));
    float2 *C = nullptr;
    ARECGB_CUDA(cudaMalloc(&C, per * batch));
    for (int z0 = 0; z0 < nz && !rc; z0 += batch) {
        const int nb = std::min(batch, nz - z0);
        const size_t off = (size_t)z0 * nx * ny;
        fs_rows<<<dim3((ny + G - 1) / G, nb), 256, row_smem, st>>>(d_in + off, C, nx, ny, twx);
        fs_cols<<<dim3((nx + kColTile - 1) / kColTile, nb), 256, col_smem, st>>>(
            C, nx, ny, d_sx + z0, d_sy + z0, twy);
        fs_rows_inv<<<dim3((ny + G - 1) / G, nb), 256, row_smem, st>>>(C, d_out + off, nx, ny,
                                                                     twx);
        count_launches(3);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(std::string("fshift2d: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
        }
    }
    cudaStreamSynchronize(st);
    cudaFree(C);
    return rc;
}

int peak_search(const float *dc, int nz, int ny, int nx, float *sx, float *sy, int *ix, int *iy,
                cudaStream_t st) {
    if (nx < 1 || ny < 1 || nz < 1) {
        set_error("speak: bad shape");
        return ARECGB_ERR_ARG;
    }
    RowStat *stats = nullptr;
    ARECGB_CUDA(cudaMalloc(&stats, sizeof(RowStat) * (size_t)ny * nz));
    k_row_stats<<<dim3((ny + 7) / 8, nz), 256, 0, st>>>(dc, stats, nx, ny);
    k_peak<<<nz, 256, 0, st>>>(dc, stats, nx, ny, sx, sy, ix, iy);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(st);
    cudaFree(stats);
    if (e != cudaSuccess) {
        set_error(std::string("speak: ") + cudaGetErrorString(e));
        return cuda_status(e);
    }
    return 0;
}


// ---------------------------------------------------------------------------
// Shift search without allocation (arecgb_cc_shifts_static).
//
// For callers that must not allocate device memory while they run: an
// alignment loop that interleaves shift searches with a reconstruction running
// on another stream (cc_shifts' cudaFree synchronises the whole device and
// would stall that solve), or a host whose memory is owned by another
// allocator (a caching allocator that already holds the free HBM).
//
// Scratch: one file-scope device array of kStaticBytes (3.5 MiB), carved into
//   Xh, Yh  float2 [kStaticSpec]   half spectra of both images
//   c       float  [kStaticPixels] correlation images
//   stats   RowStat[kStaticRows]   per-row peak statistics
//   tw      float2 [1008]          twiddles for N = 16..512, table N at offset N - 16
// Limit: nx, ny powers of two in [16, 512] and nz * ny * nx <= kStaticPixels
// (one 512 x 512 pair, or e.g. 64 pairs of 64 x 64).  Larger requests are
// rejected with ARECGB_ERR_ARG; arecgb_cc_shifts has no such limit.
// Nothing in the scratch must start at zero: every element a call reads was
// written earlier in the same call (row pass -> column pass -> inverse rows ->
// peak).  Only the twiddle tables persist; the set-up writes them.
// The scratch is shared by every call on a device: two calls that can overlap
// (different streams, or host threads without ordering) race on it.
constexpr size_t kStaticPixels = 512 * 512;
constexpr size_t kStaticRows = kStaticPixels / 16;                  // ny * nz <= pixels / nx
constexpr size_t kStaticSpec = kStaticPixels / 2 + kStaticRows;     // (nx/2 + 1) * ny * nz
constexpr size_t kStaticTw = 1024;                                  // 16 + 32 + ... + 512 = 1008
constexpr size_t kOffYh = sizeof(float2) * kStaticSpec;
constexpr size_t kOffC = 2 * kOffYh;
constexpr size_t kOffStats = kOffC + sizeof(float) * kStaticPixels;
constexpr size_t kOffTw = kOffStats + sizeof(RowStat) * kStaticRows;
constexpr size_t kStaticBytes = kOffTw + sizeof(float2) * kStaticTw;
static_assert(kOffYh % 256 == 0 && kOffC % 256 == 0 && kOffStats % 256 == 0 &&
                  kOffTw % 256 == 0,
              "scratch pieces must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_cc_static[kStaticBytes];

struct StaticScratch {
    bool ready = false;
    unsigned char *base = nullptr;
};
static std::mutex g_static_mu;
static std::map<int, StaticScratch> g_static;  // device -> scratch address

// Once per device, with that device current: resolve the scratch address and
// write the twiddle tables (a synchronous copy).  Run the first call before
// any stream capture.
static int static_setup(unsigned char **base) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("cc_shifts_static: cudaGetDevice: ") + cudaGetErrorString(e));
        return cuda_status(e);
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    StaticScratch &s = g_static[dev];
    if (s.ready) {
        *base = s.base;
        return 0;
    }
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_cc_static);
    if (e != cudaSuccess || !ptr) {
        set_error(std::string("cc_shifts_static: cudaGetSymbolAddress: ") +
                  cudaGetErrorString(e));
        return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
    }
    std::vector<float2> h(kStaticTw, make_float2(0.f, 0.f));
    for (int N = 16; N <= 512; N *= 2)
        for (int k = 0; k < N; k++) {
            const double a = 2.0 * M_PI * (double)k / (double)N;
            h[N - 16 + k] = make_float2((float)std::cos(a), (float)-std::sin(a));
        }
    e = cudaMemcpy((unsigned char *)ptr + kOffTw, h.data(), sizeof(float2) * kStaticTw,
                   cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_error(std::string("cc_shifts_static: twiddle upload: ") + cudaGetErrorString(e));
        return cuda_status(e);
    }
    s.base = (unsigned char *)ptr;
    s.ready = true;
    *base = s.base;
    return 0;
}

int cc_shifts_static(const float *d1, const float *d2, int nz, int ny, int nx, float *sx,
                     float *sy, int *ix, int *iy, cudaStream_t st) {
    const bool shape_ok = nx >= 16 && nx <= 512 && ny >= 16 && ny <= 512 &&
                          (nx & (nx - 1)) == 0 && (ny & (ny - 1)) == 0;
    if (!shape_ok || nz < 0 || !d1 || !d2 || !sx || !sy) {
        set_error("cc_shifts_static: nx and ny must be powers of two in [16, 512]");
        return ARECGB_ERR_ARG;
    }
    if ((size_t)nz * ny * nx > kStaticPixels) {
        set_error("cc_shifts_static: nz * ny * nx = " + std::to_string((size_t)nz * ny * nx) +
                  " exceeds the static scratch limit of " + std::to_string(kStaticPixels) +
                  " pixels (one 512 x 512 pair); use arecgb_cc_shifts");
        return ARECGB_ERR_ARG;
    }
    unsigned char *base = nullptr;
    int rc = static_setup(&base);
    if (rc) return rc;
    if (nz == 0) return 0;
    float2 *Xh = reinterpret_cast<float2 *>(base);
    float2 *Yh = reinterpret_cast<float2 *>(base + kOffYh);
    float *c = reinterpret_cast<float *>(base + kOffC);
    RowStat *stats = reinterpret_cast<RowStat *>(base + kOffStats);
    const float2 *tw = reinterpret_cast<const float2 *>(base + kOffTw);
    const float2 *twx = tw + (nx - 16), *twy = tw + (ny - 16);
    // shared memory: 8 * G * nx = 32 KB per row block, 64 * ny <= 32 KB per
    // column block (set_smem only ever raises the kernels' limits).
    const int G = rows_per_block(nx);
    const size_t row_smem = sizeof(float2) * (size_t)G * plen(nx);
    const size_t col_smem = sizeof(float2) * 2 * kColTile * (size_t)plen(ny);
    if ((rc = set_smem((const void *)k_cc_rows_fwd<false>, row_smem))) return rc;
    if ((rc = set_smem((const void *)k_cc_rows_inv<false>, row_smem))) return rc;
    if ((rc = set_smem((const void *)k_cc_cols<false>, col_smem))) return rc;
    const int H = nx / 2 + 1;
    k_cc_rows_fwd<false><<<dim3((ny + G - 1) / G, nz), 256, row_smem, st>>>(d1, d2, Xh, Yh, nx, ny,
                                                                           twx);
    k_cc_cols<false><<<dim3((H + kColTile - 1) / kColTile, nz), 256, col_smem, st>>>(Xh, Yh, nx, ny, twy,
                                                                            kColTile);
    k_cc_rows_inv<false><<<dim3((ny + G - 1) / G, nz), 256, row_smem, st>>>(Xh, c, stats, nx, ny,
                                                                           twx);
    k_peak<<<nz, 256, 0, st>>>(c, stats, nx, ny, sx, sy, ix, iy);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("cc_shifts_static: ") + cudaGetErrorString(e));
        return cuda_status(e);
    }
    return 0;
}

}  // namespace arecgb

extern "C" int arecgb_cc_shifts_static(const float *d_img1, const float *d_img2, int nz, int ny,
                                       int nx, float *d_sx, float *d_sy, int *d_ix, int *d_iy,
                                       void *stream) {
    return arecgb::cc_shifts_static(d_img1, d_img2, nz, ny, nx, d_sx, d_sy, d_ix, d_iy,
                                    (cudaStream_t)stream);
}
