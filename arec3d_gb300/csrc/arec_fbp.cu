// Filtered back projection (no counterpart in the reference; a cheap first
// reconstruction for the warm start): the discrete Ram-Lak ramp filter along
// detector bins, as a linear convolution, then the plan's back projector.
//
//   f[a][j][y] = c * sum_{k=0}^{nx-1} h(j - k) s[a][k][y],
//   h(0) = 1/4,  h(d) = -1 / (pi d)^2 for odd d,  h(d) = 0 for even d != 0,
//
// (the spatial form of the band-limited ramp |w| for unit bin spacing), and
// x = A^T f with c = pi / nangles, the parallel-beam inversion formula's
// weight per angle.
#include <math.h>

#include "arec_internal.cuh"

namespace arecgb {

namespace {

constexpr int kRampWarps = 8;
constexpr int kRampBinsPerWarp = 16;                          // output bins per thread
constexpr int kRampBins = kRampWarps * kRampBinsPerWarp;      // output bins per block
constexpr int kRampChunk = 32;                                // input bins per staged chunk
constexpr int kRampSlices = 128;                              // slices per block (32 lanes x 4)

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp16(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst)),
                 "l"(src), "r"(valid ? 16u : 0u)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Odd taps, index u = (d + doff) / 2 for odd d (doff odd): c * h(d).
__global__ void k_ramp_taps(float *taps, int n, int doff, double c) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const double d = 2.0 * u - doff;
    const double pi = 3.14159265358979323846;
    taps[u] = (float)(-c / (pi * pi * d * d));
}

__device__ __forceinline__ void fma4(float4 &a, float w, const float4 &v) {
    a.x = fmaf(w, v.x, a.x);
    a.y = fmaf(w, v.y, a.y);
    a.z = fmaf(w, v.z, a.z);
    a.w = fmaf(w, v.w, a.w);
}

// Block = (128 slices, 128 output bins, one angle); warp w takes bins
// jb = j0 + 16 w .. jb + 15 and lane l slices 4 l .. 4 l + 3.  The input bins
// stream through shared memory in chunks of 32 (double-buffered cp.async).
// For a pair of input bins (ke even, ke + 1) the odd distances are
// jb + i - ke for odd i and jb + i - ke - 1 for even i: nine taps
// h(D - 1), h(D + 1), ..., h(D + 15) with D = jb - ke, a window that slides by
// one tap per pair, so each pair costs one tap load, two row loads and 64
// FMAs per thread.  The centre tap h(0) is added at the end.
__global__ void __launch_bounds__(kRampWarps * 32, 2)
    k_ramp_filter(const float *__restrict__ s, float *__restrict__ f,
                  const float *__restrict__ taps, int nx, int ys, int doff, float h0) {
    constexpr int KC = kRampChunk, NB = kRampBinsPerWarp;
    __shared__ __align__(16) float4 rows[2][KC][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y0 = blockIdx.x * kRampSlices, j0 = blockIdx.y * kRampBins, a = blockIdx.z;
    const int jb = j0 + warp * NB;
    const int y = y0 + 4 * lane;
    const size_t ysz = (size_t)ys;
    const float *sa = s + (size_t)a * nx * ysz;
    const int nchunk = (nx + KC - 1) / KC;

    auto stage = [&](int c, int buf) {
        // KC rows x 32 float4: 4 per thread; rows off the detector and slices
        // past ys arrive as zeros
        for (int i = threadIdx.x; i < KC * 32; i += kRampWarps * 32) {
            const int r = i >> 5, l = i & 31, k = c * KC + r, yy = y0 + 4 * l;
            const bool ok = k < nx && yy < ys;
            cp16(&rows[buf][r][l], ok ? sa + (size_t)k * ysz + yy : sa, ok);
        }
        cp_commit();
    };

    float4 acc[NB];
#pragma unroll
    for (int i = 0; i < NB; i++) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);

    stage(0, 0);
    for (int c = 0; c < nchunk; c++) {
        if (c + 1 < nchunk) {
            stage(c + 1, (c + 1) & 1);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
        const float4(*R)[32] = rows[c & 1];
        const int k0 = c * KC;
        // window w[m] = h(D - 1 + 2 m), m = 0..8, D = jb - ke
        int D = jb - k0;
        float w[9];
#pragma unroll
        for (int m = 0; m < 9; m++) w[m] = __ldg(taps + ((D - 1 + 2 * m + doff) >> 1));
#pragma unroll
        for (int p = 0; p < KC / 2; p++) {
            const float4 pe = R[2 * p][lane], po = R[2 * p + 1][lane];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                fma4(acc[2 * m + 1], w[m + 1], pe);  // d = D + 2m + 1
                fma4(acc[2 * m], w[m], po);          // d = D - 1 + 2m
            }
            // next pair: D -= 2, the window moves down one tap
#pragma unroll
            for (int m = 8; m > 0; m--) w[m] = w[m - 1];
            D -= 2;
            w[0] = __ldg(taps + ((D - 1 + doff) >> 1));
        }
        __syncthreads();  // this buffer is refilled two chunks on
    }
    if (y >= ys) return;
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const int j = jb + i;
        if (j < nx) {
            float4 *dst = reinterpret_cast<float4 *>(f + ((size_t)a * nx + j) * ysz + y);
            const float4 v = *reinterpret_cast<const float4 *>(sa + (size_t)j * ysz + y);
            fma4(acc[i], h0, v);
            *dst = acc[i];
        }
    }
}

}  // namespace

// The plan's tap table (built once per plan): odd distances |d| <= nx + 160.
static int ramp_taps(Plan *p, int *doff, cudaStream_t st) {
    const int dmax = p->nx + 160;
    const int off = (dmax % 2 == 0) ? dmax + 1 : dmax + 2;  // odd, > dmax
    const int n = off + 1;
    if (!p->d_ramp || p->ramp_n != n) {
        cudaFree(p->d_ramp);
        p->d_ramp = nullptr;
        p->ramp_n = 0;
        ARECGB_CUDA(cudaMalloc(&p->d_ramp, sizeof(float) * n));
        k_ramp_taps<<<(n + 255) / 256, 256, 0, st>>>(p->d_ramp, n, off,
                                                     3.14159265358979323846 / p->na);
        ARECGB_CUDA(cudaGetLastError());
        count_launches(1);
        p->ramp_n = n;
    }
    *doff = off;
    return 0;
}

int ramp_filter(Plan *p, const float *d_s, float *d_f, cudaStream_t st) {
    if (p->ys % 4) return ARECGB_ERR_ARG;  // rows of float4 (ys is a multiple of 8)
    int doff = 0, rc = ramp_taps(p, &doff, st);
    if (rc) return rc;
    const dim3 grid((p->ys + kRampSlices - 1) / kRampSlices, (p->nx + kRampBins - 1) / kRampBins,
                    p->na);
    k_ramp_filter<<<grid, kRampWarps * 32, 0, st>>>(d_s, d_f, p->d_ramp, p->nx, p->ys, doff,
                                                    (float)(0.25 * 3.14159265358979323846 / p->na));
    ARECGB_CUDA(cudaGetLastError());
    count_launches(1);
    return 0;
}

// x = A^T (ramp * b); with d_norm2, also ||A^T b||^2 (a back projection of b
// into x first, overwritten).  d_work: the filtered sinogram.
int fbp(Plan *p, const float *d_b, float *d_x, float *d_work, double *d_norm2, cudaStream_t st) {
    int rc = 0;
    if (d_norm2 && (rc = back_project(p, d_b, d_x, d_norm2, nullptr, st))) return rc;
    if ((rc = ramp_filter(p, d_b, d_work, st))) return rc;
    return back_project(p, d_work, d_x, nullptr, nullptr, st);
}

}  // namespace arecgb
