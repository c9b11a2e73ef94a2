// Forward and back projector kernels (templated on weighting, slices per lane
// and slice chunks per block).  Included by one .cu file per weighting so the
// instantiations compile in parallel.
//
// Back projection  g[k][y] = sum_a sum_j w_j(k,a) s[a][iqx(k,a)-1+j][y]
//   reference: arecBackProject2D[_KB|_SQ] (AREC3D/AREC3D/arecproject.cpp:109,447,650)
//   Gather over angles.  A block owns a tile of 8x4 pixels (32 rays) and
//   256 or 512 slices; lanes are slices, so every sinogram load is a coalesced
//   row of 32*VEC slices and the per-(ray, angle) weights are warp-uniform.
//   Weights for 32 rays x 32 angles are computed once per block (lanes = rays)
//   into shared memory and reused by every slice chunk.
//
// Forward projection  q[a][b][y] = sum_{k,j: iqx(k,a)-1+j = b} w_j(k,a) x[k][y]
//   reference: arecProject2D[_KB|_SQ] (arecproject.cpp:19,351,540), which
//   scatters.  Here each output is owned by one block (no atomics): a block owns
//   a group of up to 4 consecutive angles, a tile of BT detector bins and
//   256/512 slices, and gathers the rays of the strip of the cylinder that
//   projects into the tile.  The strip is swept line by line (rows when
//   |cos| >= |sin|, columns otherwise, so consecutive pixels move <= 1 bin and a
//   line holds <= 32 candidates); candidates are bucketed by centre bin with a
//   stable counting sort in shared memory, so the accumulation loop runs over a
//   compile-time bucket index and each loaded pixel feeds up to 3 register
//   accumulators.  The four angle warps of a block read nearly the same pixels,
//   which then come from L1.
//
// Both kernels evaluate the identical ray_taps<W>() so A and A^T are exact
// transposes of each other.  Both fuse the FP64 sum of squares of their output
// (one partial per block, reduced in a fixed order afterwards).
#pragma once

#include <climits>

#include "arec_weights.cuh"

namespace arecgb {

struct OpArgs {
    const float4 *ray;
    const AngleParams *ang;
    const RowInfo *rows;
    const ColInfo *cols;
    const int4 *groups;
    const int2 *tiles;
    int nx, nrays, ys, na;
    float r_hi, r_lo;
    double *partials;
    const int *skip;
    int *err;
};

template <int VEC>
__device__ __forceinline__ void ldv(const float *__restrict__ p, float (&v)[VEC]) {
    if constexpr (VEC == 8) {
        float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        float4 b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else if constexpr (VEC == 4) {
        float4 a = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    } else if constexpr (VEC == 2) {
        float2 a = __ldg(reinterpret_cast<const float2 *>(p));
        v[0] = a.x; v[1] = a.y;
    } else {
        v[0] = __ldg(p);
    }
}

template <int VEC>
__device__ __forceinline__ void stv(float *__restrict__ p, const float (&v)[VEC]) {
    if constexpr (VEC == 8) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
        reinterpret_cast<float4 *>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else if constexpr (VEC == 4) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (VEC == 2) {
        reinterpret_cast<float2 *>(p)[0] = make_float2(v[0], v[1]);
    } else {
        p[0] = v[0];
    }
}

// Block-wide deterministic sum of one double per thread -> partials[slot].
template <int NW>
__device__ __forceinline__ void block_sum_to(double v, double *red, double *out) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < NW; w++) s += red[w];
        *out = s;
    }
}

// ---------------------------------------------------------------------------
// Back projection.
template <int W, int VEC, int NSC>
__global__ void __launch_bounds__(128 * NSC)
    bp_kernel(OpArgs A, const float *__restrict__ s, float *__restrict__ g) {
    constexpr int NT = 128 * NSC, NWARP = NT / 32, AC = 32;
    __shared__ float4 sw[AC][32];
    __shared__ double red[NWARP];
    if (A.skip && *A.skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 tile = A.tiles[blockIdx.x];
    const int ix = tile.x + (lane & (kTileX - 1)), iz = tile.y + lane / kTileX;
    int k = -1;
    if (iz < A.nx) {
        RowInfo ri = A.rows[iz];
        if (ix >= ri.lo && ix <= ri.hi) k = ri.start + ix - ri.lo;
    }
    const float4 myray = k >= 0 ? A.ray[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int rg = warp & 3, sc = warp >> 2;
    const int y0 = (blockIdx.y * NSC + sc) * 32 * VEC + lane * VEC;
    const bool yok = y0 < A.ys;
    const size_t bin_stride = (size_t)A.ys;

    float acc[8][VEC];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int q = 0; q < VEC; q++) acc[r][q] = 0.f;

    for (int a0 = 0; a0 < A.na; a0 += AC) {
        for (int ai = warp; ai < AC; ai += NWARP) {
            const int a = a0 + ai;
            float4 e = make_float4(__int_as_float(INT_MIN / 2), 0.f, 0.f, 0.f);
            if (a < A.na && k >= 0) {
                Taps t = ray_taps<W>(myray, A.ang[a], A.r_hi, A.r_lo);
                e = make_float4(__int_as_float(t.iqx - 1), t.w0, t.w1, t.w2);
            }
            sw[ai][lane] = e;
        }
        __syncthreads();
        const int nac = min(AC, A.na - a0);
        if (yok) {
            for (int ai = 0; ai < nac; ai++) {
                const float *sa = s + (size_t)(a0 + ai) * A.nx * bin_stride + y0;
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    const float4 e = sw[ai][rg * 8 + r];
                    const int b0 = __float_as_int(e.x);
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        const int b = b0 + j;
                        const float w = j == 0 ? e.y : (j == 1 ? e.z : e.w);
                        if ((unsigned)b < (unsigned)A.nx) {
                            float v[VEC];
                            ldv<VEC>(sa + (size_t)b * bin_stride, v);
#pragma unroll
                            for (int q = 0; q < VEC; q++) acc[r][q] = fmaf(w, v[q], acc[r][q]);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }

    double s2 = 0.0;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int kr = __shfl_sync(0xffffffffu, k, rg * 8 + r);
        if (kr >= 0 && yok) {
            stv<VEC>(g + (size_t)kr * bin_stride + y0, acc[r]);
#pragma unroll
            for (int q = 0; q < VEC; q++) s2 += (double)__fmul_rn(acc[r][q], acc[r][q]);
        }
    }
    block_sum_to<NWARP>(s2, red, A.partials + (size_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// ---------------------------------------------------------------------------
// Forward projection (square-pixel and Kaiser-Bessel weightings).

// Extent of the line coordinate L over {T1 <= P*ca + L*cl <= T2} within the
// disk L^2 + P^2 <= R^2 (ca, cl: direction cosines along / across lines).
__device__ __forceinline__ bool strip_line_extent(float ca, float cl, float T1, float T2, float R,
                                                  float &lmin, float &lmax) {
    const float top = R * cl, bot = -R * cl;
    if (top >= T1 && top <= T2) {
        lmax = R;
    } else {
        const float T = top < T1 ? T1 : T2;
        if (fabsf(T) > R) return false;
        lmax = T * cl + fabsf(ca) * sqrtf(fmaxf(R * R - T * T, 0.f));
    }
    if (bot >= T1 && bot <= T2) {
        lmin = -R;
    } else {
        const float T = bot < T1 ? T1 : T2;
        if (fabsf(T) > R) return false;
        lmin = T * cl - fabsf(ca) * sqrtf(fmaxf(R * R - T * T, 0.f));
    }
    return true;
}

template <int W, int VEC, int NSC, int BT>
__global__ void __launch_bounds__(32 * kGroupAngles * NSC)
    fp_kernel(OpArgs A, const float *__restrict__ x, float *__restrict__ q) {
    constexpr int NA = kGroupAngles, NWARP = NA * NSC, NG = BT + 2;
    __shared__ float4 list[NA][NSC * 32];
    __shared__ int cnt[NWARP][NG];
    __shared__ int base[NA][NG + 1];
    __shared__ int lrange[NA][2];
    __shared__ double red[NWARP];
    if (A.skip && *A.skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntile = (A.nx + BT - 1) / BT;
    const int grp = blockIdx.x / ntile, b0 = (blockIdx.x % ntile) * BT;
    const int4 G = A.groups[grp];
    const int orient = G.z;
    const float r = A.r_hi + A.r_lo;
    // The strip: centre bins iqx in [b0-1, b0+BT], i.e. xb in
    // [b0-1.5, b0+BT+0.5], with a margin; in offsets from the centre:
    const float T1 = (float)b0 - 1.5f - 0.02f - r;
    const float T2 = (float)(b0 + BT) + 0.5f + 0.02f - r;
    const float R = r + 1.5f;

    if (threadIdx.x < NA) {
        int lo = INT_MAX, hi = INT_MIN;
        if ((int)threadIdx.x < G.y) {
            const AngleParams ap = A.ang[G.x + threadIdx.x];
            const float ca = orient ? ap.s : ap.c, cl = orient ? ap.c : ap.s;
            float lmin, lmax;
            if (strip_line_extent(ca, cl, T1, T2, R, lmin, lmax)) {
                lo = max(0, (int)floorf(lmin + r) - 1);
                hi = min(A.nx - 1, (int)ceilf(lmax + r) + 1);
            }
        }
        lrange[threadIdx.x][0] = lo;
        lrange[threadIdx.x][1] = hi;
    }
    __syncthreads();
    int L0 = INT_MAX, L1 = INT_MIN;
#pragma unroll
    for (int i = 0; i < NA; i++) {
        L0 = min(L0, lrange[i][0]);
        L1 = max(L1, lrange[i][1]);
    }

    const int ai = warp % NA, sc = warp / NA;
    const bool angle_ok = ai < G.y;
    const int y0 = (blockIdx.y * NSC + sc) * 32 * VEC + lane * VEC;
    const bool yok = y0 < A.ys;
    AngleParams ap;
    float ca = 1.f, cl = 0.f;
    int my_lo = 0, my_hi = -1;
    if (angle_ok) {
        ap = A.ang[G.x + ai];
        ca = orient ? ap.s : ap.c;
        cl = orient ? ap.c : ap.s;
        my_lo = lrange[ai][0];
        my_hi = lrange[ai][1];
    }

    float acc[BT][VEC];
#pragma unroll
    for (int j = 0; j < BT; j++)
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[j][v] = 0.f;

    for (int lb = L0; lb <= L1; lb += NSC) {
        // Phase A: warp (ai, sc) enumerates line lb+sc for angle ai; lane = candidate.
        const int li = lb + sc;
        bool valid = false;
        int gk = 0;
        float4 ent = make_float4(0.f, 0.f, 0.f, 0.f);
        if (angle_ok && li >= my_lo && li <= my_hi) {
            const float Lv = (float)li - r;
            int plo, phi;
            if (orient == 0) {
                const RowInfo ri = A.rows[li];
                plo = ri.lo;
                phi = ri.hi;
            } else {
                const ColInfo ci = A.cols[li];
                plo = ci.lo;
                phi = ci.hi;
            }
            float pa = (T1 - Lv * cl) / ca, pb = (T2 - Lv * cl) / ca;
            if (pa > pb) {
                float t = pa;
                pa = pb;
                pb = t;
            }
            const int clo = max(plo, (int)floorf(pa + r) - 1);
            const int chi = min(phi, (int)ceilf(pb + r) + 1);
            const int n = chi - clo + 1;
            if (n > 32 && lane == 0) atomicOr(A.err, 1);
            if (lane < n) {
                const int pi = ca > 0.f ? clo + lane : chi - lane;
                int kk;
                if (orient == 0) {
                    const RowInfo ri = A.rows[li];
                    kk = ri.start + pi - ri.lo;
                } else {
                    const RowInfo ri = A.rows[pi];
                    kk = ri.start + li - ri.lo;
                }
                const Taps t = ray_taps<W>(A.ray[kk], ap, A.r_hi, A.r_lo);
                gk = t.iqx - b0 + 1;
                valid = gk >= 0 && gk <= BT + 1;
                ent = make_float4(__int_as_float(kk), t.w0, t.w1, t.w2);
            }
        }
        // Phase B: stable counting sort by bucket (line order, then lane order).
        const unsigned key = valid ? (unsigned)gk : 64u + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (lane < NG) cnt[warp][lane] = 0;
        __syncwarp();
        if (valid && rank == 0) cnt[warp][gk] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < NA) {
            int run = 0;
            for (int gg = 0; gg < NG; gg++) {
                base[threadIdx.x][gg] = run;
#pragma unroll
                for (int s2 = 0; s2 < NSC; s2++) run += cnt[s2 * NA + threadIdx.x][gg];
            }
            base[threadIdx.x][NG] = run;
        }
        __syncthreads();
        if (valid) {
            int pos = base[ai][gk] + rank;
            for (int w2 = ai; w2 < warp; w2 += NA) pos += cnt[w2][gk];
            list[ai][pos] = ent;
        }
        __syncthreads();
        // Phase C: accumulate, bucket index known at compile time.
        if (angle_ok && yok) {
            const float *xb = x + y0;
#pragma unroll
            for (int gg = 0; gg < NG; gg++) {
                const int e1 = base[ai][gg + 1];
                for (int i = base[ai][gg]; i < e1; i++) {
                    const float4 e = list[ai][i];
                    float v[VEC];
                    ldv<VEC>(xb + (size_t)__float_as_int(e.x) * A.ys, v);
                    if (gg >= 2) {
#pragma unroll
                        for (int c = 0; c < VEC; c++) acc[gg >= 2 ? gg - 2 : 0][c] =
                            fmaf(e.y, v[c], acc[gg >= 2 ? gg - 2 : 0][c]);
                    }
                    if (gg >= 1 && gg <= BT) {
#pragma unroll
                        for (int c = 0; c < VEC; c++) acc[(gg >= 1 && gg <= BT) ? gg - 1 : 0][c] =
                            fmaf(e.z, v[c], acc[(gg >= 1 && gg <= BT) ? gg - 1 : 0][c]);
                    }
                    if (gg <= BT - 1) {
#pragma unroll
                        for (int c = 0; c < VEC; c++) acc[gg <= BT - 1 ? gg : 0][c] =
                            fmaf(e.w, v[c], acc[gg <= BT - 1 ? gg : 0][c]);
                    }
                }
            }
        }
        __syncthreads();
    }

    double s2 = 0.0;
    if (angle_ok && yok) {
        const int a = G.x + ai;
        float *qa = q + (size_t)a * A.nx * A.ys + y0;
#pragma unroll
        for (int j = 0; j < BT; j++) {
            if (b0 + j < A.nx) {
                stv<VEC>(qa + (size_t)(b0 + j) * A.ys, acc[j]);
#pragma unroll
                for (int c = 0; c < VEC; c++) s2 += (double)__fmul_rn(acc[j][c], acc[j][c]);
            }
        }
    }
    block_sum_to<NWARP>(s2, red, A.partials + (size_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// ---------------------------------------------------------------------------
// Forward projection for the linear weighting.  Its ray coordinates are the
// reference's shifted table entries (not a pixel grid), so the strip sweep does
// not apply; this path scatters with atomics.  It exists for parity with
// pmethod=1, not for speed; its float summation order is not fixed.
template <int VEC>
__global__ void __launch_bounds__(256) fp_lin_kernel(OpArgs A, const float *__restrict__ x,
                                                     float *__restrict__ q) {
    if (A.skip && *A.skip) return;
    const int nvec = A.ys / VEC;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)A.nrays * nvec) return;
    const int k = (int)(t / nvec), y0 = (int)(t % nvec) * VEC;
    float v[VEC];
    ldv<VEC>(x + (size_t)k * A.ys + y0, v);
    bool any = false;
#pragma unroll
    for (int c = 0; c < VEC; c++) any |= v[c] != 0.f;
    if (!any) return;
    const float4 ray = A.ray[k];
    for (int a = 0; a < A.na; a++) {
        const Taps tp = ray_taps<ARECGB_LIN>(ray, A.ang[a], A.r_hi, A.r_lo);
        float *qa = q + (size_t)a * A.nx * A.ys + y0;
        const int b = tp.iqx - 1;
        if ((unsigned)b < (unsigned)A.nx)
#pragma unroll
            for (int c = 0; c < VEC; c++) atomicAdd(qa + (size_t)b * A.ys + c, tp.w0 * v[c]);
        if ((unsigned)(b + 1) < (unsigned)A.nx)
#pragma unroll
            for (int c = 0; c < VEC; c++) atomicAdd(qa + (size_t)(b + 1) * A.ys + c, tp.w1 * v[c]);
    }
}

}  // namespace arecgb

namespace arecgb {

// Launch helpers, instantiated once per weighting in arec_project_{lin,kb,sq}.cu.
template <int W>
int launch_bp(const OpArgs &A, int vec, int nsc, dim3 grid, const float *s, float *g,
              cudaStream_t st) {
#define ARECGB_BP(V, N)                                                        \
    if (vec == V && nsc == N) {                                                \
        bp_kernel<W, V, N><<<grid, 128 * N, 0, st>>>(A, s, g);                 \
        return 0;                                                              \
    }
    ARECGB_BP(1, 1) ARECGB_BP(2, 1) ARECGB_BP(4, 1) ARECGB_BP(8, 1)
    ARECGB_BP(1, 2) ARECGB_BP(2, 2) ARECGB_BP(4, 2) ARECGB_BP(8, 2)
#undef ARECGB_BP
    return -1;
}

template <int W, int BT>
int launch_fp(const OpArgs &A, int vec, int nsc, dim3 grid, const float *x, float *q,
              cudaStream_t st) {
    if constexpr (W == ARECGB_LIN) {
        (void)nsc;
        (void)grid;
        const long long n = (long long)A.nrays * (A.ys / vec);
        const unsigned blocks = (unsigned)((n + 255) / 256);
        if (vec == 1) fp_lin_kernel<1><<<blocks, 256, 0, st>>>(A, x, q);
        else if (vec == 2) fp_lin_kernel<2><<<blocks, 256, 0, st>>>(A, x, q);
        else if (vec == 4) fp_lin_kernel<4><<<blocks, 256, 0, st>>>(A, x, q);
        else fp_lin_kernel<8><<<blocks, 256, 0, st>>>(A, x, q);
        return 0;
    } else {
#define ARECGB_FP(V, N)                                                                   \
    if (vec == V && nsc == N) {                                                           \
        fp_kernel<W, V, N, BT><<<grid, 32 * kGroupAngles * N, 0, st>>>(A, x, q);          \
        return 0;                                                                         \
    }
        ARECGB_FP(1, 1) ARECGB_FP(2, 1) ARECGB_FP(4, 1) ARECGB_FP(8, 1)
        ARECGB_FP(1, 2) ARECGB_FP(2, 2) ARECGB_FP(4, 2) ARECGB_FP(8, 2)
#undef ARECGB_FP
        return -1;
    }
}

}  // namespace arecgb
