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
//   scatters.  Here each output is owned by one block per launch (no atomics): a
//   block owns a group of up to 4 consecutive angles, a tile of BT detector bins
//   and 256 slices, and gathers the rays of the strip of the cylinder that
//   projects into the tile.  The strip is swept line by line (rows when
//   |cos| >= |sin|, columns otherwise, so consecutive pixels move <= 1 bin and a
//   line holds <= 32 candidates), and the sweep is split into bands of lines,
//   one launch per (orientation, band) adding into q, so that the concurrently
//   running blocks read one band of x from L2.  Candidates arrive in centre-bin
//   order, so the accumulation loop runs over a compile-time bucket index and
//   each loaded pixel feeds up to 3 register accumulators.
//
// Both kernels evaluate the identical ray_taps<W>() so A and A^T are exact
// transposes of each other.  The back projector fuses the FP64 sum of squares
// of its output (one partial per block, reduced in a fixed order afterwards);
// the forward projector's is a separate pass over q.
#pragma once

#include <cuda.h>  // CUtensorMap (the forward projector's row tiles)

#include <climits>

#include "arec_umma.cuh"
#include "arec_weights.cuh"

namespace arecgb {

struct OpArgs {
    const float4 *ray;
    const AngleParams *ang;
    const RowInfo *rows;
    const ColInfo *cols;
    const int4 *groups;
    const int2 *tiles;
    int nx, nrays, ys, na, ngroups;
    float r_hi, r_lo;
    double *partials;
    const int *skip;
    int *err;
    // linear weighting: per angle, the rays grouped by first bin (lin_off
    // [na][nx+2]: bucket j holds the rays whose first bin is j - 1; lin_list
    // [na][nrays]: ray indices, ascending within a bucket)
    const int *lin_off;
    const int *lin_list;
    // optional per-plan tables (null when the plan has none)
    const float4 *taps;  // [ngroups][nrays][4]: ray_taps of each forward-projection angle
                         // group's (up to 4) angles per ray: (iqx, w0, w1, w2)
    const float4 *bpw;   // [ntiles][na][32]: the back projector's plan entries
    const int2 *bpf;     // [ntiles][na]: footprint (first bin, bins) per tile and angle
    const int *kinv;     // column-major ray index -> ray index
};

// A 2-D tensor map over rows of ys floats (x or its column-major copy): box =
// box_cols slices x box_rows rays; false if the CUDA driver refuses it.
bool encode_rows_map(CUtensorMap *m, const float *base, int ys, int nrows, int box_cols,
                     int box_rows);
// A 3-D tensor map over a sinogram [na][nx][ys] (device layout): box =
// box_cols slices x box_bins bins x 1 angle; false if the CUDA driver refuses it.
bool encode_sino_map(CUtensorMap *m, const float *base, int ys, int nx, int na, int box_cols,
                     int box_bins);

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

// Slices held by a lane: VEC/4 float4 pieces at c*128 + lane*4 for VEC >= 4
// (consecutive lanes read consecutive 16-byte pieces: conflict-free shared
// memory and fully coalesced global rows), lane*VEC otherwise.
template <int VEC>
__device__ __forceinline__ int lane_piece(int lane, int c) {
    return VEC >= 4 ? c * 128 + lane * 4 : lane * VEC;
}

template <int VEC>
__device__ __forceinline__ void lds_lane(const float *base, int lane, float (&v)[VEC]) {
    if constexpr (VEC >= 4) {
#pragma unroll
        for (int c = 0; c < VEC / 4; c++) {
            const float4 t = *reinterpret_cast<const float4 *>(base + lane_piece<VEC>(lane, c));
            v[4 * c] = t.x; v[4 * c + 1] = t.y; v[4 * c + 2] = t.z; v[4 * c + 3] = t.w;
        }
    } else if constexpr (VEC == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(base + lane * 2);
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = base[lane];
    }
}

// Store a lane's slices; pieces at or beyond `limit` (slices left in the row)
// are skipped.  Pieces are whole: limits are multiples of 8.
template <int VEC>
__device__ __forceinline__ void stg_lane(float *base, int lane, const float (&v)[VEC], int limit) {
    if constexpr (VEC >= 4) {
#pragma unroll
        for (int c = 0; c < VEC / 4; c++) {
            const int o = lane_piece<VEC>(lane, c);
            if (o < limit)
                *reinterpret_cast<float4 *>(base + o) =
                    make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
        }
    } else if constexpr (VEC == 2) {
        if (lane * 2 < limit) *reinterpret_cast<float2 *>(base + lane * 2) = make_float2(v[0], v[1]);
    } else {
        if (lane < limit) base[lane] = v[0];
    }
}

constexpr uint32_t kFpWait = 1u << 20;  // mbarrier polls before a wait gives up (a row lands in ~1 us)

template <int VEC>
__device__ __forceinline__ void add_lane(float *base, int lane, const float (&v)[VEC], int limit) {
    if constexpr (VEC >= 4) {
#pragma unroll
        for (int c = 0; c < VEC / 4; c++) {
            const int o = lane_piece<VEC>(lane, c);
            if (o < limit) {
                float4 *d = reinterpret_cast<float4 *>(base + o);
                float4 t = *d;
                t.x += v[4 * c];
                t.y += v[4 * c + 1];
                t.z += v[4 * c + 2];
                t.w += v[4 * c + 3];
                *d = t;
            }
        }
    } else if constexpr (VEC == 2) {
        if (lane * 2 < limit) {
            float2 *d = reinterpret_cast<float2 *>(base + lane * 2);
            float2 t = *d;
            t.x += v[0];
            t.y += v[1];
            *d = t;
        }
    } else {
        if (lane < limit) base[lane] += v[0];
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

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// 16-byte global -> shared copy, zero-filled when !valid (cp.async, sm_80+).
__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
    const unsigned n = valid ? 16u : 0u;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// lds_lane when `pred` is nonzero, else the registers keep their values: a
// predicated shared-memory load (no branch, no bandwidth when off).  VEC >= 4.
// `a` is the shared-memory address of the lane's first piece (lane_piece(lane,
// 0)); the second piece of VEC = 8 is 128 floats further.
template <int VEC>
__device__ __forceinline__ void lds_lane_if(unsigned pred, unsigned a, float (&v)[VEC]) {
    static_assert(VEC == 4 || VEC == 8, "one or two float4 pieces");
    if constexpr (VEC == 8) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %8, 0;\n\t"
            "@p ld.shared.v4.f32 {%0, %1, %2, %3}, [%9];\n\t"
            "@p ld.shared.v4.f32 {%4, %5, %6, %7}, [%9+512];\n\t}\n"
            : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]),
              "+f"(v[7])
            : "r"(pred), "r"(a));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
            "@p ld.shared.v4.f32 {%0, %1, %2, %3}, [%5];\n\t}\n"
            : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3])
            : "r"(pred), "r"(a));
    }
}

// One staged footprint row (a bin's slices) into a lane's registers; a bin off
// the detector was never copied and reads as zero.
template <int VEC>
__device__ __forceinline__ void foot_row(const float *row, bool on, int lane, float (&v)[VEC]) {
    if (on) {
        lds_lane<VEC>(row, lane, v);
    } else {
#pragma unroll
        for (int q = 0; q < VEC; q++) v[q] = 0.f;
    }
}

// acc += w * v element-wise, in pairs on the packed FP32 FMA (each lane of the
// pair is fmaf(w, v, acc), rounded once).
template <int VEC>
__device__ __forceinline__ void fma_row(float (&acc)[VEC], float w, const float (&v)[VEC]) {
    if constexpr (VEC >= 2) {
        const float2 w2 = make_float2(w, w);
#pragma unroll
        for (int q = 0; q < VEC; q += 2) {
            const float2 r = __ffma2_rn(w2, make_float2(v[q], v[q + 1]),
                                        make_float2(acc[q], acc[q + 1]));
            acc[q] = r.x;
            acc[q + 1] = r.y;
        }
    } else {
        acc[0] = fmaf(w, v[0], acc[0]);
    }
}

constexpr int kBpAngles = 32;  // angles per weight chunk
constexpr int kBpFoot = 12;    // staged footprint width in bins (an 8x4 tile spans <= 11)

constexpr int kBpBuf = 3;  // footprint buffers in flight

// The back projector's plan for one angle of one 8x4-pixel tile; lanes = the
// tile's 32 rays (lane = 8 * row + pixel; has: the lane's pixel is a ray of
// the cylinder).  The accumulating warp of each row of 8 rays keeps the three
// bins b .. b+2 of its current ray in a register ring; the plan says, per
// ray, which ring slot takes which footprint row (the centre bin moves by at
// most one bin between neighbouring pixels) and rotates the weights to the
// slots.  Entry (code, wa, wb, wc): code bits 0-2 the slots that load (0: the
// ray keeps the ring, or is skipped with zero weights; one bit: one row enters
// that slot; 7: three rows enter slots 0, 1, 2), bits 8+ footprint row of the
// (first) row entering; wa, wb, wc the weights of slots 0, 1, 2.
// Also the tile's footprint: first bin fb and bins spanned fn (<= FW; wide:
// the taps reach further, an impossible case reported by the caller).
template <int W, int FW>
__device__ __forceinline__ float4 bp_plan(const OpArgs &A, const float4 &myray, bool has,
                                          const AngleParams &ap, int lane, int &fb, int &fn,
                                          bool &wide) {
    Taps t{};
    int b = INT_MIN / 2, lo = INT_MAX, hi = INT_MIN;
    if (has) {
        t = ray_taps<W>(myray, ap, A.r_hi, A.r_lo);
        b = lo = hi = t.iqx - 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    const bool use = b != INT_MIN / 2 && b - lo <= FW - 3;
    if (!use) t.w0 = t.w1 = t.w2 = 0.f;  // code 0: the ray adds nothing
    const int gbase = lane & ~7;
    int cb = INT_MIN / 4, m = 0, my_code = 0, my_m = 0;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int br = __shfl_sync(0xffffffffu, b, gbase + r);
        const int ur = __shfl_sync(0xffffffffu, (int)use, gbase + r);
        int code = 0;
        if (ur) {
            const int d = br - cb, rr = br - lo;
            if (d == 0) {
                code = 0;
            } else if (d == 1) {  // bin cb (slot m) leaves, bin br + 2 enters
                code = (1 << m) | ((rr + 2) << 8);
                m = m == 2 ? 0 : m + 1;
            } else if (d == -1) {  // bin cb + 2 leaves, bin br enters
                m = m == 0 ? 2 : m - 1;
                code = (1 << m) | (rr << 8);
            } else {
                code = 7 | (rr << 8);
                m = 0;
            }
            cb = br;
        }
        if ((lane & 7) == r) {
            my_code = code;
            my_m = m;
        }
    }
    wide = hi - lo + 3 > FW && lo != INT_MAX;
    fb = lo == INT_MAX ? 0 : lo;
    fn = lo == INT_MAX ? 0 : min(FW, hi - lo + 3);
    // slot s holds bin b + ((s - m) mod 3): its weight is w_{(s - m) mod 3}
    const float wa = my_m == 0 ? t.w0 : (my_m == 1 ? t.w2 : t.w1);
    const float wb = my_m == 0 ? t.w1 : (my_m == 1 ? t.w0 : t.w2);
    const float wc = my_m == 0 ? t.w2 : (my_m == 1 ? t.w1 : t.w0);
    return make_float4(__int_as_float(my_code), wa, wb, wc);
}

__device__ __forceinline__ int tile_lane_ray(const OpArgs &A, int2 tile, int lane) {
    const int ix = tile.x + (lane & (kTileX - 1)), iz = tile.y + lane / kTileX;
    int k = -1;
    if (iz < A.nx) {
        const RowInfo ri = A.rows[iz];
        if (ix >= ri.lo && ix <= ri.hi) k = ri.start + ix - ri.lo;
    }
    return k;
}

// Plan tables: the back projector's entries for every (tile, angle) (one warp
// each) and the taps of every (angle group, ray, angle of the group), the rays
// in the group's line order (row-major for row sweeps, column-major for
// column sweeps): the staged pixels of a line are one contiguous record.
static_assert(kGroupAngles == 4, "the taps table holds 4 angles per group");
template <int W, int FW>
__global__ void __launch_bounds__(128) k_bp_table(OpArgs A, float4 *bpw, int2 *bpf) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x, a = blockIdx.y * 4 + warp;
    if (a >= A.na) return;  // whole warp
    const int k = tile_lane_ray(A, A.tiles[tile], lane);
    const float4 myray = k >= 0 ? A.ray[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    int f0, f1;
    bool wide;
    bpw[((size_t)tile * A.na + a) * 32 + lane] = bp_plan<W, FW>(A, myray, k >= 0, A.ang[a], lane, f0, f1, wide);
    if (lane == 0) {
        bpf[(size_t)tile * A.na + a] = make_int2(f0, f1);
        if (wide) atomicOr(A.err, 2);
    }
}

template <int W>
__global__ void __launch_bounds__(256) k_fp_taps(OpArgs A, float4 *taps) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)A.ngroups * A.nrays * 4) return;
    const int j = (int)(t & 3);
    const size_t gk = t >> 2;
    const int grp = (int)(gk / A.nrays), k = (int)(gk % A.nrays);
    const int4 G = A.groups[grp];
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < G.y) {
        // the group's line order: row-major rays for row sweeps, column-major
        // for column sweeps (k here indexes that order)
        const int kr = G.z ? A.kinv[k] : k;
        const Taps tp = ray_taps<W>(A.ray[kr], A.ang[G.x + j], A.r_hi, A.r_lo);
        e = make_float4(__int_as_float(tp.iqx), tp.w0, tp.w1, tp.w2);
    }
    taps[t] = e;
}

template <int VEC, int NSC>
constexpr size_t bp_smem_bytes() {
    return sizeof(float) * kBpBuf * kBpFoot * (NSC * 32 * VEC) + sizeof(float4) * kBpAngles * 32 +
           sizeof(int) * 2 * kBpAngles + sizeof(double) * (4 * NSC);
}

// Stage angle ai of the chunk (footprint first bin fb, bins fn) into buffer
// buf, completing on `full`; one whole warp calls it.  TMA: the footprint as
// one tile of FW bins x SPAN slices (bins off the detector are outside the
// tensor and read as zero).  Otherwise one bulk copy per bin, bins off the
// detector zero-filled, so the accumulating warps load every row they plan.
// `ok` false: arrive without copying (a wait gave up; nothing waits forever).
template <int FW, int SPAN>
__device__ __forceinline__ void bp_stage(const OpArgs &A, const float *__restrict__ s, float *dst,
                                         uint64_t *full, const CUtensorMap *tms, bool use_tma,
                                         int angle, int fb, int fn, int yb, uint32_t row_bytes,
                                         bool ok, int lane) {
    // order this block's earlier generic reads of the buffer before the copy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (use_tma) {
        if (lane == 0) {
            const bool any = ok && fn > 0;
            umma::mbar_arrive_expect_tx(full, any ? (uint32_t)(FW * SPAN * 4) : 0u);
            if (any) umma::tma_load_3d(dst, tms, yb, fb, angle, full);
        }
        __syncwarp();
        return;
    }
    const size_t ys = (size_t)A.ys;
    const int bin = fb + lane;
    const bool in = ok && lane < fn;
    const bool on = in && (unsigned)bin < (unsigned)A.nx;
    const unsigned m = __ballot_sync(0xffffffffu, on);
    unsigned off = __ballot_sync(0xffffffffu, in && !on);
    if (off) {
        for (; off; off &= off - 1) {
            float4 *z = reinterpret_cast<float4 *>(dst + (size_t)(__ffs(off) - 1) * SPAN);
            for (int c = lane; c < SPAN / 4; c += 32) z[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        // order these generic stores before later bulk copies into the rows
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncwarp();  // zero rows written before the arrival (release)
    if (lane == 0) umma::mbar_arrive_expect_tx(full, (uint32_t)__popc(m) * row_bytes);
    __syncwarp();
    if (on)
        umma::bulk_g2s(dst + (size_t)lane * SPAN, s + ((size_t)angle * A.nx + bin) * ys + yb,
                       row_bytes, full);
}

// Square-pixel and Kaiser-Bessel weightings.  Block = 4*NSC accumulating warps
// (8 rays x 32*VEC slices each).  Per chunk of 32 angles the tile's ray plans
// (lanes = rays) are copied from the plan table (or computed) into shared
// memory; the footprint of each angle (the bins the tile's taps reach, <= 12,
// each a row of the block's slices) is staged into one of three buffers:
// warp 0 primes the first three angles of the chunk, and the warp that
// releases a buffer last (a shared counter per buffer) refills it with the
// angle three ahead, completing on the buffer's "full" mbarrier.  No staging
// warp, so 4 blocks fit per SM.  Each warp walks its 8 rays through a
// three-row register ring (one shared-memory row read per ray instead of
// three).  Bins off the detector add nothing, as the reference skips them.
template <int W, int VEC, int NSC>
__global__ void __launch_bounds__(128 * NSC, NSC == 1 ? 4 : 1)
    bp_kernel(OpArgs A, const float *__restrict__ s, float *__restrict__ g,
              const __grid_constant__ CUtensorMap tms, int use_tma) {
    constexpr int NCW = 4 * NSC, AC = kBpAngles, FW = kBpFoot, NB = kBpBuf;
    constexpr int SPAN = NSC * 32 * VEC;  // slices per block
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[NB];
    __shared__ int released[NB];  // warps done with the buffer, cumulative
    float *foot = reinterpret_cast<float *>(smem_raw);               // [NB][FW][SPAN]
    float4 *sw = reinterpret_cast<float4 *>(foot + NB * FW * SPAN);  // [AC][32]
    int *fb = reinterpret_cast<int *>(sw + AC * 32);                 // [AC] first bin
    int *fn = fb + AC;                                               // [AC] bins spanned
    double *red = reinterpret_cast<double *>(fn + AC);               // [NCW]
    if (A.skip && *A.skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = tile_lane_ray(A, A.tiles[blockIdx.x], lane);
    const float4 myray = k >= 0 && !A.bpw ? A.ray[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int rg = warp & 3, sc = warp >> 2;
    const int yb = blockIdx.y * SPAN;                  // first slice of the block
    const int yw = sc * 32 * VEC;                        // this warp's slices within the block
    const bool yok = yb + yw + lane_piece<VEC>(lane, 0) < A.ys;
    const size_t ys = (size_t)A.ys;
    const uint32_t row_bytes = (uint32_t)min(SPAN, A.ys - yb) * 4u;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int b = 0; b < NB; b++) {
            umma::mbar_init(&full[b], 1);
            released[b] = 0;
        }
        umma::mbar_fence_init();
    }

    float acc[8][VEC];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int q = 0; q < VEC; q++) acc[r][q] = 0.f;
    // the register ring; zero until a ray loads it (finite for zero weights)
    float R0[VEC], R1[VEC], R2[VEC];
#pragma unroll
    for (int q = 0; q < VEC; q++) R0[q] = R1[q] = R2[q] = 0.f;

    bool ok = true;
    int t0 = 0;  // angles staged before this chunk (buffer t % NB, use t / NB)
    for (int a0 = 0; a0 < A.na; a0 += AC) {
        const int nac = min(AC, A.na - a0);
        if (A.bpw) {
            // the plan's precomputed entries for this tile and chunk
            const float4 *src = A.bpw + ((size_t)blockIdx.x * A.na + a0) * 32;
            for (int i = threadIdx.x; i < nac * 32; i += blockDim.x) cp_async16(sw + i, src + i, true);
            cp_async_commit();
            for (int i = threadIdx.x; i < nac; i += blockDim.x) {
                const int2 f = A.bpf[(size_t)blockIdx.x * A.na + a0 + i];
                fb[i] = f.x;
                fn[i] = f.y;
            }
            cp_async_wait<0>();
        } else {
            for (int ai = warp; ai < AC; ai += NCW) {
                const int a = a0 + ai;
                int f0, f1;
                bool wide;
                sw[ai * 32 + lane] =
                    bp_plan<W, FW>(A, myray, a < A.na && k >= 0, A.ang[min(a, A.na - 1)], lane,
                                   f0, f1, wide);
                if (lane == 0) {
                    if (wide) atomicOr(A.err, 2);
                    fb[ai] = f0;
                    fn[ai] = f1;
                }
            }
        }
        __syncthreads();  // plans and footprint bases of this chunk (barriers initialised)
        if (warp == 0) {
            for (int ai = 0; ai < min(NB, nac); ai++) {
                const int buf = (t0 + ai) % NB;
                bp_stage<FW, SPAN>(A, s, foot + (size_t)buf * FW * SPAN, &full[buf], &tms,
                                   use_tma != 0, a0 + ai, fb[ai], fn[ai], yb, row_bytes, ok, lane);
            }
        }
        for (int ai = 0; ai < nac; ai++) {
            const int t = t0 + ai, buf = t % NB;
            if (ok && !umma::mbar_wait(&full[buf], (uint32_t)(t / NB) & 1u, kFpWait)) {
                ok = false;
                if (lane == 0) atomicOr(A.err, 16);
            }
            if (ok && yok) {
                const float *F = foot + (size_t)buf * FW * SPAN + yw;
                // the ring (slots 0, 1, 2); a warp's first used ray loads all three
                if constexpr (VEC >= 4) {
                    // branch-free: each slot's load is predicated on its bit of
                    // the plan's code; skipped rays have zero weights (and the
                    // ring holds finite staged values), so their FMAs add nothing
                    const unsigned Fa = smem_u32(F + lane_piece<VEC>(lane, 0));
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const float4 e = sw[ai * 32 + rg * 8 + r];
                        const unsigned code = (unsigned)__float_as_int(e.x), mask = code & 7u;
                        const unsigned a = Fa + (code >> 8) * (SPAN * 4u);
                        const unsigned step = mask == 7u ? SPAN * 4u : 0u;
                        lds_lane_if<VEC>(mask & 1u, a, R0);
                        lds_lane_if<VEC>(mask & 2u, a + step, R1);
                        lds_lane_if<VEC>(mask & 4u, a + 2 * step, R2);
                        fma_row<VEC>(acc[r], e.y, R0);
                        fma_row<VEC>(acc[r], e.z, R1);
                        fma_row<VEC>(acc[r], e.w, R2);
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const float4 e = sw[ai * 32 + rg * 8 + r];
                        const int code = __float_as_int(e.x), mask = code & 7;
                        const float *row = F + (code >> 8) * SPAN;
                        if (mask == 7) {
                            lds_lane<VEC>(row, lane, R0);
                            lds_lane<VEC>(row + SPAN, lane, R1);
                            lds_lane<VEC>(row + 2 * SPAN, lane, R2);
                        } else if (mask == 1) {
                            lds_lane<VEC>(row, lane, R0);
                        } else if (mask == 2) {
                            lds_lane<VEC>(row, lane, R1);
                        } else if (mask == 4) {
                            lds_lane<VEC>(row, lane, R2);
                        }
                        fma_row<VEC>(acc[r], e.y, R0);
                        fma_row<VEC>(acc[r], e.z, R1);
                        fma_row<VEC>(acc[r], e.w, R2);
                    }
                }
            }
            __syncwarp();  // this warp's reads of the buffer are done
            // the last of the NCW warps to release the buffer refills it
            int last = 0;
            if (lane == 0) last = (atomicAdd(&released[buf], 1) + 1) % NCW == 0;
            last = __shfl_sync(0xffffffffu, last, 0);
            if (last && ai + NB < nac)
                bp_stage<FW, SPAN>(A, s, foot + (size_t)buf * FW * SPAN, &full[buf], &tms,
                                   use_tma != 0, a0 + ai + NB, fb[ai + NB], fn[ai + NB], yb,
                                   row_bytes, ok, lane);
        }
        t0 += nac;
        __syncthreads();  // the chunk's plans are no longer read
    }
    if (!ok) {
        // a wait gave up: let the copies still in flight land before the block exits
        for (int t = max(0, t0 - NB); t < t0; t++)
            umma::mbar_wait(&full[t % NB], (uint32_t)(t / NB) & 1u, kFpWait);
    }

    double s2 = 0.0;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int kr = __shfl_sync(0xffffffffu, k, rg * 8 + r);
        if (kr >= 0 && yok) {
            stg_lane<VEC>(g + (size_t)kr * ys + yb + yw, lane, acc[r], A.ys - (yb + yw));
#pragma unroll
            for (int q = 0; q < VEC; q++) s2 += (double)__fmul_rn(acc[r][q], acc[r][q]);
        }
    }
    block_sum_to<NCW>(s2, red, A.partials + (size_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// Linear weighting: its ray coordinates are the reference's shifted table
// entries, so a tile's footprint is not compact; this kernel reads the
// sinogram directly (parity path).
template <int VEC, int NSC>
__global__ void __launch_bounds__(128 * NSC)
    bp_lin_kernel(OpArgs A, const float *__restrict__ s, float *__restrict__ g) {
    constexpr int NT = 128 * NSC, NWARP = NT / 32, AC = 32;
    __shared__ float4 sw[AC][32];
    __shared__ double red[NWARP];
    if (A.skip && *A.skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = tile_lane_ray(A, A.tiles[blockIdx.x], lane);
    const float4 myray = k >= 0 && !A.bpw ? A.ray[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int rg = warp & 3, sc = warp >> 2;
    const int y0 = (blockIdx.y * NSC + sc) * 32 * VEC + lane * VEC;
    const bool yok = y0 < A.ys;
    const size_t ys = (size_t)A.ys;
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
                const Taps t = ray_taps<ARECGB_LIN>(myray, A.ang[a], A.r_hi, A.r_lo);
                e = make_float4(__int_as_float(t.iqx - 1), t.w0, t.w1, 0.f);
            }
            sw[ai][lane] = e;
        }
        __syncthreads();
        const int nac = min(AC, A.na - a0);
        if (yok) {
            for (int ai = 0; ai < nac; ai++) {
                const float *sa = s + (size_t)(a0 + ai) * A.nx * ys + y0;
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    const float4 e = sw[ai][rg * 8 + r];
                    const int b0 = __float_as_int(e.x);
#pragma unroll
                    for (int j = 0; j < 2; j++) {
                        const int b = b0 + j;
                        const float w = j == 0 ? e.y : e.z;
                        if ((unsigned)b < (unsigned)A.nx) {
                            float v[VEC];
                            ldv<VEC>(sa + (size_t)b * ys, v);
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
            stv<VEC>(g + (size_t)kr * ys + y0, acc[r]);
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

constexpr int kFpStage = 32;  // staged pixels per line: the union of the group's candidates
constexpr int kFpBox = 8;     // rays per TMA box: a line stages ceil(n / 8) boxes

// Candidate pixel range [clo, chi] on line li for one angle: pixels whose
// centre bin may fall in [b0-1, b0+BT] (a margin of one pixel each side; the
// exact test is the centre bin itself).
__device__ __forceinline__ void line_candidates(const OpArgs &A, int orient, float ca, float cl,
                                                float T1, float T2, float r, int li, int &clo,
                                                int &chi) {
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
    const float Lv = (float)li - r;
    float pa = (T1 - Lv * cl) / ca, pb = (T2 - Lv * cl) / ca;
    if (pa > pb) {
        const float t = pa;
        pa = pb;
        pb = t;
    }
    clo = max(plo, (int)floorf(pa + r) - 1);
    chi = min(phi, (int)ceilf(pb + r) + 1);
}

__device__ __forceinline__ int line_pixel_ray(const OpArgs &A, int orient, int li, int p) {
    if (orient == 0) {
        const RowInfo ri = A.rows[li];
        return ri.start + p - ri.lo;
    }
    const RowInfo ri = A.rows[p];
    return ri.start + li - ri.lo;
}

// ---------------------------------------------------------------------------
// Banded forward projection (square-pixel and Kaiser-Bessel weightings).
//
// One launch takes the angle groups of one sweep orientation and the lines
// [band_lo, band_hi) of their strips (rows for orientation 0, columns for 1),
// and ADDS its partial sums to q, which is zeroed first.  All blocks of a
// launch then read x from one band of the cylinder (band lines x nx pixels x
// the block's slices: 64 MB for 64 lines of 1024 pixels and 256 slices), which
// stays in L2, instead of every angle group streaming the whole volume from
// DRAM.  Launches run in a fixed order on one stream, so the result does not
// depend on timing.
//
// Block = 4 angle warps + 1 staging warp.  The staging warp runs up to two
// lines ahead: per line it stages the union of the group's candidate pixels
// into one of two buffers, completing on that buffer's "full" mbarrier.  With
// the plan's tables the pixels of a line are consecutive rays in the line's
// order, so the line is one 2-D TMA tile of x (or of its column-major copy)
// plus one bulk copy of their taps, and every line's staging is worked out
// before the line loop (lanes = lines); without tables, one bulk copy per
// pixel row and ray-table entry.  Each angle warp takes the taps of the
// staged rows (lanes = rows, ordered by increasing centre bin), compacts the
// rows whose centre bin falls in the tile (a contiguous run: the centre bin
// is monotonic along a line; a counting sort covers any exception) into
// per-bucket slots, accumulates them with the bucket index known at compile
// time (straight-line code when every bucket holds an entry), and arrives on
// the buffer's "empty" mbarrier.  No block-wide barrier inside the line loop;
// every wait is bounded and a timeout sets an error flag.
constexpr int kFpMaxBand = 128;  // lines per band launch at most (the staging info per line)

template <int VEC>
constexpr size_t fpb_smem_bytes() {
    return sizeof(float) * 2 * kFpStage * (32 * VEC) + sizeof(float4) * kGroupAngles * 32 +
           sizeof(float4) * 2 * kFpStage * kGroupAngles + sizeof(int) * (2 * kGroupAngles + 4) +
           sizeof(int2) * kFpMaxBand;
}

constexpr int kFpThreads = 32 * (kGroupAngles + 1);

// One staged pixel's contribution to the tile: bucket GG (centre bin b0+GG-1)
// adds w0, w1, w2 times the pixel's slices to bins GG-2, GG-1, GG of the tile.
// GG is a constant once the caller's bucket loop is unrolled, so the
// accumulator rows stay in registers.
template <int VEC, int BT>
__device__ __forceinline__ void fp_entry(float (&acc)[BT][VEC], const int GG, const float4 e,
                                         const float *S, int lane) {
    float v[VEC];
    lds_lane<VEC>(S + (__float_as_int(e.x) & 255) * (32 * VEC), lane, v);
    if (GG >= 2) fma_row<VEC>(acc[GG >= 2 ? GG - 2 : 0], e.y, v);
    if (GG >= 1 && GG <= BT) fma_row<VEC>(acc[(GG >= 1 && GG <= BT) ? GG - 1 : 0], e.z, v);
    if (GG <= BT - 1) fma_row<VEC>(acc[GG <= BT - 1 ? GG : 0], e.w, v);
}

template <int W, int VEC, int BT>
__global__ void __launch_bounds__(kFpThreads, 3)
    fp_band_kernel(OpArgs A, const float *__restrict__ x, float *__restrict__ q, int g0, int ngo,
                   int band_lo, int band_hi, const __grid_constant__ CUtensorMap tmx,
                   const __grid_constant__ CUtensorMap tmxT) {
    constexpr int NA = kGroupAngles, NG = BT + 2, SPAN = 32 * VEC, US = kFpStage;
    static_assert(NG <= 16, "two slot rows of 16 buckets per warp list");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[2], empty[2];
    float *stg = reinterpret_cast<float *>(smem_raw);                // [2][US][SPAN]
    float4 *list = reinterpret_cast<float4 *>(stg + 2 * US * SPAN);  // [NA][32]
    // [2][US][NA]: per staged row its ray-table entry (slot 0), or with the
    // plan's taps table the taps of the group's NA angles
    float4 *rayb = list + NA * 32;
    int *lrange = reinterpret_cast<int *>(rayb + 2 * US * NA);       // [NA][2]
    int *uinfo = lrange + 2 * NA;                                    // [2][2] (first pixel, rows)
    int2 *linfo = reinterpret_cast<int2 *>(uinfo + 4);               // [band lines] (first ray, rows)
    if (A.skip && *A.skip) return;
    if (band_hi - band_lo > kFpMaxBand) {  // the host keeps bands within kFpMaxBand lines
        if (threadIdx.x == 0) atomicOr(A.err, 1);
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool stager = warp == NA;
    const int ai = stager ? 0 : warp;
    const int grp = g0 + blockIdx.x % ngo, b0 = (blockIdx.x / ngo) * BT;
    const int4 G = A.groups[grp];
    const int orient = G.z;
    const float r = A.r_hi + A.r_lo;
    const float T1 = (float)b0 - 1.5f - 0.02f - r;
    const float T2 = (float)(b0 + BT) + 0.5f + 0.02f - r;
    const float R = r + 1.5f;
    const int yb = blockIdx.y * SPAN;
    const size_t ys = (size_t)A.ys;
    const uint32_t row_bytes = (uint32_t)min(SPAN, A.ys - yb) * 4u;
    const bool angle_ok = !stager && ai < G.y;
    AngleParams ap;
    float ca = 1.f, cl = 0.f;
    if (angle_ok) {
        ap = A.ang[G.x + ai];
        ca = orient ? ap.s : ap.c;
        cl = orient ? ap.c : ap.s;
    }
    if (!stager && lane == 0) {
        int lo = INT_MAX, hi = INT_MIN;
        float lmin, lmax;
        if (angle_ok && strip_line_extent(ca, cl, T1, T2, R, lmin, lmax)) {
            lo = max(band_lo, max(0, (int)floorf(lmin + r) - 1));
            hi = min(band_hi - 1, min(A.nx - 1, (int)ceilf(lmax + r) + 1));
        }
        lrange[2 * ai] = lo;
        lrange[2 * ai + 1] = hi;
    }
    if (threadIdx.x == 0) {
        umma::mbar_init(&full[0], 1);
        umma::mbar_init(&full[1], 1);
        umma::mbar_init(&empty[0], NA);
        umma::mbar_init(&empty[1], NA);
        umma::mbar_fence_init();
    }
    __syncthreads();
    int L0 = INT_MAX, L1 = INT_MIN;
#pragma unroll
    for (int i = 0; i < NA; i++) {
        L0 = min(L0, lrange[2 * i]);
        L1 = max(L1, lrange[2 * i + 1]);
    }
    if (L0 > L1) return;  // the strip misses this band (uniform over the block)
    bool ok = true;

    if (stager) {
        // lanes < NA: the angles' sweep cosines for the candidate ranges
        float cq = 1.f, lq = 0.f;
        int q_lo = INT_MAX, q_hi = INT_MIN;
        if (lane < G.y) {
            const AngleParams aq = A.ang[G.x + lane];
            cq = orient ? aq.s : aq.c;
            lq = orient ? aq.c : aq.s;
            q_lo = lrange[2 * lane];
            q_hi = lrange[2 * lane + 1];
        }
        if (A.taps) {
            // With the plan's tables every line's staging (first ray of the
            // union of the group's candidates, rows) is worked out up front,
            // lanes = lines, so the per-line loop below carries no dependent
            // chain of loads, divisions and shuffles.
            float ck[NA], lk[NA];
            int klo[NA], khi[NA];
#pragma unroll
            for (int i = 0; i < NA; i++) {
                ck[i] = 1.f;
                lk[i] = 0.f;
                klo[i] = INT_MAX;
                khi[i] = INT_MIN;
                if (i < G.y) {
                    const AngleParams aq = A.ang[G.x + i];
                    ck[i] = orient ? aq.s : aq.c;
                    lk[i] = orient ? aq.c : aq.s;
                    klo[i] = lrange[2 * i];
                    khi[i] = lrange[2 * i + 1];
                }
            }
            for (int li = L0 + lane; li <= L1; li += 32) {
                int clo = INT_MAX, chi = INT_MIN;
#pragma unroll
                for (int i = 0; i < NA; i++) {
                    if (li < klo[i] || li > khi[i]) continue;
                    int c0, c1;
                    line_candidates(A, orient, ck[i], lk[i], T1, T2, r, li, c0, c1);
                    if (c0 <= c1) {
                        clo = min(clo, c0);
                        chi = max(chi, c1);
                    }
                }
                int n = chi >= clo ? chi - clo + 1 : 0;
                if (n > US) {
                    atomicOr(A.err, 1);
                    n = US;
                }
                int j0 = 0;
                if (n) {
                    if (orient == 0) {
                        const RowInfo ri = A.rows[li];
                        j0 = ri.start + clo - ri.lo;
                    } else {
                        const ColInfo ci = A.cols[li];
                        j0 = ci.start + clo - ci.lo;
                    }
                }
                linfo[li - L0] = make_int2(j0, n);
            }
            __syncwarp();
            for (int li = L0; li <= L1; li++) {
                const int it = li - L0, buf = it & 1;
                const int2 lf = linfo[it];
                if (it >= 2 && ok &&
                    !umma::mbar_wait(&empty[buf], (uint32_t)((it - 2) >> 1) & 1u, kFpWait)) {
                    ok = false;
                    if (lane == 0) atomicOr(A.err, 16);
                }
                // the staged pixels of a line are consecutive rays in the
                // line's order: ceil(n / 8) tiles of 8 rays x SPAN slices from
                // x (row sweeps) or its column-major copy (column sweeps), and
                // one contiguous taps record
                const int n = ok ? lf.y : 0;  // a wait gave up: stage nothing more
                const int nbox = (n + kFpBox - 1) / kFpBox;
                if (lane == 0) {
                    uinfo[2 * buf + 1] = n;
                    __threadfence_block();  // counts before the arrival
                    umma::mbar_arrive_expect_tx(
                        &full[buf],
                        n ? (uint32_t)(nbox * kFpBox * SPAN * 4 + n * 16 * NA) : 0u);
                }
                __syncwarp();
                if (lane < nbox)
                    umma::tma_load_2d(stg + ((size_t)buf * US + lane * kFpBox) * SPAN,
                                      orient ? &tmxT : &tmx, yb, lf.x + lane * kFpBox, &full[buf]);
                if (lane == 0 && n)
                    umma::bulk_g2s(rayb + buf * US * NA, A.taps + ((size_t)grp * A.nrays + lf.x) * NA,
                                   (uint32_t)n * 16u * NA, &full[buf]);
                __syncwarp();
            }
            return;
        }
        for (int li = L0; li <= L1; li++) {
            const int it = li - L0, buf = it & 1;
            int clo = INT_MAX, chi = INT_MIN;
            if (lane < NA && li >= q_lo && li <= q_hi) {
                line_candidates(A, orient, cq, lq, T1, T2, r, li, clo, chi);
                if (clo > chi) {
                    clo = INT_MAX;
                    chi = INT_MIN;
                }
            }
#pragma unroll
            for (int o = 1; o < NA; o <<= 1) {
                clo = min(clo, __shfl_xor_sync(0xffffffffu, clo, o));
                chi = max(chi, __shfl_xor_sync(0xffffffffu, chi, o));
            }
            const int ulo = __shfl_sync(0xffffffffu, clo, 0);
            const int uhi = __shfl_sync(0xffffffffu, chi, 0);
            int n = uhi >= ulo ? uhi - ulo + 1 : 0;
            if (n > US) {
                if (lane == 0) atomicOr(A.err, 1);
                n = US;
            }
            if (it >= 2 && ok &&
                !umma::mbar_wait(&empty[buf], (uint32_t)((it - 2) >> 1) & 1u, kFpWait)) {
                ok = false;
                if (lane == 0) atomicOr(A.err, 16);
            }
            if (!ok) n = 0;  // a wait gave up: stage nothing more
            const int k = lane < n ? line_pixel_ray(A, orient, li, ulo + lane) : 0;
            if (lane == 0) {
                uinfo[2 * buf] = ulo;
                uinfo[2 * buf + 1] = n;
                __threadfence_block();  // counts before the arrival
                umma::mbar_arrive_expect_tx(&full[buf], (uint32_t)n * (row_bytes + 16u));
            }
            __syncwarp();
            if (lane < n) {
                umma::bulk_g2s(stg + ((size_t)buf * US + lane) * SPAN, x + (size_t)k * ys + yb,
                               row_bytes, &full[buf]);
                umma::bulk_g2s(rayb + (buf * US + lane) * NA, A.ray + k, 16u, &full[buf]);
            }
        }
        return;
    }

    const int my_lo = lrange[2 * ai], my_hi = lrange[2 * ai + 1];
    float acc[BT][VEC];
#pragma unroll
    for (int j = 0; j < BT; j++)
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[j][v] = 0.f;

    for (int li = L0; li <= L1; li++) {
        const int it = li - L0, buf = it & 1;
        if (ok && !umma::mbar_wait(&full[buf], (uint32_t)(it >> 1) & 1u, kFpWait)) {
            ok = false;
            if (lane == 0) atomicOr(A.err, 16);
        }
        const int un = ok ? uinfo[2 * buf + 1] : 0;
        // Phase A: lanes = staged rows in increasing centre-bin order for this angle.
        bool valid = false;
        int gk = 0;
        float4 ent = make_float4(0.f, 0.f, 0.f, 0.f);
        if (angle_ok && lane < un && li >= my_lo && li <= my_hi) {
            const int row = ca > 0.f ? lane : un - 1 - lane;
            Taps t;
            if (A.taps) {
                const float4 tt = rayb[(buf * US + row) * NA + ai];
                t.iqx = __float_as_int(tt.x);
                t.w0 = tt.y;
                t.w1 = tt.z;
                t.w2 = tt.w;
            } else {
                t = ray_taps<W>(rayb[(buf * US + row) * NA], ap, A.r_hi, A.r_lo);
            }
            gk = t.iqx - b0 + 1;
            valid = gk >= 0 && gk <= BT + 1;
            ent = make_float4(__int_as_float(row | (gk << 8)), t.w0, t.w1, t.w2);
        }
        // Phase B: compaction.  Expected: the valid lanes are one run with
        // non-decreasing centre bins; otherwise a stable counting sort.
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const int cnt = __popc(vm);
        const int f = vm ? __ffs(vm) - 1 : 0;
        const int gprev = __shfl_up_sync(0xffffffffu, gk, 1);
        const bool run = vm == 0 || (vm >> f) == (cnt == 32 ? 0xffffffffu : (1u << cnt) - 1u);
        const bool sorted = run && !__any_sync(0xffffffffu, valid && lane > f && gk < gprev);
        // Slots: with the entries in bucket order and at most two per bucket
        // (the rule whenever pixels on a line step by >= 0.5 bin; sweep
        // orientations keep |step| >= 0.707), entry k of bucket g goes to slot
        // [k][g] of the warp's list, so the accumulation below walks a fixed
        // bucket sequence without a data-dependent loop.
        const unsigned firsts =
            __ballot_sync(0xffffffffu, valid && (lane == f || gk != gprev));
        const int rank = lane - (31 - __clz(firsts & ((2u << lane) - 1u)));
        const bool slots = sorted && !__any_sync(0xffffffffu, valid && rank > 1);
        const unsigned maskA = __reduce_or_sync(0xffffffffu, valid && rank == 0 ? 1u << gk : 0u);
        const unsigned maskB = __reduce_or_sync(0xffffffffu, valid && rank == 1 ? 1u << gk : 0u);
        if (slots) {
            if (valid) list[ai * 32 + rank * 16 + gk] = ent;
        } else if (sorted) {
            if (valid) list[ai * 32 + lane - f] = ent;
        } else {
            const unsigned key = valid ? (unsigned)gk : 64u + lane;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const int rank = __popc(peers & ((1u << lane) - 1u));
            int mybase = 0;
#pragma unroll
            for (int gg = 0; gg <= NG; gg++) {
                const int c = __popc(__ballot_sync(0xffffffffu, valid && gk < gg));
                if (valid && gg == gk) mybase = c;
            }
            if (valid) list[ai * 32 + mybase + rank] = ent;
        }
        __syncwarp();
        // Phase C: entries in bucket order; the bucket index is a compile-time
        // constant.  In the slot layout a line that fills every bucket (the
        // usual case: the strip crosses the whole line) runs as straight-line
        // code, so the loads of later buckets overlap the FMAs of earlier ones.
        if (slots) {
            const float *S = stg + (size_t)buf * US * SPAN;
            const float4 *E = list + ai * 32;
            if (maskA == (1u << NG) - 1u) {
#pragma unroll
                for (int gg = 0; gg < NG; gg++) fp_entry<VEC, BT>(acc, gg, E[gg], S, lane);
            } else {
#pragma unroll
                for (int gg = 0; gg < NG; gg++)
                    if (maskA >> gg & 1u) fp_entry<VEC, BT>(acc, gg, E[gg], S, lane);
            }
            if (maskB) {
#pragma unroll
                for (int gg = 0; gg < NG; gg++)
                    if (maskB >> gg & 1u) fp_entry<VEC, BT>(acc, gg, E[16 + gg], S, lane);
            }
        } else if (cnt) {
            // Each entry's slices are loaded as it is reached (a prefetch into
            // a second register set cost more in register moves than it saved).
            const float *S = stg + (size_t)buf * US * SPAN;
            const float4 *E = list + ai * 32;
            int i = 0;
            float4 e = E[0];
#pragma unroll
            for (int gg = 0; gg < NG; gg++) {
                while (i < cnt && (__float_as_int(e.x) >> 8) == gg) {
                    float v[VEC];
                    lds_lane<VEC>(S + (__float_as_int(e.x) & 255) * SPAN, lane, v);
                    const float4 ec = e;
                    i++;
                    if (i < cnt) e = E[i];
                    if (gg >= 2) fma_row<VEC>(acc[gg >= 2 ? gg - 2 : 0], ec.y, v);
                    if (gg >= 1 && gg <= BT)
                        fma_row<VEC>(acc[(gg >= 1 && gg <= BT) ? gg - 1 : 0], ec.z, v);
                    if (gg <= BT - 1) fma_row<VEC>(acc[gg <= BT - 1 ? gg : 0], ec.w, v);
                }
            }
        }
        __syncwarp();  // this warp's reads of the buffer and of its list are done
        if (lane == 0) umma::mbar_arrive(&empty[buf]);
    }
    if (!ok) {
        // a wait gave up: let the copies still in flight land before the block exits
        for (int it = max(0, L1 - L0 - 1); it <= L1 - L0; it++)
            umma::mbar_wait(&full[it & 1], (uint32_t)(it >> 1) & 1u, kFpWait);
        return;
    }
    if (angle_ok) {
        float *qa = q + (size_t)(G.x + ai) * A.nx * ys + yb;
#pragma unroll
        for (int j = 0; j < BT; j++)
            if (b0 + j < A.nx) add_lane<VEC>(qa + (size_t)(b0 + j) * ys, lane, acc[j], A.ys - yb);
    }
}

// ---------------------------------------------------------------------------
// Forward projection for the linear weighting.  Its ray coordinates are the
// reference's shifted table entries (not a pixel grid), so the strip sweep does
// not apply.  With the plan's ray index (k_lin_index) each output bin gathers
// its rays in a fixed order (fp_lin_gather, deterministic); without it this
// kernel scatters with atomics, whose float summation order is not fixed.
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

// The linear weighting's ray index, one thread per angle: count the rays of
// each first bin b0 = iqx - 1 in [-1, nx - 1] (the rays that reach the
// detector), prefix sums, then place the rays in ascending order (a second
// pass, the offsets advancing as cursors and shifted back afterwards).  The
// first bins come from the projectors' own ray_taps, so the gather below and
// the back projector use identical coefficients.
static __global__ void __launch_bounds__(64) k_lin_index(OpArgs A, int *off, int *list) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A.na) return;
    const int nb = A.nx + 1;  // buckets j = b0 + 1
    int *o = off + (size_t)a * (nb + 1);
    int *l = list + (size_t)a * A.nrays;
    const AngleParams ap = A.ang[a];
    for (int j = 0; j <= nb; j++) o[j] = 0;
    for (int k = 0; k < A.nrays; k++) {
        const int j = ray_taps<ARECGB_LIN>(A.ray[k], ap, A.r_hi, A.r_lo).iqx;  // b0 + 1
        if (j >= 0 && j < nb) o[j + 1]++;
    }
    for (int j = 1; j <= nb; j++) o[j] += o[j - 1];
    for (int k = 0; k < A.nrays; k++) {
        const int j = ray_taps<ARECGB_LIN>(A.ray[k], ap, A.r_hi, A.r_lo).iqx;
        if (j >= 0 && j < nb) l[o[j]++] = k;
    }
    for (int j = nb; j > 0; j--) o[j] = o[j - 1];  // o[j] was the end of bucket j
    o[0] = 0;
}

// Linear weighting, gather: one warp per (angle, bin, slice chunk); bin b
// takes w0 of the rays whose first bin is b, then w1 of those whose first bin
// is b - 1, each in ascending ray order, as the reference's per-ray products
// added in float (arecproject.cpp:75-95).
template <int VEC>
__global__ void __launch_bounds__(256) fp_lin_gather(OpArgs A, const float *__restrict__ x,
                                                     float *__restrict__ q) {
    if (A.skip && *A.skip) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * 8 + warp;
    const int nchunk = (A.ys + 32 * VEC - 1) / (32 * VEC);
    if (gw >= (long long)A.na * A.nx * nchunk) return;
    const int c = (int)(gw % nchunk);
    const int b = (int)((gw / nchunk) % A.nx);
    const int a = (int)(gw / ((long long)nchunk * A.nx));
    const int y0 = c * 32 * VEC + lane * VEC;
    const bool yok = y0 < A.ys;
    const int *o = A.lin_off + (size_t)a * (A.nx + 2);
    const int *l = A.lin_list + (size_t)a * A.nrays;
    const AngleParams ap = A.ang[a];
    float acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = 0.f;
#pragma unroll
    for (int t = 0; t < 2; t++) {
        const int j = b + 1 - t;  // t = 0: first bin b (w0); t = 1: first bin b - 1 (w1)
        const int e = o[j + 1];
        for (int i = o[j]; i < e; i++) {
            const int k = l[i];
            const Taps tp = ray_taps<ARECGB_LIN>(A.ray[k], ap, A.r_hi, A.r_lo);
            const float w = t == 0 ? tp.w0 : tp.w1;
            if (yok) {
                float v[VEC];
                ldv<VEC>(x + (size_t)k * A.ys + y0, v);
#pragma unroll
                for (int u = 0; u < VEC; u++) acc[u] = __fadd_rn(acc[u], __fmul_rn(w, v[u]));
            }
        }
    }
    if (yok) stv<VEC>(q + ((size_t)a * A.nx + b) * A.ys + y0, acc);
}

}  // namespace arecgb

namespace arecgb {

// Launch helpers, instantiated once per weighting in arec_project_{lin,kb,sq}.cu.
template <int W, int V, int N>
int launch_bp_one(const OpArgs &A, dim3 grid, const float *s, float *g, const CUtensorMap &tms,
                  int use_tma, cudaStream_t st) {
    if constexpr (W == ARECGB_LIN) {
        bp_lin_kernel<V, N><<<grid, 128 * N, 0, st>>>(A, s, g);
    } else {
        constexpr size_t smem = bp_smem_bytes<V, N>();
        static bool configured = false;  // per instantiation, once per process
        if (!configured) {
            if (cudaFuncSetAttribute(bp_kernel<W, V, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem) != cudaSuccess)
                return -2;
            configured = true;
        }
        bp_kernel<W, V, N><<<grid, 128 * N, smem, st>>>(A, s, g, tms, use_tma);
    }
    return 0;
}

template <int W>
int launch_bp(const OpArgs &A, int vec, int nsc, dim3 grid, const float *s, float *g,
              const CUtensorMap &tms, int use_tma, cudaStream_t st) {
#define ARECGB_BP(V, N) \
    if (vec == V && nsc == N) return launch_bp_one<W, V, N>(A, grid, s, g, tms, use_tma, st);
    ARECGB_BP(1, 1) ARECGB_BP(2, 1) ARECGB_BP(4, 1) ARECGB_BP(8, 1)
    ARECGB_BP(1, 2) ARECGB_BP(2, 2) ARECGB_BP(4, 2) ARECGB_BP(8, 2)
#undef ARECGB_BP
    return -1;
}

// x in column-major ray order: xT[j] = x[kinv[j]] (rows of ys floats).
static __global__ void __launch_bounds__(256) k_ray_gather(const float4 *__restrict__ x,
                                                    float4 *__restrict__ xT,
                                                    const int *__restrict__ kinv, int nrays,
                                                    int ys4) {
    const size_t n = (size_t)nrays * ys4;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t j = t / ys4;
        const int c = (int)(t - j * ys4);
        xT[t] = x[(size_t)kinv[j] * ys4 + c];
    }
}

// The plan's tables for weighting W (one launch each).
template <int W>
int launch_tables(const OpArgs &A, int ntiles, float4 *taps, float4 *bpw, int2 *bpf,
                  cudaStream_t st) {
    const size_t n = (size_t)A.ngroups * A.nrays * 4;
    k_fp_taps<W><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A, taps);
    k_bp_table<W, kBpFoot><<<dim3(ntiles, (A.na + 3) / 4), 128, 0, st>>>(A, bpw, bpf);
    return 0;
}

template <int W, int V, int BT>
int launch_fpb_one(const OpArgs &A, dim3 grid, const float *x, float *q, int g0, int ngo, int lo,
                   int hi, const CUtensorMap &tmx, const CUtensorMap &tmxT, cudaStream_t st) {
    constexpr size_t smem = fpb_smem_bytes<V>();
    static bool configured = false;  // per instantiation, once per process
    if (!configured) {
        if (cudaFuncSetAttribute(fp_band_kernel<W, V, BT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return -2;
        configured = true;
    }
    fp_band_kernel<W, V, BT><<<grid, kFpThreads, smem, st>>>(A, x, q, g0, ngo, lo, hi, tmx, tmxT);
    return 0;
}

template <int W, int BT>
int launch_fpb(const OpArgs &A, int vec, dim3 grid, const float *x, float *q, int g0, int ngo,
               int lo, int hi, const CUtensorMap &tmx, const CUtensorMap &tmxT, cudaStream_t st) {
    if (vec == 1) return launch_fpb_one<W, 1, BT>(A, grid, x, q, g0, ngo, lo, hi, tmx, tmxT, st);
    if (vec == 2) return launch_fpb_one<W, 2, BT>(A, grid, x, q, g0, ngo, lo, hi, tmx, tmxT, st);
    if (vec == 4) return launch_fpb_one<W, 4, BT>(A, grid, x, q, g0, ngo, lo, hi, tmx, tmxT, st);
    return launch_fpb_one<W, 8, BT>(A, grid, x, q, g0, ngo, lo, hi, tmx, tmxT, st);
}

// Linear weighting: the gather when the plan has its ray index, else the
// scatter (q zeroed by the caller either way).
template <int W>
int launch_fp(const OpArgs &A, int vec, const float *x, float *q, cudaStream_t st) {
    static_assert(W == ARECGB_LIN, "the other weightings use the banded kernel");
    if (A.lin_off && A.lin_list) {
        const long long nw = (long long)A.na * A.nx * ((A.ys + 32 * vec - 1) / (32 * vec));
        const unsigned blocks = (unsigned)((nw + 7) / 8);
        if (vec == 1) fp_lin_gather<1><<<blocks, 256, 0, st>>>(A, x, q);
        else if (vec == 2) fp_lin_gather<2><<<blocks, 256, 0, st>>>(A, x, q);
        else if (vec == 4) fp_lin_gather<4><<<blocks, 256, 0, st>>>(A, x, q);
        else fp_lin_gather<8><<<blocks, 256, 0, st>>>(A, x, q);
        return 0;
    }
    const long long n = (long long)A.nrays * (A.ys / vec);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (vec == 1) fp_lin_kernel<1><<<blocks, 256, 0, st>>>(A, x, q);
    else if (vec == 2) fp_lin_kernel<2><<<blocks, 256, 0, st>>>(A, x, q);
    else if (vec == 4) fp_lin_kernel<4><<<blocks, 256, 0, st>>>(A, x, q);
    else fp_lin_kernel<8><<<blocks, 256, 0, st>>>(A, x, q);
    return 0;
}

}  // namespace arecgb
