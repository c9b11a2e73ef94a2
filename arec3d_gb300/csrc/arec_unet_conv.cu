// 3x3 convolution (stride 1, zero padding 1) as an implicit GEMM on the
// 5th-generation tensor cores: tcgen05.mma (BF16 x BF16 -> FP32 in TMEM).
//
//   Y[p][co] = act( bias[co] + sum_{tap, ci} X[p + tap][ci] * Wt[co][tap][ci] )
//
// X, Y: NHWC bf16 ([P = n*H*W pixels][C]); Wt: [Cout][9][Cin] bf16.
// A block owns 128 consecutive pixels (GEMM M = 128) and all Cout output
// channels (GEMM N = Cout in {32, 64, 128, 256}); K = 9*Cin runs in chunks of
// 32 channels of one tap.  Per chunk, 128 threads gather the A slab (the 128
// pixels' shifted neighbours, zeros outside the image) and the B slab (weights)
// into shared memory in the tensor core's K-major layout; one thread issues two
// tcgen05.mma (K = 16 each) into the TMEM accumulator and commits them to the
// stage's mbarrier, so the next chunk's gather overlaps the MMAs (two stages).
// The epilogue reads TMEM with tcgen05.ld (warp w: pixels 32w..32w+31), adds
// the bias, applies ReLU and stores bf16.
//
// The same kernel computes the data gradient of a convolution from the
// spatially flipped, channel-transposed weights.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's entry point)
#include <cuda_bf16.h>
#include <stdint.h>

#include <mutex>

#include "arec_internal.cuh"
#include "arec_umma.cuh"

namespace arecgb {

constexpr int kConvKC = 32;          // input channels per K chunk
constexpr uint32_t kWaitLimit = 4u << 20;

template <int COUT>
struct ConvCfg {
    static constexpr int A_BYTES = 128 * kConvKC * 2;  // 8 KB
    static constexpr int B_BYTES = COUT * kConvKC * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int SMEM = 2 * STAGE;
    static constexpr uint32_t NCOLS = COUT < 32 ? 32 : COUT;
};

// byte offset of element (row, k) (k < 32) in a K-major no-swizzle slab with
// `rows` rows: two MMA slabs (K = 16 each) of rows/8 core-matrix groups.
__device__ __forceinline__ int kmaj_offset(int row, int kpiece /*0..3, 8 elements*/, int rows) {
    const int s = kpiece >> 1, j = kpiece & 1;
    return s * (rows / 8) * 256 + (row >> 3) * 256 + j * 128 + (row & 7) * 16;
}

template <int COUT, int LBO, int SBO>
__global__ void __launch_bounds__(128)
    conv3x3_umma_kernel(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ Wt,
                        const float *__restrict__ bias, __nv_bfloat16 *__restrict__ Y, int H,
                        int Wd, int Cin, int P, int relu, int ystride, int *err) {
    using Cfg = ConvCfg<COUT>;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int p0 = blockIdx.x * 128;

    if (warp == 0) {
        umma::tmem_alloc(&tmem_base, Cfg::NCOLS);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        umma::mbar_init(&mbar[0], 1);
        umma::mbar_init(&mbar[1], 1);
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;

    // this thread's pixel (row of A)
    const int p = p0 + tid;
    const bool pvalid = p < P;
    const int hw = H * Wd;
    const int n = p / hw, h = (p / Wd) % H, w = p % Wd;
    const int cchunks = Cin / kConvKC;
    const int nchunks = 9 * cchunks;
    constexpr uint32_t idesc = umma::idesc_bf16(128, COUT);
    bool ok = true;

    for (int c = 0; c < nchunks; c++) {
        const int st = c & 1;
        if (c >= 2 && ok) {
            if (!umma::mbar_wait(&mbar[st], ((c - 2) >> 1) & 1, kWaitLimit)) ok = false;
        }
        unsigned char *A = sm + st * Cfg::STAGE;
        unsigned char *B = A + Cfg::A_BYTES;
        const int tap = c / cchunks, c0 = (c % cchunks) * kConvKC;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        // A: pixel tid, its neighbour at (dy, dx), channels c0..c0+31 (4 x 16 B)
        {
            const int hh = h + dy, ww = w + dx;
            const bool inside = pvalid && hh >= 0 && hh < H && ww >= 0 && ww < Wd;
            const uint4 *src = reinterpret_cast<const uint4 *>(
                X + ((size_t)n * hw + (size_t)(inside ? hh : 0) * Wd + (inside ? ww : 0)) * Cin + c0);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                uint4 v = inside ? __ldg(src + q) : make_uint4(0, 0, 0, 0);
                *reinterpret_cast<uint4 *>(A + kmaj_offset(tid, q, 128)) = v;
            }
        }
        // B: weights Wt[co][tap][c0..c0+31]
        for (int i = tid; i < COUT * 4; i += 128) {
            const int co = i >> 2, q = i & 3;
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(
                Wt + ((size_t)co * 9 + tap) * Cin + c0 + q * 8));
            *reinterpret_cast<uint4 *>(B + kmaj_offset(co, q, COUT)) = v;
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (tid == 0 && ok) {
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint64_t ad = umma::smem_desc(umma::smem_addr(A + s * (128 / 8) * 256), LBO, SBO);
                const uint64_t bd =
                    umma::smem_desc(umma::smem_addr(B + s * (COUT / 8) * 256), LBO, SBO);
                umma::mma_bf16(tmem, ad, bd, idesc, (c > 0 || s > 0) ? 1u : 0u);
            }
            umma::mma_commit(&mbar[st]);
        }
    }
    // all MMAs done (the last commit covers every earlier MMA of the issuing thread)
    if (nchunks > 0 && ok) {
        const int last = nchunks - 1;
        if (!umma::mbar_wait(&mbar[last & 1], (last >> 1) & 1, kWaitLimit)) ok = false;
    }
    if (!ok && lane == 0) atomicOr(err, 4);
    umma::fence_after_sync();

    // epilogue: warp w reads TMEM lanes 32w.. (pixels p0 + 32w + lane)
    if (ok) {
#pragma unroll 1
        for (int cc = 0; cc < COUT / 32; cc++) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(cc * 32), v);
            if (pvalid) {
                __align__(16) __nv_bfloat16 out[32];
#pragma unroll
                for (int i = 0; i < 32; i++) {
                    float t = v[i] + (bias ? bias[cc * 32 + i] : 0.f);
                    if (relu) t = fmaxf(t, 0.f);
                    out[i] = __float2bfloat16(t);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(Y + (size_t)p * ystride + cc * 32);
#pragma unroll
                for (int q = 0; q < 4; q++) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, Cfg::NCOLS);
}

template <int COUT, int LBO, int SBO>
static int launch_conv(const __nv_bfloat16 *X, const __nv_bfloat16 *Wt, const float *bias,
                       __nv_bfloat16 *Y, int H, int Wd, int Cin, int P, int relu, int ystride,
                       int *err, cudaStream_t st) {
    using Cfg = ConvCfg<COUT>;
    static bool configured = false;
    if (!configured) {
        ARECGB_CUDA(cudaFuncSetAttribute(conv3x3_umma_kernel<COUT, LBO, SBO>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
        configured = true;
    }
    conv3x3_umma_kernel<COUT, LBO, SBO><<<(P + 127) / 128, 128, Cfg::SMEM, st>>>(
        X, Wt, bias, Y, H, Wd, Cin, P, relu, ystride, err);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// TMA path (image widths that are multiples of 128): a tile is 128 consecutive
// pixels of one image row.  Per K chunk (one tap, 32 input channels) one TMA
// load brings the tile's shifted neighbours from an NHWC tensor map (box 32
// channels x 128 pixels; rows and columns outside the image arrive as zeros,
// which is the convolution's padding) and one the chunk's weights from a
// [Cout][9][Cin] tensor map, both with the 64-byte swizzle the tensor core
// reads directly.  Four stages: thread 0 of warp 0 issues the loads, thread 0
// of warp 1 the MMAs; each stage's commit frees it for the loads four chunks
// later.  All four warps run the epilogue from TMEM.
//
// A block lives a few microseconds (9 or 18 chunks, each waiting on an L2
// load), so throughput comes from blocks resident per SM: the narrow layers
// take two stages (21-25 KB of shared memory: 8-10 blocks per SM within the
// 512 TMEM columns), the wide ones four.
template <int COUT>
struct TmaCfg {
    static constexpr int STAGES = COUT <= 64 ? 2 : 4;
    static constexpr int A_BYTES = 128 * 64;  // 128 pixels x 32 channels
    static constexpr int B_BYTES = COUT * 64;
    static constexpr int STAGE = A_BYTES + B_BYTES;  // a multiple of 1024
    static constexpr int SMEM = STAGES * STAGE + 1024;
    static constexpr uint32_t NCOLS = COUT < 32 ? 32 : COUT;
};

template <int COUT>
__global__ void __launch_bounds__(128)
    conv3x3_tma_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW,
                       const float *__restrict__ bias, __nv_bfloat16 *__restrict__ Y, int H,
                       int Wd, int Cin, int relu, int ystride, int *err) {
    using Cfg = TmaCfg<COUT>;
    extern __shared__ unsigned char sm_raw[];
    __shared__ __align__(8) uint64_t full[Cfg::STAGES], empty[Cfg::STAGES], done;
    __shared__ uint32_t tmem_base;
    const uint32_t raw = umma::smem_addr(sm_raw);
    unsigned char *sm = sm_raw + ((1024u - (raw & 1023u)) & 1023u);  // 1024-byte aligned stages
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int p0 = blockIdx.x * 128;
    const int hw = H * Wd;
    const int n = p0 / hw, h = (p0 / Wd) % H, w0 = p0 % Wd;

    if (warp == 0) {
        umma::tmem_alloc(&tmem_base, Cfg::NCOLS);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        for (int st = 0; st < Cfg::STAGES; st++) {
            umma::mbar_init(&full[st], 1);
            umma::mbar_init(&empty[st], 1);
        }
        umma::mbar_init(&done, 1);
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const int cchunks = Cin / kConvKC, nchunks = 9 * cchunks;

    if (warp == 0 && lane == 0) {
        bool ok = true;
        for (int c = 0; c < nchunks && ok; c++) {
            const int st = c % Cfg::STAGES;
            if (c >= Cfg::STAGES &&
                !umma::mbar_wait(&empty[st], (uint32_t)(c / Cfg::STAGES - 1) & 1u, kWaitLimit)) {
                ok = false;
                atomicOr(err, 4);
                break;
            }
            const int tap = c / cchunks, c0 = (c % cchunks) * kConvKC;
            unsigned char *A = sm + st * Cfg::STAGE;
            umma::mbar_arrive_expect_tx(&full[st], (uint32_t)Cfg::STAGE);
            umma::tma_load_4d(A, &tmX, c0, w0 + tap % 3 - 1, h + tap / 3 - 1, n, &full[st]);
            umma::tma_load_3d(A + Cfg::A_BYTES, &tmW, c0, tap, 0, &full[st]);
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = umma::idesc_bf16(128, COUT);
        for (int c = 0; c < nchunks; c++) {
            const int st = c % Cfg::STAGES;
            if (!umma::mbar_wait(&full[st], (uint32_t)(c / Cfg::STAGES) & 1u, kWaitLimit)) {
                atomicOr(err, 4);
                break;
            }
            umma::fence_after_sync();
            const uint32_t a = umma::smem_addr(sm + st * Cfg::STAGE), b = a + Cfg::A_BYTES;
#pragma unroll
            for (int k = 0; k < 2; k++)
                umma::mma_bf16(tmem, umma::smem_desc_sw64(a + 32 * k),
                               umma::smem_desc_sw64(b + 32 * k), idesc, (c > 0 || k > 0) ? 1u : 0u);
            umma::mma_commit(&empty[st]);
        }
        umma::mma_commit(&done);  // arrives when every MMA above has completed
    }
    __syncwarp();
    const bool dok = __all_sync(0xffffffffu, umma::mbar_wait(&done, 0, kWaitLimit));
    umma::fence_after_sync();
    if (!dok && lane == 0) atomicOr(err, 4);
    if (dok) {
        const int p = p0 + tid;  // TMEM lane = pixel
#pragma unroll 1
        for (int cc = 0; cc < COUT / 32; cc++) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(cc * 32), v);
            __align__(16) __nv_bfloat16 out[32];
#pragma unroll
            for (int i = 0; i < 32; i++) {
                float t = v[i] + (bias ? bias[cc * 32 + i] : 0.f);
                if (relu) t = fmaxf(t, 0.f);
                out[i] = __float2bfloat16(t);
            }
            uint4 *dst = reinterpret_cast<uint4 *>(Y + (size_t)p * ystride + cc * 32);
#pragma unroll
            for (int q = 0; q < 4; q++) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, Cfg::NCOLS);
}

// Several output rows per block (TMA path, narrow layers): R consecutive rows
// of one image x 128 pixels x COUT channels, one accumulator per row in TMEM
// (R x COUT columns).  K runs over (column shift dx, 32-channel chunk): one
// TMA box brings the R + 2 input rows the R output rows need, shifted by dx
// (rows outside the image arrive as zeros), and three more the weights of
// the taps (dy, dx), dy = 0, 1, 2; output row r then takes input row r + dy
// with tap (dy, dx).  Each input row is loaded 3 (R + 2) / R times per output
// row instead of 9 times, and a block's fixed costs are shared by R rows.
template <int COUT, int R>
struct RowsCfg {
    static constexpr int STAGES = 2;
    static constexpr int A_ROW = 128 * 64;              // one input row tile: 128 px x 32 ch
    static constexpr int A_BYTES = (R + 2) * A_ROW;
    static constexpr int B_TAP = COUT * 64;             // one tap's weights for 32 channels
    static constexpr int STAGE = A_BYTES + 3 * B_TAP;   // a multiple of 1024
    static constexpr int SMEM = STAGES * STAGE + 1024;
    static constexpr uint32_t NCOLS = R * COUT;          // a power of two in [32, 512]
};

template <int COUT, int R>
__global__ void __launch_bounds__(128)
    conv3x3_rows_kernel(const __grid_constant__ CUtensorMap tmX,
                        const __grid_constant__ CUtensorMap tmW, const float *__restrict__ bias,
                        __nv_bfloat16 *__restrict__ Y, int H, int Wd, int Cin, int relu,
                        int ystride, int *err) {
    using Cfg = RowsCfg<COUT, R>;
    static_assert(Cfg::NCOLS >= 32 && Cfg::NCOLS <= 512 && (Cfg::NCOLS & (Cfg::NCOLS - 1)) == 0,
                  "TMEM columns: a power of two in [32, 512]");
    static_assert(Cfg::STAGE % 1024 == 0, "stages stay 1024-byte aligned");
    extern __shared__ unsigned char sm_raw[];
    __shared__ __align__(8) uint64_t full[Cfg::STAGES], empty[Cfg::STAGES], done;
    __shared__ uint32_t tmem_base;
    const uint32_t raw = umma::smem_addr(sm_raw);
    unsigned char *sm = sm_raw + ((1024u - (raw & 1023u)) & 1023u);  // 1024-byte aligned stages
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wtiles = Wd / 128, hgroups = H / R;
    const int b = blockIdx.x;
    const int wt = b % wtiles, hg = (b / wtiles) % hgroups, n = b / (wtiles * hgroups);
    const int h0 = hg * R, w0 = wt * 128;

    if (warp == 0) {
        umma::tmem_alloc(&tmem_base, Cfg::NCOLS);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        for (int st = 0; st < Cfg::STAGES; st++) {
            umma::mbar_init(&full[st], 1);
            umma::mbar_init(&empty[st], 1);
        }
        umma::mbar_init(&done, 1);
        umma::mbar_fence_init();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const int cchunks = Cin / kConvKC, nchunks = 3 * cchunks;  // (dx, channel chunk)

    if (warp == 0 && lane == 0) {
        for (int c = 0; c < nchunks; c++) {
            const int st = c % Cfg::STAGES;
            if (c >= Cfg::STAGES &&
                !umma::mbar_wait(&empty[st], (uint32_t)(c / Cfg::STAGES - 1) & 1u, kWaitLimit)) {
                atomicOr(err, 4);
                break;
            }
            const int dx = c / cchunks, c0 = (c % cchunks) * kConvKC;
            unsigned char *A = sm + st * Cfg::STAGE;
            umma::mbar_arrive_expect_tx(&full[st], (uint32_t)Cfg::STAGE);
            umma::tma_load_4d(A, &tmX, c0, w0 + dx - 1, h0 - 1, n, &full[st]);
#pragma unroll
            for (int dy = 0; dy < 3; dy++)
                umma::tma_load_3d(A + Cfg::A_BYTES + dy * Cfg::B_TAP, &tmW, c0, 3 * dy + dx, 0,
                                  &full[st]);
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = umma::idesc_bf16(128, COUT);
        for (int c = 0; c < nchunks; c++) {
            const int st = c % Cfg::STAGES;
            if (!umma::mbar_wait(&full[st], (uint32_t)(c / Cfg::STAGES) & 1u, kWaitLimit)) {
                atomicOr(err, 4);
                break;
            }
            umma::fence_after_sync();
            const uint32_t a = umma::smem_addr(sm + st * Cfg::STAGE), bw = a + Cfg::A_BYTES;
#pragma unroll
            for (int r = 0; r < R; r++)
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                    for (int k = 0; k < 2; k++)
                        umma::mma_bf16(tmem + (uint32_t)(r * COUT),
                                       umma::smem_desc_sw64(a + (r + dy) * Cfg::A_ROW + 32 * k),
                                       umma::smem_desc_sw64(bw + dy * Cfg::B_TAP + 32 * k), idesc,
                                       (c > 0 || dy > 0 || k > 0) ? 1u : 0u);
            umma::mma_commit(&empty[st]);
        }
        umma::mma_commit(&done);  // arrives when every MMA above has completed
    }
    __syncwarp();
    const bool dok = __all_sync(0xffffffffu, umma::mbar_wait(&done, 0, kWaitLimit));
    umma::fence_after_sync();
    if (!dok && lane == 0) atomicOr(err, 4);
    if (dok) {
#pragma unroll 1
        for (int r = 0; r < R; r++) {
            const size_t p = ((size_t)n * H + h0 + r) * Wd + w0 + tid;  // TMEM lane = pixel
#pragma unroll 1
            for (int cc = 0; cc < COUT / 32; cc++) {
                float v[32];
                umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(r * COUT + cc * 32),
                                v);
                __align__(16) __nv_bfloat16 out[32];
#pragma unroll
                for (int i = 0; i < 32; i++) {
                    float t = v[i] + (bias ? bias[cc * 32 + i] : 0.f);
                    if (relu) t = fmaxf(t, 0.f);
                    out[i] = __float2bfloat16(t);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(Y + p * ystride + cc * 32);
#pragma unroll
                for (int q = 0; q < 4; q++) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, Cfg::NCOLS);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

bool encode_rows_map(CUtensorMap *m, const float *base, int ys, int nrows, int box_cols,
                     int box_rows) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t d[2] = {(cuuint64_t)ys, (cuuint64_t)nrows};
    const cuuint64_t st[1] = {(cuuint64_t)ys * 4};
    const cuuint32_t b[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t one[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, d, st, b, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_sino_map(CUtensorMap *m, const float *base, int ys, int nx, int na, int box_cols,
                     int box_bins) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t d[3] = {(cuuint64_t)ys, (cuuint64_t)nx, (cuuint64_t)na};
    const cuuint64_t st[2] = {(cuuint64_t)ys * 4, (cuuint64_t)nx * ys * 4};
    const cuuint32_t b[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_bins, 1};
    const cuuint32_t one[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)base, d, st, b, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of one convolution; false if the CUDA driver refuses them (the
// caller then uses the gather kernel).
static bool conv_tensor_maps(const __nv_bfloat16 *x, const __nv_bfloat16 *w, int N, int H, int Wd,
                             int Cin, int Cout, CUtensorMap *tx, CUtensorMap *tw, int box_rows = 1) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t xd[4] = {(cuuint64_t)Cin, (cuuint64_t)Wd, (cuuint64_t)H, (cuuint64_t)N};
    const cuuint64_t xs[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)Wd * Cin * 2,
                              (cuuint64_t)H * Wd * Cin * 2};
    const cuuint32_t xb[4] = {(cuuint32_t)kConvKC, 128, (cuuint32_t)box_rows, 1};
    const cuuint32_t one[4] = {1, 1, 1, 1};
    if (enc(tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)x, xd, xs, xb, one,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t wd[3] = {(cuuint64_t)Cin, 9, (cuuint64_t)Cout};
    const cuuint64_t ws[2] = {(cuuint64_t)Cin * 2, (cuuint64_t)9 * Cin * 2};
    const cuuint32_t wb[3] = {(cuuint32_t)kConvKC, 1, (cuuint32_t)Cout};
    return enc(tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)w, wd, ws, wb, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int COUT>
static int launch_conv_tma(const CUtensorMap &tx, const CUtensorMap &tw, const float *bias,
                           __nv_bfloat16 *Y, int H, int Wd, int Cin, int P, int relu, int ystride,
                           int *err, cudaStream_t st) {
    using Cfg = TmaCfg<COUT>;
    static bool configured = false;
    if (!configured) {
        ARECGB_CUDA(cudaFuncSetAttribute(conv3x3_tma_kernel<COUT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
        configured = true;
    }
    conv3x3_tma_kernel<COUT><<<P / 128, 128, Cfg::SMEM, st>>>(tx, tw, bias, Y, H, Wd, Cin, relu,
                                                              ystride, err);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

template <int COUT, int R>
static int launch_conv_rows(const CUtensorMap &tx, const CUtensorMap &tw, const float *bias,
                            __nv_bfloat16 *Y, int N, int H, int Wd, int Cin, int relu, int ystride,
                            int *err, cudaStream_t st) {
    using Cfg = RowsCfg<COUT, R>;
    static bool configured = false;
    if (!configured) {
        ARECGB_CUDA(cudaFuncSetAttribute(conv3x3_rows_kernel<COUT, R>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
        configured = true;
    }
    conv3x3_rows_kernel<COUT, R><<<N * (H / R) * (Wd / 128), 128, Cfg::SMEM, st>>>(
        tx, tw, bias, Y, H, Wd, Cin, relu, ystride, err);
    ARECGB_CUDA(cudaGetLastError());
    return 0;
}

// Output rows per block of the multi-row TMA kernel: 4 for 32 output channels,
// 2 for 64 (two blocks per SM fit in shared memory), else 1 (the one-row kernel).
static int conv_rows_for(int Cout) { return Cout == 32 ? 4 : (Cout == 64 ? 2 : 1); }

// layout: 0 = TMA path when the width is a multiple of 128, else the gather
//         kernel with (LBO 128, SBO 256) [K-halves 128 B apart, row groups 256 B
//         apart]; 1 = the gather kernel with the two offsets exchanged (for
//         validating the descriptor fields); 2 = the gather kernel always.
int conv3x3_bf16(const void *X, const void *Wt, const float *bias, void *Y, int N, int H, int Wd,
                 int Cin, int Cout, int relu, int layout, int *err, cudaStream_t st, int ystride) {
    if (ystride <= 0) ystride = Cout;
    if (Cin % kConvKC || Cin < kConvKC || N < 1 || H < 1 || Wd < 1 || ystride < Cout ||
        ystride % 8) {
        set_error("conv3x3: Cin must be a positive multiple of 32");
        return ARECGB_ERR_ARG;
    }
    const auto *x = reinterpret_cast<const __nv_bfloat16 *>(X);
    const auto *w = reinterpret_cast<const __nv_bfloat16 *>(Wt);
    auto *y = reinterpret_cast<__nv_bfloat16 *>(Y);
    const int P = N * H * Wd;
    if (layout == 0 && Wd % 128 == 0) {
        CUtensorMap tx, tw;
        const int R = conv_rows_for(Cout);
        if (R > 1 && H % R == 0 && conv_tensor_maps(x, w, N, H, Wd, Cin, Cout, &tx, &tw, R + 2)) {
            if (Cout == 32)
                return launch_conv_rows<32, 4>(tx, tw, bias, y, N, H, Wd, Cin, relu, ystride, err, st);
            if (Cout == 64)
                return launch_conv_rows<64, 2>(tx, tw, bias, y, N, H, Wd, Cin, relu, ystride, err, st);
        }
        if (conv_tensor_maps(x, w, N, H, Wd, Cin, Cout, &tx, &tw)) {
#define ARECGB_CONV_TMA(C) \
    if (Cout == C) return launch_conv_tma<C>(tx, tw, bias, y, H, Wd, Cin, P, relu, ystride, err, st);
            ARECGB_CONV_TMA(32) ARECGB_CONV_TMA(64) ARECGB_CONV_TMA(128) ARECGB_CONV_TMA(256)
#undef ARECGB_CONV_TMA
        }
    }
    if (layout == 2) layout = 0;
#define ARECGB_CONV(C)                                                                     \
    if (Cout == C)                                                                         \
        return layout ? launch_conv<C, 256, 128>(x, w, bias, y, H, Wd, Cin, P, relu, ystride, err, st) \
                      : launch_conv<C, 128, 256>(x, w, bias, y, H, Wd, Cin, P, relu, ystride, err, st);
    ARECGB_CONV(32) ARECGB_CONV(64) ARECGB_CONV(128) ARECGB_CONV(256)
#undef ARECGB_CONV
    set_error("conv3x3: Cout must be 32, 64, 128 or 256");
    return ARECGB_ERR_ARG;
}

}  // namespace arecgb

extern "C" int arecgb_conv3x3_bf16(const void *X, const void *Wt, const float *bias, void *Y, int N,
                                   int H, int W, int Cin, int Cout, int relu, int layout, int *err,
                                   void *stream) {
    return arecgb::conv3x3_bf16(X, Wt, bias, Y, N, H, W, Cin, Cout, relu, layout, err,
                                (cudaStream_t)stream, Cout);
}
