// Blackwell (sm_100 family) tensor-core primitives used by the U-Net kernels:
// TMEM allocation, tcgen05.mma with shared-memory matrix descriptors,
// tcgen05.commit to an mbarrier, tcgen05.ld of the accumulator, and bounded
// mbarrier waits.  Inline PTX per the PTX ISA (tcgen05 family).
//
// Operand layout in shared memory: K-major, no swizzle ("interleaved"): the
// matrix is tiled into core matrices of 8 rows x 16 bytes (8 bf16), each stored
// as 128 contiguous bytes (row r at +16r).  For one MMA (K = 16 bf16) a
// 128-row operand is 16 row groups x 2 K-halves: core matrix (group i, half j)
// at  base + i*SBO + j*LBO  with LBO = 128 B and SBO = 256 B here.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace arecgb {
namespace umma {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start >> 4 in [0,14), leading
// byte offset >> 4 in [16,30), stride byte offset >> 4 in [32,46), the fixed
// version field 0b001 in [46,49), base offset 0, LBO mode 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Shared-memory matrix descriptor for a K-major operand stored with the 64-byte
// swizzle (rows of 64 bytes = 32 bf16 of K, 8-row atoms of 512 bytes, as a TMA
// load with CU_TENSOR_MAP_SWIZZLE_64B writes it): stride byte offset 512 between
// 8-row groups, leading byte offset unused (1), layout type 4 in [61,64).  The
// tile base must be 512-byte aligned; the k-th 16-element step starts 32*k
// bytes further.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for this layout)
    d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;            // version
    d |= (uint64_t)4 << 61;            // 64-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major,
// N >> 3 in [17,23), M >> 4 in [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)                        // D format: F32
           | (1u << 7)                      // A format: BF16
           | (1u << 10)                     // B format: BF16
           | ((uint32_t)(N >> 3) << 17)     // N
           | ((uint32_t)(M >> 4) << 24);    // M
}

// --- TMEM ---------------------------------------------------------------------------------
// One warp allocates `ncols` (power of two >= 32) columns; the address lands in
// shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Make generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier when all previously issued tcgen05.mma of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_addr(mbar))
        : "memory");
}

// --- mbarrier -------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(mbar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.b32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after `limit` polls and returns false (the caller
// records the failure; no kernel waits forever).
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}

// Plain arrival (release semantics) on an mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(mbar)) : "memory");
}

// Arrive on an mbarrier and add `bytes` to the transaction count the phase
// waits for (the bulk copies below complete it).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(mbar)),
                 "r"(bytes)
                 : "memory");
}

// Bulk (TMA, non-tensor) copy global -> shared of `bytes` (a multiple of 16,
// both addresses 16-byte aligned), completing on `mbar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(mbar))
        : "memory");
}

// Tiled TMA loads (cp.async.bulk.tensor), completing on `mbar`.
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, int c0, int c1,
                                            uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(smem_addr(mbar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int c0, int c1, int c2,
                                            uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(mbar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const void *tmap, int c0, int c1, int c2,
                                            int c3, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(mbar))
        : "memory");
}

// --- TMEM -> registers ------------------------------------------------------------------------
// Warp w of a warpgroup reads TMEM lanes 32w..32w+31; each thread gets 32
// consecutive 32-bit columns starting at `taddr`'s column.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace arecgb
