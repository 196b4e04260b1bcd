// tcgen05 (5th-generation tensor core) helpers for sm_103a: tensor-memory allocation,
// shared-memory matrix descriptors, instruction descriptors for kind::f16 (BF16 operands,
// FP32 accumulate), MMA issue, commit to an mbarrier, tensor-memory loads, and the bulk
// and tiled (TMA) copies global -> shared that stage the operands.
//
// Descriptor formats follow the PTX ISA's tcgen05 chapter (shared-memory descriptor and
// instruction descriptor tables).  Operands here are always in the no-swizzle canonical
// layout: a "core matrix" is 8 rows of 16 bytes stored contiguously (128 B).  For a
// K-major operand a row is one M (or N) index holding 8 consecutive K elements; for an
// MN-major operand a row is one K index holding 8 consecutive M (or N) elements.  The two
// strides of the descriptor place the core matrices: the leading byte offset (LBO) is the
// stride between neighbours along K and the stride byte offset (SBO) the one along M/N,
// for K-major and MN-major operands alike (pinned by the known-answer test of
// bpgb_diag_umma_probe).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bpgb {

// ---- descriptors (host and device) ------------------------------------------------

// Shared-memory matrix descriptor: start address, leading- and stride-dimension byte
// offsets (all in 16-byte units, 14 bits each), descriptor version 1 (bits 46-47), no
// swizzle (bits 61-63 = 0), base offset 0.
__host__ __device__ constexpr uint64_t umma_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: dense, FP32 D (bits 4-5 = 1), A and B
// BF16 (bits 7-9, 10-12 = 1), A / B major-ness (bit 15 / 16: 0 = K-major, 1 = MN-major),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(uint32_t M, uint32_t N, bool a_mn,
                                                       bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
           ((b_mn ? 1u : 0u) << 16) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

#if defined(__CUDACC__)

// ---- tensor memory --------------------------------------------------------------
// Allocation and release are warp-wide (.sync.aligned): call from one full warp.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     dst_smem),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Generic-proxy writes to shared memory become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- MMA ------------------------------------------------------------------------
// D[tmem] (+)= A[smem] x B[smem], one thread issues.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                          uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

// ---- tensor memory -> registers ----------------------------------------------------
// 32 lanes x 32 bit, 16 consecutive columns: thread i of the warp gets lane (base lane + i),
// columns col .. col + 15.  The warp's lane window is 32 x (warp index mod 4).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- bulk copy ----------------------------------------------------------------------
// Untiled global -> shared copy completing on an mbarrier's transaction count; both
// addresses 16-byte aligned and bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// 4-D tiled TMA load of one box at coordinates (c0 innermost .. c3) into shared memory,
// completing on bar.  c0 x element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const void *map, int32_t c0, int32_t c1,
                                            int32_t c2, int32_t c3, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

// 5-D tiled TMA load of one box at coordinates (c0 innermost .. c4) into shared memory,
// completing on bar.  c0 x element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const void *map, int32_t c0, int32_t c1,
                                            int32_t c2, int32_t c3, int32_t c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

#endif  // __CUDACC__

}  // namespace bpgb
