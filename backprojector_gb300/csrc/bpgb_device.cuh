// Device-side helpers for sm_103a: mbarriers, TMA tensor loads, shared-memory gathers.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bpgb {

// Adding 1.5 * 2^23 to a float in [-2^22, 2^22] leaves round-to-nearest-even(x) in the
// low mantissa bits: bits(x + kMagic) = kMagicBits + round(x).
constexpr float kMagic = 12582912.0f;
constexpr uint32_t kMagicBits = 0x4B400000u;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of the given parity; false when `limit` polls ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// The same wait with a short sleep between polls, for a warp whose wait is long against
// its own work (a producer waiting for consumers to release a stage): its polls would
// otherwise take issue slots from the warps it waits for.
__device__ __forceinline__ bool mbar_wait_backoff(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        __nanosleep(128);
    }
    return false;
}

// 2-D tiled TMA load of a {box, 1} tile at (x, y) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int32_t x,
                                            int32_t y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ---- typed shared-memory gathers accumulated in FP32 -----------------------------
// Storage element type in shared memory, its size, and the FP32 accumulate of one
// gathered element (FP16/BF16 use sm_100's mixed-precision add, one instruction).
template <typename HT>
struct Acc;

template <>
struct Acc<float> {
    using Elem = float;
    float v;
    static constexpr uint32_t kBytes = 4;
    __device__ __forceinline__ void zero() { v = 0.0f; }
    __device__ __forceinline__ void add(const Elem *base, uint32_t i) { v += base[i]; }
};

template <>
struct Acc<__half> {
    using Elem = unsigned short;
    float v;
    static constexpr uint32_t kBytes = 2;
    __device__ __forceinline__ void zero() { v = 0.0f; }
    __device__ __forceinline__ void add(const Elem *base, uint32_t i) {
        const unsigned short x = base[i];
        asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(v) : "h"(x));
    }
};

template <>
struct Acc<__nv_bfloat16> {
    using Elem = unsigned short;
    float v;
    static constexpr uint32_t kBytes = 2;
    __device__ __forceinline__ void zero() { v = 0.0f; }
    __device__ __forceinline__ void add(const Elem *base, uint32_t i) {
        const unsigned short x = base[i];
        asm("add.rn.f32.bf16 %0, %1, %0;" : "+f"(v) : "h"(x));
    }
};

template <>
struct Acc<float2> {
    using Elem = float2;
    float2 v;
    static constexpr uint32_t kBytes = 8;
    __device__ __forceinline__ void zero() { v = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void add(const Elem *base, uint32_t i) {
        const float2 x = base[i];
        v.x += x.x;
        v.y += x.y;
    }
};

}  // namespace bpgb
