// Pipe-rate probe: measured per-SM throughput of the three pipes the FAST kernel's update
// uses -- rsqrt.approx (XU), packed FP32x2 FMA (FMA pipe, counted in FP32 lanes) and
// conflict-free 32-bit shared loads -- for the roofline denominator.
//
// Each probe launches 4 CTAs of 256 threads per SM; every thread runs 8 independent
// dependency chains of the probed operation.  Each CTA times itself with clock64; the
// per-SM rate is (operations of the CTAs on that SM) / (the longest CTA's cycles).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bpgb_device.cuh"
#include "bpgb_internal.h"
#include "bpgb_umma.cuh"

namespace bpgb {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeBlocksPerSm = 4;
constexpr int kChains = 8;

__device__ __forceinline__ uint32_t smid() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

struct ProbeOut {
    unsigned long long cycles;
    uint32_t sm;
    float sink;
};

template <int OP>
__global__ void __launch_bounds__(kProbeThreads) pipe_probe_kernel(int iters, ProbeOut *out) {
    __shared__ uint32_t ring[1024];
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) ring[i] = ((i + 32) & 1023) * 4;
    __syncthreads();
    const unsigned long long t0 = clock64();
    float acc = 0.0f;
    if (OP == 0) {  // rsqrt.approx chains
        float x[kChains];
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = 1.5f + 0.01f * (threadIdx.x + c);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) x[c] = rsqrt_approx(x[c]);
        }
#pragma unroll
        for (int c = 0; c < kChains; c++) acc += x[c];
    } else if (OP == 1) {  // packed FP32x2 FMA chains
        float2 x[kChains];
        const float2 m = make_float2(0.999f, 0.998f), b = make_float2(0.001f, 0.002f);
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = make_float2(0.5f + c, 0.25f + threadIdx.x);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) x[c] = __ffma2_rn(x[c], m, b);
        }
#pragma unroll
        for (int c = 0; c < kChains; c++) acc += x[c].x + x[c].y;
    } else {  // conflict-free shared loads: each lane follows its own bank
        uint32_t o[kChains];
#pragma unroll
        for (int c = 0; c < kChains; c++) o[c] = (((threadIdx.x & 31) + 32 * c) & 1023) * 4;
        const unsigned char *base = reinterpret_cast<const unsigned char *>(ring);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) o[c] = *reinterpret_cast<const uint32_t *>(base + o[c]);
        }
#pragma unroll
        for (int c = 0; c < kChains; c++) acc += (float)o[c];
    }
    __syncthreads();
    const unsigned long long t1 = clock64();
    if (threadIdx.x == 0) {
        out[blockIdx.x].cycles = t1 - t0;
        out[blockIdx.x].sm = smid();
    }
    if (acc == -1.0f) out[blockIdx.x].sink = acc;  // keeps the chains live
}

// MUFU operations one at a time, in chains that stay bounded: OP 0 rsqrt x 8 chains,
// 1 rsqrt x 16 chains, 2 ex2(-x), 3 sqrt, 4 rcp, 5 sin.  Same timing scheme as
// pipe_probe_kernel; the per-SM rate is MUFU results per clock.
template <int OP>
__global__ void __launch_bounds__(kProbeThreads) mufu_probe_kernel(int iters, ProbeOut *out) {
    constexpr int C = OP == 1 ? 16 : kChains;
    float x[C];
#pragma unroll
    for (int c = 0; c < C; c++) x[c] = 0.5f + 0.001f * (threadIdx.x + c);
    __syncthreads();
    const unsigned long long t0 = clock64();
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < C; c++) {
            float y;
            if (OP <= 1) asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            if (OP == 2) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-x[c]));
            if (OP == 3) asm volatile("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            if (OP == 4) asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            if (OP == 5) asm volatile("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            x[c] = y;
        }
    }
    __syncthreads();
    const unsigned long long t1 = clock64();
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < C; c++) acc += x[c];
    if (threadIdx.x == 0) {
        out[blockIdx.x].cycles = t1 - t0;
        out[blockIdx.x].sm = smid();
    }
    if (acc == -1.0f) out[blockIdx.x].sink = acc;
}

template <int OP>
void launch_mufu_probe(int blocks, int iters, ProbeOut *d) {
    mufu_probe_kernel<OP><<<blocks, kProbeThreads>>>(iters, d);
}

// Per-SM rate of a probe launch: (operations of the CTAs on an SM) / (its longest CTA's
// cycles), averaged over SMs.
double per_sm_rate(const std::vector<ProbeOut> &h, int sms, double ops_per_cta) {
    std::vector<unsigned long long> longest(sms, 0);
    std::vector<int> count(sms, 0);
    for (const ProbeOut &o : h) {
        if ((int)o.sm >= sms) continue;
        longest[o.sm] = std::max(longest[o.sm], o.cycles);
        count[o.sm]++;
    }
    double sum = 0.0;
    int used = 0;
    for (int s = 0; s < sms; s++)
        if (count[s] && longest[s]) {
            sum += (double)count[s] * ops_per_cta / (double)longest[s];
            used++;
        }
    return used ? sum / used : 0.0;
}

// ---- tcgen05 known-answer probe ------------------------------------------------------
// One CTA copies a 48 KB operand image into shared memory (the rest of its 96 KB zeroed),
// issues `nk` tcgen05.mma kind::f16 (BF16, K = 16 each) with descriptors built from the
// given offsets and strides, and dumps the 128 lanes x ncols FP32 columns of the
// accumulator.  The host checks every stride combination against the 96 KB before the
// launch, so any reading of the descriptors stays inside the CTA's shared memory.
constexpr uint32_t kUmmaImage = 48 * 1024;
constexpr uint32_t kUmmaSmem = 96 * 1024;
constexpr uint32_t kUmmaCols = 256;
constexpr uint32_t kUmmaRateSmem = 64 * 1024;

struct UmmaProbeArgs {
    uint32_t a_off, a_lbo, a_sbo, a_kstep;
    uint32_t b_off, b_lbo, b_sbo, b_kstep;
    uint32_t idesc, nk, ncols;
};

__global__ void __launch_bounds__(128) umma_probe_kernel(const uint4 *__restrict__ image,
                                                         UmmaProbeArgs a, float *__restrict__ out,
                                                         uint32_t *__restrict__ status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint4 *s4 = reinterpret_cast<uint4 *>(smem);
    for (uint32_t i = tid; i < kUmmaSmem / 16; i += 128)
        s4[i] = i < kUmmaImage / 16 ? image[i] : make_uint4(0, 0, 0, 0);
    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), kUmmaCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(smem_addr(&bar), 1);
        mbar_fence_init();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;
    if (tid == 0) {
        const uint32_t base = smem_addr(smem);
        for (uint32_t k = 0; k < a.nk; k++)
            umma_bf16(taddr, umma_smem_desc(base + a.a_off + k * a.a_kstep, a.a_lbo, a.a_sbo),
                      umma_smem_desc(base + a.b_off + k * a.b_kstep, a.b_lbo, a.b_sbo), a.idesc,
                      k > 0);
        umma_commit(smem_addr(&bar));
    }
    bool done = mbar_wait(smem_addr(&bar), 0, 1u << 24);
    tc_fence_after();
    if (done) {
        for (uint32_t c = 0; c < a.ncols; c += 16) {
            float v[16];
            tmem_ld16(taddr + ((warp * 32u) << 16) + c, v);
            tmem_ld_wait();
            float *o = out + (uint64_t)(warp * 32 + lane) * a.ncols + c;
#pragma unroll
            for (int j = 0; j < 16; j++) o[j] = v[j];
        }
    } else {
        if (lane == 0) atomicOr(status, 1u);
        // the MMAs may still read shared memory and write the accumulator: wait (bounded)
        // before the columns are released
        done = mbar_wait(smem_addr(&bar), 0, 1u << 26);
        if (!done && lane == 0) atomicOr(status, 2u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, kUmmaCols);
    }
}

// ---- tcgen05 issue rate -----------------------------------------------------------------
// One thread per CTA (one CTA per SM) issues `reps` back-to-back MMAs of one shape over
// NACC independent accumulators, operands zero in shared memory; clock64 around the
// issue loop and the commit wait gives cycles per MMA.
template <uint32_t M, uint32_t N, bool MN, uint32_t NACC>
__global__ void __launch_bounds__(128) umma_rate_kernel(uint32_t reps, unsigned long long *out,
                                                        uint32_t *status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    for (uint32_t i = tid; i < kUmmaRateSmem / 16; i += 128)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
    fence_async_smem();
    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), 512);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(smem_addr(&bar), 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;
    if (tid == 0) {
        const uint32_t base = smem_addr(smem);
        // A at 0 and B at 32 KB; the widest reading (16 / 32 core matrices) stays below 48 KB
        const uint64_t ad = MN ? umma_smem_desc(base, 128, 512) : umma_smem_desc(base, 2048, 128);
        const uint64_t bd = MN ? umma_smem_desc(base + 32768, 128, 512)
                               : umma_smem_desc(base + 32768, 4096, 128);
        constexpr uint32_t idesc = umma_idesc_bf16(M, N, MN, MN);
#pragma unroll
        for (uint32_t u = 0; u < NACC; u++) umma_bf16(taddr + u * N, ad, bd, idesc, 0);
        const unsigned long long t0 = clock64();
        for (uint32_t r = 0; r < reps; r += NACC) {
#pragma unroll
            for (uint32_t u = 0; u < NACC; u++) umma_bf16(taddr + u * N, ad, bd, idesc, 1);
        }
        umma_commit(smem_addr(&bar));
        const bool ok = mbar_wait(smem_addr(&bar), 0, 1u << 24);
        const unsigned long long t1 = clock64();
        if (!ok) atomicOr(status, 1u);
        out[blockIdx.x] = t1 - t0;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, 512);
    }
}

template <uint32_t M, uint32_t N, bool MN, uint32_t NACC>
int umma_rate(int sms, unsigned long long *d, uint32_t *st, double *cycles) {
    const uint32_t reps = 2048;
    cudaError_t e = cudaFuncSetAttribute(umma_rate_kernel<M, N, MN, NACC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kUmmaRateSmem);
    for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {  // the first launch warms up
        umma_rate_kernel<M, N, MN, NACC><<<sms, 128, kUmmaRateSmem>>>(reps, d, st);
        count_launches(1);
        e = cudaGetLastError();
    }
    std::vector<unsigned long long> h(sms);
    uint32_t hs = 0;
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, sms * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hs, st, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "umma rate probe");
    if (hs) return set_error(BPGB_ERR_TIMEOUT, "umma rate probe: commit wait ran out");
    double sum = 0.0;
    for (unsigned long long c : h) sum += (double)c;
    *cycles = sum / sms / reps;
    return BPGB_OK;
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

// params: a_off, a_lbo, a_sbo, a_kstep, b_off, b_lbo, b_sbo, b_kstep, idesc, nk, ncols.
extern "C" int bpgb_diag_umma_probe(const void *h_image, uint32_t image_bytes,
                                    const uint32_t *params, float *h_out, uint32_t *h_status) {
    clear_error();
    if (!h_image || !params || !h_out || !h_status || image_bytes > kUmmaImage ||
        image_bytes % 16)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad umma probe arguments");
    UmmaProbeArgs a{params[0], params[1], params[2], params[3], params[4], params[5],
                    params[6], params[7], params[8], params[9], params[10]};
    if (a.nk == 0 || a.nk > 8 || a.ncols == 0 || a.ncols > kUmmaCols || a.ncols % 16)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "umma probe: nk in 1..8, ncols in 16..256");
    // whichever stride the hardware applies along either dimension, at most 32 core
    // matrices (256 rows) are stepped along M/N and 2 along K per MMA
    const uint64_t far_a = (uint64_t)a.a_off + (uint64_t)(a.nk - 1) * a.a_kstep +
                           32ull * (a.a_lbo + a.a_sbo) + 128;
    const uint64_t far_b = (uint64_t)a.b_off + (uint64_t)(a.nk - 1) * a.b_kstep +
                           32ull * (a.b_lbo + a.b_sbo) + 128;
    if (far_a > kUmmaSmem || far_b > kUmmaSmem || a.a_off % 16 || a.b_off % 16 ||
        a.a_lbo % 16 || a.a_sbo % 16 || a.b_lbo % 16 || a.b_sbo % 16 || a.a_kstep % 16 ||
        a.b_kstep % 16)
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "umma probe: operand extents must stay inside 96 KB, 16-byte units");
    int st = require_device();
    if (st) return st;
    uint4 *d_img = nullptr;
    float *d_out = nullptr;
    uint32_t *d_st = nullptr;
    const size_t out_bytes = (size_t)128 * a.ncols * sizeof(float);
    cudaError_t e = cudaMalloc(&d_img, kUmmaImage);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, out_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&d_st, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(d_img, 0, kUmmaImage);
    if (e == cudaSuccess) e = cudaMemcpy(d_img, h_image, image_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_out, 0xFF, out_bytes);
    if (e == cudaSuccess) e = cudaMemset(d_st, 0, sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(umma_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kUmmaSmem);
    if (e == cudaSuccess) {
        umma_probe_kernel<<<1, 128, kUmmaSmem>>>(d_img, a, d_out, d_st);
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h_out, d_out, out_bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_status, d_st, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_img);
    cudaFree(d_out);
    cudaFree(d_st);
    if (e != cudaSuccess) return cuda_error(e, "umma probe");
    return BPGB_OK;
}

extern "C" int bpgb_diag_mufu_rates(double *rates, int n) {
    clear_error();
    if (!rates || n < 1) return set_error(BPGB_ERR_INVALID_ARGUMENT, "rates is null or n < 1");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    const int blocks = sms * kProbeBlocksPerSm;
    ProbeOut *d = nullptr;
    BPGB_CUDA_TRY(cudaMalloc(&d, blocks * sizeof(ProbeOut)));
    std::vector<ProbeOut> h(blocks);
    const int iters = 2048;
    void (*launch[6])(int, int, ProbeOut *) = {launch_mufu_probe<0>, launch_mufu_probe<1>,
                                                launch_mufu_probe<2>, launch_mufu_probe<3>,
                                                launch_mufu_probe<4>, launch_mufu_probe<5>};
    for (int op = 0; op < 6 && op < n; op++) {
        for (int rep = 0; rep < 2; rep++) {  // first launch warms up
            launch[op](blocks, iters, d);
            count_launches(1);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, blocks * sizeof(ProbeOut), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_error(e, "mufu probe");
        }
        const double chains = op == 1 ? 16.0 : (double)kChains;
        rates[op] = per_sm_rate(h, sms, (double)kProbeThreads * iters * chains);
    }
    cudaFree(d);
    return BPGB_OK;
}

extern "C" int bpgb_diag_pipe_rates(double *rates) {
    clear_error();
    if (!rates) return set_error(BPGB_ERR_INVALID_ARGUMENT, "rates is null");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    const int blocks = sms * kProbeBlocksPerSm;
    ProbeOut *d = nullptr;
    BPGB_CUDA_TRY(cudaMalloc(&d, blocks * sizeof(ProbeOut)));
    std::vector<ProbeOut> h(blocks);
    const int iters = 4096;
    // operations per thread-iteration in the unit reported: rsqrt results, FP32 lanes, loads
    const double per_iter[3] = {kChains, 2.0 * kChains, kChains};
    for (int op = 0; op < 3; op++) {
        for (int rep = 0; rep < 2; rep++) {  // first launch warms up
            if (op == 0) pipe_probe_kernel<0><<<blocks, kProbeThreads>>>(iters, d);
            if (op == 1) pipe_probe_kernel<1><<<blocks, kProbeThreads>>>(iters, d);
            if (op == 2) pipe_probe_kernel<2><<<blocks, kProbeThreads>>>(iters, d);
            count_launches(1);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, blocks * sizeof(ProbeOut), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_error(e, "pipe probe");
        }
        std::vector<unsigned long long> longest(sms, 0);
        std::vector<int> count(sms, 0);
        for (const ProbeOut &o : h) {
            if ((int)o.sm >= sms) continue;
            longest[o.sm] = std::max(longest[o.sm], o.cycles);
            count[o.sm]++;
        }
        double sum = 0.0;
        int used = 0;
        for (int s = 0; s < sms; s++)
            if (count[s] && longest[s]) {
                sum += (double)count[s] * kProbeThreads * iters * per_iter[op] / (double)longest[s];
                used++;
            }
        rates[op] = used ? sum / used : 0.0;
    }
    cudaFree(d);
    return BPGB_OK;
}

// Cycles per tcgen05.mma (BF16, K = 16) issued back to back by one thread per SM over
// independent accumulators: [0] M128 N48 MN-major, [1] M64 N48 MN-major, [2] M128 N48
// K-major, [3] M128 N96 K-major, [4] M128 N128 K-major, [5] M128 N256 K-major.
extern "C" int bpgb_diag_umma_issue_rates(double *cycles, int n) {
    clear_error();
    if (!cycles || n < 1) return set_error(BPGB_ERR_INVALID_ARGUMENT, "cycles is null or n < 1");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    unsigned long long *d = nullptr;
    uint32_t *ds = nullptr;
    cudaError_t e = cudaMalloc(&d, sms * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&ds, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ds, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaFree(d);
        cudaFree(ds);
        return cuda_error(e, "umma rate probe");
    }
    int (*run[6])(int, unsigned long long *, uint32_t *, double *) = {
        umma_rate<128, 48, true, 8>,  umma_rate<64, 48, true, 8>,   umma_rate<128, 48, false, 8>,
        umma_rate<128, 96, false, 4>, umma_rate<128, 128, false, 2>, umma_rate<128, 256, false, 2>};
    for (int i = 0; i < 6 && i < n && !st; i++) st = run[i](sms, d, ds, &cycles[i]);
    cudaFree(d);
    cudaFree(ds);
    return st;
}
