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

}  // namespace
}  // namespace bpgb

using namespace bpgb;

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
