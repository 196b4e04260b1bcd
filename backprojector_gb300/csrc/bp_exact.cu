// Reference-exact dense backprojection (FP32 and complex64).
//
// Semantics of cuda_backprojection_impl<FT> (backproject_cuda.cu:117-175): for every
// voxel v = zero + inc[0:3]*x + inc[3:6]*y + inc[6:9]*z (:144-148) and every pair p,
//   d = laser_wall + |l_p - v| + |v - c_p| + camera_wall        (:31-46, norm3df)
//   b = (int) round((d - t0 - 0) / deltaT)                       (:155-158)
// and H[p, b] is added when 0 <= b <= T-1 (:157-159).  The arithmetic below is the same
// expression in the same order (FMA-contracted voxel position, norm3df, IEEE division,
// round-half-away), so every bin index equals the reference's; only the summation order
// differs (register sums in pair order instead of strided partial sums plus a serial
// shared-memory reduction).  This file must be compiled without fast-math flags.
//
// Layout: one CTA = 256 threads = a 4 x 8 x 8 voxel tile (z fastest, x slowest), one
// voxel per thread.  Pair records are staged 256 at a time in shared memory and read as
// warp-uniform broadcasts; each warp's 32 voxels gather from one H row at neighbouring
// bins, so the global gathers coalesce into few sectors.  All pairs are used (the
// reference skips the last P mod blockDim) and every voxel is visited for any N.
#include <cuda_runtime.h>

#include <algorithm>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

constexpr int kTX = 4, kTY = 8, kTZ = 8;
constexpr int kThreads = kTX * kTY * kTZ;

struct ExactArgs {
    uint32_t n[3];
    uint32_t tiles[3];
    float zero[3];
    float inc[9];
    float t0, dT;
    uint32_t T;
    uint64_t pitch;
    uint64_t P;
};

__device__ __forceinline__ void voxel_position(const ExactArgs &a, uint32_t x, uint32_t y,
                                               uint32_t z, float v[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float s = __fmaf_rn(a.inc[k], (float)x, a.zero[k]);
        s = __fmaf_rn(a.inc[3 + k], (float)y, s);
        v[k] = __fmaf_rn(a.inc[6 + k], (float)z, s);
    }
}

__device__ __forceinline__ int exact_bin(const bpgb_pair &pr, const float v[3], float t0,
                                         float dT) {
    float lpv = norm3df(pr.laser_point[0] - v[0], pr.laser_point[1] - v[1],
                        pr.laser_point[2] - v[2]);
    float vcp = norm3df(v[0] - pr.camera_point[0], v[1] - pr.camera_point[1],
                        v[2] - pr.camera_point[2]);
    float total = pr.laser_wall + lpv + vcp + pr.camera_wall;
    float r = roundf((total - t0 - 0.0f / 2) / dT);
    return (int)r;
}

__device__ __forceinline__ void tile_voxel(const ExactArgs &a, uint32_t &x, uint32_t &y,
                                           uint32_t &z) {
    uint32_t t = blockIdx.x;
    uint32_t tz = t % a.tiles[2];
    t /= a.tiles[2];
    uint32_t tx = t % a.tiles[0];
    uint32_t ty = t / a.tiles[0];
    uint32_t lz = threadIdx.x % kTZ;
    uint32_t ly = (threadIdx.x / kTZ) % kTY;
    uint32_t lx = threadIdx.x / (kTZ * kTY);
    x = tx * kTX + lx;
    y = ty * kTY + ly;
    z = tz * kTZ + lz;
}

__device__ __forceinline__ float load_h(const float *H, uint64_t i) { return __ldg(H + i); }
__device__ __forceinline__ float2 load_h(const float2 *H, uint64_t i) { return __ldg(H + i); }
__device__ __forceinline__ void add_to(float &a, float b) { a += b; }
__device__ __forceinline__ void add_to(float2 &a, float2 b) {
    a.x += b.x;
    a.y += b.y;
}
template <typename HT>
__device__ __forceinline__ HT zero_h();
template <>
__device__ __forceinline__ float zero_h<float>() { return 0.0f; }
template <>
__device__ __forceinline__ float2 zero_h<float2>() { return make_float2(0.0f, 0.0f); }

template <typename HT>
__global__ void __launch_bounds__(kThreads)
    bp_exact_kernel(const HT *__restrict__ H, const bpgb_pair *__restrict__ pairs,
                    HT *__restrict__ out, const ExactArgs a) {
    __shared__ bpgb_pair sp[kThreads];
    uint32_t x, y, z;
    tile_voxel(a, x, y, z);
    const bool valid = x < a.n[0] && y < a.n[1] && z < a.n[2];
    float v[3];
    voxel_position(a, x, y, z, v);
    HT acc = zero_h<HT>();
    const int last = (int)a.T - 1;
    for (uint64_t base = 0; base < a.P; base += kThreads) {
        __syncthreads();
        if (base + threadIdx.x < a.P) sp[threadIdx.x] = pairs[base + threadIdx.x];
        __syncthreads();
        const uint32_t n = (uint32_t)(a.P - base < (uint64_t)kThreads ? a.P - base : (uint64_t)kThreads);
        for (uint32_t j = 0; j < n; j++) {
            const int b = exact_bin(sp[j], v, a.t0, a.dT);
            if (b >= 0 && b <= last) add_to(acc, load_h(H, (base + j) * a.pitch + (uint64_t)b));
        }
    }
    if (valid) out[((uint64_t)x * a.n[1] + y) * a.n[2] + z] = acc;
}

// bins[i * P + p] for voxel ids[i]; same expression as bp_exact_kernel.
__global__ void bp_exact_bins_kernel(const bpgb_pair *__restrict__ pairs,
                                     const int64_t *__restrict__ ids, int64_t n,
                                     int32_t *__restrict__ bins, const ExactArgs a) {
    const uint64_t total = (uint64_t)n * a.P;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < total;
         w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = w / a.P, p = w % a.P;
        const int64_t id = ids[i];
        const uint32_t z = (uint32_t)(id % a.n[2]);
        const uint32_t y = (uint32_t)((id / a.n[2]) % a.n[1]);
        const uint32_t x = (uint32_t)(id / ((int64_t)a.n[1] * a.n[2]));
        float v[3];
        voxel_position(a, x, y, z, v);
        const bpgb_pair pr = pairs[p];
        const int b = exact_bin(pr, v, a.t0, a.dT);
        bins[w] = (b >= 0 && b <= (int)a.T - 1) ? b : -1;
    }
}

ExactArgs make_args(uint64_t pitch, uint64_t P, const Volume &vol, const BinParams &bp) {
    ExactArgs a{};
    for (int k = 0; k < 3; k++) {
        a.n[k] = vol.n[k];
        a.zero[k] = vol.zero[k];
    }
    for (int k = 0; k < 9; k++) a.inc[k] = vol.inc[k];
    a.tiles[0] = (vol.n[0] + kTX - 1) / kTX;
    a.tiles[1] = (vol.n[1] + kTY - 1) / kTY;
    a.tiles[2] = (vol.n[2] + kTZ - 1) / kTZ;
    a.t0 = bp.t0;
    a.dT = bp.dT;
    a.T = bp.T;
    a.pitch = pitch;
    a.P = P;
    return a;
}

}  // namespace

int launch_exact(const void *d_H, bool is_complex, uint64_t pitch, const bpgb_pair *d_pairs,
                 uint64_t P, const Volume &vol, const BinParams &bp, void *d_out,
                 cudaStream_t stream) {
    const ExactArgs a = make_args(pitch, P, vol, bp);
    const uint64_t tiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    if (tiles == 0) return BPGB_OK;
    if (tiles > 0x7fffffffull)
        return set_error(BPGB_ERR_UNSUPPORTED, "volume too large for the exact kernel grid");
    if (is_complex)
        bp_exact_kernel<float2><<<(unsigned)tiles, kThreads, 0, stream>>>(
            (const float2 *)d_H, d_pairs, (float2 *)d_out, a);
    else
        bp_exact_kernel<float><<<(unsigned)tiles, kThreads, 0, stream>>>(
            (const float *)d_H, d_pairs, (float *)d_out, a);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int launch_exact_bins(const bpgb_pair *d_pairs, uint64_t P, const Volume &vol,
                      const BinParams &bp, const int64_t *d_ids, int64_t n, int32_t *d_bins,
                      cudaStream_t stream) {
    if (n <= 0 || P == 0) return BPGB_OK;
    const ExactArgs a = make_args(0, P, vol, bp);
    const uint64_t total = (uint64_t)n * P;
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 16);
    bp_exact_bins_kernel<<<blocks, 256, 0, stream>>>(d_pairs, d_ids, n, d_bins, a);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

}  // namespace bpgb
