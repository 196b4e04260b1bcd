// Transient-row storage conversion: FP32 rows to FP16 / BF16 with a per-capture scale
// (the FAST kernels multiply the volume back by that scale, bpgb_options.h_scale).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

// out[0] = max |in| over rows x T (float bits compare as unsigned for |x|).
__global__ void absmax_kernel(const float *__restrict__ in, uint64_t rows, uint32_t T,
                              uint32_t pitch, unsigned int *__restrict__ out) {
    float m = 0.0f;
    const uint64_t n = rows * T;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / T, t = i - r * T;
        const float v = fabsf(in[r * pitch + t]);
        if (v > m || v != v) m = v != v ? INFINITY : v;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__device__ __forceinline__ void store_h(__half *p, float v) { *p = __float2half_rn(v); }
__device__ __forceinline__ void store_h(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }

// The scale is `scale`, or *d_absmax / target when d_absmax is set (read on the device).
__device__ __forceinline__ float scale_of(float scale, const float *d_absmax, float target) {
    if (!d_absmax) return scale;
    const float m = *d_absmax;
    return m > 0.0f ? m / target : 1.0f;
}

template <typename HT>
__global__ void to_half_kernel(const float *__restrict__ in, uint64_t rows, uint32_t T,
                               uint32_t in_pitch, float scale, const float *__restrict__ d_absmax,
                               float target, HT *__restrict__ out, uint32_t out_pitch) {
    const float inv_scale = 1.0f / scale_of(scale, d_absmax, target);
    const uint64_t n = rows * out_pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / out_pitch, t = i - r * out_pitch;
        const float v = t < T ? in[r * in_pitch + t] * inv_scale : 0.0f;
        store_h(out + i, v);
    }
}

// out[r][t] = in[r][from + t] for 0 <= from + t < T, else 0 (t < out_pitch).
__global__ void crop_kernel(const float *__restrict__ in, uint64_t rows, uint32_t T,
                            uint32_t in_pitch, int64_t from, uint32_t len,
                            float *__restrict__ out, uint32_t out_pitch) {
    const uint64_t n = rows * out_pitch;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / out_pitch, t = i - r * out_pitch;
        const int64_t src = from + (int64_t)t;
        out[i] = (t < len && src >= 0 && src < (int64_t)T) ? in[r * in_pitch + src] : 0.0f;
    }
}

__global__ void scale_kernel(float *__restrict__ v, uint64_t n, float scale,
                             const float *__restrict__ d_absmax, float target) {
    const float f = scale_of(scale, d_absmax, target);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        v[i] *= f;
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" {

int bpgb_rows_absmax(const float *d_H, uint64_t rows, uint32_t T, uint32_t pitch,
                     float *d_max, void *stream) {
    clear_error();
    if (!d_H || !d_max || T == 0 || pitch < T)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad absmax arguments");
    cudaStream_t s = (cudaStream_t)stream;
    BPGB_CUDA_TRY(cudaMemsetAsync(d_max, 0, sizeof(float), s));
    const uint64_t n = rows * T;
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
    absmax_kernel<<<grid, 256, 0, s>>>(d_H, rows, T, pitch, (unsigned int *)d_max);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_rows_to_half(const float *d_H, uint64_t rows, uint32_t T, uint32_t in_pitch, float scale,
                      const float *d_absmax, float target, int dtype, void *d_out,
                      uint32_t out_pitch, void *stream) {
    clear_error();
    if (!d_H || !d_out || T == 0 || in_pitch < T || out_pitch < T ||
        (d_absmax ? !(target > 0.0f) : !(scale > 0.0f)) ||
        (dtype != BPGB_DTYPE_F16 && dtype != BPGB_DTYPE_BF16))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad row conversion arguments");
    const uint64_t n = rows * out_pitch;
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == BPGB_DTYPE_F16)
        to_half_kernel<__half><<<grid, 256, 0, s>>>(d_H, rows, T, in_pitch, scale, d_absmax,
                                                  target, (__half *)d_out, out_pitch);
    else
        to_half_kernel<__nv_bfloat16><<<grid, 256, 0, s>>>(d_H, rows, T, in_pitch, scale,
                                                         d_absmax, target,
                                                         (__nv_bfloat16 *)d_out, out_pitch);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_volume_scale(float *d_volume, uint64_t n, float scale, const float *d_absmax,
                      float target, void *stream) {
    clear_error();
    if (!d_volume || (d_absmax ? !(target > 0.0f) : !(scale == scale)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad volume scale arguments");
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
    scale_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_volume, n, scale, d_absmax, target);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_rows_crop(const float *d_in, uint64_t rows, uint32_t T, uint32_t in_pitch, int64_t from,
                   uint32_t len, float *d_out, uint32_t out_pitch, void *stream) {
    clear_error();
    if (!d_in || !d_out || T == 0 || in_pitch < T || len == 0 || out_pitch < len)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad crop arguments");
    const uint64_t n = rows * out_pitch;
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
    crop_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_in, rows, T, in_pitch, from, len, d_out,
                                                      out_pitch);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

}  // extern "C"
