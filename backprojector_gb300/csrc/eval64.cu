// FP64 evaluation of listed voxels: the reference kernel's quantity
// (backproject_cuda.cu:117-175) with every geometric step in double, for measuring the
// FP32 paths' error on the GPU (bench, tests).  Not a reconstruction path.
//
// Per voxel v = zero + inc[0:3] x + inc[3:6] y + inc[6:9] z (backproject_cuda.cu:144-148)
// and pair p: d = lw + |l - v| + |v - c| + cw (:25-46), b = round((d - t0) / dT) half away
// from zero, kept iff 0 <= b <= T - 1 (:155-159); V[v] = sum over p in pair order of
// H[p, b], accumulated in double.  Each operation is rounded separately (no contraction),
// in a fixed order, one thread per voxel summing sequentially.
#include <cuda_runtime.h>

#include <algorithm>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

__device__ __forceinline__ double dist_f64(const float *p, const double v[3]) {
    const double dx = __dsub_rn((double)p[0], v[0]);
    const double dy = __dsub_rn((double)p[1], v[1]);
    const double dz = __dsub_rn((double)p[2], v[2]);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

template <bool CPLX>
__global__ void eval_f64_kernel(const float *__restrict__ H, uint32_t T, uint64_t pitch,
                                const bpgb_pair *__restrict__ pairs, uint64_t P, uint32_t n1,
                                uint32_t n2, Volume vol, double t0, double dT,
                                const int64_t *__restrict__ ids, int64_t n,
                                double *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id = ids[i];
        const uint32_t iz = (uint32_t)(id % n2);
        const uint32_t iy = (uint32_t)((id / n2) % n1);
        const uint32_t ix = (uint32_t)(id / ((int64_t)n1 * n2));
        double v[3];
        for (int k = 0; k < 3; k++) {
            double a = __dadd_rn((double)vol.zero[k], __dmul_rn((double)vol.inc[k], (double)ix));
            a = __dadd_rn(a, __dmul_rn((double)vol.inc[3 + k], (double)iy));
            v[k] = __dadd_rn(a, __dmul_rn((double)vol.inc[6 + k], (double)iz));
        }
        double re = 0.0, im = 0.0;
        for (uint64_t p = 0; p < P; p++) {
            const bpgb_pair pr = pairs[p];
            double d = __dadd_rn((double)pr.laser_wall, dist_f64(pr.laser_point, v));
            d = __dadd_rn(d, dist_f64(pr.camera_point, v));
            d = __dadd_rn(d, (double)pr.camera_wall);
            const double b = round(__ddiv_rn(__dsub_rn(d, t0), dT));
            if (b < 0.0 || b > (double)T - 1.0) continue;
            const uint64_t at = p * pitch + (uint64_t)b;
            if (CPLX) {
                re = __dadd_rn(re, (double)H[2 * at]);
                im = __dadd_rn(im, (double)H[2 * at + 1]);
            } else {
                re = __dadd_rn(re, (double)H[at]);
            }
        }
        if (CPLX) {
            out[2 * i] = re;
            out[2 * i + 1] = im;
        } else {
            out[i] = re;
        }
    }
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" int bpgb_eval_f64_voxels(const void *d_H, int is_complex, uint32_t T, uint32_t h_pitch,
                                    const bpgb_pair *d_pairs, uint64_t num_pairs,
                                    const uint32_t *voxels_per_side, const float *volume_zero_pos,
                                    const float *voxel_inc, float t0, float deltaT,
                                    const int64_t *d_voxel_ids, int64_t n, double *d_out,
                                    void *stream) {
    clear_error();
    if (n < 0) return set_error(BPGB_ERR_INVALID_ARGUMENT, "negative voxel count");
    if (n == 0) return BPGB_OK;
    if (!d_H || !d_pairs || !voxels_per_side || !volume_zero_pos || !voxel_inc || !d_voxel_ids ||
        !d_out)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (T == 0 || (h_pitch && h_pitch < T))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "need T > 0 and h_pitch 0 or >= T");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    Volume vol{};
    for (int k = 0; k < 3; k++) {
        vol.n[k] = voxels_per_side[k];
        vol.zero[k] = volume_zero_pos[k];
        if (!vol.n[k]) return set_error(BPGB_ERR_INVALID_ARGUMENT, "empty volume");
    }
    for (int k = 0; k < 9; k++) vol.inc[k] = voxel_inc[k];
    const uint64_t pitch = h_pitch ? h_pitch : T;
    const unsigned blocks =
        (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, (int64_t)sms * 32));
    cudaStream_t s = (cudaStream_t)stream;
    if (is_complex)
        eval_f64_kernel<true><<<blocks, 128, 0, s>>>((const float *)d_H, T, pitch, d_pairs,
                                                      num_pairs, vol.n[1], vol.n[2], vol,
                                                      (double)t0, (double)deltaT, d_voxel_ids, n,
                                                      d_out);
    else
        eval_f64_kernel<false><<<blocks, 128, 0, s>>>((const float *)d_H, T, pitch, d_pairs,
                                                       num_pairs, vol.n[1], vol.n[2], vol,
                                                       (double)t0, (double)deltaT, d_voxel_ids,
                                                       n, d_out);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}
