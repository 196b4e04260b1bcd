// Device kernels of the learned-octree reconstruction and its training data:
//
//   * a scene renderer (transients of point scatterers, the GPU form of
//     bpgb_synth_render) so that thousands of seeded training scenes render in
//     milliseconds each;
//   * block max-pooling of a volume (occupancy labels and block scores);
//   * trilinear fill of a fine volume from a coarse one over the same box (the value
//     of blocks the block-sparse pass skips).
//
// The reference's octree (octree_volume.hpp, backproject.hpp:264-335 on the CPU,
// backproject_cuda.cu:183-367 on the GPU) refines a volume level by level and drops
// regions whose mean falls under a threshold; these kernels serve its learned
// replacement, which predicts occupied blocks from one coarse pass.
#include <cuda_runtime.h>

#include <cstdint>

#include "bpgb_internal.h"
#include "bpgb_synth.h"

namespace bpgb {
namespace {

// One warp per pair.  Lanes evaluate 32 consecutive scatterers at a time; the hits are
// added to the pair's row (FP64, shared memory) in scatterer order per bin, so the
// result does not depend on thread timing.  Geometry in FP32: |l - q| and |q - c| from
// FP32 differences, squares summed x, y, z in order.
__global__ void render_kernel(const bpgb_pair *__restrict__ pairs, uint64_t P, uint32_t T,
                              float t0, float inv_dT, const float *__restrict__ points,
                              const float *__restrict__ albedo, uint64_t n_points,
                              float *__restrict__ out, uint32_t pitch) {
    extern __shared__ double row[];
    const uint32_t lane = threadIdx.x;
    for (uint64_t p = blockIdx.x; p < P; p += gridDim.x) {
        for (uint32_t t = lane; t < T; t += 32) row[t] = 0.0;
        __syncwarp();
        const bpgb_pair pr = pairs[p];
        const float lw_cw = __fadd_rn(pr.laser_wall, pr.camera_wall);
        for (uint64_t base = 0; base < n_points; base += 32) {
            const uint64_t i = base + lane;
            int32_t bin = -1;
            double v = 0.0;
            if (i < n_points) {
                const float qx = points[3 * i], qy = points[3 * i + 1], qz = points[3 * i + 2];
                const float ax = __fsub_rn(pr.laser_point[0], qx);
                const float ay = __fsub_rn(pr.laser_point[1], qy);
                const float az = __fsub_rn(pr.laser_point[2], qz);
                const float bx = __fsub_rn(qx, pr.camera_point[0]);
                const float by = __fsub_rn(qy, pr.camera_point[1]);
                const float bz = __fsub_rn(qz, pr.camera_point[2]);
                const float a2 = __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)),
                                           __fmul_rn(az, az));
                const float b2 = __fadd_rn(__fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by)),
                                           __fmul_rn(bz, bz));
                const float d = __fadd_rn(__fadd_rn(lw_cw, __fsqrt_rn(a2)), __fsqrt_rn(b2));
                const float b = roundf(__fmul_rn(__fsub_rn(d, t0), inv_dT));
                if (a2 > 0.0f && b2 > 0.0f && b >= 0.0f && b < (float)T) {
                    bin = (int32_t)b;
                    v = (double)albedo[i] / ((double)a2 * (double)b2);
                }
            }
            // lanes hitting the same bin add in lane (= scatterer) order
            const uint32_t valid = __ballot_sync(0xffffffffu, bin >= 0);
            if (!valid) continue;
            const uint32_t peers = __match_any_sync(0xffffffffu, bin);
            const uint32_t rank = bin >= 0 ? __popc(peers & ((1u << lane) - 1u)) : 0u;
            for (uint32_t r = 0; __any_sync(0xffffffffu, rank >= r); r++) {
                if (bin >= 0 && rank == r) row[bin] += v;
                __syncwarp();
            }
        }
        __syncwarp();
        float *o = out + p * (uint64_t)pitch;
        for (uint32_t t = lane; t < T; t += 32) o[t] = (float)row[t];
        for (uint32_t t = T + lane; t < pitch; t += 32) o[t] = 0.0f;
        __syncwarp();
    }
}

// out[b] = max over the bs^3 voxels of block b of vol (blocks clipped at the volume edge).
__global__ void block_max_kernel(const float *__restrict__ vol, uint32_t n0, uint32_t n1,
                                 uint32_t n2, uint32_t bs, uint32_t b0, uint32_t b1, uint32_t b2,
                                 float *__restrict__ out) {
    const uint64_t nb = (uint64_t)b0 * b1 * b2;
    for (uint64_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const uint32_t bz = (uint32_t)(b % b2), by = (uint32_t)((b / b2) % b1),
                       bx = (uint32_t)(b / ((uint64_t)b2 * b1));
        float m = -INFINITY;
        const uint32_t vox = bs * bs * bs;
        for (uint32_t i = threadIdx.x; i < vox; i += blockDim.x) {
            const uint32_t x = bx * bs + i / (bs * bs), y = by * bs + (i / bs) % bs,
                           z = bz * bs + i % bs;
            if (x < n0 && y < n1 && z < n2) m = fmaxf(m, vol[((uint64_t)x * n1 + y) * n2 + z]);
        }
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        __shared__ float part[32];
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            float r = part[0];
            for (uint32_t w = 1; w < (blockDim.x + 31) / 32; w++) r = fmaxf(r, part[w]);
            out[b] = r;
        }
        __syncthreads();
    }
}

// fine[i, j, k] = trilinear sample of coarse at (i (c0-1)/(f0-1), ...): both grids span
// the same box with the reference's spacing size / (n - 1).  One CTA per fine (i, j) line:
// the four coarse z-lines around it are blended in x and y once into shared memory, then
// the threads interpolate along z and write the line with coalesced stores.
__global__ void upsample_kernel(const float *__restrict__ coarse, uint32_t c0, uint32_t c1,
                                uint32_t c2, float *__restrict__ fine, uint32_t f0, uint32_t f1,
                                uint32_t f2) {
    extern __shared__ float line[];  // c2 floats
    const uint32_t j = blockIdx.x, i = blockIdx.y;
    const float s0 = f0 > 1 ? (float)(c0 - 1) / (float)(f0 - 1) : 0.0f;
    const float s1 = f1 > 1 ? (float)(c1 - 1) / (float)(f1 - 1) : 0.0f;
    const float s2 = f2 > 1 ? (float)(c2 - 1) / (float)(f2 - 1) : 0.0f;
    const float u0 = i * s0, u1 = j * s1;
    const float fl0 = floorf(u0), fl1 = floorf(u1);
    const uint32_t x0 = min((uint32_t)fl0, c0 - 1), x1 = min(x0 + 1, c0 - 1);
    const uint32_t y0 = min((uint32_t)fl1, c1 - 1), y1 = min(y0 + 1, c1 - 1);
    const float w0 = u0 - fl0, w1 = u1 - fl1;
    for (uint32_t z = threadIdx.x; z < c2; z += blockDim.x) {
        auto at = [&](uint32_t x, uint32_t y) { return coarse[((uint64_t)x * c1 + y) * c2 + z]; };
        const float a0 = at(x0, y0) * (1 - w1) + at(x0, y1) * w1;
        const float a1 = at(x1, y0) * (1 - w1) + at(x1, y1) * w1;
        line[z] = a0 * (1 - w0) + a1 * w0;
    }
    __syncthreads();
    float *out = fine + ((uint64_t)i * f1 + j) * f2;
    for (uint32_t k = threadIdx.x; k < f2; k += blockDim.x) {
        const float u2 = k * s2, fl2 = floorf(u2);
        const uint32_t z0 = min((uint32_t)fl2, c2 - 1), z1 = min(z0 + 1, c2 - 1);
        const float w2 = u2 - fl2;
        out[k] = line[z0] * (1 - w2) + line[z1] * w2;
    }
}

// out[v] = sum over the in-volume face neighbours u of (vol[v] - vol[u]): the negated
// 7-point Laplacian (positive at local maxima), neighbours outside the volume omitted.
__global__ void laplacian7_kernel(const float *__restrict__ vol, uint32_t n0, uint32_t n1,
                                  uint32_t n2, float *__restrict__ out) {
    const uint64_t n = (uint64_t)n0 * n1 * n2;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t z = (uint32_t)(v % n2), y = (uint32_t)((v / n2) % n1),
                       x = (uint32_t)(v / ((uint64_t)n2 * n1));
        const float c = vol[v];
        float s = 0.0f;
        if (x > 0) s += c - vol[v - (uint64_t)n1 * n2];
        if (x + 1 < n0) s += c - vol[v + (uint64_t)n1 * n2];
        if (y > 0) s += c - vol[v - n2];
        if (y + 1 < n1) s += c - vol[v + n2];
        if (z > 0) s += c - vol[v - 1];
        if (z + 1 < n2) s += c - vol[v + 1];
        out[v] = s;
    }
}

// Trilinear sample of a coarse grid spanning the fine grid's box at fine index
// (x, y, z), with upsample_kernel's coordinate mapping and clamping.
__device__ __forceinline__ float trilinear_at(const float *__restrict__ c, uint32_t c0,
                                              uint32_t c1, uint32_t c2, float s0, float s1,
                                              float s2, uint32_t x, uint32_t y, uint32_t z) {
    const float u0 = x * s0, u1 = y * s1, u2 = z * s2;
    const float f0 = floorf(u0), f1 = floorf(u1), f2 = floorf(u2);
    const uint32_t x0 = min((uint32_t)f0, c0 - 1), x1 = min(x0 + 1, c0 - 1);
    const uint32_t y0 = min((uint32_t)f1, c1 - 1), y1 = min(y0 + 1, c1 - 1);
    const uint32_t z0 = min((uint32_t)f2, c2 - 1), z1 = min(z0 + 1, c2 - 1);
    const float w0 = u0 - f0, w1 = u1 - f1, w2 = u2 - f2;
    auto at = [&](uint32_t i, uint32_t j, uint32_t k) { return c[((uint64_t)i * c1 + j) * c2 + k]; };
    auto line = [&](uint32_t i, uint32_t j) { return at(i, j, z0) * (1 - w2) + at(i, j, z1) * w2; };
    const float a0 = line(x0, y0) * (1 - w1) + line(x0, y1) * w1;
    const float a1 = line(x1, y0) * (1 - w1) + line(x1, y1) * w1;
    return a0 * (1 - w0) + a1 * w0;
}

// One warp per fine block of bs^3 voxels: the mean over ns^3 evenly spread voxels of the
// block of (fill_hi - fill_lo)^2, the squared difference between the trilinear fills of
// two coarse passes over the same box -- the detail the finer pass adds there, a
// predictor of the fill's error.  Blocks whose logit reaches logit_lo (when logits are
// given, one per block) score +inf, so a top-k selection takes them first.
__global__ void block_detail_kernel(const float *__restrict__ lo, uint32_t l0, uint32_t l1,
                                    uint32_t l2, const float *__restrict__ hi, uint32_t h0,
                                    uint32_t h1, uint32_t h2, uint32_t f0, uint32_t f1,
                                    uint32_t f2, uint32_t bs, uint32_t ns, uint32_t b0,
                                    uint32_t b1, uint32_t b2, const float *__restrict__ logits,
                                    float logit_lo, float *__restrict__ out) {
    const uint64_t nb = (uint64_t)b0 * b1 * b2;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    auto scale = [](uint32_t c, uint32_t f) { return f > 1 ? (float)(c - 1) / (float)(f - 1) : 0.0f; };
    const float ls0 = scale(l0, f0), ls1 = scale(l1, f1), ls2 = scale(l2, f2);
    const float hs0 = scale(h0, f0), hs1 = scale(h1, f1), hs2 = scale(h2, f2);
    const uint32_t npts = ns * ns * ns;
    for (uint64_t b = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < nb;
         b += warps) {
        const uint32_t bz = (uint32_t)(b % b2), by = (uint32_t)((b / b2) % b1),
                       bx = (uint32_t)(b / ((uint64_t)b2 * b1));
        float acc = 0.0f;
        uint32_t cnt = 0;
        for (uint32_t i = lane; i < npts; i += 32) {
            // sample k of ns along an axis sits at (2k + 1) bs / (2 ns) inside the block
            const uint32_t x = bx * bs + (2 * (i / (ns * ns)) + 1) * bs / (2 * ns);
            const uint32_t y = by * bs + (2 * ((i / ns) % ns) + 1) * bs / (2 * ns);
            const uint32_t z = bz * bs + (2 * (i % ns) + 1) * bs / (2 * ns);
            if (x < f0 && y < f1 && z < f2) {
                const float d = trilinear_at(hi, h0, h1, h2, hs0, hs1, hs2, x, y, z) -
                                trilinear_at(lo, l0, l1, l2, ls0, ls1, ls2, x, y, z);
                acc += d * d;
                cnt++;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            float sc = cnt ? acc / (float)cnt : 0.0f;
            if (!(sc >= 0.0f)) sc = 0.0f;  // NaN-safe: scores are non-negative
            if (logits && logits[b] >= logit_lo) sc = INFINITY;
            out[b] = sc;
        }
    }
}

__global__ void complex_abs_kernel(const float2 *__restrict__ in, uint64_t n,
                                   float *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 z = in[i];
        out[i] = sqrtf(z.x * z.x + z.y * z.y);
    }
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" {

int bpgb_synth_render_device(const bpgb_pair *d_pairs, uint64_t num_pairs, uint32_t T, float t0,
                             float deltaT, const float *d_points, const float *d_albedo,
                             uint64_t num_points, float *d_out, uint32_t pitch, void *stream) {
    clear_error();
    if ((num_pairs && (!d_pairs || !d_out)) || (num_points && (!d_points || !d_albedo)) ||
        T == 0 || !(deltaT > 0.0f) || pitch < T)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad render arguments");
    if (num_pairs == 0) return BPGB_OK;
    const size_t smem = (size_t)T * sizeof(double);
    if (smem > 200 * 1024) return set_error(BPGB_ERR_UNSUPPORTED, "T too large for the device renderer");
    int st = require_device();
    if (st) return st;
    st = reserve_dynamic_smem((const void *)render_kernel, (uint32_t)smem);
    if (st) return st;
    const unsigned grid = (unsigned)(num_pairs < (1u << 20) ? num_pairs : (1u << 20));
    render_kernel<<<grid, 32, smem, (cudaStream_t)stream>>>(d_pairs, num_pairs, T, t0,
                                                          1.0f / deltaT, d_points, d_albedo,
                                                          num_points, d_out, pitch);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_block_max(const float *d_volume, const uint32_t *voxels_per_side, uint32_t block_size,
                   float *d_out, void *stream) {
    clear_error();
    if (!d_volume || !voxels_per_side || !d_out || block_size == 0 || block_size > 64)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad block_max arguments");
    const uint32_t *n = voxels_per_side;
    const uint32_t b0 = (n[0] + block_size - 1) / block_size, b1 = (n[1] + block_size - 1) / block_size,
                   b2 = (n[2] + block_size - 1) / block_size;
    const uint64_t nb = (uint64_t)b0 * b1 * b2;
    if (nb == 0) return BPGB_OK;
    const unsigned grid = (unsigned)(nb < (1u << 20) ? nb : (1u << 20));
    block_max_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_volume, n[0], n[1], n[2], block_size,
                                                           b0, b1, b2, d_out);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_upsample_trilinear(const float *d_coarse, const uint32_t *coarse_dims, float *d_fine,
                            const uint32_t *fine_dims, void *stream) {
    clear_error();
    if (!d_coarse || !coarse_dims || !d_fine || !fine_dims)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    for (int a = 0; a < 3; a++)
        if (!coarse_dims[a] || !fine_dims[a])
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "empty grid");
    if (fine_dims[0] > 65535 || fine_dims[1] > (1u << 31) - 1 || coarse_dims[2] > 12288)
        return set_error(BPGB_ERR_UNSUPPORTED, "upsample grid too large");
    const dim3 grid(fine_dims[1], fine_dims[0]);
    upsample_kernel<<<grid, 256, coarse_dims[2] * sizeof(float), (cudaStream_t)stream>>>(
        d_coarse, coarse_dims[0], coarse_dims[1], coarse_dims[2], d_fine, fine_dims[0],
        fine_dims[1], fine_dims[2]);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_laplacian7(const float *d_volume, const uint32_t *voxels_per_side, float *d_out,
                    void *stream) {
    clear_error();
    if (!d_volume || !voxels_per_side || !d_out || d_volume == d_out)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad laplacian arguments");
    const uint32_t *n = voxels_per_side;
    const uint64_t total = (uint64_t)n[0] * n[1] * n[2];
    if (total == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((total + 255) / 256 < 152 * 16 ? (total + 255) / 256 : 152 * 16);
    laplacian7_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_volume, n[0], n[1], n[2], d_out);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_block_detail(const float *d_coarse_lo, const uint32_t *lo_dims, const float *d_coarse_hi,
                      const uint32_t *hi_dims, const uint32_t *fine_dims, uint32_t block_size,
                      uint32_t samples, const float *d_logits, float logit_lo, float *d_score,
                      void *stream) {
    clear_error();
    if (!d_coarse_lo || !lo_dims || !d_coarse_hi || !hi_dims || !fine_dims || !d_score ||
        block_size == 0 || samples == 0 || samples > block_size)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad block_detail arguments");
    for (int a = 0; a < 3; a++)
        if (!lo_dims[a] || !hi_dims[a] || !fine_dims[a])
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "empty grid");
    const uint32_t *f = fine_dims;
    const uint32_t b0 = (f[0] + block_size - 1) / block_size, b1 = (f[1] + block_size - 1) / block_size,
                   b2 = (f[2] + block_size - 1) / block_size;
    const uint64_t nb = (uint64_t)b0 * b1 * b2;
    const unsigned grid = (unsigned)((nb + 7) / 8 < 152 * 16 ? (nb + 7) / 8 : 152 * 16);
    block_detail_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        d_coarse_lo, lo_dims[0], lo_dims[1], lo_dims[2], d_coarse_hi, hi_dims[0], hi_dims[1],
        hi_dims[2], f[0], f[1], f[2], block_size, samples, b0, b1, b2, d_logits, logit_lo, d_score);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_complex_abs(const float *d_in, uint64_t n, float *d_out, void *stream) {
    clear_error();
    if (!d_in || !d_out || ((uintptr_t)d_in) % 8)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad complex_abs arguments");
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
    complex_abs_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const float2 *)d_in, n, d_out);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

}  // extern "C"
