// BF16 tensor-core kernels of the occupancy CNN (learned octree): 3x3x3 convolutions
// (zero padding, stride 1) as implicit GEMMs on mma.sync m16n8k16 (BF16 operands, FP32
// accumulate), their weight gradients, BCE-with-logits gradients and Adam.
//
// Layout.  Activations are channels-last BF16 [V][C] (voxel v = ((s n0 + x) n1 + y) n2 + z
// for sample s of a batch, z fastest) with a channel stride xs >= C.  A layer with CIN
// input and COUT output channels has the GEMM shape M = voxels, N = COUT padded to NP
// (8 or 16), K = 27 CIN + 1 padded to KP (multiple of 16): row k < 27 CIN holds tap
// k / CIN (offsets (k/CIN)/9-1, (k/CIN)/3%3-1, (k/CIN)%3-1 in x, y, z) and input channel
// k % CIN; row 27 CIN multiplies a constant 1 (the bias); the rest are zero.  The master
// weights are FP32 [KP][COUT]; the kernels read a packed BF16 copy Wt[NP][KP] (k
// contiguous per output channel).  The backward-data pass of a layer is the forward
// kernel run on the gradient with the flipped, channel-transposed weights (tap 26 - t,
// CIN <-> COUT, no bias) and the previous layer's ReLU mask.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

constexpr int kTaps = 27;

struct Geo {
    uint32_t n0, n1, n2;
    uint32_t batch;
    uint64_t vox;  // n0 n1 n2
};

__device__ __forceinline__ void coords(const Geo &g, uint64_t v, uint64_t &s, int &x, int &y,
                                       int &z) {
    s = v / g.vox;
    const uint64_t r = v - s * g.vox;
    z = (int)(r % g.n2);
    y = (int)((r / g.n2) % g.n1);
    x = (int)(r / ((uint64_t)g.n2 * g.n1));
}

// Voxel index of v shifted by tap t, or -1 outside the sample's volume.
__device__ __forceinline__ int64_t shifted(const Geo &g, uint64_t s, int x, int y, int z, int t) {
    x += t / 9 - 1;
    y += (t / 3) % 3 - 1;
    z += t % 3 - 1;
    if (x < 0 || y < 0 || z < 0 || x >= (int)g.n0 || y >= (int)g.n1 || z >= (int)g.n2) return -1;
    return (int64_t)(s * g.vox + ((uint64_t)x * g.n1 + y) * g.n2 + z);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<const uint32_t *>(&p);
}

__device__ __forceinline__ float bf(const __nv_bfloat16 *p, int64_t i) {
    return __bfloat162float(p[i]);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Element (v, k) of the implicit im2col matrix (bias row = 1, padding = 0).
template <int CIN>
__device__ __forceinline__ float im2col(const __nv_bfloat16 *X, uint32_t xs, const Geo &g,
                                        uint64_t s, int x, int y, int z, int k) {
    if (k < kTaps * CIN) {
        const int64_t u = shifted(g, s, x, y, z, k / CIN);
        return u < 0 ? 0.0f : bf(X, u * xs + k % CIN);
    }
    return k == kTaps * CIN ? 1.0f : 0.0f;
}

template <int CIN>
__host__ __device__ constexpr int kp_of() {
    return (kTaps * CIN + 1 + 15) / 16 * 16;
}

// ---- forward (and backward-data) ------------------------------------------------
// Each warp computes 16 voxels x NP outputs per tile; 4 warps per CTA.
template <int CIN, int NP>
__global__ void __launch_bounds__(128)
    conv_fwd_kernel(const __nv_bfloat16 *__restrict__ X, uint32_t xs, Geo g,
                    const __nv_bfloat16 *__restrict__ Wt, int relu,
                    const __nv_bfloat16 *__restrict__ mask, uint32_t mstride,
                    __nv_bfloat16 *__restrict__ Y, float *__restrict__ Yf) {
    constexpr int KP = kp_of<CIN>();
    constexpr int NT = NP / 8;
    __shared__ __align__(16) __nv_bfloat16 w_s[NP * KP];
    for (int i = threadIdx.x; i < NP * KP; i += blockDim.x) w_s[i] = Wt[i];
    __syncthreads();
    const uint64_t V = g.vox * g.batch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
    for (uint64_t m0 = ((uint64_t)blockIdx.x * 4 + warp) * 16; m0 < V;
         m0 += (uint64_t)gridDim.x * 64) {
        const uint64_t r[2] = {m0 + grp, m0 + grp + 8};
        uint64_t sr[2];
        int xr[2], yr[2], zr[2];
        bool ok[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            ok[h] = r[h] < V;
            coords(g, ok[h] ? r[h] : 0, sr[h], xr[h], yr[h], zr[h]);
        }
        float acc[NT][4];
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int i = 0; i < 4; i++) acc[nt][i] = 0.0f;
#pragma unroll 1
        for (int ks = 0; ks < KP / 16; ks++) {
            uint32_t a[4];
            if (CIN == 16 && ks < kTaps) {
                // one tap, 16 channels: two 32-bit loads per row
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int64_t u = ok[h] ? shifted(g, sr[h], xr[h], yr[h], zr[h], ks) : -1;
                    a[h] = a[h + 2] = 0u;
                    if (u >= 0) {
                        const uint32_t *row = reinterpret_cast<const uint32_t *>(X + u * xs);
                        a[h] = row[tig];
                        a[h + 2] = row[tig + 4];
                    }
                }
            } else {
                const int k0 = ks * 16 + 2 * tig;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    float e[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                    if (ok[h]) {
                        e[0] = im2col<CIN>(X, xs, g, sr[h], xr[h], yr[h], zr[h], k0);
                        e[1] = im2col<CIN>(X, xs, g, sr[h], xr[h], yr[h], zr[h], k0 + 1);
                        e[2] = im2col<CIN>(X, xs, g, sr[h], xr[h], yr[h], zr[h], k0 + 8);
                        e[3] = im2col<CIN>(X, xs, g, sr[h], xr[h], yr[h], zr[h], k0 + 9);
                    }
                    a[h] = pack2(e[0], e[1]);
                    a[h + 2] = pack2(e[2], e[3]);
                }
            }
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const uint32_t *wr =
                    reinterpret_cast<const uint32_t *>(w_s + (nt * 8 + grp) * KP + ks * 16);
                mma_bf16(acc[nt], a, wr[tig], wr[tig + 4]);
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!ok[h]) continue;
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const int c = nt * 8 + 2 * tig;
                float v0 = acc[nt][2 * h], v1 = acc[nt][2 * h + 1];
                if (relu) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                if (mask) {
                    if (!(bf(mask, r[h] * mstride + c) > 0.0f)) v0 = 0.0f;
                    if (!(bf(mask, r[h] * mstride + c + 1) > 0.0f)) v1 = 0.0f;
                }
                if (Y) *reinterpret_cast<uint32_t *>(Y + r[h] * NP + c) = pack2(v0, v1);
                if (Yf && c == 0) Yf[r[h]] = v0;
            }
        }
    }
}

// ---- weight gradient ----------------------------------------------------------------
// dW[k][n] = sum_v im2col(v, k) dY[v][n].  CTA (split, mt): rows mt*16 .. +15 of dW over
// the voxels [split * vpc, (split + 1) * vpc); partial sums land in
// partial[split][KP][NP] and are reduced in split order.
template <int CIN, int NP>
__global__ void __launch_bounds__(128)
    conv_wgrad_kernel(const __nv_bfloat16 *__restrict__ X, uint32_t xs, Geo g,
                      const __nv_bfloat16 *__restrict__ dY, uint32_t vpc,
                      float *__restrict__ partial) {
    constexpr int KP = kp_of<CIN>();
    constexpr int NT = NP / 8;
    __shared__ float red[4][16][NP];
    const uint64_t V = g.vox * g.batch;
    const uint32_t split = blockIdx.x, mt = blockIdx.y;
    const uint64_t vbeg = (uint64_t)split * vpc;
    const uint64_t vend = vbeg + vpc < V ? vbeg + vpc : V;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
    const int kr0 = mt * 16 + grp, kr1 = kr0 + 8;
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc[nt][i] = 0.0f;
    for (uint64_t v0 = vbeg + (uint64_t)warp * 16; v0 < vend; v0 += 64) {
        const uint64_t vv[4] = {v0 + 2 * tig, v0 + 2 * tig + 1, v0 + 2 * tig + 8, v0 + 2 * tig + 9};
        float e0[4], e1[4];
        uint32_t bb[NT][2];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            e0[j] = e1[j] = 0.0f;
            if (vv[j] < vend) {
                uint64_t s;
                int x, y, z;
                coords(g, vv[j], s, x, y, z);
                e0[j] = im2col<CIN>(X, xs, g, s, x, y, z, kr0);
                e1[j] = im2col<CIN>(X, xs, g, s, x, y, z, kr1);
            }
        }
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
            const int n = nt * 8 + grp;
            float d[4];
#pragma unroll
            for (int j = 0; j < 4; j++) d[j] = vv[j] < vend ? bf(dY, vv[j] * NP + n) : 0.0f;
            bb[nt][0] = pack2(d[0], d[1]);
            bb[nt][1] = pack2(d[2], d[3]);
        }
        const uint32_t a[4] = {pack2(e0[0], e0[1]), pack2(e1[0], e1[1]), pack2(e0[2], e0[3]),
                               pack2(e1[2], e1[3])};
#pragma unroll
        for (int nt = 0; nt < NT; nt++) mma_bf16(acc[nt], a, bb[nt][0], bb[nt][1]);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const int c = nt * 8 + 2 * tig;
        red[warp][grp][c] = acc[nt][0];
        red[warp][grp][c + 1] = acc[nt][1];
        red[warp][grp + 8][c] = acc[nt][2];
        red[warp][grp + 8][c + 1] = acc[nt][3];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 16 * NP; i += blockDim.x) {
        const int row = i / NP, n = i % NP;
        const float sum = ((red[0][row][n] + red[1][row][n]) + red[2][row][n]) + red[3][row][n];
        partial[((uint64_t)split * KP + mt * 16 + row) * NP + n] = sum;
    }
    (void)kr1;
}

__global__ void reduce_partials_kernel(const float *__restrict__ partial, uint32_t splits,
                                       uint32_t KP, uint32_t NP, uint32_t cout,
                                       float *__restrict__ dW) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= KP * cout) return;
    const uint32_t k = i / cout, n = i % cout;
    float s = 0.0f;
    for (uint32_t p = 0; p < splits; p++) s += partial[((uint64_t)p * KP + k) * NP + n];
    dW[i] = s;  // [KP][COUT]
}

// ---- weights, loss, optimiser -----------------------------------------------------
// Wt[n][k] = W[k][n] (BF16, zero for n >= cout); Wb (when non-null) = the backward-data
// weights: Wb[ci][k'] with k' = t' cout + co = W[(26 - t') cin + ci][co], bias row 0.
__global__ void pack_weights_kernel(const float *__restrict__ W, uint32_t cin, uint32_t cout,
                                    uint32_t KP, uint32_t NP, __nv_bfloat16 *__restrict__ Wt,
                                    uint32_t KPb, uint32_t NPb, __nv_bfloat16 *__restrict__ Wb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < NP * KP) {
        const uint32_t n = i / KP, k = i % KP;
        Wt[i] = __float2bfloat16_rn(n < cout ? W[(uint64_t)k * cout + n] : 0.0f);
    }
    if (Wb && i < NPb * KPb) {
        const uint32_t ci = i / KPb, kb = i % KPb;
        float w = 0.0f;
        if (ci < cin && kb < kTaps * cout) {
            const uint32_t tb = kb / cout, co = kb % cout;
            w = W[((uint64_t)(26 - tb) * cin + ci) * cout + co];
        }
        Wb[i] = __float2bfloat16_rn(w);
    }
}

// dZ[v][0] = w (sigmoid(z) - y) * scale with w = pos_weight for y = 1 (channels 1..7 zero);
// loss[v] = w (softplus(z) - y z) * scale.
__global__ void bce_grad_kernel(const float *__restrict__ logits, const uint8_t *__restrict__ y,
                                uint64_t n, float pos_weight, float scale,
                                __nv_bfloat16 *__restrict__ dZ, float *__restrict__ loss) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float z = logits[i];
        const float t = y[i] ? 1.0f : 0.0f;
        const float w = y[i] ? pos_weight : 1.0f;
        const float sig = 1.0f / (1.0f + expf(-z));
        const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
        uint4 *row = reinterpret_cast<uint4 *>(dZ + i * 8);
        const __nv_bfloat16 g = __float2bfloat16_rn(w * (sig - t) * scale);
        uint4 r = make_uint4(0, 0, 0, 0);
        r.x = (uint32_t)__bfloat16_as_ushort(g);
        *row = r;
        if (loss) loss[i] = w * (sp - t * z) * scale;
    }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, uint64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// X[v] = coarse[v] / max over the sample (BF16), one CTA per sample.
__global__ void normalize_kernel(const float *__restrict__ coarse, uint64_t vox,
                                 __nv_bfloat16 *__restrict__ X) {
    const float *c = coarse + blockIdx.x * vox;
    float m = 0.0f;
    for (uint64_t i = threadIdx.x; i < vox; i += blockDim.x) m = fmaxf(m, c[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        float r = threadIdx.x < (blockDim.x + 31) / 32 ? part[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
        if (threadIdx.x == 0) part[0] = r;
    }
    __syncthreads();
    const float inv = part[0] > 0.0f ? 1.0f / part[0] : 0.0f;
    for (uint64_t i = threadIdx.x; i < vox; i += blockDim.x)
        X[blockIdx.x * vox + i] = __float2bfloat16_rn(c[i] * inv);
}

// X[v][0] = coarse / max(coarse), X[v][1] = F / max|F| with F the negated 7-point
// Laplacian of the coarse volume (in-volume neighbours), per sample (one CTA each).
__global__ void features_kernel(const float *__restrict__ coarse, Geo g,
                                __nv_bfloat16 *__restrict__ X) {
    const float *c = coarse + blockIdx.x * g.vox;
    auto lap = [&](uint64_t r) {
        const uint32_t z = (uint32_t)(r % g.n2), y = (uint32_t)((r / g.n2) % g.n1),
                       x = (uint32_t)(r / ((uint64_t)g.n2 * g.n1));
        const float v = c[r];
        float s = 0.0f;
        if (x > 0) s += v - c[r - (uint64_t)g.n1 * g.n2];
        if (x + 1 < g.n0) s += v - c[r + (uint64_t)g.n1 * g.n2];
        if (y > 0) s += v - c[r - g.n2];
        if (y + 1 < g.n1) s += v - c[r + g.n2];
        if (z > 0) s += v - c[r - 1];
        if (z + 1 < g.n2) s += v - c[r + 1];
        return s;
    };
    float m0 = 0.0f, m1 = 0.0f;
    for (uint64_t i = threadIdx.x; i < g.vox; i += blockDim.x) {
        m0 = fmaxf(m0, c[i]);
        m1 = fmaxf(m1, fabsf(lap(i)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    }
    __shared__ float part[2][32];
    if ((threadIdx.x & 31) == 0) {
        part[0][threadIdx.x >> 5] = m0;
        part[1][threadIdx.x >> 5] = m1;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = threadIdx.x < (blockDim.x + 31) / 32;
        float r0 = in ? part[0][threadIdx.x] : 0.0f, r1 = in ? part[1][threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) {
            r0 = fmaxf(r0, __shfl_xor_sync(0xffffffffu, r0, o));
            r1 = fmaxf(r1, __shfl_xor_sync(0xffffffffu, r1, o));
        }
        __syncwarp();
        if (threadIdx.x == 0) {
            part[0][0] = r0;
            part[1][0] = r1;
        }
    }
    __syncthreads();
    const float i0 = part[0][0] > 0.0f ? 1.0f / part[0][0] : 0.0f;
    const float i1 = part[1][0] > 0.0f ? 1.0f / part[1][0] : 0.0f;
    __nv_bfloat16 *x = X + blockIdx.x * g.vox * 2;
    for (uint64_t i = threadIdx.x; i < g.vox; i += blockDim.x) {
        x[2 * i] = __float2bfloat16_rn(c[i] * i0);
        x[2 * i + 1] = __float2bfloat16_rn(lap(i) * i1);
    }
}

// Grid-wide form of features_kernel: pass 1 folds each sample's max(c, 0) and max |F|
// into scratch[2 s], scratch[2 s + 1] (float bits compare as unsigned for values >= 0),
// pass 2 writes both channels.
__device__ __forceinline__ float lap7(const float *c, const Geo &g, uint64_t r) {
    const uint32_t z = (uint32_t)(r % g.n2), y = (uint32_t)((r / g.n2) % g.n1),
                   x = (uint32_t)(r / ((uint64_t)g.n2 * g.n1));
    const float v = c[r];
    float s = 0.0f;
    if (x > 0) s += v - c[r - (uint64_t)g.n1 * g.n2];
    if (x + 1 < g.n0) s += v - c[r + (uint64_t)g.n1 * g.n2];
    if (y > 0) s += v - c[r - g.n2];
    if (y + 1 < g.n1) s += v - c[r + g.n2];
    if (z > 0) s += v - c[r - 1];
    if (z + 1 < g.n2) s += v - c[r + 1];
    return s;
}

__global__ void features_max_kernel(const float *__restrict__ coarse, Geo g,
                                    unsigned int *__restrict__ scratch) {
    const float *c = coarse + blockIdx.y * g.vox;
    float m0 = 0.0f, m1 = 0.0f;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < g.vox;
         i += (uint64_t)gridDim.x * blockDim.x) {
        m0 = fmaxf(m0, c[i]);
        m1 = fmaxf(m1, fabsf(lap7(c, g, i)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&scratch[2 * blockIdx.y], __float_as_uint(m0));
        atomicMax(&scratch[2 * blockIdx.y + 1], __float_as_uint(m1));
    }
}

__global__ void features_write_kernel(const float *__restrict__ coarse, Geo g,
                                      const unsigned int *__restrict__ scratch,
                                      __nv_bfloat16 *__restrict__ X) {
    const float *c = coarse + blockIdx.y * g.vox;
    const float mx0 = __uint_as_float(scratch[2 * blockIdx.y]);
    const float mx1 = __uint_as_float(scratch[2 * blockIdx.y + 1]);
    const float i0 = mx0 > 0.0f ? 1.0f / mx0 : 0.0f, i1 = mx1 > 0.0f ? 1.0f / mx1 : 0.0f;
    __nv_bfloat16 *x = X + blockIdx.y * g.vox * 2;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < g.vox;
         i += (uint64_t)gridDim.x * blockDim.x)
        *reinterpret_cast<__nv_bfloat162 *>(x + 2 * i) =
            __floats2bfloat162_rn(c[i] * i0, lap7(c, g, i) * i1);
}

template <int CIN, int NP>
int launch_fwd(const void *X, uint32_t xs, const Geo &g, const void *Wt, int relu,
               const void *mask, uint32_t ms, void *Y, float *Yf, cudaStream_t s) {
    const uint64_t V = g.vox * g.batch;
    const uint64_t tiles = (V + 63) / 64;
    const unsigned grid = (unsigned)(tiles < 152 * 16 ? tiles : 152 * 16);
    conv_fwd_kernel<CIN, NP><<<grid, 128, 0, s>>>(
        (const __nv_bfloat16 *)X, xs, g, (const __nv_bfloat16 *)Wt, relu,
        (const __nv_bfloat16 *)mask, ms, (__nv_bfloat16 *)Y, Yf);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

template <int CIN, int NP>
int launch_wgrad(const void *X, uint32_t xs, const Geo &g, const void *dY, float *partial,
                 uint32_t splits, uint32_t vpc, uint32_t cout, float *dW, cudaStream_t s) {
    constexpr int KP = kp_of<CIN>();
    conv_wgrad_kernel<CIN, NP><<<dim3(splits, KP / 16), 128, 0, s>>>(
        (const __nv_bfloat16 *)X, xs, g, (const __nv_bfloat16 *)dY, vpc, partial);
    count_launches(1);
    reduce_partials_kernel<<<(KP * cout + 255) / 256, 256, 0, s>>>(partial, splits, KP, NP, cout,
                                                                   dW);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

constexpr uint32_t kWgradVoxelsPerCta = 2048;

bool geo_of(const uint32_t *dims, uint32_t batch, Geo *g) {
    if (!dims || !batch || !dims[0] || !dims[1] || !dims[2]) return false;
    g->n0 = dims[0];
    g->n1 = dims[1];
    g->n2 = dims[2];
    g->batch = batch;
    g->vox = (uint64_t)dims[0] * dims[1] * dims[2];
    return true;
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" {

uint32_t bpgb_cnn_kp(uint32_t cin) { return (kTaps * cin + 1 + 15) / 16 * 16; }

int bpgb_cnn_conv3d(const void *d_X, uint32_t cin, uint32_t x_stride, const uint32_t *dims,
                    uint32_t batch, const void *d_Wt, uint32_t np, int relu, const void *d_mask,
                    uint32_t mask_stride, void *d_Y, float *d_Yf, void *stream) {
    clear_error();
    Geo g;
    if (!d_X || !d_Wt || !geo_of(dims, batch, &g) || (!d_Y && !d_Yf) || x_stride < cin ||
        (d_mask && mask_stride < np))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad conv3d arguments");
    if (cin == 16 && (x_stride % 2 || ((uintptr_t)d_X) % 4))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "16-channel input needs 4-byte aligned pairs");
    if (d_Y && ((uintptr_t)d_Y) % 4) return set_error(BPGB_ERR_INVALID_ARGUMENT, "Y misaligned");
    cudaStream_t s = (cudaStream_t)stream;
    if (cin == 1 && np == 16) return launch_fwd<1, 16>(d_X, x_stride, g, d_Wt, relu, d_mask, mask_stride, d_Y, d_Yf, s);
    if (cin == 2 && np == 16) return launch_fwd<2, 16>(d_X, x_stride, g, d_Wt, relu, d_mask, mask_stride, d_Y, d_Yf, s);
    if (cin == 16 && np == 16) return launch_fwd<16, 16>(d_X, x_stride, g, d_Wt, relu, d_mask, mask_stride, d_Y, d_Yf, s);
    if (cin == 16 && np == 8) return launch_fwd<16, 8>(d_X, x_stride, g, d_Wt, relu, d_mask, mask_stride, d_Y, d_Yf, s);
    return set_error(BPGB_ERR_UNSUPPORTED, "conv3d shapes: (cin, np) in {(1,16), (2,16), (16,16), (16,8)}");
}

uint64_t bpgb_cnn_wgrad_scratch_bytes(uint32_t cin, uint32_t np, const uint32_t *dims,
                                      uint32_t batch) {
    Geo g;
    if (!geo_of(dims, batch, &g)) return 0;
    const uint64_t splits = (g.vox * batch + kWgradVoxelsPerCta - 1) / kWgradVoxelsPerCta;
    return splits * bpgb_cnn_kp(cin) * np * sizeof(float);
}

int bpgb_cnn_conv3d_wgrad(const void *d_X, uint32_t cin, uint32_t x_stride, const uint32_t *dims,
                          uint32_t batch, const void *d_dY, uint32_t np, uint32_t cout,
                          float *d_scratch, uint64_t scratch_bytes, float *d_dW, void *stream) {
    clear_error();
    Geo g;
    if (!d_X || !d_dY || !d_dW || !d_scratch || !geo_of(dims, batch, &g) || x_stride < cin ||
        cout == 0 || cout > np)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad conv3d_wgrad arguments");
    if (scratch_bytes < bpgb_cnn_wgrad_scratch_bytes(cin, np, dims, batch))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "wgrad scratch too small");
    const uint64_t splits = (g.vox * batch + kWgradVoxelsPerCta - 1) / kWgradVoxelsPerCta;
    if (splits >= (1u << 31)) return set_error(BPGB_ERR_UNSUPPORTED, "batch too large");
    cudaStream_t s = (cudaStream_t)stream;
    if (cin == 1 && np == 16) return launch_wgrad<1, 16>(d_X, x_stride, g, d_dY, d_scratch, (uint32_t)splits, kWgradVoxelsPerCta, cout, d_dW, s);
    if (cin == 2 && np == 16) return launch_wgrad<2, 16>(d_X, x_stride, g, d_dY, d_scratch, (uint32_t)splits, kWgradVoxelsPerCta, cout, d_dW, s);
    if (cin == 16 && np == 16) return launch_wgrad<16, 16>(d_X, x_stride, g, d_dY, d_scratch, (uint32_t)splits, kWgradVoxelsPerCta, cout, d_dW, s);
    if (cin == 16 && np == 8) return launch_wgrad<16, 8>(d_X, x_stride, g, d_dY, d_scratch, (uint32_t)splits, kWgradVoxelsPerCta, cout, d_dW, s);
    return set_error(BPGB_ERR_UNSUPPORTED, "conv3d_wgrad shapes: (cin, np) in {(1,16), (2,16), (16,16), (16,8)}");
}

int bpgb_cnn_pack_weights(const float *d_W, uint32_t cin, uint32_t cout, uint32_t np,
                          void *d_Wt, uint32_t np_back, void *d_Wb, void *stream) {
    clear_error();
    if (!d_W || !d_Wt || cin == 0 || cout == 0 || cout > np || (d_Wb && cin > np_back))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad pack_weights arguments");
    const uint32_t KP = bpgb_cnn_kp(cin), KPb = bpgb_cnn_kp(cout);
    const uint32_t n = std::max(np * KP, d_Wb ? np_back * KPb : 0u);
    pack_weights_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        d_W, cin, cout, KP, np, (__nv_bfloat16 *)d_Wt, KPb, np_back, (__nv_bfloat16 *)d_Wb);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_bce_grad(const float *d_logits, const uint8_t *d_labels, uint64_t n,
                      float pos_weight, float scale, void *d_dZ, float *d_loss, void *stream) {
    clear_error();
    if (!d_logits || !d_labels || !d_dZ) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (((uintptr_t)d_dZ) % 16) return set_error(BPGB_ERR_INVALID_ARGUMENT, "dZ must be 16-byte aligned");
    if (n == 0) return BPGB_OK;
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
    bce_grad_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_logits, d_labels, n, pos_weight, scale,
                                                          (__nv_bfloat16 *)d_dZ, d_loss);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_adam(float *d_p, const float *d_g, float *d_m, float *d_v, uint64_t n, float lr,
                  float beta1, float beta2, float eps, uint32_t step, void *stream) {
    clear_error();
    if (!d_p || !d_g || !d_m || !d_v || step == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad adam arguments");
    if (n == 0) return BPGB_OK;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    const unsigned grid = (unsigned)((n + 255) / 256 < 152 * 4 ? (n + 255) / 256 : 152 * 4);
    adam_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_p, d_g, d_m, d_v, n, lr, beta1, beta2,
                                                      eps, c1, c2);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_normalize(const float *d_coarse, const uint32_t *dims, uint32_t batch, void *d_X,
                       void *stream) {
    clear_error();
    Geo g;
    if (!d_coarse || !d_X || !geo_of(dims, batch, &g))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad normalize arguments");
    normalize_kernel<<<batch, 256, 0, (cudaStream_t)stream>>>(d_coarse, g.vox,
                                                            (__nv_bfloat16 *)d_X);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_features(const float *d_coarse, const uint32_t *dims, uint32_t batch, void *d_X,
                      float *d_scratch, void *stream) {
    clear_error();
    Geo g;
    if (!d_coarse || !d_X || !geo_of(dims, batch, &g) || ((uintptr_t)d_X) % 4)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad features arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (!d_scratch || batch > 65535) {
        features_kernel<<<batch, 256, 0, s>>>(d_coarse, g, (__nv_bfloat16 *)d_X);
        count_launches(1);
    } else {
        BPGB_CUDA_TRY(cudaMemsetAsync(d_scratch, 0, 2 * sizeof(float) * batch, s));
        const uint64_t per = (g.vox + 255) / 256;
        const dim3 grid((unsigned)(per < 64 ? per : 64), batch);
        features_max_kernel<<<grid, 256, 0, s>>>(d_coarse, g, (unsigned int *)d_scratch);
        features_write_kernel<<<grid, 256, 0, s>>>(d_coarse, g, (const unsigned int *)d_scratch,
                                                   (__nv_bfloat16 *)d_X);
        count_launches(2);
    }
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

}  // extern "C"
