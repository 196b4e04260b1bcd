// tcgen05 kernels of the occupancy CNN's training step: 3x3x3 convolutions (forward and
// backward-data) and their weight gradients on the 5th-generation tensor cores (BF16
// operands staged in shared memory by bulk copies, FP32 accumulators in tensor memory).
//
// Line-planes layout (Lp).  Volumes are n0 x n1 x 32 voxels per sample (z fastest, one
// z-line = 32 voxels).  A tensor of C <= 16 channels is stored as rows of 16 bytes holding
// 8 BF16 channels ("planes": 1 for C <= 8, 2 for C <= 16), zero-padded by one voxel in x
// and y and by zp (0 or 1) rows at both ends of each z-line:
//   row(s, x', y', h, z') = (((s (n0+2) + x') (n1+2) + y') npl + h) (32 + 2 zp) + z'
// with x' = x + 1, y' = y + 1, z' = z + zp; a tail of zero lines follows the last sample.
// The padding rows are zero (the buffer is cleared once; kernels write interior rows only),
// so every 3x3 neighbourhood in x and y is a fixed row offset.  Activations (inputs of
// the forward convolutions) use zp = 0, gradients zp = 1.
//
// Convolution (conv_tc_kernel): per output z-line, for each of the 9 (dx, dy) taps one
// tcgen05.mma with M = 64 (rows dz x 16 output channels, 48 used), N = 32 (the line's
// voxels), K = 16 (input channels; for single-plane inputs K = 8 channels x 2 taps):
//   D[dz, co][z] += sum_ci W[dx, dy, dz][ci][co] X[x + dx, y + dy, z][ci]
// Both operands are K-major and read in place: A is the packed weight image, B the staged
// input lines (8 voxels x 16 B core matrices along the line).  The z taps are folded
// into M and recombined in the epilogue: Y[z] = D[dz=-1][z-1] + D[0][z] + D[+1][z+1]
// (zero outside the line), then bias, ReLU or the ReLU mask of the backward pass.
//
// Weight gradient (wgrad_tc_kernel): for each output line and each (dx, dz), one
// tcgen05.mma with M = 64 (rows dy'' x plane x 8 channels; dy'' = 0..2 used, 3 in range
// but unused), N = 16 output channels, K = 16 voxels of the line, both operands MN-major
// and read in place from the staged lines:
//   D[dx, dz][dy'', ci][co] += sum_z X[x + dx, y + dy'' - 1, z][ci] dY[x, y, z - dz][co]
// (z - dz reads the gradient's zero z-padding at the ends), plus one MMA with an all-ones
// A for the bias gradient.  Each CTA accumulates its lines in tensor memory and writes
// one partial [kp][16]; a second kernel sums the partials in CTA order.
//
// Descriptor and accumulator layouts are the ones bpgb_diag_umma_probe pins: LBO = the
// K-direction core-matrix stride and SBO = the M/N-direction stride for both K-major and
// MN-major operands; with M = 64, row r of D is tensor-memory lane 32 (r / 16) + r % 16.
//
// Each CTA runs 4 epilogue warps and one producer/MMA warp (one elected thread issues the
// bulk copies and the MMAs).  Every mbarrier wait is bounded; a wait that gives up sets
// g_tc_status (read by bpgb_cnn_tc_status) and the CTA drains its MMAs before it frees
// its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "bpgb_device.cuh"
#include "bpgb_internal.h"
#include "bpgb_umma.cuh"

namespace bpgb {
namespace {

constexpr uint32_t kZLine = 32;      // voxels per z-line (n2)
constexpr uint32_t kTailLines = 16;  // zero line-pairs after the last sample
constexpr uint32_t kSpin = 1u << 22;
constexpr uint32_t kMinSmem = 80 * 1024;  // at most 2 CTAs per SM (256 TMEM columns each)

__device__ uint32_t g_tc_status;

struct Lp {
    uint32_t n0, n1, batch;
    uint32_t npl;  // planes of 8 channels
    uint32_t zp;   // z padding rows at each end of a line
    __host__ __device__ uint32_t L() const { return kZLine + 2 * zp; }
    __host__ __device__ uint32_t line_rows() const { return npl * L(); }
    __host__ __device__ uint64_t row(uint32_t s, uint32_t xp, uint32_t yp, uint32_t h,
                                     uint32_t zq) const {
        return ((((uint64_t)s * (n0 + 2) + xp) * (n1 + 2) + yp) * npl + h) * L() + zq;
    }
    __host__ __device__ uint64_t rows() const {
        return ((uint64_t)batch * (n0 + 2) * (n1 + 2) + kTailLines) * line_rows();
    }
};

__device__ __forceinline__ void fail(uint32_t bit) { atomicOr(&g_tc_status, bit); }

__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&p);
}

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// ---- convolution --------------------------------------------------------------------
constexpr uint32_t kConvLB = 4;                // output lines per block (same s, x)
constexpr uint32_t kConvSlabLines = kConvLB + 3;  // y' lines staged per x' (last one spare)
constexpr uint32_t kConvThreads = 160;
constexpr uint32_t kConvCols = 2 * kConvLB * 32;  // two accumulator buffers
constexpr uint32_t kEStride = 33;                 // floats per (dz, co) row of the exchange

struct ConvArgs {
    const uint8_t *X;
    Lp in;
    const uint8_t *W;  // weight image: groups x 2 KB
    const float *bias;  // cout values or null
    uint32_t cout;
    int relu;
    const uint8_t *mask;  // activation-layout tensor of the output's channels, or null
    Lp mk;
    uint8_t *Y;  // output tensor or null
    Lp out;
    float *Yf;  // channel 0 in FP32 [batch n0 n1 32], or null
    uint32_t nblocks;
};

template <int NPL>
struct ConvShape {
    static constexpr uint32_t kGroups = NPL == 2 ? 9 : 5;
    static constexpr uint32_t kWBytes = kGroups * 2048;
    static __host__ __device__ uint32_t line_bytes(uint32_t zp) { return NPL * (kZLine + 2 * zp) * 16; }
    static __host__ __device__ uint32_t slabx(uint32_t zp) { return kConvSlabLines * line_bytes(zp); }
    static __host__ __device__ uint32_t slab(uint32_t zp) { return 3 * slabx(zp); }
    static constexpr uint32_t kEBytes = kConvLB * 3 * 16 * kEStride * 4;
    static __host__ __device__ uint32_t smem(uint32_t zp) {
        return kWBytes + 2 * slab(zp) + kEBytes;
    }
};

__device__ __forceinline__ void conv_block(uint32_t b, const Lp &in, uint32_t &s, uint32_t &x,
                                           uint32_t &y0) {
    const uint32_t per_x = in.n1 / kConvLB;
    const uint32_t per_s = in.n0 * per_x;
    s = b / per_s;
    const uint32_t r = b - s * per_s;
    x = r / per_x;
    y0 = (r - x * per_x) * kConvLB;
}

template <int NPL>
__global__ void __launch_bounds__(kConvThreads) conv_tc_kernel(ConvArgs a) {
    using S = ConvShape<NPL>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[2], empty[2], acc_full[2], acc_empty[2], drain;
    __shared__ uint32_t taddr_s;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t zp = a.in.zp;
    const uint32_t line_bytes = S::line_bytes(zp), slabx = S::slabx(zp), slab_bytes = S::slab(zp);
    uint8_t *w_s = smem;
    uint8_t *slab_s = smem + S::kWBytes;
    float *E = reinterpret_cast<float *>(slab_s + 2 * slab_bytes);

    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), kConvCols);
        tmem_relinquish();
    }
    if (tid == 128) {
        for (int i = 0; i < 2; i++) {
            mbar_init(smem_addr(&full[i]), 1);
            mbar_init(smem_addr(&empty[i]), 1);
            mbar_init(smem_addr(&acc_full[i]), 1);
            mbar_init(smem_addr(&acc_empty[i]), 128);
        }
        mbar_init(smem_addr(&drain), 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;

    if (tid == 128) {
        // ---- producer and MMA issue
        auto copy = [&](uint32_t buf, uint32_t b, bool weights) {
            uint32_t s, x, y0;
            conv_block(b, a.in, s, x, y0);
            const uint32_t bar = smem_addr(&full[buf]);
            mbar_expect_tx(bar, slab_bytes + (weights ? S::kWBytes : 0u));
            if (weights) bulk_g2s(smem_addr(w_s), a.W, S::kWBytes, bar);
            const uint32_t dst = smem_addr(slab_s + buf * slab_bytes);
            for (uint32_t dx = 0; dx < 3; dx++)
                bulk_g2s(dst + dx * slabx, a.X + a.in.row(s, x + dx, y0, 0, 0) * 16, slabx, bar);
            mbar_arrive(bar);
        };
        const uint32_t idesc = umma_idesc_bf16(64, 32, false, false);
        const uint32_t wbase = smem_addr(w_s);
        uint32_t it = 0;
        if (blockIdx.x < a.nblocks) copy(0, blockIdx.x, true);
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t buf = it & 1, use = it >> 1;
            if (!mbar_wait(smem_addr(&full[buf]), use & 1, kSpin)) {
                fail(1);
                break;
            }
            if (use > 0 && !mbar_wait(smem_addr(&acc_empty[buf]), (use - 1) & 1, kSpin)) {
                fail(2);
                break;
            }
            tc_fence_after();
            const uint32_t sb = smem_addr(slab_s + buf * slab_bytes) + zp * 16;
            for (uint32_t j = 0; j < kConvLB; j++) {
                const uint32_t d = taddr + buf * (kConvLB * 32) + j * 32;
                for (uint32_t g = 0; g < S::kGroups; g++) {
                    uint32_t b0, lbo;
                    if (NPL == 2) {
                        b0 = sb + (g / 3) * slabx + (j + g % 3) * line_bytes;
                        lbo = (kZLine + 2 * zp) * 16;  // plane 1 of the same line
                    } else {
                        const uint32_t ta = 2 * g, tb = 2 * g + 1;
                        b0 = sb + (ta / 3) * slabx + (j + ta % 3) * line_bytes;
                        // second K group: the next tap (the tenth is a zero-weight slot that
                        // reads the rows one voxel further on)
                        lbo = tb < 9 ? sb + (tb / 3) * slabx + (j + tb % 3) * line_bytes - b0 : 16u;
                    }
                    umma_bf16(d, umma_smem_desc(wbase + g * 2048, 1024, 128),
                              umma_smem_desc(b0, lbo, 128), idesc, g > 0);
                }
            }
            umma_commit(smem_addr(&empty[buf]));
            umma_commit(smem_addr(&acc_full[buf]));
            const uint32_t nb = b + gridDim.x;
            if (nb < a.nblocks) {
                const uint32_t nbuf = (it + 1) & 1, nuse = (it + 1) >> 1;
                if (nuse > 0 && !mbar_wait(smem_addr(&empty[nbuf]), (nuse - 1) & 1, kSpin)) {
                    fail(4);
                    break;
                }
                copy(nbuf, nb, false);
            }
        }
        umma_commit(smem_addr(&drain));
        if (!mbar_wait(smem_addr(&drain), 0, kSpin)) fail(8);
    } else if (tid < 128) {
        // ---- epilogue: tensor memory -> z recombination -> bias / ReLU / mask -> BF16 rows
        uint32_t it = 0;
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t buf = it & 1, use = it >> 1;
            if (!mbar_wait(smem_addr(&acc_full[buf]), use & 1, kSpin)) {
                fail(16);
                break;
            }
            tc_fence_after();
            uint32_t s, x, y0;
            conv_block(b, a.in, s, x, y0);
            if (warp < 3) {
                for (uint32_t j = 0; j < kConvLB; j++) {
                    float v[32];
                    __syncwarp();
                    const uint32_t t = taddr + ((warp * 32u) << 16) + buf * (kConvLB * 32) + j * 32;
                    tmem_ld16(t, *reinterpret_cast<float(*)[16]>(&v[0]));
                    tmem_ld16(t + 16, *reinterpret_cast<float(*)[16]>(&v[16]));
                    tmem_ld_wait();
                    if (lane < 16) {
                        float *e = E + ((j * 3 + warp) * 16 + lane) * kEStride;
#pragma unroll
                        for (int z = 0; z < 32; z++) e[z] = v[z];
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(smem_addr(&acc_empty[buf]));
            epi_sync();
            if (a.Y) {
                const uint32_t chunks = kConvLB * 32 * a.out.npl;
                for (uint32_t c = tid; c < chunks; c += 128) {
                    const uint32_t h = c % a.out.npl, z = (c / a.out.npl) % 32,
                                   j = c / (a.out.npl * 32);
                    const float *e = E + (j * 3 * 16 + h * 8) * kEStride;
                    float o[8];
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const uint32_t co = h * 8 + k;
                        const float *r = e + k * kEStride;
                        float y = r[16 * kEStride + z];
                        if (z > 0) y = r[z - 1] + y;
                        if (z < 31) y = y + r[32 * kEStride + z + 1];
                        if (a.bias && co < a.cout) y += a.bias[co];
                        if (co >= a.cout) y = 0.0f;
                        if (a.relu) y = fmaxf(y, 0.0f);
                        o[k] = y;
                    }
                    if (a.mask) {
                        const uint4 m = *reinterpret_cast<const uint4 *>(
                            a.mask + a.mk.row(s, x + 1, y0 + j + 1, h, z + a.mk.zp) * 16);
                        const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (!(bf_lo(mw[k]) > 0.0f)) o[2 * k] = 0.0f;
                            if (!(bf_hi(mw[k]) > 0.0f)) o[2 * k + 1] = 0.0f;
                        }
                    }
                    *reinterpret_cast<uint4 *>(a.Y +
                                               a.out.row(s, x + 1, y0 + j + 1, h, z + a.out.zp) * 16) =
                        make_uint4(pack_bf2(o[0], o[1]), pack_bf2(o[2], o[3]), pack_bf2(o[4], o[5]),
                                   pack_bf2(o[6], o[7]));
                }
            }
            if (a.Yf) {
                const uint32_t j = tid / 32, z = tid % 32;  // 128 threads = 4 lines x 32
                const float *r = E + (j * 3 * 16) * kEStride;
                float y = r[16 * kEStride + z];
                if (z > 0) y = r[z - 1] + y;
                if (z < 31) y = y + r[32 * kEStride + z + 1];
                if (a.bias && a.cout > 0) y += a.bias[0];
                a.Yf[(((uint64_t)s * a.in.n0 + x) * a.in.n1 + y0 + j) * 32 + z] = y;
            }
            epi_sync();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, kConvCols);
    }
}

// ---- weight gradient ----------------------------------------------------------------
constexpr uint32_t kWgLB = 8;  // output lines per block
constexpr uint32_t kWgThreads = 160;
constexpr uint32_t kWgCols = 256;  // 10 accumulators x 16 columns, rounded up
constexpr uint32_t kOnesBytes = 2048;

struct WgradArgs {
    const uint8_t *X;  // activation (zp 0)
    Lp xin;
    const uint8_t *dY;  // gradient (zp 1)
    Lp dy;
    uint32_t cin, cout, kp;
    float *partial;  // [gridDim.x][kp][16]
    uint32_t nblocks;
};

template <int NPLX, int NPLD>
struct WgShape {
    static constexpr uint32_t kXL = NPLX == 2 ? kWgLB + 3 : kWgLB + 8;  // y' lines per x'
    static constexpr uint32_t kXLine = NPLX * 32 * 16;
    static constexpr uint32_t kDLine = NPLD * 34 * 16;
    // a single-plane gradient is read as N = 16 too: its second core matrix is the next
    // line (columns 8..15 of D, unused), so one more line is staged
    static constexpr uint32_t kDLines = NPLD == 2 ? kWgLB : kWgLB + 1;
    static constexpr uint32_t kSlabX = kXL * kXLine;
    static constexpr uint32_t kXBytes = 3 * kSlabX;
    static constexpr uint32_t kDBytes = kDLines * kDLine;
    static constexpr uint32_t kBuf = kXBytes + kDBytes;
    static constexpr uint32_t kSmem = kOnesBytes + 2 * kBuf;
};

__device__ __forceinline__ void wg_block(uint32_t b, const Lp &g, uint32_t &s, uint32_t &x,
                                         uint32_t &y0) {
    const uint32_t per_x = g.n1 / kWgLB;
    const uint32_t per_s = g.n0 * per_x;
    s = b / per_s;
    const uint32_t r = b - s * per_s;
    x = r / per_x;
    y0 = (r - x * per_x) * kWgLB;
}

template <int NPLX, int NPLD>
__global__ void __launch_bounds__(kWgThreads) wgrad_tc_kernel(WgradArgs a) {
    using S = WgShape<NPLX, NPLD>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[2], empty[2], done;
    __shared__ uint32_t taddr_s;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *ones = smem;
    uint8_t *buf_s = smem + kOnesBytes;

    for (uint32_t i = tid; i < kOnesBytes / 4; i += kWgThreads)
        reinterpret_cast<uint32_t *>(ones)[i] = 0x3F803F80u;  // BF16 1.0 pairs
    fence_async_smem();
    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), kWgCols);
        tmem_relinquish();
    }
    if (tid == 128) {
        for (int i = 0; i < 2; i++) {
            mbar_init(smem_addr(&full[i]), 1);
            mbar_init(smem_addr(&empty[i]), 1);
        }
        mbar_init(smem_addr(&done), 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;
    const bool any = blockIdx.x < a.nblocks;

    if (tid == 128) {
        auto copy = [&](uint32_t buf, uint32_t b) {
            uint32_t s, x, y0;
            wg_block(b, a.dy, s, x, y0);
            const uint32_t bar = smem_addr(&full[buf]);
            mbar_expect_tx(bar, S::kBuf);
            const uint32_t dst = smem_addr(buf_s + buf * S::kBuf);
            for (uint32_t dx = 0; dx < 3; dx++)
                bulk_g2s(dst + dx * S::kSlabX, a.X + a.xin.row(s, x + dx, y0, 0, 0) * 16, S::kSlabX,
                         bar);
            bulk_g2s(dst + S::kXBytes, a.dY + a.dy.row(s, x + 1, y0 + 1, 0, 0) * 16, S::kDBytes, bar);
            mbar_arrive(bar);
        };
        const uint32_t idesc = umma_idesc_bf16(64, 16, true, true);
        const uint32_t ones_a = smem_addr(ones);
        uint32_t it = 0, acc = 0;
        if (any) copy(0, blockIdx.x);
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t buf = it & 1, use = it >> 1;
            if (!mbar_wait(smem_addr(&full[buf]), use & 1, kSpin)) {
                fail(32);
                break;
            }
            tc_fence_after();
            const uint32_t xs = smem_addr(buf_s + buf * S::kBuf);
            const uint32_t ds = xs + S::kXBytes;
            for (uint32_t j = 0; j < kWgLB; j++) {
                for (uint32_t ks = 0; ks < 2; ks++) {
                    for (uint32_t dx = 0; dx < 3; dx++) {
                        const uint64_t ad = umma_smem_desc(
                            xs + dx * S::kSlabX + j * S::kXLine + ks * 256, 128, 512);
                        for (uint32_t dz = 0; dz < 3; dz++) {
                            const uint64_t bd = umma_smem_desc(
                                ds + j * S::kDLine + (2 - dz) * 16 + ks * 256, 128, S::kDLine / NPLD);
                            umma_bf16(taddr + (dx * 3 + dz) * 16, ad, bd, idesc, acc);
                        }
                    }
                    umma_bf16(taddr + 9 * 16, umma_smem_desc(ones_a, 128, 256),
                              umma_smem_desc(ds + j * S::kDLine + 16 + ks * 256, 128, S::kDLine / NPLD),
                              idesc, acc);
                    acc = 1;
                }
            }
            umma_commit(smem_addr(&empty[buf]));
            const uint32_t nb = b + gridDim.x;
            if (nb < a.nblocks) {
                const uint32_t nbuf = (it + 1) & 1, nuse = (it + 1) >> 1;
                if (nuse > 0 && !mbar_wait(smem_addr(&empty[nbuf]), (nuse - 1) & 1, kSpin)) {
                    fail(64);
                    break;
                }
                copy(nbuf, nb);
            }
        }
        umma_commit(smem_addr(&done));
    } else if (tid < 128) {
        float *P = a.partial + (uint64_t)blockIdx.x * a.kp * 16;
        const bool ok = mbar_wait(smem_addr(&done), 0, kSpin * 4);
        if (!ok) fail(128);
        tc_fence_after();
        if (!any || !ok) {
            for (uint32_t i = tid; i < a.kp * 16; i += 128) P[i] = 0.0f;
        } else {
            for (uint32_t ai = 0; ai < 10; ai++) {
                float v[16];
                __syncwarp();
                tmem_ld16(taddr + ((warp * 32u) << 16) + ai * 16, v);
                tmem_ld_wait();
                uint32_t row = 0;
                bool valid = false;
                if (ai < 9) {
                    uint32_t dyi, ci;
                    if (NPLX == 2) {
                        dyi = warp;
                        ci = lane;
                    } else {
                        const uint32_t r = 16 * warp + lane;
                        dyi = r / 8;
                        ci = r % 8;
                    }
                    valid = lane < 16 && dyi < 3 && ci < a.cin;
                    row = ((ai / 3) * 9 + dyi * 3 + ai % 3) * a.cin + ci;
                } else {
                    valid = warp == 0 && lane == 0;
                    row = 27 * a.cin;
                }
                if (valid) {
                    float *p = P + (uint64_t)row * 16;
#pragma unroll
                    for (int c = 0; c < 16; c++) p[c] = c < NPLD * 8 ? v[c] : 0.0f;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, kWgCols);
    }
}

// dW[k][n] = sum over CTAs of partial[p][k][n] (k <= 27 cin), 0 on the padding rows.
__global__ void wgrad_tc_reduce_kernel(const float *__restrict__ partial, uint32_t parts,
                                       uint32_t kp, uint32_t cin, uint32_t cout,
                                       float *__restrict__ dW) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp * cout) return;
    const uint32_t k = i / cout, n = i % cout;
    float s = 0.0f;
    if (k <= 27 * cin)
        for (uint32_t p = 0; p < parts; p++) s += partial[((uint64_t)p * kp + k) * 16 + n];
    dW[i] = s;
}

// ---- layout conversion, weights, loss ----------------------------------------------------
// Interior rows of an Lp tensor from channels-last BF16 [V][x_stride] (channels >= C zero).
__global__ void lp_pack_kernel(const __nv_bfloat16 *__restrict__ X, uint32_t C, uint32_t xs, Lp g,
                               uint8_t *__restrict__ out) {
    const uint64_t n = (uint64_t)g.batch * g.n0 * g.n1 * 32 * g.npl;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t h = (uint32_t)(i % g.npl);
        const uint64_t v = i / g.npl;
        const uint32_t z = (uint32_t)(v % 32), y = (uint32_t)((v / 32) % g.n1);
        const uint64_t sx = v / (32ull * g.n1);
        const uint32_t x = (uint32_t)(sx % g.n0), s = (uint32_t)(sx / g.n0);
        float c[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t ch = h * 8 + k;
            c[k] = ch < C ? __bfloat162float(X[v * xs + ch]) : 0.0f;
        }
        *reinterpret_cast<uint4 *>(out + g.row(s, x + 1, y + 1, h, z + g.zp) * 16) =
            make_uint4(pack_bf2(c[0], c[1]), pack_bf2(c[2], c[3]), pack_bf2(c[4], c[5]),
                       pack_bf2(c[6], c[7]));
    }
}

__global__ void lp_unpack_kernel(const uint8_t *__restrict__ in, Lp g, uint32_t C,
                                 __nv_bfloat16 *__restrict__ X) {
    const uint64_t n = (uint64_t)g.batch * g.n0 * g.n1 * 32 * C;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ch = (uint32_t)(i % C);
        const uint64_t v = i / C;
        const uint32_t z = (uint32_t)(v % 32), y = (uint32_t)((v / 32) % g.n1);
        const uint64_t sx = v / (32ull * g.n1);
        const uint32_t x = (uint32_t)(sx % g.n0), s = (uint32_t)(sx / g.n0);
        const __nv_bfloat16 *r = reinterpret_cast<const __nv_bfloat16 *>(
            in + g.row(s, x + 1, y + 1, ch / 8, z + g.zp) * 16);
        X[i] = r[ch % 8];
    }
}

// Weight image of a convolution with `in_ch` input channels (groups x 2 KB): element
// (group g, row m = dz 16 + oc, column k) at g 2048 + (k/8) 1024 + (m/8) 128 + (m%8) 16 +
// (k%8) 2; column k = input channel (two planes) or (tap of the pair, channel) for one
// plane.  Forward: W[t cin + ic][oc]; backward-data: W[(26 - t) cin + oc][ic].
__global__ void pack_tc_weights_kernel(const float *__restrict__ W, uint32_t cin, uint32_t cout,
                                       int backward, uint32_t groups,
                                       __nv_bfloat16 *__restrict__ img) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= groups * 1024) return;
    const uint32_t g = e / 1024, m = (e / 16) % 64, k = e % 16;
    const uint32_t in_ch = backward ? cout : cin, out_ch = backward ? cin : cout;
    const bool two = in_ch > 8;
    const uint32_t tap9 = two ? g : 2 * g + k / 8, ic = two ? k : k % 8;
    const uint32_t dz = m / 16, oc = m % 16;
    float w = 0.0f;
    if (tap9 < 9 && m < 48 && ic < in_ch && oc < out_ch) {
        const uint32_t t = (tap9 / 3) * 9 + (tap9 % 3) * 3 + dz;
        w = backward ? W[((uint64_t)(26 - t) * cin + oc) * cout + ic]
                     : W[((uint64_t)t * cin + ic) * cout + oc];
    }
    const uint32_t off = g * 2048 + (k / 8) * 1024 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2;
    img[off / 2] = __float2bfloat16_rn(w);
}

// dZ (single-plane gradient, zp 1) and the per-voxel loss of BCE-with-logits:
// dZ = w (sigmoid(z) - y) scale, loss = w (softplus(z) - y z) scale, w = pos_weight for y = 1.
__global__ void bce_lp_kernel(const float *__restrict__ logits, const uint8_t *__restrict__ y,
                              Lp g, float pos_weight, float scale, uint8_t *__restrict__ dZ,
                              float *__restrict__ loss) {
    const uint64_t n = (uint64_t)g.batch * g.n0 * g.n1 * 32;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float z = logits[i];
        const float t = y[i] ? 1.0f : 0.0f;
        const float w = y[i] ? pos_weight : 1.0f;
        const float sig = 1.0f / (1.0f + expf(-z));
        const float sp = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
        const uint32_t zz = (uint32_t)(i % 32), yy = (uint32_t)((i / 32) % g.n1);
        const uint64_t sx = i / (32ull * g.n1);
        const uint32_t x = (uint32_t)(sx % g.n0), s = (uint32_t)(sx / g.n0);
        const __nv_bfloat16 gr = __float2bfloat16_rn(w * (sig - t) * scale);
        *reinterpret_cast<uint4 *>(dZ + g.row(s, x + 1, yy + 1, 0, zz + 1) * 16) =
            make_uint4((uint32_t)__bfloat16_as_ushort(gr), 0u, 0u, 0u);
        if (loss) loss[i] = w * (sp - t * z) * scale;
    }
}

// ---- host -----------------------------------------------------------------------------
bool lp_of(const uint32_t *dims, uint32_t batch, uint32_t channels, uint32_t zp, Lp *g) {
    if (!dims || !batch || !dims[0] || !dims[1] || dims[2] != kZLine || channels == 0 ||
        channels > 16 || zp > 1 || dims[1] % kWgLB)
        return false;
    g->n0 = dims[0];
    g->n1 = dims[1];
    g->batch = batch;
    g->npl = channels > 8 ? 2 : 1;
    g->zp = zp;
    return true;
}

int sm_count_cached() {
    static int n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            n = 0;
    });
    return n > 0 ? n : 148;
}

template <typename K>
int set_smem(K kernel, uint32_t bytes) {
    BPGB_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes));
    return BPGB_OK;
}

unsigned grid_for(uint64_t n, unsigned threads, unsigned cap) {
    const uint64_t b = (n + threads - 1) / threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, cap));
}

bool aligned16(const void *p) { return ((uintptr_t)p % 16) == 0; }

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" {

uint64_t bpgb_cnn_lp_bytes(uint32_t channels, uint32_t zpad, const uint32_t *dims,
                           uint32_t batch) {
    Lp g;
    if (!lp_of(dims, batch, channels, zpad, &g)) return 0;
    return g.rows() * 16;
}

uint64_t bpgb_cnn_tc_weight_bytes(uint32_t in_channels) {
    if (in_channels == 0 || in_channels > 16) return 0;
    return (in_channels > 8 ? 9u : 5u) * 2048u;
}

int bpgb_cnn_lp_pack(const void *d_X, uint32_t channels, uint32_t x_stride, const uint32_t *dims,
                     uint32_t batch, uint32_t zpad, void *d_lp, void *stream) {
    clear_error();
    Lp g;
    if (!d_X || !d_lp || x_stride < channels || !lp_of(dims, batch, channels, zpad, &g) ||
        !aligned16(d_lp))
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "bad lp_pack arguments (dims[2] must be 32, dims[1] a multiple of 8)");
    const uint64_t n = (uint64_t)batch * g.n0 * g.n1 * 32 * g.npl;
    lp_pack_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)d_X, channels, x_stride, g, (uint8_t *)d_lp);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_lp_unpack(const void *d_lp, uint32_t channels, uint32_t zpad, const uint32_t *dims,
                       uint32_t batch, void *d_X, void *stream) {
    clear_error();
    Lp g;
    if (!d_X || !d_lp || !lp_of(dims, batch, channels, zpad, &g) || !aligned16(d_lp))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad lp_unpack arguments");
    const uint64_t n = (uint64_t)batch * g.n0 * g.n1 * 32 * channels;
    lp_unpack_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, (cudaStream_t)stream>>>(
        (const uint8_t *)d_lp, g, channels, (__nv_bfloat16 *)d_X);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_tc_pack_weights(const float *d_W, uint32_t cin, uint32_t cout, void *d_Wf,
                             void *d_Wb, void *stream) {
    clear_error();
    if (!d_W || !d_Wf || cin == 0 || cin > 16 || cout == 0 || cout > 16 || !aligned16(d_Wf) ||
        (d_Wb && !aligned16(d_Wb)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_pack_weights arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t gf = (uint32_t)(bpgb_cnn_tc_weight_bytes(cin) / 2048);
    pack_tc_weights_kernel<<<(gf * 1024 + 255) / 256, 256, 0, s>>>(d_W, cin, cout, 0, gf,
                                                                   (__nv_bfloat16 *)d_Wf);
    count_launches(1);
    if (d_Wb) {
        const uint32_t gb = (uint32_t)(bpgb_cnn_tc_weight_bytes(cout) / 2048);
        pack_tc_weights_kernel<<<(gb * 1024 + 255) / 256, 256, 0, s>>>(d_W, cin, cout, 1, gb,
                                                                       (__nv_bfloat16 *)d_Wb);
        count_launches(1);
    }
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_tc_conv3d(const void *d_X, uint32_t in_channels, uint32_t in_zpad,
                       const uint32_t *dims, uint32_t batch, const void *d_W, const float *d_bias,
                       uint32_t out_channels, int relu, const void *d_mask, void *d_Y,
                       uint32_t out_zpad, float *d_Yf, void *stream) {
    clear_error();
    ConvArgs a{};
    if (!d_X || !d_W || (!d_Y && !d_Yf) || !lp_of(dims, batch, in_channels, in_zpad, &a.in) ||
        !lp_of(dims, batch, out_channels, out_zpad, &a.out) ||
        !lp_of(dims, batch, out_channels, 0, &a.mk) || !aligned16(d_X) || !aligned16(d_W) ||
        (d_Y && !aligned16(d_Y)) || (d_mask && !aligned16(d_mask)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "bad tc_conv3d arguments (channels 1..16, dims[2] = 32, dims[1] % 8 = 0, "
                         "16-byte aligned tensors)");
    a.X = (const uint8_t *)d_X;
    a.W = (const uint8_t *)d_W;
    a.bias = d_bias;
    a.cout = out_channels;
    a.relu = relu;
    a.mask = (const uint8_t *)d_mask;
    a.Y = (uint8_t *)d_Y;
    a.Yf = d_Yf;
    a.nblocks = batch * dims[0] * (dims[1] / kConvLB);
    const unsigned grid = (unsigned)std::min<uint64_t>(a.nblocks, 2ull * sm_count_cached());
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if (a.in.npl == 2) {
        const uint32_t sm = std::max(kMinSmem, ConvShape<2>::smem(in_zpad));
        if ((st = set_smem(conv_tc_kernel<2>, sm))) return st;
        conv_tc_kernel<2><<<grid, kConvThreads, sm, s>>>(a);
    } else {
        const uint32_t sm = std::max(kMinSmem, ConvShape<1>::smem(in_zpad));
        if ((st = set_smem(conv_tc_kernel<1>, sm))) return st;
        conv_tc_kernel<1><<<grid, kConvThreads, sm, s>>>(a);
    }
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

uint64_t bpgb_cnn_tc_wgrad_scratch_bytes(uint32_t in_channels, const uint32_t *dims,
                                         uint32_t batch) {
    Lp g;
    if (!lp_of(dims, batch, in_channels, 0, &g)) return 0;
    const uint64_t nb = (uint64_t)batch * dims[0] * (dims[1] / kWgLB);
    const uint64_t parts = std::min<uint64_t>(nb, 2ull * sm_count_cached());
    return parts * bpgb_cnn_kp(in_channels) * 16 * sizeof(float);
}

int bpgb_cnn_tc_conv3d_wgrad(const void *d_X, uint32_t in_channels, const void *d_dY,
                             uint32_t out_channels, const uint32_t *dims, uint32_t batch,
                             float *d_scratch, uint64_t scratch_bytes, float *d_dW, void *stream) {
    clear_error();
    WgradArgs a{};
    if (!d_X || !d_dY || !d_dW || !d_scratch || !lp_of(dims, batch, in_channels, 0, &a.xin) ||
        !lp_of(dims, batch, out_channels, 1, &a.dy) || !aligned16(d_X) || !aligned16(d_dY))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_conv3d_wgrad arguments");
    if (scratch_bytes < bpgb_cnn_tc_wgrad_scratch_bytes(in_channels, dims, batch))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "tc wgrad scratch too small");
    a.X = (const uint8_t *)d_X;
    a.dY = (const uint8_t *)d_dY;
    a.cin = in_channels;
    a.cout = out_channels;
    a.kp = bpgb_cnn_kp(in_channels);
    a.partial = d_scratch;
    a.nblocks = batch * dims[0] * (dims[1] / kWgLB);
    const unsigned grid = (unsigned)std::min<uint64_t>(a.nblocks, 2ull * sm_count_cached());
    cudaStream_t s = (cudaStream_t)stream;
    int st;
#define BPGB_WG(PX, PD)                                                                \
    do {                                                                               \
        const uint32_t sm = std::max(kMinSmem, WgShape<PX, PD>::kSmem);                \
        if ((st = set_smem(wgrad_tc_kernel<PX, PD>, sm))) return st;                   \
        wgrad_tc_kernel<PX, PD><<<grid, kWgThreads, sm, s>>>(a);                       \
    } while (0)
    if (a.xin.npl == 2 && a.dy.npl == 2) BPGB_WG(2, 2);
    else if (a.xin.npl == 2) BPGB_WG(2, 1);
    else if (a.dy.npl == 2) BPGB_WG(1, 2);
    else BPGB_WG(1, 1);
#undef BPGB_WG
    count_launches(1);
    wgrad_tc_reduce_kernel<<<(a.kp * out_channels + 255) / 256, 256, 0, s>>>(
        d_scratch, grid, a.kp, in_channels, out_channels, d_dW);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_tc_bce_grad(const float *d_logits, const uint8_t *d_labels, const uint32_t *dims,
                         uint32_t batch, float pos_weight, float scale, void *d_dZ, float *d_loss,
                         void *stream) {
    clear_error();
    Lp g;
    if (!d_logits || !d_labels || !d_dZ || !lp_of(dims, batch, 1, 1, &g) || !aligned16(d_dZ))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_bce_grad arguments");
    const uint64_t n = (uint64_t)batch * g.n0 * g.n1 * 32;
    bce_lp_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, (cudaStream_t)stream>>>(
        d_logits, d_labels, g, pos_weight, scale, (uint8_t *)d_dZ, d_loss);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_tc_status(uint32_t *status, int reset) {
    clear_error();
    if (!status) return set_error(BPGB_ERR_INVALID_ARGUMENT, "status is null");
    BPGB_CUDA_TRY(cudaDeviceSynchronize());
    BPGB_CUDA_TRY(cudaMemcpyFromSymbol(status, g_tc_status, sizeof(uint32_t)));
    if (reset) {
        const uint32_t zero = 0;
        BPGB_CUDA_TRY(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(uint32_t)));
    }
    return BPGB_OK;
}

}  // extern "C"
