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
// Convolution (conv_tc_kernel): a block is 4 output z-lines of one (sample, x); for each
// of the 9 (dx, dy) taps one tcgen05.mma with M = 128 (the block's voxels), N = 48 (3 z
// taps x 16 output channels), K = 16 (input channels; for single-plane inputs 8 channels
// x 2 taps):
//   D[z][dz, co] += sum_ci X[x + dx, y + dy, z][ci] W[dx, dy, dz][ci][co]
// Both operands are K-major and read in place: A the staged input lines (core matrices of
// 8 voxels along a line), B the packed weight image.  The z taps are recombined in the
// epilogue, where thread = voxel: Y[z] = D[z-1][-1] + D[z][0] + D[z+1][+1] by warp
// shuffles (zero outside the line), then bias, ReLU or the ReLU mask of the backward pass.
//
// Weight gradient (wgrad_tc_kernel): for each output line and each 16-voxel K step,
// tcgen05.mma with both operands MN-major and read in place from TMA-staged lines: A = the
// activation's (dy, dx, plane) core matrices (M = 128 + 64), B = the gradient line at its
// three z shifts (N = 48):
//   D[dy, dx, ci][dz, co] += sum_z X[x + dx, y + dy, z][ci] dY[x, y, z - dz][co]
// (z - dz reads the gradient's zero z-padding at the ends).  The bias gradient is summed
// from the staged gradient by the otherwise idle epilogue warps.  Each CTA accumulates its
// lines in tensor memory and writes one partial [kp][16]; a second kernel sums the
// partials in CTA order.
//
// Descriptor and accumulator layouts are the ones bpgb_diag_umma_probe pins: LBO = the
// K-direction core-matrix stride and SBO = the M/N-direction stride for both K-major and
// MN-major operands; with M = 64, row r of D is tensor-memory lane 32 (r / 16) + r % 16.
//
// Each CTA runs one thread that issues the TMA copies, one that issues the MMAs and
// commits them to mbarriers, and epilogue warps; stages and accumulators are rings.  Every
// mbarrier wait is bounded; a wait that gives up sets g_tc_status (read by
// bpgb_cnn_tc_status) and the CTA drains its MMAs before it frees its tensor memory.
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

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&p);
}

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// ---- convolution --------------------------------------------------------------------
constexpr uint32_t kConvLB = 4;                       // output lines per block (M = 128)
constexpr uint32_t kConvLines = kConvLB + 3;          // y' lines staged per (x', plane), 1 spare
constexpr uint32_t kConvBox = kConvLines * 32 * 16;   // bytes of one staged (x', plane) box
constexpr uint32_t kConvStages = 4;
constexpr uint32_t kConvThreads = 352;  // 8 epilogue warps, 2 MMA warps, the TMA warp
constexpr uint32_t kConvMma = 256;      // MMA-issuing threads: 256 (even blocks), 288 (odd)
constexpr uint32_t kConvTma = 320;      // the TMA-issuing thread
constexpr uint32_t kConvN = 48;                       // dz x 16 output channels
constexpr uint32_t kConvAccs = 4;                     // accumulators in flight
constexpr uint32_t kConvAcc = 64;                     // columns per accumulator
constexpr uint32_t kConvCols = kConvAccs * kConvAcc;  // 256: two CTAs per SM
constexpr uint32_t kConvGroup = kConvN * 16 * 2;      // one K = 16 weight group: 1536 B

struct ConvArgs {
    Lp in;
    const uint8_t *W;    // weight image: groups x 1536 B
    const float *bias;   // cout values or null
    uint32_t cout;
    int relu;
    const uint8_t *mask; // activation-layout tensor of the output's channels, or null
    Lp mk;
    uint8_t *Y;          // output tensor or null
    Lp out;
    float *Yf;           // channel 0 in FP32 [batch n0 n1 32], or null
    uint32_t nblocks;
};

template <int NPL>
struct ConvShape {
    static constexpr uint32_t kGroups = NPL == 2 ? 9 : 5;
    static constexpr uint32_t kWBytes = kGroups * kConvGroup;
    static constexpr uint32_t kStage = 3 * NPL * kConvBox;
    static constexpr uint32_t kSmem = kWBytes + kConvStages * kStage;
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

// One block = 4 consecutive output lines (y0 .. y0 + 3) of one (sample, x): M = 128 voxels
// (row 32 j + z = line j, voxel z), N = 48 = (dz, co), K = 16.  The stage holds, for each
// dx and plane h, the box of lines y' = y0 .. y0 + 6 without z-padding ([line][z][8 ch]),
// so tap (dx, dy) is the A operand at box(dx, plane 0) + dy x 512 B (core matrices of 8
// voxels at 128 B, the second plane at +kConvBox); single-plane inputs pair two taps as
// the two K groups.  Accumulator row = TMEM lane, so warp j's lane z holds voxel z of line
// j: the dz recombination is a shuffle up / down within the warp.
template <int NPL>
__global__ void __launch_bounds__(kConvThreads)
    conv_tc_kernel(const __grid_constant__ CUtensorMap tmap, ConvArgs a) {
    using S = ConvShape<NPL>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[kConvStages], empty[kConvStages], acc_full[kConvAccs],
        acc_empty[kConvAccs], drain[2], wbar;
    __shared__ uint32_t taddr_s;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *w_s = smem;
    uint8_t *stage_s = smem + S::kWBytes;

    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), kConvCols);
        tmem_relinquish();
    }
    if (tid == kConvMma) {
        for (uint32_t i = 0; i < kConvStages; i++) {
            mbar_init(smem_addr(&full[i]), 1);
            mbar_init(smem_addr(&empty[i]), 1);
        }
        for (uint32_t i = 0; i < kConvAccs; i++) {
            mbar_init(smem_addr(&acc_full[i]), 1);
            mbar_init(smem_addr(&acc_empty[i]), 128);
        }
        mbar_init(smem_addr(&drain[0]), 1);
        mbar_init(smem_addr(&drain[1]), 1);
        mbar_init(smem_addr(&wbar), 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;

    auto copy = [&](uint32_t st, uint32_t b) {
        uint32_t s, x, y0;
        conv_block(b, a.in, s, x, y0);
        const uint32_t bar = smem_addr(&full[st]);
        mbar_expect_tx(bar, S::kStage);
        const uint32_t dst = smem_addr(stage_s + st * S::kStage);
        const int32_t xg = (int32_t)(s * (a.in.n0 + 2) + x);
        // one box: 3 x' x the planes x 7 lines x 32 voxels, landing [dx][plane][line][z]
        tma_load_4d(dst, &tmap, (int32_t)(a.in.zp * 8), (int32_t)y0, 0, xg, bar);
        mbar_arrive(bar);
    };
    if (tid == kConvTma) {
        // ---- TMA producer: the weights once, then the stage of local block i is
        // i % kConvStages, refilled as soon as the MMAs of block i - kConvStages completed
        mbar_expect_tx(smem_addr(&wbar), S::kWBytes);
        bulk_g2s(smem_addr(w_s), a.W, S::kWBytes, smem_addr(&wbar));
        mbar_arrive(smem_addr(&wbar));
        uint32_t it = 0;
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t st = it % kConvStages;
            if (it >= kConvStages &&
                !mbar_wait(smem_addr(&empty[st]), ((it / kConvStages) - 1) & 1, kSpin)) {
                fail(4);
                break;
            }
            copy(st, b);
        }
    } else if (tid == kConvMma || tid == kConvMma + 32) {
        // ---- MMA issue: two threads take alternate blocks (their stages, accumulators
        // and epilogue groups alternate with them), each committing its own MMAs
        const uint32_t m = (tid - kConvMma) / 32;
        const uint32_t idesc = umma_idesc_bf16(128, kConvN, false, false);
        const uint64_t b_base = umma_smem_desc(smem_addr(w_s), kConvN * 16, 128);
        if (!mbar_wait(smem_addr(&wbar), 0, kSpin)) fail(1);
        uint32_t it = m;
        for (uint64_t b = blockIdx.x + (uint64_t)m * gridDim.x; b < a.nblocks;
             b += 2ull * gridDim.x, it += 2) {
            const uint32_t st = it % kConvStages, ab = it % kConvAccs;
            if (!mbar_wait(smem_addr(&full[st]), (it / kConvStages) & 1, kSpin)) {
                fail(1);
                break;
            }
            if (it >= kConvAccs &&
                !mbar_wait(smem_addr(&acc_empty[ab]), ((it / kConvAccs) - 1) & 1, kSpin)) {
                fail(2);
                break;
            }
            tc_fence_after();
            const uint32_t d = taddr + ab * kConvAcc;
            // descriptors: the stage's base descriptor plus compile-time start and LBO
            // offsets (the fields cannot carry: addresses stay below 256 KB)
            const uint64_t a_base = umma_smem_desc(smem_addr(stage_s + st * S::kStage), 0, 128);
#pragma unroll
            for (uint32_t g = 0; g < S::kGroups; g++) {
                uint32_t off, lbo;
                if (NPL == 2) {
                    off = (g / 3) * 2 * kConvBox + (g % 3) * 512;
                    lbo = kConvBox;  // plane 1 of the same lines
                } else {
                    const uint32_t ta = 2 * g, tb = 2 * g + 1;
                    off = (ta / 3) * kConvBox + (ta % 3) * 512;
                    // second K group: the next tap (the tenth is a zero-weight slot that
                    // reads the rows one voxel further on)
                    lbo = tb < 9 ? (tb / 3) * kConvBox + (tb % 3) * 512 - off : 16u;
                }
                umma_bf16(d, a_base + (off >> 4) + ((uint64_t)(lbo >> 4) << 16),
                          b_base + ((g * kConvGroup) >> 4), idesc, g > 0);
            }
            umma_commit(smem_addr(&empty[st]));
            umma_commit(smem_addr(&acc_full[ab]));
        }
        umma_commit(smem_addr(&drain[m]));
        if (!mbar_wait(smem_addr(&drain[m]), 0, kSpin)) fail(8);
    } else if (warp < 8) {
        // ---- epilogue: two groups of 4 warps take alternate blocks; in a group, warp q
        // reads tensor-memory lanes 32 q.. (line q of the block), lane = z: one voxel each
        const uint32_t grp = warp >> 2, q = warp & 3;
        uint32_t it = grp;
        for (uint64_t b = blockIdx.x + (uint64_t)grp * gridDim.x; b < a.nblocks;
             b += 2ull * gridDim.x, it += 2) {
            const uint32_t ab = it % kConvAccs;
            uint32_t s, x, y0;
            conv_block((uint32_t)b, a.in, s, x, y0);
            const uint32_t y = y0 + q, z = lane;
            uint4 mk[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
            if (a.mask) {  // the ReLU mask is known before the accumulator: fetch it first
#pragma unroll
                for (uint32_t h = 0; h < 2; h++)
                    if (h < a.out.npl)
                        mk[h] = *reinterpret_cast<const uint4 *>(
                            a.mask + a.mk.row(s, x + 1, y + 1, h, z + a.mk.zp) * 16);
            }
            if (!mbar_wait(smem_addr(&acc_full[ab]), (it / kConvAccs) & 1, kSpin)) {
                fail(16);
                break;
            }
            tc_fence_after();
            float dm[16], d0[16], dp[16];
            const uint32_t t = taddr + ((q * 32u) << 16) + ab * kConvAcc;
            tmem_ld16(t, dm);
            tmem_ld16(t + 16, d0);
            tmem_ld16(t + 32, dp);
            tmem_ld_wait();
            tc_fence_before();
            mbar_arrive(smem_addr(&acc_empty[ab]));
            float o[16];
#pragma unroll
            for (int co = 0; co < 16; co++) {
                float up = __shfl_up_sync(0xffffffffu, dm[co], 1);
                float dn = __shfl_down_sync(0xffffffffu, dp[co], 1);
                if (lane == 0) up = 0.0f;
                if (lane == 31) dn = 0.0f;
                o[co] = (up + d0[co]) + dn;
            }
            if (a.Yf)
                a.Yf[(((uint64_t)s * a.in.n0 + x) * a.in.n1 + y) * 32 + z] =
                    a.bias && a.cout > 0 ? o[0] + a.bias[0] : o[0];
            if (a.Y) {
#pragma unroll
                for (int co = 0; co < 16; co++) {
                    float v = o[co];
                    if (a.bias && (uint32_t)co < a.cout) v += a.bias[co];
                    if ((uint32_t)co >= a.cout) v = 0.0f;
                    if (a.relu) v = fmaxf(v, 0.0f);
                    o[co] = v;
                }
#pragma unroll
                for (uint32_t h = 0; h < 2; h++) {
                    if (h >= a.out.npl) break;
                    float *oh = o + 8 * h;
                    if (a.mask) {
                        const uint4 m = mk[h];
                        const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (!(bf_lo(mw[k]) > 0.0f)) oh[2 * k] = 0.0f;
                            if (!(bf_hi(mw[k]) > 0.0f)) oh[2 * k + 1] = 0.0f;
                        }
                    }
                    *reinterpret_cast<uint4 *>(a.Y + a.out.row(s, x + 1, y + 1, h, z + a.out.zp) * 16) =
                        make_uint4(pack_bf2(oh[0], oh[1]), pack_bf2(oh[2], oh[3]),
                                   pack_bf2(oh[4], oh[5]), pack_bf2(oh[6], oh[7]));
                }
            }
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
constexpr uint32_t kWgLB = 4;       // output lines per block
constexpr uint32_t kWgStages = 3;
constexpr uint32_t kWgThreads = 192;  // 4 epilogue warps, the MMA warp, the TMA warp
constexpr uint32_t kWgMma = 128;      // the MMA-issuing thread
constexpr uint32_t kWgTma = 160;      // the TMA-issuing thread
constexpr uint32_t kWgCols = 128;   // M = 128 and M = 64 accumulators (48 columns each)
constexpr uint32_t kWgAcc64 = 48;   // column of the M = 64 accumulator
constexpr uint32_t kWgBLine = 3 * 2 * 512;  // per output line: (k, plane) blocks of 32 rows

struct WgradArgs {
    Lp xin;            // activation (zp 0), read through its tensor map
    Lp dy;             // gradient (zp 1), read through its tensor map
    int dy_one_box;    // the gradient map is the 5-D one-box form (two planes)
    uint32_t cin, cout, kp;
    float *partial;    // [gridDim.x][kp][16]
    uint32_t nblocks;
};

template <int NPLX>
struct WgShape {
    // staged activation lines y' = y0 .. y0 + kXL - 1, each as [dx][plane][32 voxels]: M-core
    // i = (dy'' 3 + dx) planes + plane of output line j sits at (j planes 3 + i) x 512 B
    static constexpr uint32_t kXL = NPLX == 2 ? kWgLB + 3 : kWgLB + 5;
    static constexpr uint32_t kXLine = 3 * NPLX * 512;
    static constexpr uint32_t kXBytes = kXL * kXLine;
    static constexpr uint32_t kBBytes = kWgLB * kWgBLine;
    static constexpr uint32_t kStage = kXBytes + kBBytes;
    static constexpr uint32_t kSmem = kWgStages * kStage;
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

// Bounded wait that sleeps between polls (for threads with nothing else to do).
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        __nanosleep(256);
    }
    return false;
}

// One block = 4 output lines of one (sample, x).  Per line j and K step (16 voxels):
//   A (MN-major): the activation, staged [y'][dx][plane][32 voxels] by one TMA box, so
//     M-core (dy'', dx, plane) -- channels 8 plane .. + 7 of line y + dy'' - 1 of x + dx - 1
//     -- is at +512 B per core in the order (dy'', dx, plane), K groups of 8 voxels at
//     +128 B.  Two planes: 18 useful cores = one M = 128 MMA (cores 0..15) and one M = 64
//     (cores 16..23, of which 16 and 17 are used); one plane: 9 useful cores, one M = 128;
//   B (MN-major, N = 48): the gradient line at three z shifts, staged as blocks
//     (k, plane) of 32 rows starting at z' = k (k = 1 - dz) -- N-core (k, plane) at +512 B;
// so D (48 columns: dz, co) accumulates two (one) MMAs per K step.  The bias gradient
// (the sum of the gradient over voxels) is summed from the staged k = 1 blocks by the
// epilogue warps, which have nothing else to do until the last MMA: thread t adds
// channel t % 16 of 16 fixed voxels of every block, and a stage is refilled only after
// both the MMAs and these four warps have released it.
// (Measured and dropped: staging only the k = 1 blocks and building the shifted ones in
// these warps -- 24% fewer TMA bytes -- put the copies on the critical path: 27.1 against
// 23.8 us for the 16-channel layer.)
template <int NPLX>
__global__ void __launch_bounds__(kWgThreads)
    wgrad_tc_kernel(const __grid_constant__ CUtensorMap xmap,
                    const __grid_constant__ CUtensorMap dymap, WgradArgs a) {
    using S = WgShape<NPLX>;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[kWgStages], empty[kWgStages], done;
    __shared__ uint32_t taddr_s;
    __shared__ float bias_part[8][16];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *stage_s = smem;

    if (warp == 0) {
        tmem_alloc(smem_addr(&taddr_s), kWgCols);
        tmem_relinquish();
    }
    if (tid == kWgMma) {
        for (uint32_t i = 0; i < kWgStages; i++) {
            mbar_init(smem_addr(&full[i]), 1);
            mbar_init(smem_addr(&empty[i]), 1 + 4);  // the MMA commit + the 4 epilogue warps
        }
        mbar_init(smem_addr(&done), 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_s;
    const bool any = blockIdx.x < a.nblocks;
    const uint32_t npd = a.dy.npl;

    if (tid == kWgTma) {
        // ---- TMA producer: the stage of local block i is i % kWgStages, refilled as soon
        // as block i - kWgStages has been released
        uint32_t it = 0;
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t st = it % kWgStages;
            if (it >= kWgStages &&
                !mbar_wait(smem_addr(&empty[st]), ((it / kWgStages) - 1) & 1, kSpin)) {
                fail(64);
                break;
            }
            uint32_t s, x, y0;
            wg_block(b, a.dy, s, x, y0);
            const uint32_t bar = smem_addr(&full[st]);
            mbar_expect_tx(bar, S::kXBytes + kWgLB * 3 * npd * 512);
            const uint32_t dst = smem_addr(stage_s + st * S::kStage);
            const int32_t xg = (int32_t)(s * (a.dy.n0 + 2) + x);
            tma_load_4d(dst, &xmap, 0, 0, xg, (int32_t)y0, bar);
            if (a.dy_one_box)  // [line][k][plane][32 rows] in one box (k = a 16-byte shift)
                tma_load_5d(dst + S::kXBytes, &dymap, 0, 0, 0, (int32_t)(y0 + 1), xg + 1, bar);
            else
                for (uint32_t j = 0; j < kWgLB; j++)
                    for (uint32_t k = 0; k < 3; k++)
                        tma_load_4d(dst + S::kXBytes + j * kWgBLine + k * 1024, &dymap,
                                    (int32_t)(k * 8), 0, (int32_t)(y0 + 1 + j), xg + 1, bar);
            mbar_arrive(bar);
        }
    } else if (tid == kWgMma) {
        // ---- MMA issue
        const uint32_t idesc128 = umma_idesc_bf16(128, 48, true, true);
        const uint32_t idesc64 = umma_idesc_bf16(64, 48, true, true);
        uint32_t it = 0, acc = 0;
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t st = it % kWgStages;
            if (!mbar_wait(smem_addr(&full[st]), (it / kWgStages) & 1, kSpin)) {
                fail(32);
                break;
            }
            tc_fence_after();
            const uint32_t xs = smem_addr(stage_s + st * S::kStage);
            // descriptors of line 0, K step 0; later lines / steps add to the start field
            const uint64_t ad0 = umma_smem_desc(xs, 128, 512);
            const uint64_t bd0 = umma_smem_desc(xs + S::kXBytes, 128, 512);
#pragma unroll
            for (uint32_t j = 0; j < kWgLB; j++) {
#pragma unroll
                for (uint32_t ks = 0; ks < 2; ks++) {
                    const uint64_t bd = bd0 + ((j * kWgBLine + ks * 256) >> 4);
                    const uint64_t ad = ad0 + ((j * S::kXLine + ks * 256) >> 4);
                    umma_bf16(taddr, ad, bd, idesc128, acc);
                    if (NPLX == 2) umma_bf16(taddr + kWgAcc64, ad + ((16 * 512) >> 4), bd, idesc64, acc);
                    acc = 1;
                }
            }
            umma_commit(smem_addr(&empty[st]));
        }
        umma_commit(smem_addr(&done));
    } else if (tid < 128) {
        // ---- bias gradient from the staged gradient lines, then the accumulators
        const uint32_t c = tid % 16, grp = tid / 16;  // channel, voxel group (8 x 16 voxels)
        const bool chan = c < npd * 8 && c < a.cout;
        float bsum = 0.0f;
        bool ok = true;
        uint32_t it = 0;
        for (uint32_t b = blockIdx.x; b < a.nblocks; b += gridDim.x, it++) {
            const uint32_t st = it % kWgStages;
            if (!mbar_wait(smem_addr(&full[st]), (it / kWgStages) & 1, kSpin)) {
                fail(256);
                ok = false;
                break;
            }
            const unsigned char *bb = stage_s + st * S::kStage + S::kXBytes;
            if (chan) {
                // voxels 16 grp .. 16 grp + 15 of the block's 4 x 32: line j, z
                const unsigned char *blk = bb + 1024 + (c / 8) * 512 + (c % 8) * 2;
#pragma unroll
                for (uint32_t v = 0; v < 16; v++) {
                    const uint32_t vox = grp * 16 + v, j = vox / 32, z = vox % 32;
                    const uint16_t h =
                        *reinterpret_cast<const uint16_t *>(blk + j * kWgBLine + z * 16);
                    bsum += __uint_as_float((uint32_t)h << 16);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&empty[st]));
        }
        bias_part[grp][c] = bsum;
        float *P = a.partial + (uint64_t)blockIdx.x * a.kp * 16;
        ok = mbar_wait_sleep(smem_addr(&done), 0, kSpin) && ok;
        if (!ok) fail(128);
        tc_fence_after();
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (!any || !ok) {
            for (uint32_t i = tid; i < a.kp * 16; i += 128) P[i] = 0.0f;
        } else {
            if (tid < 16) {
                float bs = 0.0f;
                for (uint32_t g = 0; g < 8; g++) bs += bias_part[g][tid];
                P[27 * a.cin * 16 + tid] = tid < npd * 8 ? bs : 0.0f;
            }
            // chunk c: 0..2 = M = 128 accumulator (k = c), 3..5 = M = 64 (k = c - 3)
            const uint32_t chunks = NPLX == 2 ? 6 : 3;
            for (uint32_t ck = 0; ck < chunks; ck++) {
                const bool m64 = ck >= 3;
                float v[16];
                __syncwarp();
                tmem_ld16(taddr + ((warp * 32u) << 16) + (m64 ? kWgAcc64 + (ck - 3) * 16 : ck * 16), v);
                tmem_ld_wait();
                // accumulator row -> M-core i and channel within the core
                uint32_t i, c8;
                bool valid;
                if (m64) {
                    valid = lane < 16;
                    i = 16 + (warp * 16 + lane) / 8;
                    c8 = lane % 8;
                } else {
                    valid = true;
                    i = (warp * 32 + lane) / 8;
                    c8 = lane % 8;
                }
                const uint32_t dyi = i / (3 * NPLX), dx = (i / NPLX) % 3, h = i % NPLX;
                const uint32_t ci = h * 8 + c8;
                const uint32_t dzi = 2 - (m64 ? ck - 3 : ck);  // chunk k holds dz = 1 - k
                valid = valid && dyi < 3 && ci < a.cin;
                if (valid) {
                    float *p = P + (uint64_t)((dx * 9 + dyi * 3 + dzi) * a.cin + ci) * 16;
#pragma unroll
                    for (int co = 0; co < 16; co++) p[co] = co < (int)(npd * 8) ? v[co] : 0.0f;
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
// One CTA per row k: thread (p0, q) sums the float4 of channels 4q .. 4q + 3 over
// p = p0, p0 + 64, ... in order, then a fixed tree over p0 (deterministic).
__global__ void __launch_bounds__(256) wgrad_tc_reduce_kernel(const float *__restrict__ partial,
                                                              uint32_t parts, uint32_t kp,
                                                              uint32_t cin, uint32_t cout,
                                                              float *__restrict__ dW) {
    __shared__ float4 red[64][4];
    const uint32_t k = blockIdx.x, q = threadIdx.x % 4, p0 = threadIdx.x / 4;
    float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (k <= 27 * cin)
        for (uint32_t p = p0; p < parts; p += 64) {
            const float4 v =
                reinterpret_cast<const float4 *>(partial + ((uint64_t)p * kp + k) * 16)[q];
            s.x += v.x;
            s.y += v.y;
            s.z += v.z;
            s.w += v.w;
        }
    red[p0][q] = s;
    __syncthreads();
    for (uint32_t w = 32; w > 0; w >>= 1) {
        if (p0 < w) {
            const float4 o = red[p0 + w][q];
            float4 &r = red[p0][q];
            r.x += o.x;
            r.y += o.y;
            r.z += o.z;
            r.w += o.w;
        }
        __syncthreads();
    }
    if (threadIdx.x < 16 && threadIdx.x < cout) {
        const float4 r = red[0][threadIdx.x / 4];
        const uint32_t c = threadIdx.x % 4;
        dW[(uint64_t)k * cout + threadIdx.x] = c == 0 ? r.x : c == 1 ? r.y : c == 2 ? r.z : r.w;
    }
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

// Weight image of a convolution with `in_ch` input channels (groups x 1536 B, the B
// operand, K-major): element (group g, row n = dz 16 + oc, column k) at g 1536 +
// (k/8) 768 + (n/8) 128 + (n%8) 16 + (k%8) 2; column k = input channel (two planes) or
// (tap of the pair, channel) for one plane.  Forward: W[t cin + ic][oc]; backward-data:
// W[(26 - t) cin + oc][ic].
__global__ void pack_tc_weights_kernel(const float *__restrict__ W, uint32_t cin, uint32_t cout,
                                       int backward, uint32_t groups,
                                       __nv_bfloat16 *__restrict__ img) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= groups * kConvN * 16) return;
    const uint32_t g = e / (kConvN * 16), n = (e / 16) % kConvN, k = e % 16;
    const uint32_t in_ch = backward ? cout : cin, out_ch = backward ? cin : cout;
    const bool two = in_ch > 8;
    const uint32_t tap9 = two ? g : 2 * g + k / 8, ic = two ? k : k % 8;
    const uint32_t dz = n / 16, oc = n % 16;
    float w = 0.0f;
    if (tap9 < 9 && ic < in_ch && oc < out_ch) {
        const uint32_t t = (tap9 / 3) * 9 + (tap9 % 3) * 3 + dz;
        w = backward ? W[((uint64_t)(26 - t) * cin + oc) * cout + ic]
                     : W[((uint64_t)t * cin + ic) * cout + oc];
    }
    const uint32_t off = g * kConvGroup + (k / 8) * (kConvN * 16) + (n / 8) * 128 + (n % 8) * 16 +
                         (k % 8) * 2;
    img[off / 2] = __float2bfloat16_rn(w);
}

// Several images in one launch: job j packs W[j / 2] forward (j even) or backward-data
// (j odd, when img[j] is non-null); element e of the launch belongs to the job whose range
// [start[j], start[j + 1]) holds it.
constexpr uint32_t kMaxPackJobs = 16;
struct PackJobs {
    const float *W[kMaxPackJobs];
    __nv_bfloat16 *img[kMaxPackJobs];
    uint32_t cin[kMaxPackJobs], cout[kMaxPackJobs], groups[kMaxPackJobs];
    uint32_t start[kMaxPackJobs + 1];
    uint32_t jobs;
};

__global__ void pack_tc_jobs_kernel(PackJobs p) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= p.start[p.jobs]) return;
    uint32_t j = 0;
    while (e >= p.start[j + 1]) j++;
    const uint32_t q = e - p.start[j];
    const uint32_t g = q / (kConvN * 16), n = (q / 16) % kConvN, k = q % 16;
    const bool backward = j & 1;
    const uint32_t cin = p.cin[j], cout = p.cout[j];
    const uint32_t in_ch = backward ? cout : cin, out_ch = backward ? cin : cout;
    const bool two = in_ch > 8;
    const uint32_t tap9 = two ? g : 2 * g + k / 8, ic = two ? k : k % 8;
    const uint32_t dz = n / 16, oc = n % 16;
    float w = 0.0f;
    if (tap9 < 9 && ic < in_ch && oc < out_ch) {
        const uint32_t t = (tap9 / 3) * 9 + (tap9 % 3) * 3 + dz;
        w = backward ? p.W[j][((uint64_t)(26 - t) * cin + oc) * cout + ic]
                     : p.W[j][((uint64_t)t * cin + ic) * cout + oc];
    }
    const uint32_t off = g * kConvGroup + (k / 8) * (kConvN * 16) + (n / 8) * 128 + (n % 8) * 16 +
                         (k % 8) * 2;
    p.img[j][off / 2] = __float2bfloat16_rn(w);
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
        channels > 16 || zp > 1 || dims[1] % 8)
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
    return (in_channels > 8 ? 9u : 5u) * kConvGroup;
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
    const uint32_t gf = (uint32_t)(bpgb_cnn_tc_weight_bytes(cin) / kConvGroup);
    pack_tc_weights_kernel<<<(gf * kConvN * 16 + 255) / 256, 256, 0, s>>>(
        d_W, cin, cout, 0, gf, (__nv_bfloat16 *)d_Wf);
    count_launches(1);
    if (d_Wb) {
        const uint32_t gb = (uint32_t)(bpgb_cnn_tc_weight_bytes(cout) / kConvGroup);
        pack_tc_weights_kernel<<<(gb * kConvN * 16 + 255) / 256, 256, 0, s>>>(
            d_W, cin, cout, 1, gb, (__nv_bfloat16 *)d_Wb);
        count_launches(1);
    }
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int bpgb_cnn_tc_pack_layers(const float *const *d_W, const uint32_t *cin, const uint32_t *cout,
                            void *const *d_Wf, void *const *d_Wb, uint32_t layers, void *stream) {
    clear_error();
    if (!d_W || !cin || !cout || !d_Wf || layers == 0 || 2 * layers > kMaxPackJobs)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_pack_layers arguments (1..8 layers)");
    PackJobs p{};
    uint32_t n = 0;
    for (uint32_t l = 0; l < layers; l++) {
        if (!d_W[l] || !d_Wf[l] || cin[l] == 0 || cin[l] > 16 || cout[l] == 0 || cout[l] > 16 ||
            !aligned16(d_Wf[l]) || (d_Wb && d_Wb[l] && !aligned16(d_Wb[l])))
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_pack_layers layer");
        for (uint32_t b = 0; b < 2; b++) {
            void *img = b ? (d_Wb ? d_Wb[l] : nullptr) : d_Wf[l];
            const uint32_t j = 2 * l + b;
            p.W[j] = d_W[l];
            p.img[j] = (__nv_bfloat16 *)img;
            p.cin[j] = cin[l];
            p.cout[j] = cout[l];
            p.groups[j] = img ? (uint32_t)(bpgb_cnn_tc_weight_bytes(b ? cout[l] : cin[l]) / kConvGroup) : 0;
            p.start[j] = n;
            n += p.groups[j] * kConvN * 16;
        }
    }
    p.jobs = 2 * layers;
    p.start[p.jobs] = n;
    pack_tc_jobs_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(p);
    count_launches(1);
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
    if (!tensor_map_encoder()) return set_error(BPGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    // the input as [x' (with sample)][y'][plane][z' x 8 channels]: boxes of 7 lines x the
    // line's 32 voxels (256 elements, 512 B contiguous) of one plane
    // (dimension 1 is y', dimension 2 the plane: one box lands [x'][plane][y'][z])
    const Lp &g = a.in;
    const cuuint64_t gdims[4] = {g.L() * 8ull, g.n1 + 2ull, g.npl, (cuuint64_t)batch * (g.n0 + 2)};
    const cuuint64_t gstr[3] = {(cuuint64_t)g.line_rows() * 16, g.L() * 16ull,
                                (g.n1 + 2ull) * g.line_rows() * 16};
    const cuuint32_t box[4] = {256, kConvLines, g.npl, 3};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap map;
    CUresult r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                                      const_cast<void *>(d_X), gdims, gstr, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(BPGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (cnn)");
    a.W = (const uint8_t *)d_W;
    a.bias = d_bias;
    a.cout = out_channels;
    a.relu = relu;
    a.mask = (const uint8_t *)d_mask;
    a.Y = (uint8_t *)d_Y;
    a.Yf = d_Yf;
    a.nblocks = batch * dims[0] * (dims[1] / kConvLB);
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    auto launch = [&](auto kernel, uint32_t smem) -> int {
        smem = std::max(kMinSmem, smem);
        if ((st = reserve_dynamic_smem((const void *)kernel, smem))) return st;
        const unsigned grid = (unsigned)std::min<uint64_t>(a.nblocks, 2ull * sm_count_cached());
        kernel<<<grid, kConvThreads, smem, s>>>(map, a);
        return BPGB_OK;
    };
    st = a.in.npl == 2 ? launch(conv_tc_kernel<2>, ConvShape<2>::kSmem)
                       : launch(conv_tc_kernel<1>, ConvShape<1>::kSmem);
    if (st) return st;
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
        !lp_of(dims, batch, out_channels, 1, &a.dy) || !aligned16(d_X) || !aligned16(d_dY) ||
        !aligned16(d_scratch))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad tc_conv3d_wgrad arguments");
    if (scratch_bytes < bpgb_cnn_tc_wgrad_scratch_bytes(in_channels, dims, batch))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "tc wgrad scratch too small");
    if (!tensor_map_encoder()) return set_error(BPGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    // the gradient as [x' (with sample)][y'][plane][z' x 8 channels]: boxes of one line's
    // planes x 32 rows (256 elements) starting at row k
    const Lp &g = a.dy;
    const cuuint64_t gdims[4] = {g.L() * 8ull, g.npl, g.n1 + 2ull, (cuuint64_t)batch * (g.n0 + 2)};
    const cuuint64_t gstr[3] = {g.L() * 16ull, (cuuint64_t)g.line_rows() * 16,
                                (g.n1 + 2ull) * g.line_rows() * 16};
    const cuuint32_t box[4] = {256, g.npl, 1, 1};
    // the activation as [y'][x' (with sample)][plane][32 voxels x 8 channels] (dimension 2 is
    // x', dimension 3 y'): one box = 3 x' x the staged y' lines, landing [y'][dx][plane][z]
    const Lp &gx = a.xin;
    const cuuint64_t xdims[4] = {256, gx.npl, (cuuint64_t)batch * (gx.n0 + 2), gx.n1 + 2ull};
    const cuuint64_t xstr[3] = {512, (gx.n1 + 2ull) * gx.line_rows() * 16,
                                (cuuint64_t)gx.line_rows() * 16};
    const cuuint32_t xbox[4] = {256, gx.npl, 3,
                                gx.npl == 2 ? WgShape<2>::kXL : WgShape<1>::kXL};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap map, xmap;
    CUresult r = CUDA_ERROR_INVALID_VALUE;
    if (g.npl == 2) {
        // one box per block: [line 4][k 3][plane][32 rows], k a dimension of stride 16 B
        // (the row shift of the three z taps; its windows overlap by design)
        const cuuint64_t d5[5] = {256, 2, 3, g.n1 + 2ull, (cuuint64_t)batch * (g.n0 + 2)};
        const cuuint64_t s5[4] = {g.L() * 16ull, 16, (cuuint64_t)g.line_rows() * 16,
                                  (g.n1 + 2ull) * g.line_rows() * 16};
        const cuuint32_t b5[5] = {256, 2, 3, kWgLB, 1};
        const cuuint32_t e5[5] = {1, 1, 1, 1, 1};
        r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5,
                                 const_cast<void *>(d_dY), d5, s5, b5, e5,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        a.dy_one_box = r == CUDA_SUCCESS;
    }
    if (!a.dy_one_box)
        r = tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                                 const_cast<void *>(d_dY), gdims, gstr, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS)
        r = tensor_map_encoder()(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4,
                                 const_cast<void *>(d_X), xdims, xstr, xbox, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(BPGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (cnn wgrad)");
    a.cin = in_channels;
    a.cout = out_channels;
    a.kp = bpgb_cnn_kp(in_channels);
    a.partial = d_scratch;
    a.nblocks = batch * dims[0] * (dims[1] / kWgLB);
    const unsigned grid = (unsigned)std::min<uint64_t>(a.nblocks, 2ull * sm_count_cached());
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    auto launch = [&](auto kernel, uint32_t smem) -> int {
        smem = std::max(kMinSmem, smem);
        if ((st = reserve_dynamic_smem((const void *)kernel, smem))) return st;
        kernel<<<grid, kWgThreads, smem, s>>>(xmap, map, a);
        return BPGB_OK;
    };
    st = a.xin.npl == 2 ? launch(wgrad_tc_kernel<2>, WgShape<2>::kSmem)
                        : launch(wgrad_tc_kernel<1>, WgShape<1>::kSmem);
    if (st) return st;
    count_launches(1);
    wgrad_tc_reduce_kernel<<<a.kp, 256, 0, s>>>(d_scratch, grid, a.kp, in_channels, out_channels,
                                                d_dW);
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

