// Factored, TMA-staged dense backprojection for sm_103a.
//
// Same quantity as the reference kernel (backproject_cuda.cu:117-175):
//   V[v] = sum_p H[p, round((lw_p + |l_p - v| + |v - c_p| + cw_p - t0) / dT)]
// restricted to in-range bins, for pair lists that factor as p = l * S + s (the
// exhaustive and single-laser orders of precompute_distances, backproject.hpp:374-397)
// or are confocal (:399-413, laser point = camera point, d = 2|v - c| + 2 cw).
//
// Work decomposition
//   * A CTA owns one voxel tile and, when `splits` > 1, a contiguous range of
//     (laser, SPAD-chunk) items.  Each consumer thread holds K voxels on a line along
//     one axis (`kax`); a warp's lanes cover the other axes at each step of that line.
//     The grouped form (preset 13, block-sparse passes) gives a CTA four 8^3 tiles, each
//     with its own two consumer warps, sharing the producer and the stage ring: a stage
//     holds `chunk` rows of every tile, so an SM runs as many consumer warps as with the
//     wide tiles while the tiles stay the size of the occupancy CNN's blocks.
//   * Warp 0 is the producer.  For every item it computes, per SPAD row of the chunk,
//     the range of bins the tile can reach (exact distance bounds from the SPAD and
//     the laser point to the tile's box), aligns it for TMA, writes a 32-byte row record
//     (SPAD position relative to the tile centre in bin units, row constant, pre-splatted
//     for packed FP32x2 arithmetic) and issues 2-D TMA tile loads of H[p, lo : lo + W]
//     into a shared-memory stage.  Out-of-range bins (< 0 or >= T) arrive as zeros from
//     the TMA unit, which is exactly the reference's "skip out-of-range bins" rule.
//   * Warps 1..n are consumers.  Per thread: the laser leg A_k = |v_k - l| / dT +
//     lw / dT - t0 / dT (recomputed per laser), the voxels' coordinates relative to the
//     tile centre (bin units) and the accumulators, all as voxel pairs.  Per row and
//     voxel pair (sm_100 packed FP32x2 ops, one instruction for two voxels):
//       dz = vk - ck; q = dz*dz + D; r = rsqrt(q) (MUFU, per voxel);
//       x = q*r + A; y = x + row constant; z = y + 1.5*2^23 (round to nearest);
//     then one shifted-add per voxel forms the shared address and one load gathers.
//     That is 6 FP32x2 + 2 MUFU + 2 address + 2 gathers = 12 issue slots per two updates;
//     FP16/BF16 rows accumulate with sm_100's one-op mixed-precision add.
//   * Stages are handed over with mbarriers (full: TMA bytes + producer arrive; empty:
//     one arrive per consumer warp; the producer sleeps briefly between its polls, so
//     that they take no issue slots from the consumers).  Every wait is bounded; a wait
//     that gives up sets an error counter the host reads (bpgb_plan_check) and the CTA
//     drains its own in-flight copies before returning.
//
// Numerics: FP32 geometry relative to the tile centre, rsqrt.approx; FP32 or Kahan-
// folded chunk sums.  Rounding is round-half-even instead of the reference's half-away
// (ties need an exact .5 in FP32 and are measured with the mis-binned fraction).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bpgb_device.cuh"
#include "bpgb_internal.h"

namespace bpgb {

namespace {

constexpr int kPlanRows = 16;  // rows per unrolled consumer iteration: plans
constexpr int kBatchRows = 4;  // and the batch kernel
constexpr int kC32Rows = 4;    // complex rows (FP16 pairs / complex64), whose accumulators
constexpr int kC64Rows = 1;    // already double the registers
constexpr uint32_t kMaxChunk = 64;                         // rows per stage (two per lane)
constexpr uint32_t kMaxGroupEntries = 128;  // grouped stages: (tile, row) entries, four per lane
constexpr uint32_t kMaxGroups = 4;          // tiles per CTA
constexpr uint32_t kFactS = 4;  // SPADs per block of the factored lasers x SPADs form
constexpr uint32_t kRecordBytes = 32;                      // two float4 per row
constexpr uint32_t kPlanDiagWords = 8;  // a plan's device counters (see fast_plan_build)
constexpr uint32_t kPlanThresholdWord = 5;  // ... and the top-k selection's threshold
// row records of a chunk of c rows, padded so that the TMA rows after them stay aligned
__host__ __device__ constexpr uint32_t table_bytes_of(uint32_t c) {
    return (c * kRecordBytes + 127) / 128 * 128;
}
constexpr float kMargin = 2.0f;                            // bins of slack around each window
constexpr float kQEps = 1e-6f;                             // keeps q > 0 (bins^2)

struct FastArgs {
    uint32_t n[3];      // voxels per side
    uint32_t tiles[3];  // tiles per axis
    uint32_t tdim[3];   // tile size in voxels
    uint32_t lane[3];   // lane layout (product 32)
    uint32_t warp[3];   // consumer warp layout
    uint32_t kax;       // axis of each thread's voxel line
    uint32_t planar;    // every SPAD has the same frame coordinate along kax
    uint32_t oax0, oax1;  // the two other axes
    float h[3];         // voxel step length along each frame axis (m)
    float hs[3];        // h * sb (bins)
    float sb;           // SPAD-leg scale: 1/dT (2/dT confocal)
    float sa;           // laser-leg scale: 1/dT (0 confocal)
    uint32_t W;         // staged bins per row
    uint32_t BW;        // TMA box width (elements)
    uint32_t nbox;      // boxes per row
    uint32_t row_bytes; // shared bytes per row (W * esz)
    uint32_t chunk;     // rows per stage
    uint32_t stages;
    uint32_t stage_bytes;
    uint32_t table_bytes;  // row records at the start of each stage
    uint32_t align;     // TMA x alignment (elements)
    uint64_t L, S;
    uint32_t nchunks;   // ceil(S / chunk)
    uint32_t splits;
    uint32_t spin_limit;
    uint32_t T;
    float out_scale;
    uint64_t nvox;
    // tile-list launches (block-sparse passes): CTA i runs the tiles in list slots
    // groups x (i / splits) + g (g < groups) below min(*tile_count, max_tiles); null =
    // every tile of the volume
    const uint32_t *tile_list;
    const uint32_t *tile_count;
    uint32_t max_tiles;
    uint32_t groups;  // tiles per CTA, each with its own wx x wy x wz consumer warps
    // tile-list launches with pair splits: partial sums are stored per list slot and
    // split at tile-local voxel offsets (slot-major, then split, then voxel)
    uint32_t tile_local;
    // lasers x SPADs with factored legs (bp_fact_kernel); nchunks then counts laser groups
    uint32_t fact;
};

// (laser, SPAD chunk) items of one tile, or (SPAD block, laser group) items when factored
__host__ __device__ inline uint64_t fast_items(const FastArgs &a) {
    return a.fact ? (a.S / kFactS) * (uint64_t)a.nchunks : a.L * (uint64_t)a.nchunks;
}

struct TileGeo {
    uint32_t org[3];
    float ctr[3];  // tile centre in voxel-index units
};

__device__ __forceinline__ void tile_of_block(const FastArgs &a, uint32_t tile, TileGeo &g) {
    const uint32_t tz = tile % a.tiles[2];
    tile /= a.tiles[2];
    const uint32_t tx = tile % a.tiles[0];
    const uint32_t ty = tile / a.tiles[0];
    g.org[0] = tx * a.tdim[0];
    g.org[1] = ty * a.tdim[1];
    g.org[2] = tz * a.tdim[2];
#pragma unroll
    for (int k = 0; k < 3; k++) g.ctr[k] = __fmaf_rn(0.5f, (float)(a.tdim[k] - 1), (float)g.org[k]);
}

// Distance bounds from point p (frame coordinates, metres) to the tile's box of voxel
// centres: min to the clamped point, max to the farthest corner.
__device__ __forceinline__ void box_bounds(const FastArgs &a, const TileGeo &g, float px,
                                           float py, float pz, float &dmin, float &dmax) {
    const float p[3] = {px, py, pz};
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float lo = __fmul_rn((float)g.org[k], a.h[k]);
        const float hi = __fmul_rn((float)(g.org[k] + a.tdim[k] - 1), a.h[k]);
        const float c = fminf(fmaxf(p[k], lo), hi);
        const float d0 = p[k] - c;
        const float e0 = p[k] - lo, e1 = p[k] - hi;
        s0 = __fmaf_rn(d0, d0, s0);
        s1 = __fadd_rn(s1, fmaxf(__fmul_rn(e0, e0), __fmul_rn(e1, e1)));
    }
    dmin = sqrtf(s0);
    dmax = sqrtf(s1);
}

// lo rounded down to a multiple of al, a power of two (the TMA alignment in elements).
__device__ __forceinline__ int32_t align_down(int32_t lo, uint32_t al) {
    return lo & -(int32_t)al;
}

// A tile's box of voxel centres and its centre in frame coordinates (metres), formed once
// per tile for the producer's row records (the same products box_bounds forms).
struct TileBox {
    float lo[3], hi[3], ch[3];
};

__device__ __forceinline__ void tile_box(const FastArgs &a, const TileGeo &g, TileBox &b) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        b.lo[k] = __fmul_rn((float)g.org[k], a.h[k]);
        b.hi[k] = __fmul_rn((float)(g.org[k] + a.tdim[k] - 1), a.h[k]);
        b.ch[k] = __fmul_rn(g.ctr[k], a.h[k]);
    }
}

// box_bounds' minimum distance, from the precomputed box.
__device__ __forceinline__ float box_dmin(const TileBox &b, float px, float py, float pz) {
    const float p[3] = {px, py, pz};
    float s0 = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float d0 = p[k] - fminf(fmaxf(p[k], b.lo[k]), b.hi[k]);
        s0 = __fmaf_rn(d0, d0, s0);
    }
    return sqrtf(s0);
}

// The laser's part of a tile's window start: sa x (min distance to the box) + Lt.w; one per
// (tile, laser), shared by every SPAD row of that laser.
__device__ __forceinline__ float laser_term(const FastArgs &a, const TileBox &b, float4 Lt) {
    return __fmaf_rn(a.sa, box_dmin(b, Lt.x, Lt.y, Lt.z), Lt.w);
}

// Row record of SPAD entry G (frame position, row constant Cs) for a tile (box b) and the
// laser's laser_term lt: e[a] = SPAD coordinate a relative to the tile centre in bin units,
// ew = Cs - lo; returns lo, the window's first bin, aligned down to a.align.
__device__ __forceinline__ int32_t row_record(const FastArgs &a, const TileBox &b, float4 G,
                                              float lt, float e[3], float &ew) {
    const float bmin = __fmaf_rn(a.sb, box_dmin(b, G.x, G.y, G.z), G.w) + lt;
    const int32_t lo = align_down((int32_t)floorf(bmin - kMargin), a.align);
    const float gp[3] = {G.x, G.y, G.z};
#pragma unroll
    for (int k = 0; k < 3; k++) e[k] = __fmul_rn(gp[k] - b.ch[k], a.sb);
    ew = G.w - (float)lo;
    return lo;
}

// Laser leg of voxel idx[3] for laser entry Lt = (frame position, lw/dT - t0/dT).
__device__ __forceinline__ float laser_leg(const FastArgs &a, const uint32_t idx[3], float4 Lt) {
    const float dx = __fmaf_rn((float)idx[0], a.h[0], -Lt.x);
    const float dy = __fmaf_rn((float)idx[1], a.h[1], -Lt.y);
    const float dz = __fmaf_rn((float)idx[2], a.h[2], -Lt.z);
    const float d = sqrtf(__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz))));
    return __fmaf_rn(a.sa, d, Lt.w);
}

// x_i for i = 0, 1, 2 without indexing a local array (runtime axis choices would
// otherwise place small arrays in local memory).
template <typename T>
__device__ __forceinline__ T sel3(T x0, T x1, T x2, uint32_t i) {
    return i == 0 ? x0 : (i == 1 ? x1 : x2);
}

__device__ __forceinline__ float rel_coord(const FastArgs &a, const TileGeo &g, uint32_t ax,
                                           uint32_t idx) {
    return __fmul_rn((float)idx - sel3(g.ctr[0], g.ctr[1], g.ctr[2], ax),
                     sel3(a.hs[0], a.hs[1], a.hs[2], ax));
}

// D = d0^2 + d1^2 + eps over the two axes across a thread's voxel line.
__device__ __forceinline__ float row_d(float v0, float v1, float e0, float e1) {
    const float d0 = v0 - e0, d1 = v1 - e1;
    return __fmaf_rn(d0, d0, __fmaf_rn(d1, d1, kQEps));
}

// Window index (as float bits of x + 1.5*2^23) of one voxel; the scalar form of the
// packed consumer arithmetic, used by the bin dump.
__device__ __forceinline__ uint32_t window_bits(float vk, float D, float A, float ek, float ew,
                                                bool planar) {
    const float dz = __fadd_rn(vk, -ek);
    // planar walls: dz^2 is per voxel, formed once, then one add per row
    const float q = planar ? __fadd_rn(D, __fmul_rn(dz, dz)) : __fmaf_rn(dz, dz, D);
    const float r = rsqrt_approx(q);
    const float y = __fmaf_rn(q, r, __fadd_rn(A, ew));
    return __float_as_uint(__fadd_rn(y, kMagic));
}

// ---- shared-memory gathers ------------------------------------------------------------
// `ld.shared` at a 32-bit shared-window address (the dynamic base's window address plus a
// byte offset): one address add per gather.  Written as volatile asm they keep their
// order against the stage's full-barrier wait and empty-barrier arrive (volatile asm
// too); the backend still interleaves the independent voxel chains around them.  The same
// loads written as C++ dereferences of the generic base pointer ran 9-12% slower (dense
// 256^3 79.3 against 71.9 ms, the 64-capture batch 115.5 against 101.3 ms).
template <typename T>
__device__ __forceinline__ T lds(const unsigned char *smem, uint32_t off);
template <>
__device__ __forceinline__ float lds<float>(const unsigned char *smem, uint32_t off) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(smem_addr(smem) + off));
    return v;
}
template <>
__device__ __forceinline__ unsigned short lds<unsigned short>(const unsigned char *smem, uint32_t off) {
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(smem_addr(smem) + off));
    return v;
}
template <>
__device__ __forceinline__ uint32_t lds<uint32_t>(const unsigned char *smem, uint32_t off) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(smem_addr(smem) + off));
    return v;
}
template <>
__device__ __forceinline__ float2 lds<float2>(const unsigned char *smem, uint32_t off) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(smem_addr(smem) + off));
    return v;
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// Accumulators of one voxel pair, per storage type.
template <typename HT>
struct Pair;

template <>
struct Pair<float> {
    static constexpr uint32_t kEsz = 4, kShift = 2;
    static constexpr bool kCplx = false;
    float2 a;
    __device__ __forceinline__ void zero() { a = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void gather2(const unsigned char *sm, uint32_t p0, uint32_t p1) {
        const float v0 = lds<float>(sm, p0), v1 = lds<float>(sm, p1);
        a = __fadd2_rn(a, make_float2(v0, v1));
    }
    __device__ __forceinline__ void fold(Pair &comp, const Pair &part) {
        kahan_add(a.x, comp.a.x, part.a.x);
        kahan_add(a.y, comp.a.y, part.a.y);
    }
    __device__ __forceinline__ void finish(const Pair &comp) {
        a.x -= comp.a.x;
        a.y -= comp.a.y;
    }
    __device__ __forceinline__ void store(void *out, uint64_t i, int which, float s) const {
        ((float *)out)[i] = (which ? a.y : a.x) * s;
    }
};

template <int IS_BF16>
struct PairHalf {
    static constexpr uint32_t kEsz = 2, kShift = 1;
    static constexpr bool kCplx = false;
    float2 a;
    __device__ __forceinline__ void zero() { a = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void gather2(const unsigned char *sm, uint32_t p0, uint32_t p1) {
        const unsigned short h0 = lds<unsigned short>(sm, p0), h1 = lds<unsigned short>(sm, p1);
        if (IS_BF16) {
            asm("add.rn.f32.bf16 %0, %1, %0;" : "+f"(a.x) : "h"(h0));
            asm("add.rn.f32.bf16 %0, %1, %0;" : "+f"(a.y) : "h"(h1));
        } else {
            asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(a.x) : "h"(h0));
            asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(a.y) : "h"(h1));
        }
    }
    __device__ __forceinline__ void fold(PairHalf &comp, const PairHalf &part) {
        kahan_add(a.x, comp.a.x, part.a.x);
        kahan_add(a.y, comp.a.y, part.a.y);
    }
    __device__ __forceinline__ void finish(const PairHalf &comp) {
        a.x -= comp.a.x;
        a.y -= comp.a.y;
    }
    __device__ __forceinline__ void store(void *out, uint64_t i, int which, float s) const {
        ((float *)out)[i] = (which ? a.y : a.x) * s;
    }
};
template <>
struct Pair<__half> : PairHalf<0> {};
template <>
struct Pair<__nv_bfloat16> : PairHalf<1> {};

template <>
struct Pair<float2> {
    static constexpr uint32_t kEsz = 8, kShift = 3;
    static constexpr bool kCplx = true;
    float2 a0, a1;
    __device__ __forceinline__ void zero() { a0 = a1 = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void gather2(const unsigned char *sm, uint32_t p0, uint32_t p1) {
        const float2 v0 = lds<float2>(sm, p0), v1 = lds<float2>(sm, p1);
        a0 = __fadd2_rn(a0, v0);
        a1 = __fadd2_rn(a1, v1);
    }
    __device__ __forceinline__ void fold(Pair &comp, const Pair &part) {
        kahan_add(a0.x, comp.a0.x, part.a0.x);
        kahan_add(a0.y, comp.a0.y, part.a0.y);
        kahan_add(a1.x, comp.a1.x, part.a1.x);
        kahan_add(a1.y, comp.a1.y, part.a1.y);
    }
    __device__ __forceinline__ void finish(const Pair &comp) {
        a0.x -= comp.a0.x;
        a0.y -= comp.a0.y;
        a1.x -= comp.a1.x;
        a1.y -= comp.a1.y;
    }
    __device__ __forceinline__ void store(void *out, uint64_t i, int which, float s) const {
        const float2 v = which ? a1 : a0;
        ((float2 *)out)[i] = make_float2(v.x * s, v.y * s);
    }
};

// Complex rows stored as FP16 pairs (re, im) in one 32-bit word: each half is added to
// its FP32 accumulator with the mixed-precision add.
template <>
struct Pair<__half2> {
    static constexpr uint32_t kEsz = 4, kShift = 2;
    static constexpr bool kCplx = true;
    float2 a0, a1;
    __device__ __forceinline__ void zero() { a0 = a1 = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ static void add_c16(float2 &acc, uint32_t w) {
        asm("{\n\t.reg .f16 re, im;\n\t"
            "mov.b32 {re, im}, %2;\n\t"
            "add.rn.f32.f16 %0, re, %0;\n\t"
            "add.rn.f32.f16 %1, im, %1;\n\t}"
            : "+f"(acc.x), "+f"(acc.y)
            : "r"(w));
    }
    __device__ __forceinline__ void gather2(const unsigned char *sm, uint32_t p0, uint32_t p1) {
        add_c16(a0, lds<uint32_t>(sm, p0));
        add_c16(a1, lds<uint32_t>(sm, p1));
    }
    __device__ __forceinline__ void fold(Pair &comp, const Pair &part) {
        kahan_add(a0.x, comp.a0.x, part.a0.x);
        kahan_add(a0.y, comp.a0.y, part.a0.y);
        kahan_add(a1.x, comp.a1.x, part.a1.x);
        kahan_add(a1.y, comp.a1.y, part.a1.y);
    }
    __device__ __forceinline__ void finish(const Pair &comp) {
        a0.x -= comp.a0.x;
        a0.y -= comp.a0.y;
        a1.x -= comp.a1.x;
        a1.y -= comp.a1.y;
    }
    __device__ __forceinline__ void store(void *out, uint64_t i, int which, float s) const {
        const float2 v = which ? a1 : a0;
        ((float2 *)out)[i] = make_float2(v.x * s, v.y * s);
    }
};

// Resident CTAs per SM of the 8-consumer-warp presets: K = 8 three CTAs (27 warps, 72
// registers, no spills for real rows; with the shared-load gathers this measured 256^3
// 71.8 -> 70.5 ms and the phasor capture's 8-row stages 16.8 -> 13.1 ms against two CTAs
// at 96 registers), Kahan-compensated variants two (at 72 registers they spill 36-364 B),
// K = 16 one CTA with room for its 16 chains.  The 2- and 4-warp block-sparse presets run
// the two-CTA build (96 registers; the learned octree's fine pass measured 3.94 against
// 4.10 ms per reconstruction with the 72-register one), and the factored lasers x SPADs
// body keeps two (kFactCtas: its SPAD legs alone take 32 registers).
__host__ __device__ constexpr int fast_ctas_per_sm(int k, bool kahan, int esz) {
    return (void)esz, k == 16 ? 1 : (kahan ? 2 : 3);
}
constexpr int kFactCtas = 2;

// Shared-memory state of a CTA's pipeline: stage ring, its mbarriers, the abort flag.
struct PipeShared {
    unsigned char *smem_raw;    // dynamic shared memory base
    unsigned char *stage_base;  // 128-byte aligned stage ring
    uint32_t pad;               // stage_base - smem_raw
    uint64_t *full_bar, *empty_bar;
    int *abort_flag;
};

// Tile and output base of tile g of a CTA's group: tile t0 + g of the volume, or in a
// tile-list launch the tile in list slot t0 + g (with pair splits, partial sums at the
// slot's own tile-local block); false when there is none.
template <typename PairT>
__device__ __forceinline__ bool group_tile(const FastArgs &a, void *out, uint32_t t0, uint32_t g,
                                           uint32_t &tile, void *&dst) {
    const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    dst = out;
    tile = t0 + g;
    if (!a.tile_list) return tile < ntiles;
    const uint32_t slot = t0 + g;
    if (slot >= a.max_tiles || slot >= *a.tile_count) return false;
    tile = a.tile_list[slot];
    if (tile >= ntiles) return false;
    if (a.tile_local) {
        constexpr uint32_t kOutEsz = PairT::kCplx ? 8 : 4;
        const uint64_t tvox = (uint64_t)a.tdim[0] * a.tdim[1] * a.tdim[2];
        dst = (unsigned char *)out + (uint64_t)slot * a.splits * tvox * kOutEsz;
    }
    return true;
}

// First tile (full-volume launch) or list slot (tile-list launch) of a grouped CTA's
// tiles, and its pair split.
__device__ __forceinline__ uint32_t group_origin(const FastArgs &a, uint32_t &split) {
    if (a.tile_list) {
        split = blockIdx.x % a.splits;
        return blockIdx.x / a.splits * a.groups;
    }
    const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    const uint64_t ngroups = (ntiles + a.groups - 1) / a.groups;
    split = (uint32_t)(blockIdx.x / ngroups);
    return (uint32_t)(blockIdx.x % ngroups) * a.groups;
}

// One work unit -- a voxel tile (group_tile(t0, 0)) and a range of (laser, SPAD-chunk)
// items -- through the producer / consumer pipeline.  GROUPED: a group of a.groups tiles
// (group_tile(t0, g)), each with its own wx x wy x wz consumer warps; a stage then holds
// `chunk` rows for every tile of the group, entry e = g x chunk + row (record and
// window), so one producer and one stage ring serve them all.  `step` is the CTA's
// running pipeline step (stage = step % stages, phase = step / stages); consecutive units
// of a persistent CTA continue it, so the stage ring and its barriers carry over.  Rows
// of H are read at row_base + l * S + s (the capture's first row in a packed buffer).
// Returns false when a bounded wait gave up (the CTA must stop).
template <typename HT, int K, bool KAHAN, bool CHECKED, bool PLANAR, int ROWS, bool GROUPED>
__device__ __forceinline__ bool fast_unit(const FastArgs &a, const CUtensorMap *tmap,
                                          const float4 *__restrict__ spads,
                                          const float4 *__restrict__ lasers, void *out,
                                          unsigned long long *diag, uint32_t t0,
                                          uint32_t split, uint32_t row_base, uint64_t &step,
                                          const PipeShared &sh) {
    using PairT = Pair<HT>;
    constexpr uint32_t esz = PairT::kEsz;
    constexpr int NP = K / 2;
    // stage entries per producer lane
    constexpr uint32_t kLane = GROUPED ? kMaxGroupEntries / 32 : kMaxChunk / 32;
    unsigned char *const smem_raw = sh.smem_raw;
    unsigned char *const stage_base = sh.stage_base;
    const uint32_t pad = sh.pad;
    uint64_t *const full_bar = sh.full_bar;
    uint64_t *const empty_bar = sh.empty_bar;
    int &abort_flag = *sh.abort_flag;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t items = a.L * a.nchunks;
    const uint64_t i0 = items * split / a.splits, i1 = items * (split + 1) / a.splits;
    const uint64_t step0 = step;
    step += i1 - i0;
    const uint32_t count = (uint32_t)(i1 - i0);  // items < 2^32 (checked at plan build)

    TileGeo g;
    uint32_t tile = t0;  // the tile itself when not GROUPED
    if constexpr (!GROUPED) tile_of_block(a, tile, g);

    if (warp == 0) {
        // ---------------- producer ----------------
        // The tile's box, and the laser's part of every window start (laser_term) while
        // the laser stays the same.  GROUPED: entry lane + 32 q of a stage is row
        // (lane + 32 q) % chunk of tile (lane + 32 q) / chunk of the group; the tiles'
        // boxes, laser terms and whether they exist are kept in shared memory.
        uint32_t nvalid = 1;  // tiles of the group that exist
        TileBox box;
        float lt = 0.0f;
        uint32_t cur_l = ~0u;
        TileBox *box_g = nullptr;
        float *lt_g = nullptr;
        const uint32_t *ok_g = nullptr;
        uint32_t cshift = 0;
        if constexpr (GROUPED) {
            __shared__ TileBox box_s[kMaxGroups];
            __shared__ float lt_s[kMaxGroups];
            __shared__ uint32_t ok_s[kMaxGroups];
            if (lane < kMaxGroups) {
                void *unused;
                ok_s[lane] = lane < a.groups && group_tile<PairT>(a, out, t0, lane, tile, unused);
                if (ok_s[lane]) {
                    TileGeo gt;
                    tile_of_block(a, tile, gt);
                    tile_box(a, gt, box_s[lane]);
                }
            }
            __syncwarp();
            nvalid = ok_s[0] + ok_s[1] + ok_s[2] + ok_s[3];
            box_g = box_s;
            lt_g = lt_s;
            ok_g = ok_s;
            cshift = __ffs(a.chunk) - 1;  // chunk = 2^cshift
        } else {
            tile_box(a, g, box);
        }
        // stage / round of the ring and (laser, chunk) of the item advance by counting: no
        // 64-bit division per stage
        uint32_t stage = (uint32_t)(step0 % a.stages);
        uint64_t round = step0 / a.stages;
        uint32_t l = (uint32_t)(i0 / a.nchunks);
        uint32_t c = (uint32_t)(i0 % a.nchunks);
        for (uint32_t n = 0; n < count; n++) {
            const uint64_t i = step0 + n;
            if (round > 0) {
                // Every lane observes the consumers' release before its TMA overwrites
                // the stage.
                bool ok = mbar_wait_backoff(smem_addr(&empty_bar[stage]),
                                            (uint32_t)(round - 1) & 1, a.spin_limit);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    if (lane == 0) {
                        atomicAdd(&diag[0], 1ull);
                        *(volatile int *)&abort_flag = 1;
                    }
                    step = i;
                    return false;
                }
            }
            if (*(volatile int *)&abort_flag) {
                step = i;
                return false;
            }
            if (l != cur_l) {  // a new laser: its part of the window starts
                const float4 Lt = lasers[l];
                if constexpr (GROUPED) {
                    __syncwarp();  // every lane is done with the previous laser's terms
                    if (lane < kMaxGroups && ok_g[lane])
                        lt_g[lane] = laser_term(a, box_g[lane], Lt);
                    __syncwarp();
                } else {
                    lt = laser_term(a, box, Lt);
                }
                cur_l = l;
            }
            const uint64_t s0 = (uint64_t)c * a.chunk;
            const uint32_t nrows =
                (uint32_t)(a.S - s0 < (uint64_t)a.chunk ? a.S - s0 : (uint64_t)a.chunk);
            unsigned char *st = stage_base + (size_t)stage * a.stage_bytes;
            float4 *table = reinterpret_cast<float4 *>(st);
            const uint32_t data = smem_addr(st + a.table_bytes);
            const uint32_t fb = smem_addr(&full_bar[stage]);
            if constexpr (GROUPED) {
                // one entry at a time (four per lane): record, then its window
                if (lane == 0) mbar_expect_tx(fb, nrows * nvalid * a.nbox * a.BW * esz);
                __syncwarp();
#pragma unroll 1
                for (uint32_t q = 0; q < kLane; q++) {
                    const uint32_t e = lane + 32 * q, r = e & (a.chunk - 1), gi = e >> cshift;
                    if (r < nrows && gi < kMaxGroups && ok_g[gi]) {
                        const float4 G = spads[s0 + r];
                        float ev[3], ew;
                        const int32_t lo = row_record(a, box_g[gi], G, lt_g[gi], ev, ew);
                        const float ek = sel3(ev[0], ev[1], ev[2], a.kax);
                        table[2 * e] = make_float4(sel3(ev[0], ev[1], ev[2], a.oax0),
                                                   sel3(ev[0], ev[1], ev[2], a.oax1), ew, ew);
                        table[2 * e + 1] = make_float4(-ek, -ek, ew, ew);
                        const int32_t row = (int32_t)(row_base + l * a.S + s0 + r);
                        const uint32_t dst = data + e * a.row_bytes;
                        for (uint32_t b = 0; b < a.nbox; b++)
                            tma_load_2d(dst + b * a.BW * esz, tmap, lo + (int32_t)(b * a.BW),
                                        row, fb);
                    }
                }
            } else {
                // entries lane + 32 q of the stage: row r of the chunk
                int32_t lo[kLane] = {};
#pragma unroll
                for (uint32_t q = 0; q < kLane; q++) {
                    const uint32_t e = lane + 32 * q, r = e;
                    if (r < nrows) {
                        const float4 G = spads[s0 + r];
                        float ev[3], ew;
                        lo[q] = row_record(a, box, G, lt, ev, ew);
                        const float ek = sel3(ev[0], ev[1], ev[2], a.kax);
                        table[2 * e] = make_float4(sel3(ev[0], ev[1], ev[2], a.oax0),
                                                   sel3(ev[0], ev[1], ev[2], a.oax1), ew, ew);
                        table[2 * e + 1] = make_float4(-ek, -ek, ew, ew);
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_expect_tx(fb, nrows * a.nbox * a.BW * esz);
                __syncwarp();
#pragma unroll
                for (uint32_t q = 0; q < kLane; q++) {
                    const uint32_t e = lane + 32 * q, r = e;
                    if (r < nrows) {
                        const int32_t row = (int32_t)(row_base + l * a.S + s0 + r);
                        const uint32_t dst = data + e * a.row_bytes;
                        for (uint32_t b = 0; b < a.nbox; b++)
                            tma_load_2d(dst + b * a.BW * esz, tmap, lo[q] + (int32_t)(b * a.BW),
                                        row, fb);
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(fb);
            if (++stage == a.stages) stage = 0, round++;
            if (++c == a.nchunks) c = 0, l++;
        }
        return true;
    }
    // ---------------- consumers ----------------
    // GROUPED: warp cw of tile grp = (warp - 1) / (wx wy wz) of the group, reading that
    // tile's entries of each stage (records and windows grp x chunk ..)
    uint32_t cw = warp - 1, grp = 0;
    bool live = true;
    unsigned char *tab_base = stage_base;
    uint32_t data_base = pad;  // offset from smem_raw
    if constexpr (GROUPED) {
        const uint32_t twarps = a.warp[0] * a.warp[1] * a.warp[2];
        grp = cw / twarps;
        cw -= grp * twarps;
        void *unused;
        live = group_tile<PairT>(a, out, t0, grp, tile, unused);
        tile_of_block(a, live ? tile : 0u, g);
        tab_base += grp * a.chunk * kRecordBytes;
        data_base += grp * a.chunk * a.row_bytes;
    }
    const uint32_t li[3] = {lane % a.lane[0], (lane / a.lane[0]) % a.lane[1],
                            lane / (a.lane[0] * a.lane[1])};
    const uint32_t wi[3] = {cw % a.warp[0], (cw / a.warp[0]) % a.warp[1],
                            cw / (a.warp[0] * a.warp[1])};
    const uint32_t bx = g.org[0] + wi[0] * a.lane[0] * (a.kax == 0 ? K : 1) + li[0];
    const uint32_t by = g.org[1] + wi[1] * a.lane[1] * (a.kax == 1 ? K : 1) + li[1];
    const uint32_t bz = g.org[2] + wi[2] * a.lane[2] * (a.kax == 2 ? K : 1) + li[2];
    const uint32_t bk = sel3(bx, by, bz, a.kax);
    const uint32_t kstep = sel3(a.lane[0], a.lane[1], a.lane[2], a.kax);
    const float v0 = rel_coord(a, g, a.oax0, sel3(bx, by, bz, a.oax0));
    const float v1 = rel_coord(a, g, a.oax1, sel3(bx, by, bz, a.oax1));
    float2 vk[NP], A[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) {
        vk[i].x = rel_coord(a, g, a.kax, bk + (2 * i) * kstep);
        vk[i].y = rel_coord(a, g, a.kax, bk + (2 * i + 1) * kstep);
    }
    // Planar wall: every row has the same kax coordinate (row_record's arithmetic on the
    // first SPAD), so (v_k - c_k)^2 is formed once per voxel.
    float2 dzsq[PLANAR ? NP : 1];
    if (PLANAR) {
        const float4 G0 = spads[0];
        const float ek = __fmul_rn(sel3(G0.x, G0.y, G0.z, a.kax) -
                                       __fmul_rn(sel3(g.ctr[0], g.ctr[1], g.ctr[2], a.kax),
                                                 sel3(a.h[0], a.h[1], a.h[2], a.kax)),
                                   a.sb);
        const float2 nk = make_float2(-ek, -ek);
#pragma unroll
        for (int i = 0; i < (PLANAR ? NP : 1); i++) {
            const float2 dz = __fadd2_rn(vk[i], nk);
            dzsq[i] = __fmul2_rn(dz, dz);
        }
    }

    PairT acc[NP], comp[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) {
        acc[i].zero();
        comp[i].zero();
    }
    uint32_t cur_l = ~0u;
    uint32_t violations = 0;
    const float2 magic2 = make_float2(kMagic, kMagic);

    uint32_t stage = (uint32_t)(step0 % a.stages);
    uint32_t phase = (uint32_t)(step0 / a.stages) & 1;
    uint32_t l = (uint32_t)(i0 / a.nchunks);
    uint32_t c = (uint32_t)(i0 % a.nchunks);
    for (uint32_t n = 0; n < count; n++) {
        if (l != cur_l) {
            const float4 Lt = lasers[l];
#pragma unroll
            for (int p = 0; p < NP; p++) {
#pragma unroll
                for (int w = 0; w < 2; w++) {
                    const uint32_t kv = bk + (2 * p + w) * kstep;
                    const uint32_t idx[3] = {a.kax == 0 ? kv : bx, a.kax == 1 ? kv : by,
                                             a.kax == 2 ? kv : bz};
                    const float v = laser_leg(a, idx, Lt);
                    if (w == 0)
                        A[p].x = v;
                    else
                        A[p].y = v;
                }
            }
            cur_l = l;
        }
        // Every lane acquires the stage (TMA bytes and the producer's row records).
        bool ok = mbar_wait(smem_addr(&full_bar[stage]), phase, a.spin_limit);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok || *(volatile int *)&abort_flag) {
            if (lane == 0 && !ok) {
                atomicAdd(&diag[0], 1ull);
                *(volatile int *)&abort_flag = 1;
            }
            return false;
        }
        const uint64_t s0 = (uint64_t)c * a.chunk;
        const uint32_t nrows =
            (uint32_t)(a.S - s0 < (uint64_t)a.chunk ? a.S - s0 : (uint64_t)a.chunk);
        const float4 *table =
            reinterpret_cast<const float4 *>(tab_base + (size_t)stage * a.stage_bytes);
        const uint32_t data = data_base + stage * a.stage_bytes + a.table_bytes;

        PairT part[NP];
        if (KAHAN) {
#pragma unroll
            for (int p = 0; p < NP; p++) part[p].zero();
        }
        // ROWS rows per unrolled iteration give the scheduler ROWS x NP independent
        // voxel-pair chains to interleave (one row for complex rows, whose accumulators
        // already double the registers).  Measured on the 256^3 capture: 2 rows 86.7 ms,
        // 4 rows 84.5, 8 rows 80.9, 16 rows 80.4 (the batch kernel: 4 rows best).
        const uint32_t jn = live ? nrows : 0u;  // a tile past the list or volume idles
#pragma unroll(PairT::kCplx ? (PairT::kEsz == 8 ? kC64Rows : kC32Rows) : ROWS)
        for (uint32_t j = 0; j < jn; j++) {
            const float4 r0 = table[2 * j];  // (c_o0, c_o1, ew, ew)
            const float D = row_d(v0, v1, r0.x, r0.y);
            const float2 D2 = make_float2(D, D);
            const float2 ew = make_float2(r0.z, r0.w);
            float2 nk = make_float2(0.0f, 0.0f);
            if (!PLANAR) {
                const float4 r1 = table[2 * j + 1];  // (-c_k, -c_k, ew, ew)
                nk = make_float2(r1.x, r1.y);
            }
            const uint32_t rbase = data + j * a.row_bytes - kMagicBits * esz;
#pragma unroll
            for (int p = 0; p < NP; p++) {
                // laser leg + row constant ahead of the rsqrt: one dependent op after it
                const float2 Ae = __fadd2_rn(A[p], ew);
                float2 q;
                if (PLANAR) {
                    q = __fadd2_rn(D2, dzsq[p]);
                } else {
                    const float2 dz = __fadd2_rn(vk[p], nk);
                    q = __ffma2_rn(dz, dz, D2);
                }
                const float2 r = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
                const float2 y = __ffma2_rn(q, r, Ae);
                const float2 z = __fadd2_rn(y, magic2);
                uint32_t b0 = __float_as_uint(z.x), b1 = __float_as_uint(z.y);
                if (CHECKED) {
                    const uint32_t r0i = b0 - kMagicBits, r1i = b1 - kMagicBits;
                    if (r0i >= a.W) {
                        violations++;
                        b0 = kMagicBits + ((int32_t)r0i < 0 ? 0u : a.W - 1);
                    }
                    if (r1i >= a.W) {
                        violations++;
                        b1 = kMagicBits + ((int32_t)r1i < 0 ? 0u : a.W - 1);
                    }
                }
                const uint32_t p0 = rbase + (b0 << PairT::kShift);
                const uint32_t p1 = rbase + (b1 << PairT::kShift);
                if (KAHAN)
                    part[p].gather2(smem_raw, p0, p1);
                else
                    acc[p].gather2(smem_raw, p0, p1);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&empty_bar[stage]));
        if (KAHAN) {
#pragma unroll
            for (int p = 0; p < NP; p++) acc[p].fold(comp[p], part[p]);
        }
        if (++stage == a.stages) stage = 0, phase ^= 1;
        if (++c == a.nchunks) c = 0, l++;
    }
    if (CHECKED && violations) atomicAdd(&diag[1], (unsigned long long)violations);
    if (KAHAN) {
#pragma unroll
        for (int p = 0; p < NP; p++) acc[p].finish(comp[p]);
    }
    const float scale = a.splits > 1 ? 1.0f : a.out_scale;
    if constexpr (GROUPED) {  // the tile's output base, re-derived rather than held
        if (!live) return true;
        uint32_t sp;
        const uint32_t tw = a.warp[0] * a.warp[1] * a.warp[2];
        group_tile<PairT>(a, out, group_origin(a, sp), (threadIdx.x / 32 - 1) / tw, tile, out);
    }
    const uint64_t tvox = (uint64_t)a.tdim[0] * a.tdim[1] * a.tdim[2];
    const uint64_t part_off = a.splits > 1 ? (uint64_t)split * (a.tile_local ? tvox : a.nvox) : 0;
#pragma unroll
    for (int p = 0; p < NP; p++) {
#pragma unroll
        for (int w = 0; w < 2; w++) {
            const uint32_t kv = bk + (2 * p + w) * kstep;
            const uint32_t x = a.kax == 0 ? kv : bx, y = a.kax == 1 ? kv : by,
                           z = a.kax == 2 ? kv : bz;
            if (x < a.n[0] && y < a.n[1] && z < a.n[2]) {
                const uint64_t idx =
                    a.tile_local
                        ? ((uint64_t)(x - g.org[0]) * a.tdim[1] + (y - g.org[1])) * a.tdim[2] +
                              (z - g.org[2])
                        : ((uint64_t)x * a.n[1] + y) * a.n[2] + z;
                acc[p].store(out, part_off + idx, w, scale);
            }
        }
    }
    return true;
}

// ---- lasers x SPADs captures with factored legs ------------------------------------
// Bin of voxel v for pair (l, s): round(A(v, l) + B(v, s)) with
//   A = sa |v - l| + (lw - t0) / dT - lo_L(l),   B = sb |v - s| + cw / dT - lo_S(s),
// where lo = lo_L + lo_S is the pair's staged window start (both parts aligned, so their
// sum is).  A stage holds the rows of cl = chunk / kFactS lasers x kFactS SPADs; its table
// carries one record per laser and per SPAD (position relative to the tile centre in bin
// units, constant).  A consumer thread keeps B of its 8 voxels for the current SPAD block
// in registers (formed when the block changes, reused across every laser of the capture)
// and forms A once per laser, so an update costs two packed adds, the address and the
// gather instead of a square root: 1 / kFactS reciprocal square roots per update.
template <typename HT, bool CHECKED>
__device__ __forceinline__ bool fact_unit(const FastArgs &a, const CUtensorMap *tmap,
                                          const float4 *__restrict__ spads,
                                          const float4 *__restrict__ lasers, void *out,
                                          unsigned long long *diag, uint32_t tile,
                                          uint32_t split, uint32_t row_base, uint64_t &step,
                                          const PipeShared &sh) {
    using PairT = Pair<HT>;
    constexpr uint32_t esz = PairT::kEsz;
    constexpr int K = 8, NP = K / 2;
    unsigned char *const smem_raw = sh.smem_raw;
    unsigned char *const stage_base = sh.stage_base;
    const uint32_t pad = sh.pad;
    uint64_t *const full_bar = sh.full_bar;
    uint64_t *const empty_bar = sh.empty_bar;
    int &abort_flag = *sh.abort_flag;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t cl = a.chunk / kFactS;  // lasers per stage
    // items: (SPAD block, laser group), SPAD block slowest
    const uint64_t items = fast_items(a);
    const uint64_t i0 = items * split / a.splits, i1 = items * (split + 1) / a.splits;
    const uint64_t step0 = step;
    step += i1 - i0;
    const uint32_t count = (uint32_t)(i1 - i0);

    TileGeo g;
    tile_of_block(a, tile, g);

    if (warp == 0) {
        // ---------------- producer ----------------
        uint32_t stage = (uint32_t)(step0 % a.stages);
        uint64_t round = step0 / a.stages;
        uint32_t sb = (uint32_t)(i0 / a.nchunks), lg = (uint32_t)(i0 % a.nchunks);
        const int32_t al = (int32_t)a.align;
        for (uint32_t n = 0; n < count; n++) {
            const uint64_t i = step0 + n;
            if (round > 0) {
                bool ok = mbar_wait_backoff(smem_addr(&empty_bar[stage]),
                                            (uint32_t)(round - 1) & 1, a.spin_limit);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) {
                    if (lane == 0) {
                        atomicAdd(&diag[0], 1ull);
                        *(volatile int *)&abort_flag = 1;
                    }
                    step = i;
                    return false;
                }
            }
            if (*(volatile int *)&abort_flag) {
                step = i;
                return false;
            }
            const uint32_t l0 = lg * cl;
            const uint32_t ncl = (uint32_t)(a.L - l0 < (uint64_t)cl ? a.L - l0 : (uint64_t)cl);
            const uint32_t s0 = sb * kFactS;
            unsigned char *st = stage_base + (size_t)stage * a.stage_bytes;
            float4 *table = reinterpret_cast<float4 *>(st);
            const uint32_t data = smem_addr(st + a.table_bytes);
            const uint32_t fb = smem_addr(&full_bar[stage]);
            // laser records in lanes < ncl, SPAD records in lanes < kFactS
            int32_t lo_l = 0, lo_s = 0;
            if (lane < ncl) {
                const float4 Lt = lasers[l0 + lane];
                float dmin, dmax;
                box_bounds(a, g, Lt.x, Lt.y, Lt.z, dmin, dmax);
                lo_l = (int32_t)floorf(__fmaf_rn(a.sa, dmin, Lt.w) - kMargin);
                lo_l = align_down(lo_l, al);
                const float lp[3] = {Lt.x, Lt.y, Lt.z};
                float e[3];
#pragma unroll
                for (int k = 0; k < 3; k++)
                    e[k] = __fmul_rn(lp[k] - __fmul_rn(g.ctr[k], a.h[k]), a.sa);
                table[lane] = make_float4(sel3(e[0], e[1], e[2], a.oax0),
                                          sel3(e[0], e[1], e[2], a.oax1),
                                          sel3(e[0], e[1], e[2], a.kax), Lt.w - (float)lo_l);
            }
            if (lane < kFactS) {
                const float4 G = spads[s0 + lane];
                float dmin, dmax;
                box_bounds(a, g, G.x, G.y, G.z, dmin, dmax);
                lo_s = (int32_t)floorf(__fmaf_rn(a.sb, dmin, G.w));
                lo_s = align_down(lo_s, al);
                const float gp[3] = {G.x, G.y, G.z};
                float e[3];
#pragma unroll
                for (int k = 0; k < 3; k++)
                    e[k] = __fmul_rn(gp[k] - __fmul_rn(g.ctr[k], a.h[k]), a.sb);
                table[cl + lane] = make_float4(sel3(e[0], e[1], e[2], a.oax0),
                                               sel3(e[0], e[1], e[2], a.oax1),
                                               sel3(e[0], e[1], e[2], a.kax), G.w - (float)lo_s);
            }
            const uint32_t nrows = ncl * kFactS;
            __syncwarp();
            if (lane == 0) mbar_expect_tx(fb, nrows * a.nbox * a.BW * esz);
            __syncwarp();
#pragma unroll
            for (uint32_t q = 0; q < kMaxChunk / 32; q++) {
                const uint32_t r = lane + 32 * q;  // row r = laser r / kFactS, SPAD r % kFactS
                const int32_t x = __shfl_sync(0xffffffffu, lo_l, (r / kFactS) & 31) +
                                  __shfl_sync(0xffffffffu, lo_s, r % kFactS);
                if (r < nrows) {
                    const int32_t row = (int32_t)(row_base + (uint64_t)(l0 + r / kFactS) * a.S +
                                                  s0 + r % kFactS);
                    const uint32_t dst = data + r * a.row_bytes;
                    for (uint32_t b = 0; b < a.nbox; b++)
                        tma_load_2d(dst + b * a.BW * esz, tmap, x + (int32_t)(b * a.BW), row, fb);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(fb);
            if (++stage == a.stages) stage = 0, round++;
            if (++lg == a.nchunks) lg = 0, sb++;
        }
        return true;
    }
    // ---------------- consumers ----------------
    const uint32_t cw = warp - 1;
    const uint32_t li[3] = {lane % a.lane[0], (lane / a.lane[0]) % a.lane[1],
                            lane / (a.lane[0] * a.lane[1])};
    const uint32_t wi[3] = {cw % a.warp[0], (cw / a.warp[0]) % a.warp[1],
                            cw / (a.warp[0] * a.warp[1])};
    const uint32_t bx = g.org[0] + wi[0] * a.lane[0] * (a.kax == 0 ? K : 1) + li[0];
    const uint32_t by = g.org[1] + wi[1] * a.lane[1] * (a.kax == 1 ? K : 1) + li[1];
    const uint32_t bz = g.org[2] + wi[2] * a.lane[2] * (a.kax == 2 ? K : 1) + li[2];
    const uint32_t bk = sel3(bx, by, bz, a.kax);
    const uint32_t kstep = sel3(a.lane[0], a.lane[1], a.lane[2], a.kax);
    const float v0 = rel_coord(a, g, a.oax0, sel3(bx, by, bz, a.oax0));
    const float v1 = rel_coord(a, g, a.oax1, sel3(bx, by, bz, a.oax1));
    float2 vk[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) {
        vk[i].x = rel_coord(a, g, a.kax, bk + (2 * i) * kstep);
        vk[i].y = rel_coord(a, g, a.kax, bk + (2 * i + 1) * kstep);
    }
    // leg of the 8 voxels to the point of record rec: q * rsqrt(q) + rec.w
    auto legs = [&](const float4 rec, float2 (&out)[NP]) {
        const float D = row_d(v0, v1, rec.x, rec.y);
        const float2 D2 = make_float2(D, D), nk = make_float2(-rec.z, -rec.z);
        const float2 c2 = make_float2(rec.w, rec.w);
#pragma unroll
        for (int p = 0; p < NP; p++) {
            const float2 dz = __fadd2_rn(vk[p], nk);
            const float2 q = __ffma2_rn(dz, dz, D2);
            const float2 r = make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y));
            out[p] = __ffma2_rn(q, r, c2);
        }
    };

    PairT acc[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) acc[i].zero();
    float2 B[kFactS][NP];
    uint32_t cur_sb = ~0u;
    uint32_t violations = 0;
    const float2 magic2 = make_float2(kMagic, kMagic);

    uint32_t stage = (uint32_t)(step0 % a.stages);
    uint32_t phase = (uint32_t)(step0 / a.stages) & 1;
    uint32_t sb = (uint32_t)(i0 / a.nchunks), lg = (uint32_t)(i0 % a.nchunks);
    for (uint32_t n = 0; n < count; n++) {
        bool ok = mbar_wait(smem_addr(&full_bar[stage]), phase, a.spin_limit);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok || *(volatile int *)&abort_flag) {
            if (lane == 0 && !ok) {
                atomicAdd(&diag[0], 1ull);
                *(volatile int *)&abort_flag = 1;
            }
            return false;
        }
        const uint32_t l0 = lg * cl;
        const uint32_t ncl = (uint32_t)(a.L - l0 < (uint64_t)cl ? a.L - l0 : (uint64_t)cl);
        const float4 *table =
            reinterpret_cast<const float4 *>(stage_base + (size_t)stage * a.stage_bytes);
        const uint32_t data = pad + stage * a.stage_bytes + a.table_bytes;  // offset from smem_raw
        if (sb != cur_sb) {
#pragma unroll
            for (uint32_t si = 0; si < kFactS; si++) legs(table[cl + si], B[si]);
            cur_sb = sb;
        }
        for (uint32_t lj = 0; lj < ncl; lj++) {
            float2 A[NP];
            legs(table[lj], A);
#pragma unroll
            for (uint32_t si = 0; si < kFactS; si++) {
                const uint32_t rbase = data + (lj * kFactS + si) * a.row_bytes - kMagicBits * esz;
#pragma unroll
                for (int p = 0; p < NP; p++) {
                    const float2 z = __fadd2_rn(__fadd2_rn(A[p], B[si][p]), magic2);
                    uint32_t b0 = __float_as_uint(z.x), b1 = __float_as_uint(z.y);
                    if (CHECKED) {
                        const uint32_t r0i = b0 - kMagicBits, r1i = b1 - kMagicBits;
                        if (r0i >= a.W) {
                            violations++;
                            b0 = kMagicBits + ((int32_t)r0i < 0 ? 0u : a.W - 1);
                        }
                        if (r1i >= a.W) {
                            violations++;
                            b1 = kMagicBits + ((int32_t)r1i < 0 ? 0u : a.W - 1);
                        }
                    }
                    acc[p].gather2(smem_raw, rbase + (b0 << PairT::kShift),
                                   rbase + (b1 << PairT::kShift));
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&empty_bar[stage]));
        if (++stage == a.stages) stage = 0, phase ^= 1;
        if (++lg == a.nchunks) lg = 0, sb++;
    }
    if (CHECKED && violations) atomicAdd(&diag[1], (unsigned long long)violations);
    const float scale = a.splits > 1 ? 1.0f : a.out_scale;
    const uint64_t tvox = (uint64_t)a.tdim[0] * a.tdim[1] * a.tdim[2];
    const uint64_t part_off = a.splits > 1 ? (uint64_t)split * (a.tile_local ? tvox : a.nvox) : 0;
#pragma unroll
    for (int p = 0; p < NP; p++) {
#pragma unroll
        for (int w = 0; w < 2; w++) {
            const uint32_t kv = bk + (2 * p + w) * kstep;
            const uint32_t x = a.kax == 0 ? kv : bx, y = a.kax == 1 ? kv : by,
                           z = a.kax == 2 ? kv : bz;
            if (x < a.n[0] && y < a.n[1] && z < a.n[2]) {
                const uint64_t idx =
                    a.tile_local
                        ? ((uint64_t)(x - g.org[0]) * a.tdim[1] + (y - g.org[1])) * a.tdim[2] +
                              (z - g.org[2])
                        : ((uint64_t)x * a.n[1] + y) * a.n[2] + z;
                acc[p].store(out, part_off + idx, w, scale);
            }
        }
    }
    return true;
}

// Producer lane 0 before the CTA exits: every stage the CTA filled must have landed
// (bounded waits; the last `stages` steps are the only ones that can be in flight).
__device__ __forceinline__ void pipeline_drain(uint32_t stages, uint64_t issued,
                                               uint64_t *full_bar, unsigned long long *diag,
                                               uint32_t spin_limit) {
    if (threadIdx.x != 0) return;
    const uint64_t first = issued > stages ? issued - stages : 0;
    for (uint64_t i = first; i < issued; i++) {
        const uint32_t stage = (uint32_t)(i % stages);
        if (!mbar_wait(smem_addr(&full_bar[stage]), (uint32_t)(i / stages) & 1, spin_limit))
            atomicAdd(&diag[0], 1ull);
    }
}

// The CTA's voxel tile, pair split and output base; false when a tile-list CTA has no
// tile (it exits before any barrier is initialised).
template <typename PairT>
__device__ __forceinline__ bool plan_block(const FastArgs &a, void *out, uint32_t &tile,
                                           uint32_t &split, void *&dst) {
    const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    tile = (uint32_t)(blockIdx.x % ntiles);
    split = (uint32_t)(blockIdx.x / ntiles);
    dst = out;
    if (a.tile_list) {
        split = blockIdx.x % a.splits;
        return group_tile<PairT>(a, out, blockIdx.x / a.splits, 0, tile, dst);
    }
    return true;
}

// Grouped launches: the CTA's first tile (full-volume launch) or list slot (tile-list
// launch) and pair split; false when none of its group's tiles exists.
template <typename PairT>
__device__ __forceinline__ bool plan_group(const FastArgs &a, void *out, uint32_t &t0,
                                           uint32_t &split) {
    t0 = group_origin(a, split);
    bool any = false;
    for (uint32_t g = 0; g < a.groups; g++) {
        uint32_t tile;
        void *dst;
        any = any || group_tile<PairT>(a, out, t0, g, tile, dst);
    }
    return any;
}

// Stage ring (128-byte aligned) and its mbarriers; ends with a CTA barrier.
__device__ __forceinline__ void pipeline_init(PipeShared &sh, unsigned char *smem_raw,
                                              uint64_t *full_bar, uint64_t *empty_bar,
                                              int *abort_flag, uint32_t stages) {
    sh.smem_raw = smem_raw;
    sh.pad = (128u - (smem_addr(smem_raw) & 127u)) & 127u;
    sh.stage_base = smem_raw + sh.pad;
    sh.full_bar = full_bar;
    sh.empty_bar = empty_bar;
    sh.abort_flag = abort_flag;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < stages; s++) {
            mbar_init(smem_addr(&full_bar[s]), 1);
            mbar_init(smem_addr(&empty_bar[s]), blockDim.x / 32 - 1);
        }
        *abort_flag = 0;
        mbar_fence_init();
    }
    __syncthreads();
}

// CTAS: resident CTAs per SM the variant is compiled for (its register budget).  GROUPED:
// several tiles per CTA (fast_unit).
template <typename HT, int K, bool KAHAN, bool CHECKED, bool PLANAR, int CTAS, bool GROUPED>
__global__ void __launch_bounds__(288, CTAS)
    bp_fast_kernel(const __grid_constant__ CUtensorMap tmap, const float4 *__restrict__ spads,
                   const float4 *__restrict__ lasers, void *__restrict__ out,
                   unsigned long long *__restrict__ diag, const FastArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[8];
    __shared__ __align__(8) uint64_t empty_bar[8];
    __shared__ int abort_flag;
    uint32_t t0, split;
    void *dst = out;
    if constexpr (GROUPED) {
        if (!plan_group<Pair<HT>>(a, out, t0, split)) return;
    } else {
        if (!plan_block<Pair<HT>>(a, out, t0, split, dst)) return;
    }
    PipeShared sh;
    pipeline_init(sh, smem_raw, full_bar, empty_bar, &abort_flag, a.stages);
    uint64_t step = 0;
    fast_unit<HT, K, KAHAN, CHECKED, PLANAR, kPlanRows, GROUPED>(a, &tmap, spads, lasers, dst,
                                                                 diag, t0, split, 0, step, sh);
    pipeline_drain(a.stages, step, full_bar, diag, a.spin_limit);
}

// Lasers x SPADs captures with factored legs (fact_unit): same launch shape as the plan
// kernel with K = 8.
template <typename HT, bool CHECKED>
__global__ void __launch_bounds__(288, kFactCtas)
    bp_fact_kernel(const __grid_constant__ CUtensorMap tmap, const float4 *__restrict__ spads,
                   const float4 *__restrict__ lasers, void *__restrict__ out,
                   unsigned long long *__restrict__ diag, const FastArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[8];
    __shared__ __align__(8) uint64_t empty_bar[8];
    __shared__ int abort_flag;
    uint32_t tile, split;
    void *dst;
    if (!plan_block<Pair<HT>>(a, out, tile, split, dst)) return;
    PipeShared sh;
    pipeline_init(sh, smem_raw, full_bar, empty_bar, &abort_flag, a.stages);
    uint64_t step = 0;
    fact_unit<HT, CHECKED>(a, &tmap, spads, lasers, dst, diag, tile, split, 0, step, sh);
    pipeline_drain(a.stages, step, full_bar, diag, a.spin_limit);
}

// out[v] = scale * sum_s partial[s][v], in split order (optionally Kahan).
template <bool COMPLEX, bool KAHAN>
__global__ void reduce_splits_kernel(const float *__restrict__ partial, float *__restrict__ out,
                                     uint64_t nvox, uint32_t splits, float scale) {
    constexpr int C = COMPLEX ? 2 : 1;
    const uint64_t n = nvox * C;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float s = 0.0f, c = 0.0f;
        for (uint32_t k = 0; k < splits; k++) {
            const float x = partial[(uint64_t)k * n + i];
            if (KAHAN)
                kahan_add(s, c, x);
            else
                s += x;
        }
        if (KAHAN) s -= c;
        out[i] = s * scale;
    }
}

// Tile-list form of reduce_splits_kernel: slot s < *count holds tile list[s]; the
// partial sums of its splits (slot-major, then split, then tile-local voxel) are added in split order
// with the same arithmetic, so a voxel equals the full-volume reduction bit for bit.
template <bool COMPLEX, bool KAHAN>
__global__ void reduce_tiles_kernel(const float *__restrict__ partial,
                                    const uint32_t *__restrict__ list,
                                    const uint32_t *__restrict__ count, uint32_t max_tiles,
                                    const FastArgs a, float *__restrict__ out) {
    constexpr int C = COMPLEX ? 2 : 1;
    const uint64_t tvox = (uint64_t)a.tdim[0] * a.tdim[1] * a.tdim[2];
    const uint64_t n = (uint64_t)max_tiles * tvox * C;
    const uint32_t cnt = *count;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t slot = i / (tvox * C);
        if (slot >= cnt) break;
        const uint64_t r = i - slot * tvox * C;
        const uint64_t local = r / C;
        const uint32_t c = (uint32_t)(r - local * C);
        const uint32_t tile = list[slot];
        if (tile >= (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2]) continue;  // skipped entry
        const uint32_t tz = tile % a.tiles[2], tx = (tile / a.tiles[2]) % a.tiles[0],
                       ty = tile / (a.tiles[2] * a.tiles[0]);
        const uint32_t lz = (uint32_t)(local % a.tdim[2]),
                       ly = (uint32_t)((local / a.tdim[2]) % a.tdim[1]),
                       lx = (uint32_t)(local / ((uint64_t)a.tdim[2] * a.tdim[1]));
        const uint32_t x = tx * a.tdim[0] + lx, y = ty * a.tdim[1] + ly, z = tz * a.tdim[2] + lz;
        if (x >= a.n[0] || y >= a.n[1] || z >= a.n[2]) continue;
        float s = 0.0f, cmp = 0.0f;
        for (uint32_t k = 0; k < a.splits; k++) {
            const float v = partial[((slot * a.splits + k) * tvox + local) * C + c];
            if (KAHAN)
                kahan_add(s, cmp, v);
            else
                s += v;
        }
        if (KAHAN) s -= cmp;
        out[(((uint64_t)x * a.n[1] + y) * a.n[2] + z) * C + c] = s * a.out_scale;
    }
}

// bins[i * P + p] with the fast kernel's arithmetic for voxel ids[i] and pair p.
__global__ void bp_fast_bins_kernel(const float4 *__restrict__ spads,
                                    const float4 *__restrict__ lasers,
                                    const int64_t *__restrict__ ids, int64_t n,
                                    int32_t *__restrict__ bins, const FastArgs a) {
    const uint64_t P = a.L * a.S;
    const uint64_t total = (uint64_t)n * P;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < total;
         w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = w / P, p = w % P;
        const int64_t id = ids[i];
        const uint32_t idx[3] = {(uint32_t)(id / ((int64_t)a.n[1] * a.n[2])),
                                 (uint32_t)((id / a.n[2]) % a.n[1]), (uint32_t)(id % a.n[2])};
        const uint32_t tile =
            ((idx[1] / a.tdim[1]) * a.tiles[0] + idx[0] / a.tdim[0]) * a.tiles[2] +
            idx[2] / a.tdim[2];
        TileGeo g;
        tile_of_block(a, tile, g);
        const uint64_t l = p / a.S, s = p % a.S;
        const float4 Lt = lasers[l];
        if (a.fact) {  // fact_unit's arithmetic: window start and legs split per laser / SPAD
            const float4 G = spads[s];
            const int32_t al = (int32_t)a.align;
            float lmin, lmax, dmin, dmax;
            box_bounds(a, g, Lt.x, Lt.y, Lt.z, lmin, lmax);
            box_bounds(a, g, G.x, G.y, G.z, dmin, dmax);
            int32_t lo_l = (int32_t)floorf(__fmaf_rn(a.sa, lmin, Lt.w) - kMargin);
            lo_l = align_down(lo_l, al);
            int32_t lo_s = (int32_t)floorf(__fmaf_rn(a.sb, dmin, G.w));
            lo_s = align_down(lo_s, al);
            const float v[3] = {rel_coord(a, g, 0, idx[0]), rel_coord(a, g, 1, idx[1]),
                                rel_coord(a, g, 2, idx[2])};
            auto leg = [&](float4 P4, float sc, float c) {
                const float pp[3] = {P4.x, P4.y, P4.z};
                float e3[3];
                for (int k = 0; k < 3; k++) e3[k] = __fmul_rn(pp[k] - __fmul_rn(g.ctr[k], a.h[k]), sc);
                const float D = row_d(sel3(v[0], v[1], v[2], a.oax0), sel3(v[0], v[1], v[2], a.oax1),
                                      sel3(e3[0], e3[1], e3[2], a.oax0),
                                      sel3(e3[0], e3[1], e3[2], a.oax1));
                const float dz = __fadd_rn(sel3(v[0], v[1], v[2], a.kax), -sel3(e3[0], e3[1], e3[2], a.kax));
                const float q = __fmaf_rn(dz, dz, D);
                return __fmaf_rn(q, rsqrt_approx(q), c);
            };
            const float A = leg(Lt, a.sa, Lt.w - (float)lo_l);
            const float B = leg(G, a.sb, G.w - (float)lo_s);
            const int32_t rel =
                (int32_t)(__float_as_uint(__fadd_rn(__fadd_rn(A, B), kMagic)) - kMagicBits);
            const int32_t b = lo_l + lo_s + rel;
            bins[w] = (b >= 0 && b < (int32_t)a.T) ? b : -1;
            continue;
        }
        float e[3], ew;
        TileBox tb;
        tile_box(a, g, tb);
        const int32_t lo = row_record(a, tb, spads[s], laser_term(a, tb, Lt), e, ew);
        const float A = laser_leg(a, idx, Lt);
        const float v0 = rel_coord(a, g, a.oax0, sel3(idx[0], idx[1], idx[2], a.oax0));
        const float v1 = rel_coord(a, g, a.oax1, sel3(idx[0], idx[1], idx[2], a.oax1));
        const float vk = rel_coord(a, g, a.kax, sel3(idx[0], idx[1], idx[2], a.kax));
        const float D = row_d(v0, v1, sel3(e[0], e[1], e[2], a.oax0), sel3(e[0], e[1], e[2], a.oax1));
        const float ek = sel3(e[0], e[1], e[2], a.kax);
        const int32_t rel = (int32_t)(window_bits(vk, D, A, ek, ew, a.planar != 0) - kMagicBits);
        const int32_t b = lo + rel;
        bins[w] = (b >= 0 && b < (int32_t)a.T) ? b : -1;
    }
}

// Failure-path probe: one warp waits (bounded) on an mbarrier that nothing arrives on,
// through the same wait helper the pipeline uses, and records whether it gave up.
__global__ void wait_timeout_probe_kernel(uint32_t limit, unsigned long long *out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_addr(&bar), 1);
        mbar_fence_init();
    }
    __syncwarp();
    bool ok = mbar_wait(smem_addr(&bar), 0, limit);
    ok = __all_sync(0xffffffffu, ok);
    if (threadIdx.x == 0) out[0] = ok ? 0ull : 1ull;
}

// ---- FP64 tables of the FAST kernels, built on the GPU --------------------------------
// SPAD entry s: (frame position relative to the volume origin, cw / dT) -- (cw + lw) / dT
// when confocal; laser entry l: (frame position, lw / dT - t0 / dT).  The pair precompute
// of the reference keeps its wall legs in double (backproject.hpp:356-418); these are the
// values the kernels' FP32 arithmetic starts from, formed in FP64 with every operation
// rounded separately (no contraction) in a fixed order.
struct TableArgs {
    double u[3][3];  // orthonormal frame rows of the voxel basis
    double zero[3];
    double dT, t0;
    uint64_t L, S;
    int confocal;
    uint32_t kax;  // voxel-line axis of the tile preset (planar-wall test)
};

__device__ __forceinline__ void frame_fp64(const TableArgs &t, const float *pt, double o[3]) {
    const double d0 = __dsub_rn((double)pt[0], t.zero[0]);
    const double d1 = __dsub_rn((double)pt[1], t.zero[1]);
    const double d2 = __dsub_rn((double)pt[2], t.zero[2]);
    for (int r = 0; r < 3; r++)
        o[r] = __dadd_rn(__dadd_rn(__dmul_rn(t.u[r][0], d0), __dmul_rn(t.u[r][1], d1)),
                         __dmul_rn(t.u[r][2], d2));
}

__device__ __forceinline__ bool same_point(const float *a, const float *b) {
    return __float_as_uint(a[0]) == __float_as_uint(b[0]) &&
           __float_as_uint(a[1]) == __float_as_uint(b[1]) &&
           __float_as_uint(a[2]) == __float_as_uint(b[2]);
}

// Tables (S SPAD entries, then L laser entries) from a device pair list in the order
// p = l * S + s (or confocal), with three checks counted in diag: diag[0] pairs that
// break that order, diag[1] non-finite pair values, diag[2] SPADs whose FP32 frame
// coordinate along kax differs from SPAD 0's (0 = planar wall for that axis).
__global__ void tables_fp64_kernel(const bpgb_pair *__restrict__ pairs, const TableArgs t,
                                   float4 *__restrict__ tab, unsigned long long *__restrict__ diag) {
    __shared__ float g0k;  // SPAD 0's kax coordinate, formed once per block
    if (threadIdx.x == 0) {
        double g0[3];
        frame_fp64(t, pairs[0].camera_point, g0);
        g0k = (float)g0[t.kax];
    }
    __syncthreads();
    const uint64_t P = t.L * t.S;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const bpgb_pair pr = pairs[p];
        const uint64_t l = p / t.S, s = p % t.S;
        const float *f = reinterpret_cast<const float *>(&pr);
        bool finite = true;
        for (int k = 0; k < 8; k++) finite = finite && isfinite(f[k]);
        if (!finite) atomicAdd(&diag[1], 1ull);
        bool ok;
        if (t.confocal) {
            ok = same_point(pr.laser_point, pr.camera_point) &&
                 __float_as_uint(pr.laser_wall) == __float_as_uint(pr.camera_wall);
        } else {
            const bpgb_pair &head = pairs[l * t.S];
            const bpgb_pair &col = pairs[s];
            ok = same_point(pr.laser_point, head.laser_point) &&
                 __float_as_uint(pr.laser_wall) == __float_as_uint(head.laser_wall) &&
                 same_point(pr.camera_point, col.camera_point) &&
                 __float_as_uint(pr.camera_wall) == __float_as_uint(col.camera_wall);
        }
        if (!ok) atomicAdd(&diag[0], 1ull);
        if (l == 0) {
            double g[3];
            frame_fp64(t, pr.camera_point, g);
            const double cs = t.confocal
                                  ? __ddiv_rn(__dadd_rn((double)pr.camera_wall, (double)pr.laser_wall), t.dT)
                                  : __ddiv_rn((double)pr.camera_wall, t.dT);
            tab[s] = make_float4((float)g[0], (float)g[1], (float)g[2], (float)cs);
            if (__float_as_uint((float)g[t.kax]) != __float_as_uint(g0k)) atomicAdd(&diag[2], 1ull);
        }
        if (s == 0) {
            double g[3] = {0.0, 0.0, 0.0};
            double c = __ddiv_rn(-t.t0, t.dT);
            if (!t.confocal) {
                frame_fp64(t, pr.laser_point, g);
                c = __dadd_rn(c, __ddiv_rn((double)pr.laser_wall, t.dT));
            }
            tab[t.S + l] = make_float4((float)g[0], (float)g[1], (float)g[2], (float)c);
        }
    }
}

// Queues tables_fp64_kernel for L lasers x S SPADs (L = 1 when confocal) on stream s;
// diag[0..2] must be zero beforehand.
int launch_tables(const bpgb_pair *d_pairs, const Volume &vol, const double u[3][3], double dT,
                  double t0, uint64_t L, uint64_t S, bool confocal, uint32_t kax, float4 *d_tab,
                  unsigned long long *d_diag, int sms, cudaStream_t s) {
    TableArgs ta{};
    for (int r = 0; r < 3; r++)
        for (int k = 0; k < 3; k++) ta.u[r][k] = u[r][k];
    for (int k = 0; k < 3; k++) ta.zero[k] = (double)vol.zero[k];
    ta.dT = dT;
    ta.t0 = t0;
    ta.L = L;
    ta.S = S;
    ta.confocal = confocal ? 1 : 0;
    ta.kax = kax;
    const uint64_t P = L * S;
    const unsigned blocks = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((P + 255) / 256, (uint64_t)std::max(sms, 1) * 16));
    tables_fp64_kernel<<<blocks, 256, 0, s>>>(d_pairs, ta, d_tab, d_diag);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

EncodeTiledFn encode_fn() { return tensor_map_encoder(); }

uint32_t dtype_bytes(int dt) {
    switch (dt) {
        case BPGB_DTYPE_F32: return 4;
        case BPGB_DTYPE_F16:
        case BPGB_DTYPE_BF16: return 2;
        case BPGB_DTYPE_C64: return 8;
        case BPGB_DTYPE_C32: return 4;
    }
    return 0;
}

CUtensorMapDataType tma_type(int dt) {
    switch (dt) {
        case BPGB_DTYPE_F16: return CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
        case BPGB_DTYPE_BF16: return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
        case BPGB_DTYPE_C64: return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
        case BPGB_DTYPE_C32: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;  // one (re, im) FP16 pair
        default: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    }
}

int encode_rows(CUtensorMap *map, int dtype, const void *d_H, uint32_t T, uint64_t P,
                uint32_t pitch, uint32_t box) {
    const uint32_t esz = dtype_bytes(dtype);
    const cuuint64_t dims[2] = {T, P};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * esz};
    const cuuint32_t boxd[2] = {box, 1};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(map, tma_type(dtype), 2, const_cast<void *>(d_H), dims, strides, boxd,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(BPGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return BPGB_OK;
}

// Tile presets: {lx, ly, lz, k, wx, wy, wz, kaxis, chunk, stages}.  The voxel line of a
// thread runs along `kaxis`; lanes cover the other two axes.
const FastConfig kPresets[] = {
    {8, 1, 4, 8, 2, 1, 4, 1, 64, 4},  // 16 x 8 x 16, lanes over x-z, lines along y (depth)
    {8, 4, 1, 8, 2, 2, 2, 2, 64, 4},  // 16 x 8 x 16, lanes over x-y, lines along z
    {4, 1, 8, 8, 4, 1, 2, 1, 64, 4},  // 16 x 8 x 16, 4 x 8 lane blocks over x-z
    {8, 1, 4, 8, 2, 2, 2, 1, 64, 4},  // 16 x 16 x 8
    {8, 1, 4, 8, 4, 1, 2, 1, 64, 4},  // 32 x 8 x 8
    {4, 1, 8, 8, 2, 1, 4, 1, 64, 4},  // 8 x 8 x 32
    {8, 1, 4, 8, 1, 2, 4, 1, 64, 4},  // 8 x 16 x 16
    {8, 1, 4, 16, 2, 1, 4, 1, 64, 4}, // 16 x 16 x 16, 16 voxels per thread
    {8, 1, 4, 16, 1, 1, 8, 1, 64, 4}, // 8 x 16 x 32, 16 voxels per thread
    {4, 1, 8, 16, 2, 1, 4, 1, 64, 4}, // 8 x 16 x 32, 4 x 8 lane blocks
    // small tiles for block-sparse passes (2 or 4 consumer warps per CTA)
    {8, 1, 4, 8, 1, 1, 2, 1, 64, 4},  // 8 x 8 x 8
    {8, 1, 4, 8, 1, 1, 4, 1, 64, 4},  // 8 x 8 x 16
    {8, 1, 4, 8, 2, 1, 2, 1, 64, 4},  // 16 x 8 x 8
    // 8 x 8 x 8 tiles, four per CTA (2 consumer warps each, one producer and stage ring)
    {8, 1, 4, 8, 1, 1, 2, 1, 32, 2, 4},
};

// wide: a preset with 8 consumer warps per CTA (three CTAs per SM unless
// Kahan-compensated); grouped: several tiles per CTA, built for real rows with plain sums
template <typename HT, int K, bool PLANAR>
void *kernel_ptr(bool kahan, bool checked, bool wide, bool grouped) {
    if (grouped) {
        if constexpr (K != 8 || Pair<HT>::kCplx) {
            return nullptr;
        } else {
            if (kahan || !wide) return nullptr;
            return checked ? (void *)bp_fast_kernel<HT, K, false, true, PLANAR, 3, true>
                           : (void *)bp_fast_kernel<HT, K, false, false, PLANAR, 3, true>;
        }
    }
    if (kahan)
        return checked ? (void *)bp_fast_kernel<HT, K, true, true, PLANAR, 2, false>
                       : (void *)bp_fast_kernel<HT, K, true, false, PLANAR, 2, false>;
    if (wide)
        return checked ? (void *)bp_fast_kernel<HT, K, false, true, PLANAR, 3, false>
                       : (void *)bp_fast_kernel<HT, K, false, false, PLANAR, 3, false>;
    return checked ? (void *)bp_fast_kernel<HT, K, false, true, PLANAR, 2, false>
                   : (void *)bp_fast_kernel<HT, K, false, false, PLANAR, 2, false>;
}

template <typename HT>
void *kernel_ptr8(bool kahan, bool checked, bool planar, bool wide, bool grouped) {
    return planar ? kernel_ptr<HT, 8, true>(kahan, checked, wide, grouped)
                  : kernel_ptr<HT, 8, false>(kahan, checked, wide, grouped);
}

// Variants built: K = 8 for every row type, accumulation, check mode and wall shape, in
// the 72-register (8-warp presets, plain sums) and 96-register builds, plus the grouped
// form (several tiles per CTA) for real rows with plain sums; K = 16 (one CTA per SM, 16
// chains per thread) for FP32 rows with plain sums.
void *select_kernel(int dtype, bool kahan, bool checked, uint32_t k, bool planar, bool wide,
                    bool grouped = false) {
    if (k == 16) {
        if (dtype != BPGB_DTYPE_F32 || kahan || grouped) return nullptr;
        return checked ? (void *)bp_fast_kernel<float, 16, false, true, false, 1, false>
                       : (void *)bp_fast_kernel<float, 16, false, false, false, 1, false>;
    }
    switch (dtype) {
        case BPGB_DTYPE_F16: return kernel_ptr8<__half>(kahan, checked, planar, wide, grouped);
        case BPGB_DTYPE_BF16:
            return kernel_ptr8<__nv_bfloat16>(kahan, checked, planar, wide, grouped);
        case BPGB_DTYPE_C64: return kernel_ptr8<float2>(kahan, checked, planar, wide, grouped);
        case BPGB_DTYPE_C32: return kernel_ptr8<__half2>(kahan, checked, planar, wide, grouped);
        default: return kernel_ptr8<float>(kahan, checked, planar, wide, grouped);
    }
}

void *select_fact_kernel(int dtype, bool checked) {
    switch (dtype) {
        case BPGB_DTYPE_F32:
            return checked ? (void *)bp_fact_kernel<float, true> : (void *)bp_fact_kernel<float, false>;
        case BPGB_DTYPE_F16:
            return checked ? (void *)bp_fact_kernel<__half, true> : (void *)bp_fact_kernel<__half, false>;
        case BPGB_DTYPE_BF16:
            return checked ? (void *)bp_fact_kernel<__nv_bfloat16, true>
                           : (void *)bp_fact_kernel<__nv_bfloat16, false>;
    }
    return nullptr;
}

// Launch arguments of the fast kernel for a volume, pair factorisation and tile preset:
// everything but the pair splits.  No allocation.  chunk / stages > 0 override the
// preset; otherwise the chunk shrinks until the stages fit the shared-memory budget.
int fast_args(FastArgs &a, const FastConfig &cfg, const Volume &vol, const double hd[3],
              bool confocal, double dT, double t0, uint64_t L, uint64_t S, uint32_t T,
              uint32_t esz, bool kahan, uint32_t chunk_req, uint32_t stages_req,
              std::string *why, uint32_t bw_fixed = 0, bool fact = false) {
    auto no = [&](const std::string &m) {
        if (why) *why = m;
        return BPGB_ERR_UNSUPPORTED;
    };
    (void)t0;
    a = FastArgs{};
    const uint32_t cwarps = cfg.cta_consumer_warps();
    if ((cfg.k != 8 && cfg.k != 16) || (cfg.k == 16 && (esz != 4 || kahan || cwarps != 8)) ||
        cfg.lx * cfg.ly * cfg.lz != 32 || cfg.kaxis > 2 ||
        (cwarps != 8 && cwarps != 4 && cwarps != 2) ||
        (cfg.groups != 1 && cfg.groups != 2 && cfg.groups != 4) || (cfg.groups > 1 && fact))
        return no("tile preset not available for this row type");
    a.groups = cfg.groups;
    const uint32_t lane[3] = {cfg.lx, cfg.ly, cfg.lz}, warp[3] = {cfg.wx, cfg.wy, cfg.wz};
    for (int k = 0; k < 3; k++) {
        a.n[k] = vol.n[k];
        a.lane[k] = lane[k];
        a.warp[k] = warp[k];
        a.tdim[k] = cfg.tile(k);
        a.tiles[k] = (vol.n[k] + a.tdim[k] - 1) / a.tdim[k];
    }
    a.kax = cfg.kaxis;
    a.oax0 = cfg.kaxis == 0 ? 1 : 0;
    a.oax1 = cfg.kaxis == 2 ? 1 : 2;
    const double sb = (confocal ? 2.0 : 1.0) / dT, sa = confocal ? 0.0 : 1.0 / dT;
    a.sb = (float)sb;
    a.sa = (float)sa;
    for (int k = 0; k < 3; k++) {
        a.h[k] = (float)hd[k];
        a.hs[k] = (float)(hd[k] * sb);
    }
    a.L = L;
    a.S = S;
    a.T = T;
    a.out_scale = 1.0f;
    a.nvox = vol.count();
    a.spin_limit = 1u << 22;
    // Window width: the spread of (laser leg + SPAD leg) over a tile is at most
    // (sa + sb) * tile diagonal (triangle inequality), plus margins and alignment.
    double diag2 = 0.0;
    for (int k = 0; k < 3; k++) {
        const double e = (double)(a.tdim[k] - 1) * hd[k];
        diag2 += e * e;
    }
    const double span = (sa + sb) * std::sqrt(diag2) * (1.0 + 1e-5) + 2.0 * kMargin + 3.0;
    a.align = 16 / esz;
    // factored form: the window start is the sum of a laser part and a SPAD part, each
    // aligned down, so the window carries one more alignment of slack
    const uint32_t w_need = (uint32_t)std::ceil(span) + (fact ? 2 : 1) * a.align;
    const uint32_t bw_align = 128 / esz;
    if (bw_fixed) {  // one TMA box width shared by several captures (batches)
        a.BW = bw_fixed;
        a.nbox = (w_need + bw_fixed - 1) / bw_fixed;
    } else {
        a.nbox = (w_need + 255) / 256;
        a.BW = ((w_need + a.nbox - 1) / a.nbox + bw_align - 1) / bw_align * bw_align;
    }
    if (a.BW > 256) return no("window box too wide");
    a.W = a.BW * a.nbox;
    a.row_bytes = a.W * esz;
    // a stage holds `chunk` rows of each of the group's tiles (kMaxChunk entries at most,
    // kMaxGroupEntries with several tiles per CTA)
    auto stage_bytes = [&](uint32_t c) {
        return table_bytes_of(c * a.groups) + c * a.groups * a.row_bytes;
    };
    const uint32_t max_entries = a.groups > 1 ? kMaxGroupEntries : kMaxChunk;
    uint32_t chunk = (uint32_t)std::min<uint64_t>(
        std::min<uint32_t>(chunk_req ? chunk_req : cfg.chunk, max_entries / a.groups),
        fact ? L * kFactS : S);
    uint32_t stages = std::min<uint32_t>(stages_req ? stages_req : cfg.stages, 8);
    if (stages < 2) stages = 2;
    // Shared memory per CTA so that the variant's resident-CTA target fits one SM (228 KB).
    // Smaller CTAs (2 or 4 consumer warps, block-sparse tiles) need proportionally more
    // resident CTAs per SM: 96 registers x (1 + warps) x 32 threads each.
    const int ctas = cwarps == 8 ? (fact ? kFactCtas : fast_ctas_per_sm((int)cfg.k, kahan, (int)esz))
                                 : (cwarps == 4 ? 4 : 7);
    const uint32_t soft = ctas >= 7   ? 38 * 1024
                          : ctas >= 4 ? 56 * 1024
                          : ctas >= 3 ? 72 * 1024
                          : (ctas == 2 ? 110 * 1024 : 200 * 1024);
    const uint32_t budget = 200 * 1024;
    // Long chunks amortise the per-stage handshake (measured: 8 -> 32 rows cut the
    // 256^3 time by a quarter, pipeline depth 2..4 changed it by < 1%), so the depth
    // gives way first.
    if (!stages_req)
        while (stages > 2 && stages * stage_bytes(chunk) > soft) stages--;
    if (!chunk_req)
        while (chunk > 4 && stages * stage_bytes(chunk) > soft) chunk = (chunk + 1) / 2;
    while (chunk > 1 && stages * stage_bytes(chunk) > budget) chunk = (chunk + 1) / 2;
    if (stages * stage_bytes(chunk) > budget)
        return no("time window of one tile does not fit in shared memory (" +
                  std::to_string(a.W) + " bins)");
    if (fact) {  // whole SPAD blocks: chunk = lasers per stage x kFactS
        if (chunk < kFactS || S % kFactS) return no("factored form needs 4-SPAD blocks");
        chunk = chunk / kFactS * kFactS;
    }
    if (a.groups > 1) {  // a power of two: entry -> (tile, row) by shift and mask
        uint32_t p2 = 1;
        while (2 * p2 <= chunk) p2 *= 2;
        chunk = p2;
    }
    a.chunk = chunk;
    a.stages = stages;
    a.table_bytes = table_bytes_of(chunk * a.groups);
    a.stage_bytes = stage_bytes(chunk);
    a.fact = fact ? 1 : 0;
    // items: (laser, SPAD chunk), or (SPAD block, laser group) in the factored form
    a.nchunks = fact ? (uint32_t)((L + chunk / kFactS - 1) / (chunk / kFactS))
                     : (uint32_t)((S + chunk - 1) / chunk);
    // the kernel counts items in 32 bits
    if (fast_items(a) >= (1ull << 32)) return no("more than 2^32 (laser, chunk) items");
    return BPGB_OK;
}

uint32_t fast_threads(const FastConfig &cfg) { return 32 * (1 + cfg.cta_consumer_warps()); }
uint32_t fast_smem(const FastArgs &a) { return a.stages * a.stage_bytes + 128; }

}  // namespace

FastConfig fast_preset(int index, int dtype) {
    (void)dtype;
    const int n = (int)(sizeof(kPresets) / sizeof(kPresets[0]));
    if (index < 0 || index >= n) index = 0;
    return kPresets[index];
}

int fast_preset_count() { return (int)(sizeof(kPresets) / sizeof(kPresets[0])); }

struct FastPlan {
    FastArgs a{};
    int dtype = 0;
    bool kahan = false, checked = false;
    uint64_t P = 0;
    uint32_t pitch = 0;
    uint32_t threads = 0, smem = 0, grid = 0;
    float4 *d_tables = nullptr;  // S spad entries then L laser entries
    unsigned long long *d_diag = nullptr;
    float *d_partial = nullptr;
    uint64_t scratch = 0;
    int geom = 0;
    uint32_t k = 8;
    bool planar = false;
    bool fact = false;
    bool wide = true;      // 8 consumer warps per CTA
    bool grouped = false;  // several tiles per CTA
};

void *plan_kernel(const FastPlan *fp) {
    return fp->fact ? select_fact_kernel(fp->dtype, fp->checked)
                    : select_kernel(fp->dtype, fp->kahan, fp->checked, fp->k, fp->planar,
                                    fp->wide, fp->grouped);
}

int fast_plan_build(FastPlan **out, const bpgb_pair *d_pairs, uint64_t P,
                    const Factorization &fz, const Volume &vol, const BinParams &bp,
                    const bpgb_options &opt, int sm_count, std::string *why_not) {
    *out = nullptr;
    auto no = [&](const std::string &m) {
        if (why_not) *why_not = m;
        return BPGB_ERR_UNSUPPORTED;
    };
    if (fz.geom != GEOM_SINGLE_LASER && fz.geom != GEOM_EXHAUSTIVE && fz.geom != GEOM_CONFOCAL)
        return no("pair list does not factor as lasers x SPADs or confocal");
    double u[3][3], hd[3];
    if (!volume_frame(vol, u, hd)) return no("voxel basis is not orthogonal");
    if (!encode_fn()) return no("cuTensorMapEncodeTiled unavailable");
    const int dt = opt.h_dtype;
    const uint32_t esz = dtype_bytes(dt);
    if (!esz) return no("unknown H dtype");
    const uint32_t pitch = opt.h_pitch ? opt.h_pitch : bp.T;
    if (pitch < bp.T) return no("h_pitch < T");
    if (((uint64_t)pitch * esz) % 16) return no("H row pitch is not a multiple of 16 bytes");
    if (P >= (1ull << 31) || bp.T >= (1u << 30)) return no("P or T too large for TMA coordinates");
    if (!(bp.dT > 0.0f)) return no("deltaT must be positive");

    const FastConfig cfg = fast_preset(opt.tile, dt);
    const bool confocal = fz.geom == GEOM_CONFOCAL;
    const uint64_t L = confocal ? 1 : fz.L;
    // Lasers x SPADs captures take the factored form where it is built: K = 8 voxels per
    // thread, 8 consumer warps, real rows with FP32 sums, whole 4-SPAD blocks.
    const bool fact = fz.geom == GEOM_EXHAUSTIVE && !opt.unfactored && cfg.k == 8 &&
                      cfg.groups == 1 && cfg.consumer_warps() == 8 &&
                      opt.accum != BPGB_ACCUM_KAHAN &&
                      (dt == BPGB_DTYPE_F32 || dt == BPGB_DTYPE_F16 || dt == BPGB_DTYPE_BF16) &&
                      fz.S % kFactS == 0;
    FastArgs a;
    std::string why;
    int st = fast_args(a, cfg, vol, hd, confocal, bp.dT, bp.t0, L, fz.S, bp.T, esz,
                       opt.accum == BPGB_ACCUM_KAHAN, opt.chunk > 0 ? (uint32_t)opt.chunk : 0,
                       opt.stages > 0 ? (uint32_t)opt.stages : 0, &why, 0, fact);
    if (st) return no(why);
    a.out_scale = opt.h_scale != 0.0f ? opt.h_scale : 1.0f;
    if (opt.spin_limit) a.spin_limit = opt.spin_limit;

    auto *fp = new FastPlan();
    fp->dtype = dt;
    fp->kahan = opt.accum == BPGB_ACCUM_KAHAN;
    fp->checked = opt.checked != 0;
    fp->P = P;
    fp->pitch = pitch;
    fp->geom = fz.geom;
    fp->threads = fast_threads(cfg);
    fp->smem = fast_smem(a);

    fp->k = cfg.k;
    fp->wide = cfg.cta_consumer_warps() == 8;
    fp->grouped = cfg.groups > 1;
    // Device tables: SPAD entries (frame position relative to zero, row constant) and
    // laser entries (frame position, lw/dT - t0/dT), built in FP64 on the GPU from the
    // plan's device pair list (tables_fp64_kernel), which also tests the planar wall:
    // every SPAD's FP32 frame coordinate along the voxel-line axis is the same float.
    // d_diag: [0] timed-out waits, [1] window violations (read by fast_plan_check),
    // [2..4] the table kernel's order / non-finite / off-plane counts, [5] the top-k tile
    // selection's score threshold.
    const size_t tab_bytes = (fz.S + a.L) * sizeof(float4);
    cudaError_t e = cudaMalloc(&fp->d_tables, tab_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&fp->d_diag, kPlanDiagWords * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(fp->d_diag, 0, kPlanDiagWords * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        fast_plan_free(fp);
        return e == cudaErrorMemoryAllocation ? set_error(BPGB_ERR_OUT_OF_MEMORY, "fast plan tables")
                                              : cuda_error(e, "fast plan tables");
    }
    if (int ts = launch_tables(d_pairs, vol, u, (double)bp.dT, (double)bp.t0, a.L, fz.S, confocal,
                               cfg.kaxis, fp->d_tables, fp->d_diag + 2, sm_count, 0)) {
        fast_plan_free(fp);
        return ts;
    }
    unsigned long long tdiag[3] = {0, 0, 0};
    e = cudaMemcpy(tdiag, fp->d_diag + 2, sizeof(tdiag), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        fast_plan_free(fp);
        return cuda_error(e, "fast plan table checks");
    }
    if (tdiag[0] || tdiag[1]) {  // the host factorisation and finiteness checks passed
        fast_plan_free(fp);
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "device pair list disagrees with the host list");
    }
    const bool planar = cfg.k == 8 && tdiag[2] == 0;
    a.planar = planar && !fact ? 1 : 0;
    fp->planar = a.planar != 0;
    fp->fact = fact;
    void *kern = plan_kernel(fp);
    if (!kern) {
        fast_plan_free(fp);
        return no("tile preset not built for this row type / accumulation");
    }
    if (int rs = reserve_dynamic_smem(kern, fp->smem)) {
        fast_plan_free(fp);
        return rs;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, (int)fp->threads, fp->smem);
    if (e != cudaSuccess || occ < 1) {
        fast_plan_free(fp);
        return e != cudaSuccess ? cuda_error(e, "occupancy query")
                                : no("fast kernel does not fit on an SM");
    }

    const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    const uint64_t ngroups = (ntiles + a.groups - 1) / a.groups;  // CTAs per pair split
    const uint64_t items = fast_items(a);
    uint64_t splits = opt.pair_splits > 0 ? (uint64_t)opt.pair_splits : 1;
    if (opt.pair_splits <= 0) {
        const uint64_t want = 2ull * sm_count * occ;  // two waves of resident CTAs
        if (ngroups < want) splits = (want + ngroups - 1) / ngroups;
    }
    splits = std::max<uint64_t>(1, std::min<uint64_t>(splits, items));
    if (ngroups * splits >= (1ull << 31)) {
        fast_plan_free(fp);
        return no("grid too large");
    }
    a.splits = (uint32_t)splits;
    fp->grid = (uint32_t)(ngroups * splits);
    fp->a = a;

    // partial sums: [split][voxel] for full launches, [slot][split][tile voxel] for
    // tile-list launches (tiles x tile voxels >= voxels)
    const size_t part_bytes =
        splits > 1 ? (size_t)splits * ntiles * a.tdim[0] * a.tdim[1] * a.tdim[2] *
                         (dt == BPGB_DTYPE_C64 || dt == BPGB_DTYPE_C32 ? 8 : 4)
                   : 0;
    if (part_bytes) e = cudaMalloc(&fp->d_partial, part_bytes);
    if (e != cudaSuccess) {
        fast_plan_free(fp);
        return e == cudaErrorMemoryAllocation ? set_error(BPGB_ERR_OUT_OF_MEMORY, "fast plan scratch")
                                              : cuda_error(e, "fast plan scratch");
    }
    fp->scratch = tab_bytes + part_bytes + kPlanDiagWords * sizeof(unsigned long long);
    *out = fp;
    return BPGB_OK;
}

int fast_plan_execute(FastPlan *fp, const void *d_H, void *d_out, cudaStream_t stream) {
    const FastArgs &a = fp->a;
    if (((uintptr_t)d_H) % 16) return set_error(BPGB_ERR_INVALID_ARGUMENT, "H must be 16-byte aligned");
    CUtensorMap map;
    int st = encode_rows(&map, fp->dtype, d_H, a.T, fp->P, fp->pitch, a.BW);
    if (st) return st;
    void *target = a.splits > 1 ? (void *)fp->d_partial : d_out;
    const float4 *spads = fp->d_tables;
    const float4 *lasers = fp->d_tables + a.S;
    void *kern = plan_kernel(fp);
    unsigned long long *diag = fp->d_diag;
    void *args[] = {(void *)&map, (void *)&spads, (void *)&lasers, (void *)&target,
                    (void *)&diag, (void *)&fp->a};
    BPGB_CUDA_TRY(cudaLaunchKernel(kern, dim3(fp->grid), dim3(fp->threads), args, fp->smem, stream));
    count_launches(1);
    if (a.splits > 1) {
        const bool cplx = fp->dtype == BPGB_DTYPE_C64 || fp->dtype == BPGB_DTYPE_C32;
        const uint64_t n = a.nvox * (cplx ? 2 : 1);
        const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 8);
        if (cplx) {
            if (fp->kahan)
                reduce_splits_kernel<true, true><<<blocks, 256, 0, stream>>>(
                    fp->d_partial, (float *)d_out, a.nvox, a.splits, a.out_scale);
            else
                reduce_splits_kernel<true, false><<<blocks, 256, 0, stream>>>(
                    fp->d_partial, (float *)d_out, a.nvox, a.splits, a.out_scale);
        } else {
            if (fp->kahan)
                reduce_splits_kernel<false, true><<<blocks, 256, 0, stream>>>(
                    fp->d_partial, (float *)d_out, a.nvox, a.splits, a.out_scale);
            else
                reduce_splits_kernel<false, false><<<blocks, 256, 0, stream>>>(
                    fp->d_partial, (float *)d_out, a.nvox, a.splits, a.out_scale);
        }
        count_launches(1);
        BPGB_CUDA_TRY(cudaGetLastError());
    }
    return BPGB_OK;
}

int fast_plan_execute_tiles(FastPlan *fp, const void *d_H, void *d_out, const uint32_t *d_list,
                            const uint32_t *d_count, uint32_t max_tiles, cudaStream_t stream) {
    const FastArgs &a0 = fp->a;
    const uint64_t ntiles = (uint64_t)a0.tiles[0] * a0.tiles[1] * a0.tiles[2];
    if (!d_list || !d_count) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null tile list");
    if (max_tiles == 0) return BPGB_OK;
    const uint64_t slot_groups = ((uint64_t)max_tiles + a0.groups - 1) / a0.groups;
    if (slot_groups * a0.splits >= (1ull << 31))
        return set_error(BPGB_ERR_UNSUPPORTED, "tile list x pair splits too large for one grid");
    if (max_tiles > ntiles)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "max_tiles exceeds the plan's tile count");
    if (((uintptr_t)d_H) % 16) return set_error(BPGB_ERR_INVALID_ARGUMENT, "H must be 16-byte aligned");
    CUtensorMap map;
    int st = encode_rows(&map, fp->dtype, d_H, a0.T, fp->P, fp->pitch, a0.BW);
    if (st) return st;
    FastArgs a = a0;
    a.tile_list = d_list;
    a.tile_count = d_count;
    a.max_tiles = max_tiles;
    a.tile_local = a.splits > 1 ? 1 : 0;
    const float4 *spads = fp->d_tables;
    const float4 *lasers = fp->d_tables + a.S;
    void *target = a.splits > 1 ? (void *)fp->d_partial : d_out;
    void *kern = plan_kernel(fp);
    void *args[] = {(void *)&map, (void *)&spads, (void *)&lasers, (void *)&target,
                    (void *)&fp->d_diag, (void *)&a};
    BPGB_CUDA_TRY(cudaLaunchKernel(kern, dim3((uint32_t)(slot_groups * a.splits)),
                                   dim3(fp->threads), args, fp->smem, stream));
    count_launches(1);
    if (a.splits > 1) {
        const bool cplx = fp->dtype == BPGB_DTYPE_C64 || fp->dtype == BPGB_DTYPE_C32;
        const uint64_t n = (uint64_t)max_tiles * a.tdim[0] * a.tdim[1] * a.tdim[2] * (cplx ? 2 : 1);
        const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 8);
        float *o = (float *)d_out;
        if (cplx) {
            if (fp->kahan)
                reduce_tiles_kernel<true, true><<<blocks, 256, 0, stream>>>(fp->d_partial, d_list, d_count, max_tiles, a, o);
            else
                reduce_tiles_kernel<true, false><<<blocks, 256, 0, stream>>>(fp->d_partial, d_list, d_count, max_tiles, a, o);
        } else {
            if (fp->kahan)
                reduce_tiles_kernel<false, true><<<blocks, 256, 0, stream>>>(fp->d_partial, d_list, d_count, max_tiles, a, o);
            else
                reduce_tiles_kernel<false, false><<<blocks, 256, 0, stream>>>(fp->d_partial, d_list, d_count, max_tiles, a, o);
        }
        count_launches(1);
        BPGB_CUDA_TRY(cudaGetLastError());
    }
    return BPGB_OK;
}

namespace {

// One thread per tile of the plan (tile order of tile_of_block): the tile is listed when
// any score block it overlaps is above the threshold (at or above it when `ge`; the
// threshold read from device memory when d_thr is given).  Blocks are bs^3 voxels on the
// plan's voxel grid; list order depends on thread timing, results of a tile-list launch
// do not (every tile is computed on its own).
__global__ void select_tiles_kernel(const float *__restrict__ score, uint32_t bnx, uint32_t bny,
                                    uint32_t bnz, uint32_t bs, float threshold,
                                    const float *__restrict__ d_thr, int ge, uint32_t t0n,
                                    uint32_t t1n, uint32_t t2n, uint32_t d0, uint32_t d1,
                                    uint32_t d2, uint32_t *__restrict__ list,
                                    uint32_t *__restrict__ count) {
    const float thr = d_thr ? *d_thr : threshold;
    const uint32_t ntiles = t0n * t1n * t2n;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles;
         t += gridDim.x * blockDim.x) {
        const uint32_t tz = t % t2n, tx = (t / t2n) % t0n, ty = t / (t2n * t0n);
        const uint32_t lo[3] = {tx * d0 / bs, ty * d1 / bs, tz * d2 / bs};
        const uint32_t hi[3] = {min((tx * d0 + d0 - 1) / bs, bnx - 1),
                                min((ty * d1 + d1 - 1) / bs, bny - 1),
                                min((tz * d2 + d2 - 1) / bs, bnz - 1)};
        bool any = false;
        for (uint32_t x = lo[0]; x <= hi[0] && !any; x++)
            for (uint32_t y = lo[1]; y <= hi[1] && !any; y++)
                for (uint32_t z = lo[2]; z <= hi[2] && !any; z++) {
                    const float v = score[((uint64_t)x * bny + y) * bnz + z];
                    any = ge ? v >= thr : v > thr;
                }
        if (any) list[atomicAdd(count, 1u)] = t;
    }
}

// The k-th largest of n non-negative scores (NaN and negative values count as 0), by
// radix selection on their float bits, which order like the values: four passes over
// 8-bit digits, most significant first, each a shared-memory histogram of the scores
// that share the digits chosen so far.  One CTA; writes the score to *out.
__global__ void __launch_bounds__(1024) topk_threshold_kernel(const float *__restrict__ score,
                                                              uint32_t n, uint32_t k,
                                                              float *__restrict__ out) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t prefix, mask, rest;
    if (threadIdx.x == 0) {
        prefix = 0;
        mask = 0;
        rest = k;
    }
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const uint32_t pf = prefix, mk = mask;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const float v = score[i];
            const uint32_t key = v > 0.0f ? __float_as_uint(v) : 0u;
            if ((key & mk) == pf) atomicAdd(&hist[(key >> shift) & 0xFFu], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t cum = 0, d = 255;
            for (;; d--) {
                if (cum + hist[d] >= rest || d == 0) break;
                cum += hist[d];
            }
            rest -= cum;
            prefix = pf | (d << shift);
            mask = mk | (0xFFu << shift);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = __uint_as_float(prefix);
}

}  // namespace

int fast_plan_select_tiles(FastPlan *fp, const float *d_score, const uint32_t *block_dims,
                           uint32_t block_size, float threshold, uint32_t *d_list,
                           uint32_t *d_count, cudaStream_t stream) {
    const FastArgs &a = fp->a;
    if (!d_score || !block_dims || !d_list || !d_count || block_size == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    for (int k = 0; k < 3; k++)
        if (block_dims[k] == 0 || (uint64_t)block_dims[k] * block_size < a.n[k])
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "score blocks do not cover the volume");
    const uint32_t ntiles = a.tiles[0] * a.tiles[1] * a.tiles[2];
    BPGB_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), stream));
    const unsigned blocks = (ntiles + 255) / 256;
    select_tiles_kernel<<<blocks, 256, 0, stream>>>(d_score, block_dims[0], block_dims[1],
                                                    block_dims[2], block_size, threshold, nullptr,
                                                    0, a.tiles[0], a.tiles[1], a.tiles[2],
                                                    a.tdim[0], a.tdim[1], a.tdim[2], d_list,
                                                    d_count);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int fast_plan_select_tiles_topk(FastPlan *fp, const float *d_score, const uint32_t *block_dims,
                                uint32_t block_size, uint32_t k, uint32_t *d_list,
                                uint32_t *d_count, cudaStream_t stream) {
    const FastArgs &a = fp->a;
    if (!d_score || !block_dims || !d_list || !d_count || block_size == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    for (int q = 0; q < 3; q++)
        if (block_dims[q] == 0 || (uint64_t)block_dims[q] * block_size < a.n[q])
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "score blocks do not cover the volume");
    const uint64_t nb = (uint64_t)block_dims[0] * block_dims[1] * block_dims[2];
    if (nb >= (1ull << 32)) return set_error(BPGB_ERR_UNSUPPORTED, "too many score blocks");
    BPGB_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), stream));
    if (k == 0) return BPGB_OK;
    const uint32_t kk = (uint32_t)std::min<uint64_t>(k, nb);
    // the threshold lives in the plan's device counters (word kPlanThresholdWord)
    float *d_thr = reinterpret_cast<float *>(fp->d_diag + kPlanThresholdWord);
    topk_threshold_kernel<<<1, 1024, 0, stream>>>(d_score, (uint32_t)nb, kk, d_thr);
    const uint32_t ntiles = a.tiles[0] * a.tiles[1] * a.tiles[2];
    select_tiles_kernel<<<(ntiles + 255) / 256, 256, 0, stream>>>(
        d_score, block_dims[0], block_dims[1], block_dims[2], block_size, 0.0f, d_thr, 1,
        a.tiles[0], a.tiles[1], a.tiles[2], a.tdim[0], a.tdim[1], a.tdim[2], d_list, d_count);
    count_launches(2);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

int fast_plan_dump_bins(FastPlan *fp, const int64_t *d_ids, int64_t n, int32_t *d_bins,
                        cudaStream_t stream) {
    if (n <= 0) return BPGB_OK;
    const uint64_t total = (uint64_t)n * fp->P;
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 16);
    bp_fast_bins_kernel<<<blocks, 256, 0, stream>>>(fp->d_tables, fp->d_tables + fp->a.S, d_ids,
                                                     n, d_bins, fp->a);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

void fast_plan_info(const FastPlan *fp, bpgb_plan_info *info) {
    const FastArgs &a = fp->a;
    info->algo = BPGB_ALGO_FAST;
    info->geometry = fp->geom;
    info->num_lasers = a.L;
    info->num_spads = a.S;
    for (int k = 0; k < 3; k++) info->tile[k] = a.tdim[k];
    info->window = a.W;
    info->chunk = a.chunk;
    info->stages = a.stages;
    info->pair_splits = a.splits;
    info->grid = fp->grid;
    info->threads = fp->threads;
    info->smem_bytes = fp->smem;
    info->scratch_bytes = fp->scratch;
    info->factored = fp->fact ? 1 : 0;
}

int fast_plan_tables(const FastPlan *fp, float *host_out, uint64_t capacity, uint64_t *count) {
    const uint64_t n = fp->a.S + fp->a.L;
    if (count) *count = n;
    const uint64_t m = std::min(n, capacity);
    if (m && host_out)
        BPGB_CUDA_TRY(cudaMemcpy(host_out, fp->d_tables, m * sizeof(float4), cudaMemcpyDeviceToHost));
    return BPGB_OK;
}

int fast_plan_check(FastPlan *fp, uint64_t *violations, uint64_t *timeouts) {
    unsigned long long h[2] = {0, 0};
    BPGB_CUDA_TRY(cudaMemcpy(h, fp->d_diag, sizeof(h), cudaMemcpyDeviceToHost));
    BPGB_CUDA_TRY(cudaMemset(fp->d_diag, 0, sizeof(h)));
    if (violations) *violations = h[1];
    if (timeouts) *timeouts = h[0];
    return BPGB_OK;
}

int wait_timeout_probe(uint32_t limit, int *timed_out) {
    unsigned long long *d = nullptr;
    BPGB_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
    wait_timeout_probe_kernel<<<1, 32>>>(limit, d);
    count_launches(1);
    unsigned long long h = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_error(e, "wait timeout probe");
    *timed_out = h ? 1 : 0;
    return BPGB_OK;
}

void fast_plan_free(FastPlan *fp) {
    if (!fp) return;
    if (fp->d_tables) cudaFree(fp->d_tables);
    if (fp->d_diag) cudaFree(fp->d_diag);
    if (fp->d_partial) cudaFree(fp->d_partial);
    delete fp;
}

// ==================================================================================
// Batches: many captures of uneven grids, T and volumes in persistent launches.
//
// All captures' rows live in one packed device buffer [sum P_c, pitch] (capture c at
// rows row_base_c; bins T_c..pitch zero) behind a single TMA tensor map whose box width
// is shared.  Each capture has a launch descriptor (FastArgs, table, output and partial-sum
// offsets) in device memory.  The work lists hold (capture, tile, pair range) units, one
// list per launch (per-pair legs; factored lasers x SPADs legs), each sorted by cost
// (pairs x tile voxels / ranges) in decreasing order; each CTA takes the next unit from
// an atomic counter when it finishes one (greedy longest-first), with its pipeline (stage
// ring, mbarrier phases) continuing across units.  Captures split over pair ranges write
// partial sums that a reduction adds after their launch.  The launches allocate nothing,
// so a caller can capture them in a CUDA graph; bpgb_batch_graph_launch does that once per
// buffer pair and replays the graph.
// ==================================================================================
namespace {

struct BatchCap {
    FastArgs a;
    uint64_t row_base;  // first row of the capture in the packed H
    uint64_t out_off;   // first voxel of the capture in the packed output
    uint64_t tab_off;   // first table entry (SPADs then lasers)
    uint64_t part_off;  // a.splits > 1: first float of its split-major partial sums in scratch
};

struct BatchUnit {
    uint32_t cap, tile, split;
};

// FACT: the launch over the batch's lasers x SPADs captures (factored legs); otherwise the
// launch over the rest (per-pair legs).  Each is one persistent launch over its own
// cost-sorted unit list with its own counters; a batch with both kinds runs the two
// launches back to back.
template <typename HT, bool CHECKED, bool PLANAR, bool FACT>
__global__ void __launch_bounds__(288, FACT ? kFactCtas : 3)
    bp_batch_kernel(const __grid_constant__ CUtensorMap tmap, const BatchCap *__restrict__ caps,
                    const BatchUnit *__restrict__ units, uint32_t n_units,
                    const float4 *__restrict__ tables, float *__restrict__ out,
                    float *__restrict__ scratch, unsigned long long *__restrict__ diag,
                    unsigned int *__restrict__ sched, uint32_t stages, uint32_t spin_limit) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[8];
    __shared__ __align__(8) uint64_t empty_bar[8];
    __shared__ int abort_flag;
    PipeShared sh;
    pipeline_init(sh, smem_raw, full_bar, empty_bar, &abort_flag, stages);
    // The unit's launch descriptor is staged in shared memory: fields are reloaded from
    // there instead of held in registers (global loads would be hoisted and spill).
    __shared__ __align__(16) BatchCap cap_s;
    __shared__ uint32_t unit_s;
    uint64_t step = 0;
    bool ok = true;
    for (;;) {
        // Greedy longest-first: the next unit of the cost-sorted list goes to whichever
        // CTA asks first (sched[0] counts handed-out units).
        __syncthreads();  // every warp is done with the previous unit's descriptor
        if (threadIdx.x == 0) unit_s = atomicAdd(&sched[0], 1u);
        __syncthreads();
        const uint32_t w = unit_s;
        if (w >= n_units) break;
        const BatchUnit u = units[w];
        {
            constexpr uint32_t kWords = sizeof(BatchCap) / 4;
            const uint32_t *src = reinterpret_cast<const uint32_t *>(caps + u.cap);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&cap_s);
            for (uint32_t i = threadIdx.x; i < kWords; i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        if (*(volatile int *)&abort_flag) break;
        const float4 *tab = tables + cap_s.tab_off;
        // split captures write partial sums (reduced after the launch), the rest the volume
        float *dst = cap_s.a.splits > 1 ? scratch + cap_s.part_off : out + cap_s.out_off;
        if constexpr (FACT)
            ok = fact_unit<HT, CHECKED>(cap_s.a, &tmap, tab, tab + cap_s.a.S, dst, diag, u.tile,
                                        u.split, (uint32_t)cap_s.row_base, step, sh);
        else
            ok = fast_unit<HT, 8, false, CHECKED, PLANAR, kBatchRows, false>(
                cap_s.a, &tmap, tab, tab + cap_s.a.S, dst, diag, u.tile, u.split,
                (uint32_t)cap_s.row_base, step, sh);
        if (!ok) *(volatile int *)&abort_flag = 1;
    }
    pipeline_drain(stages, step, full_bar, diag, spin_limit);
    // The last CTA to finish re-arms the work counter for the next launch (graph replays).
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&sched[1], 1u) == gridDim.x - 1) {
            atomicExch(&sched[0], 0u);
            atomicExch(&sched[1], 0u);
        }
    }
}

template <typename HT>
void *batch_kernel_ptr(bool checked, bool planar, bool fact) {
    if (fact)  // the planar-wall form is a per-pair body detail
        return checked ? (void *)bp_batch_kernel<HT, true, false, true>
                       : (void *)bp_batch_kernel<HT, false, false, true>;
    if (planar)
        return checked ? (void *)bp_batch_kernel<HT, true, true, false>
                       : (void *)bp_batch_kernel<HT, false, true, false>;
    return checked ? (void *)bp_batch_kernel<HT, true, false, false>
                   : (void *)bp_batch_kernel<HT, false, false, false>;
}

void *select_batch_kernel(int dtype, bool checked, bool planar, bool fact) {
    return dtype == BPGB_DTYPE_F16 ? batch_kernel_ptr<__half>(checked, planar, fact)
                                   : batch_kernel_ptr<float>(checked, planar, fact);
}

}  // namespace

struct BatchPlan {
    int dtype = BPGB_DTYPE_F32;
    bool checked = false, planar = false;
    uint32_t n = 0, pitch = 0, stages = 0, chunk = 0, smem = 0, grid = 0, n_units = 0;
    // units [0, n_units - n_fact) run per-pair legs, the last n_fact factored legs (a
    // second launch with grid_fact CTAs and the counters d_sched[2..3]); each launch has
    // its own stage ring (ring[0] per-pair, ring[1] factored)
    uint32_t n_fact = 0, grid_fact = 0;
    struct {
        uint32_t chunk = 0, stages = 0, smem = 0;
    } ring[2];
    // captures whose units are split over pair ranges: partial sums in d_scratch, added
    // into the volume after their launch
    struct Split {
        int fact;
        uint32_t splits;
        uint64_t part_off, out_off, nvox;
        float scale;
    };
    std::vector<Split> splits;
    float *d_scratch = nullptr;
    uint32_t spin_limit = 1u << 22;
    uint64_t total_rows = 0, total_vox = 0, updates = 0;
    std::vector<uint64_t> row_off, vox_off;
    BatchCap *d_caps = nullptr;
    BatchUnit *d_units = nullptr;
    float4 *d_tables = nullptr;
    unsigned long long *d_diag = nullptr;
    unsigned int *d_sched = nullptr;  // work counter, finished-CTA counter
    cudaStream_t own_stream = nullptr;
    cudaStream_t side_stream = nullptr;  // the per-pair launch when both kinds run
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaGraphExec_t graph = nullptr;
    const void *graph_H = nullptr;
    const float *graph_out = nullptr;
    cudaStream_t last_stream = nullptr;
};

void batch_free(BatchPlan *b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    if (b->side_stream) cudaStreamDestroy(b->side_stream);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    cudaFree(b->d_caps);
    cudaFree(b->d_units);
    cudaFree(b->d_tables);
    cudaFree(b->d_diag);
    cudaFree(b->d_sched);
    cudaFree(b->d_scratch);
    delete b;
}

int batch_execute(BatchPlan *b, const void *d_H, float *d_out, cudaStream_t s) {
    if (!d_H || !d_out) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null batch buffer");
    if (((uintptr_t)d_H) % 16) return set_error(BPGB_ERR_INVALID_ARGUMENT, "H must be 16-byte aligned");
    const uint32_t esz = dtype_bytes(b->dtype);
    const cuuint64_t dims[2] = {b->pitch, b->total_rows};
    const cuuint64_t strides[1] = {(cuuint64_t)b->pitch * esz};
    const cuuint32_t box[2] = {128 / esz, 1};
    const cuuint32_t estr[2] = {1, 1};
    CUtensorMap map;
    CUresult r = encode_fn()(&map, tma_type(b->dtype), 2, const_cast<void *>(d_H), dims, strides, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(BPGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (batch)");
    // With both kinds of capture the two persistent launches run concurrently: the
    // factored launch (most of the work) on `s`, the per-pair launch on the batch's side
    // stream forked from and joined back into `s` (two branches of a captured graph).
    // Their CTAs cannot share an SM (registers), so the per-pair CTAs take the SMs the
    // factored launch's last CTAs leave, and neither launch ends with an idle tail.
    const uint32_t n_pp = b->n_units - b->n_fact;
    const bool fork = n_pp && b->n_fact;
    if (fork) {
        BPGB_CUDA_TRY(cudaEventRecord(b->ev_fork, s));
        BPGB_CUDA_TRY(cudaStreamWaitEvent(b->side_stream, b->ev_fork, 0));
    }
    for (int f = 1; f >= 0; f--) {
        uint32_t nu = f ? b->n_fact : n_pp;
        if (!nu) continue;
        const cudaStream_t ls = (fork && f == 0) ? b->side_stream : s;
        const BatchUnit *units = b->d_units + (f ? n_pp : 0);
        unsigned int *sched = b->d_sched + (f ? 2 : 0);
        void *kern = select_batch_kernel(b->dtype, b->checked, b->planar, f != 0);
        void *args[] = {(void *)&map,         (void *)&b->d_caps,    (void *)&units,
                        (void *)&nu,          (void *)&b->d_tables,  (void *)&d_out,
                        (void *)&b->d_scratch, (void *)&b->d_diag,   (void *)&sched,
                        (void *)&b->ring[f].stages, (void *)&b->spin_limit};
        BPGB_CUDA_TRY(cudaLaunchKernel(kern, dim3(f ? b->grid_fact : b->grid), dim3(288), args,
                                       b->ring[f].smem, ls));
        count_launches(1);
        for (const auto &sp : b->splits) {  // partial sums of this launch's split captures
            if (sp.fact != f) continue;
            const unsigned blocks = (unsigned)std::min<uint64_t>((sp.nvox + 255) / 256, 152ull * 8);
            reduce_splits_kernel<false, false><<<blocks, 256, 0, ls>>>(
                b->d_scratch + sp.part_off, d_out + sp.out_off, sp.nvox, sp.splits, sp.scale);
            count_launches(1);
        }
        BPGB_CUDA_TRY(cudaGetLastError());
    }
    if (fork) {
        BPGB_CUDA_TRY(cudaEventRecord(b->ev_join, b->side_stream));
        BPGB_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_join, 0));
    }
    b->last_stream = s;
    return BPGB_OK;
}

}  // namespace bpgb

using namespace bpgb;

struct bpgb_batch_s : BatchPlan {};

extern "C" {

int bpgb_batch_create(bpgb_batch *out, const bpgb_capture_geometry *caps, uint32_t n,
                      const bpgb_options *opt) {
    clear_error();
    if (!out || (n && !caps)) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (n == 0) return set_error(BPGB_ERR_INVALID_ARGUMENT, "empty batch");
    bpgb_options o;
    bpgb_options_default(&o);
    if (opt) o = *opt;
    if (o.h_dtype != BPGB_DTYPE_F32 && o.h_dtype != BPGB_DTYPE_F16)
        return set_error(BPGB_ERR_UNSUPPORTED, "batches take FP32 or FP16 rows");
    if (o.accum != BPGB_ACCUM_F32)
        return set_error(BPGB_ERR_UNSUPPORTED, "batches accumulate in FP32");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    const uint32_t esz = dtype_bytes(o.h_dtype);
    const uint32_t bw = 128 / esz;
    FastConfig cfg = fast_preset(o.tile, o.h_dtype);
    if (cfg.k != 8 || cfg.consumer_warps() != 8 || cfg.groups != 1) cfg = fast_preset(0, o.h_dtype);
    auto *b = new bpgb_batch_s();
    b->n = n;
    b->dtype = o.h_dtype;
    b->checked = o.checked != 0;
    if (o.spin_limit) b->spin_limit = o.spin_limit;
    std::vector<BatchCap> hc(n);
    struct TableJob {
        uint32_t c;
        Volume vol;
        double u[3][3];
        uint64_t L, S;
        bool confocal;
    };
    std::vector<TableJob> tjobs;
    uint64_t tab_count = 0;
    uint32_t max_row_bytes = 0, tmax = 0;
    for (uint32_t c = 0; c < n; c++) {
        const bpgb_capture_geometry &g = caps[c];
        auto fail = [&](int code, const std::string &m) {
            batch_free(b);
            return set_error(code, "capture " + std::to_string(c) + ": " + m);
        };
        if (!g.pairs || g.num_pairs == 0 || g.T == 0) return fail(BPGB_ERR_INVALID_ARGUMENT, "empty capture");
        Volume vol{};
        for (int k = 0; k < 3; k++) {
            vol.n[k] = g.voxels_per_side[k];
            vol.zero[k] = g.volume_zero_pos[k];
        }
        for (int k = 0; k < 9; k++) vol.inc[k] = g.voxel_inc[k];
        BinParams bp{g.t0, g.deltaT, g.T};
        std::string why;
        if (!finite_geometry(g.pairs, g.num_pairs, vol, bp, &why)) return fail(BPGB_ERR_INVALID_ARGUMENT, why);
        const Factorization fz = factorize_pairs(g.pairs, g.num_pairs);
        if (fz.geom != GEOM_SINGLE_LASER && fz.geom != GEOM_EXHAUSTIVE && fz.geom != GEOM_CONFOCAL)
            return fail(BPGB_ERR_UNSUPPORTED, "pair list does not factor as lasers x SPADs");
        double u[3][3], hd[3];
        if (!volume_frame(vol, u, hd)) return fail(BPGB_ERR_UNSUPPORTED, "voxel basis is not orthogonal");
        const bool confocal = fz.geom == GEOM_CONFOCAL;
        const uint64_t L = confocal ? 1 : fz.L;
        FastArgs &a = hc[c].a;
        bool fact = fz.geom == GEOM_EXHAUSTIVE && !o.unfactored && fz.S % kFactS == 0;
        for (;;) {  // the per-pair form where the factored one does not fit
            st = fast_args(a, cfg, vol, hd, confocal, g.deltaT, g.t0, L, fz.S, g.T, esz, false,
                           o.chunk > 0 ? (uint32_t)o.chunk : 0,
                           o.stages > 0 ? (uint32_t)o.stages : 0, &why, bw, fact);
            if (!st || !fact) break;
            fact = false;
        }
        if (st) return fail(st, why);
        a.out_scale = g.h_scale != 0.0f ? g.h_scale : 1.0f;
        a.splits = 1;
        a.spin_limit = b->spin_limit;
        max_row_bytes = std::max(max_row_bytes, a.row_bytes);
        tmax = std::max(tmax, g.T);
        // tables: built on the GPU after the loop (same FP64 kernel as a plan)
        hc[c].tab_off = tab_count;
        tab_count += fz.S + L;
        tjobs.push_back({c, vol, {{u[0][0], u[0][1], u[0][2]}, {u[1][0], u[1][1], u[1][2]},
                                  {u[2][0], u[2][1], u[2][2]}},
                         L, fz.S, confocal});
        hc[c].row_base = b->total_rows;
        hc[c].out_off = b->total_vox;
        b->row_off.push_back(b->total_rows);
        b->vox_off.push_back(b->total_vox);
        b->total_rows += g.num_pairs;
        b->total_vox += vol.count();
        b->updates += vol.count() * g.num_pairs;
    }
    if (b->total_rows >= (1ull << 31)) {
        batch_free(b);
        return set_error(BPGB_ERR_UNSUPPORTED, "batch has too many rows for TMA coordinates");
    }
    // Tables of every capture on the GPU in FP64 (tables_fp64_kernel, as for a plan) from
    // the captures' pairs staged in one temporary device buffer, and the planar-wall
    // test over all of them (each capture's SPADs against its own first SPAD).
    bool planar = true;
    {
        bpgb_pair *d_pairs = nullptr;
        cudaError_t e = cudaMalloc(&b->d_tables, tab_count * sizeof(float4));
        if (e == cudaSuccess) e = cudaMalloc(&b->d_diag, kPlanDiagWords * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(b->d_diag, 0, kPlanDiagWords * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc(&d_pairs, b->total_rows * sizeof(bpgb_pair));
        for (uint32_t c = 0; c < n && e == cudaSuccess; c++)
            e = cudaMemcpy(d_pairs + b->row_off[c], caps[c].pairs,
                           caps[c].num_pairs * sizeof(bpgb_pair), cudaMemcpyHostToDevice);
        int ts = e == cudaSuccess ? BPGB_OK : cuda_error(e, "batch table inputs");
        for (const TableJob &j : tjobs) {
            if (ts) break;
            const BinParams bp{caps[j.c].t0, caps[j.c].deltaT, caps[j.c].T};
            ts = launch_tables(d_pairs + b->row_off[j.c], j.vol, j.u, (double)bp.dT, (double)bp.t0,
                               j.L, j.S, j.confocal, cfg.kaxis, b->d_tables + hc[j.c].tab_off,
                               b->d_diag + 2, sms, 0);
        }
        unsigned long long tdiag[3] = {0, 0, 0};
        if (!ts) {
            e = cudaMemcpy(tdiag, b->d_diag + 2, sizeof(tdiag), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) ts = cuda_error(e, "batch table checks");
        }
        if (d_pairs) cudaFree(d_pairs);
        if (!ts && (tdiag[0] || tdiag[1]))
            ts = set_error(BPGB_ERR_INVALID_ARGUMENT, "device pair lists disagree with the host lists");
        if (ts) {
            batch_free(b);
            return ts;
        }
        planar = tdiag[2] == 0;
    }
    // One stage ring per launch: the widest window among that launch's captures sets its
    // row slot.  The per-pair launch targets three CTAs per SM (72 KB of shared memory
    // each), the factored one two (110 KB); factored captures need whole 4-SPAD blocks per
    // stage and run per pair (their wider windows serve that form too) when their ring
    // cannot hold them.
    auto ring_of = [&](int f, uint32_t row_bytes, uint32_t *chunk_out, uint32_t *stages_out) {
        uint32_t chunk = o.chunk > 0 ? std::min<uint32_t>((uint32_t)o.chunk, kMaxChunk) : cfg.chunk;
        uint32_t stages = o.stages > 0 ? std::min<uint32_t>((uint32_t)o.stages, 8) : cfg.stages;
        stages = std::max<uint32_t>(stages, 2);
        const uint32_t soft = f ? 110 * 1024 : 72 * 1024;
        auto sb = [&](uint32_t ch) { return table_bytes_of(ch) + ch * row_bytes; };
        if (o.stages <= 0)
            while (stages > 2 && stages * sb(chunk) > soft) stages--;
        if (o.chunk <= 0)
            while (chunk > 4 && stages * sb(chunk) > soft) chunk = (chunk + 1) / 2;
        while (chunk > 1 && stages * sb(chunk) > 200 * 1024) chunk = (chunk + 1) / 2;
        if (f) chunk = chunk / kFactS * kFactS;
        *chunk_out = chunk;
        *stages_out = stages;
        return chunk > 0 && stages * sb(chunk) <= 200 * 1024;
    };
    uint32_t row_bytes[2] = {0, 0};
    for (uint32_t c = 0; c < n; c++)
        row_bytes[hc[c].a.fact ? 1 : 0] = std::max(row_bytes[hc[c].a.fact ? 1 : 0], hc[c].a.row_bytes);
    uint32_t chunk[2] = {0, 0}, stages[2] = {0, 0};
    if (row_bytes[1] && !ring_of(1, row_bytes[1], &chunk[1], &stages[1])) {
        for (uint32_t c = 0; c < n; c++) hc[c].a.fact = 0;
        row_bytes[0] = std::max(row_bytes[0], row_bytes[1]);
        row_bytes[1] = 0;
    }
    if (row_bytes[0] && !ring_of(0, row_bytes[0], &chunk[0], &stages[0])) {
        batch_free(b);
        return set_error(BPGB_ERR_UNSUPPORTED, "widest time window does not fit in shared memory");
    }
    for (int f = 0; f < 2; f++) {
        b->ring[f].chunk = chunk[f];
        b->ring[f].stages = stages[f];
        b->ring[f].smem =
            row_bytes[f] ? stages[f] * (table_bytes_of(chunk[f]) + chunk[f] * row_bytes[f]) + 128 : 0;
    }
    const int shown = row_bytes[0] ? 0 : 1;  // the ring bpgb_batch_info reports
    b->chunk = chunk[shown];
    b->stages = stages[shown];
    b->smem = b->ring[shown].smem;
    b->planar = planar;
    b->pitch = (tmax + bw - 1) / bw * bw;
    for (uint32_t c = 0; c < n; c++) {
        FastArgs &a = hc[c].a;
        const int f = a.fact ? 1 : 0;
        a.chunk = chunk[f];
        a.stages = stages[f];
        a.table_bytes = table_bytes_of(chunk[f]);
        a.stage_bytes = table_bytes_of(chunk[f]) + chunk[f] * row_bytes[f];
        a.nchunks = a.fact ? (uint32_t)((a.L + chunk[f] / kFactS - 1) / (chunk[f] / kFactS))
                           : (uint32_t)((a.S + chunk[f] - 1) / chunk[f]);
        if (fast_items(a) >= (1ull << 32)) {
            batch_free(b);
            return set_error(BPGB_ERR_UNSUPPORTED, "more than 2^32 (laser, chunk) items");
        }
        a.planar = planar ? 1 : 0;
    }
    // resident CTAs of each launch
    cudaError_t e = cudaSuccess;
    uint64_t resident[2] = {0, 0};
    for (int f = 0; f < 2; f++) {
        if (!row_bytes[f]) continue;
        void *kern = select_batch_kernel(b->dtype, b->checked, b->planar, f != 0);
        if (int rs = reserve_dynamic_smem(kern, b->ring[f].smem)) {
            batch_free(b);
            return rs;
        }
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 288, b->ring[f].smem);
        if (e != cudaSuccess || occ < 1) {
            batch_free(b);
            return e != cudaSuccess ? cuda_error(e, "batch kernel attributes")
                                    : set_error(BPGB_ERR_UNSUPPORTED, "batch kernel does not fit on an SM");
        }
        resident[f] = (uint64_t)sms * occ;
    }
    // Units are (capture, tile, pair range).  A capture whose (capture, tile) unit is long
    // against a resident CTA's share of its launch is split into up to 8 pair ranges, so
    // the launch ends evenly (greedy longest-first over many short units); its ranges
    // write partial sums that are added, in range order, after the launch.
    auto unit_cost = [&](uint32_t c) {
        const FastArgs &a = hc[c].a;
        return (double)a.L * a.S * a.tdim[0] * a.tdim[1] * a.tdim[2];
    };
    double share[2] = {0.0, 0.0};
    for (uint32_t c = 0; c < n; c++) {
        const FastArgs &a = hc[c].a;
        share[a.fact ? 1 : 0] += unit_cost(c) * a.tiles[0] * a.tiles[1] * a.tiles[2];
    }
    for (int f = 0; f < 2; f++)
        if (resident[f]) share[f] /= (double)resident[f];
    uint64_t scratch = 0;
    std::vector<BatchUnit> units;
    for (uint32_t c = 0; c < n; c++) {
        FastArgs &a = hc[c].a;
        const int f = a.fact ? 1 : 0;
        const double target = share[f] / 24.0;  // unit length aimed at
        uint64_t sp = target > 0.0 ? (uint64_t)std::llround(unit_cost(c) / target) : 1;
        sp = std::max<uint64_t>(1, std::min<uint64_t>({sp, 8, fast_items(a)}));
        if (o.pair_splits > 0) sp = std::min<uint64_t>((uint64_t)o.pair_splits, fast_items(a));
        a.splits = (uint32_t)sp;
        hc[c].part_off = scratch;
        if (sp > 1) {
            b->splits.push_back({f, (uint32_t)sp, scratch, hc[c].out_off, a.nvox, a.out_scale});
            scratch += sp * a.nvox;
        }
        const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
        for (uint32_t k = 0; k < sp; k++)
            for (uint64_t t = 0; t < ntiles; t++) units.push_back({c, (uint32_t)t, k});
    }
    // per-pair units first, then the factored ones; each list longest first
    std::vector<uint32_t> order(units.size());
    for (uint32_t i = 0; i < order.size(); i++) order[i] = i;
    auto cost_of = [&](const BatchUnit &u) { return unit_cost(u.cap) / hc[u.cap].a.splits; };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const bool fx = hc[units[x].cap].a.fact != 0, fy = hc[units[y].cap].a.fact != 0;
        if (fx != fy) return fy;
        return cost_of(units[x]) > cost_of(units[y]);
    });
    std::vector<BatchUnit> sorted(units.size());
    for (size_t i = 0; i < order.size(); i++) sorted[i] = units[order[i]];
    if (sorted.size() >= (1ull << 32)) {
        batch_free(b);
        return set_error(BPGB_ERR_UNSUPPORTED, "too many work units");
    }
    b->n_units = (uint32_t)sorted.size();
    for (const BatchUnit &u : sorted) b->n_fact += hc[u.cap].a.fact ? 1 : 0;
    b->grid = (uint32_t)std::min<uint64_t>(b->n_units - b->n_fact, resident[0]);
    b->grid_fact = (uint32_t)std::min<uint64_t>(b->n_fact, resident[1]);
    if (scratch) e = cudaMalloc(&b->d_scratch, scratch * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_caps, n * sizeof(BatchCap));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_units, sorted.size() * sizeof(BatchUnit));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_caps, hc.data(), n * sizeof(BatchCap), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_units, sorted.data(), sorted.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_sched, 4 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(b->d_sched, 0, 4 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        batch_free(b);
        return cuda_error(e, "batch upload");
    }
    *out = b;
    return BPGB_OK;
}

int bpgb_batch_layout(bpgb_batch b, uint64_t *row_offsets, uint64_t *voxel_offsets) {
    if (!b) return set_error(BPGB_ERR_INVALID_ARGUMENT, "batch is null");
    for (uint32_t c = 0; c < b->n; c++) {
        if (row_offsets) row_offsets[c] = b->row_off[c];
        if (voxel_offsets) voxel_offsets[c] = b->vox_off[c];
    }
    return BPGB_OK;
}

int bpgb_batch_get_info(bpgb_batch b, bpgb_batch_info *info) {
    if (!b || !info) return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->captures = b->n;
    info->pitch = b->pitch;
    info->total_rows = b->total_rows;
    info->total_voxels = b->total_vox;
    info->work_units = b->n_units;
    info->grid = std::max(b->grid, b->grid_fact);
    info->stages = b->stages;
    info->chunk = b->chunk;
    info->smem_bytes = b->smem;
    info->updates = b->updates;
    info->planar = b->planar ? 1 : 0;
    return BPGB_OK;
}

int bpgb_batch_execute(bpgb_batch b, const void *d_H, float *d_volumes, void *stream) {
    clear_error();
    if (!b) return set_error(BPGB_ERR_INVALID_ARGUMENT, "batch is null");
    return batch_execute(b, d_H, d_volumes, (cudaStream_t)stream);
}

int bpgb_batch_graph_launch(bpgb_batch b, const void *d_H, float *d_volumes, void *stream) {
    clear_error();
    if (!b) return set_error(BPGB_ERR_INVALID_ARGUMENT, "batch is null");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->own_stream;
    if (!b->graph || b->graph_H != d_H || b->graph_out != d_volumes) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaStream_t cap = b->own_stream;
        BPGB_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int st = batch_execute(b, d_H, d_volumes, cap);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_error(e, "batch graph capture");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_error(e, "batch graph instantiate");
        b->graph_H = d_H;
        b->graph_out = d_volumes;
    }
    BPGB_CUDA_TRY(cudaGraphLaunch(b->graph, s));
    b->last_stream = s;
    return BPGB_OK;
}

int bpgb_batch_check(bpgb_batch b, uint64_t *violations) {
    clear_error();
    if (!b) return set_error(BPGB_ERR_INVALID_ARGUMENT, "batch is null");
    BPGB_CUDA_TRY(cudaStreamSynchronize(b->last_stream));
    unsigned long long h[2] = {0, 0};
    BPGB_CUDA_TRY(cudaMemcpy(h, b->d_diag, sizeof(h), cudaMemcpyDeviceToHost));
    BPGB_CUDA_TRY(cudaMemset(b->d_diag, 0, sizeof(h)));
    if (violations) *violations = h[1];
    if (h[0]) return set_error(BPGB_ERR_TIMEOUT, std::to_string(h[0]) + " device waits timed out");
    if (h[1]) return set_error(BPGB_ERR_WINDOW, std::to_string(h[1]) + " bins fell outside their window");
    return BPGB_OK;
}

int bpgb_batch_destroy(bpgb_batch b) {
    batch_free(b);
    return BPGB_OK;
}

}  // extern "C"

namespace bpgb {

}  // namespace bpgb

// ==================================================================================
// Allocation-free entry point (bpgb_backproject_noalloc).
//
// For callers that cannot allocate device memory at call time -- code running under a
// custom or pre-sized memory pool, host integrations whose allocator is owned by someone
// else, long-running services that forbid cudaMalloc after start-up.  The call runs the
// same FAST kernel as bpgb_plan_execute (FP32 rows, FP32 sums), but everything it needs
// beyond the caller's input and output buffers lives in one file-scope device array:
// the SPAD / laser tables (built on the GPU from the caller's device pair list), the
// diagnostic counters, and the per-split partial sums.  Nothing is allocated on the
// device or the host heap.
// ==================================================================================
namespace bpgb {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)BPGB_NOALLOC_SCRATCH_BYTES;
constexpr size_t kNoAllocDiagBytes = 256;  // counters; the tables start 256 B in

// Shared by every call of every thread of the process on a given device.  The host
// never names it directly as a pointer: its device address comes from
// cudaGetSymbolAddress (noalloc_scratch_ptr below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch, resolved once per device with that device
// current (the symbol's host-side name is only a stand-in, never a device pointer).
int noalloc_scratch_ptr(unsigned char **out) {
    static std::mutex mu;
    static unsigned char *ptrs[64] = {nullptr};
    int dev = 0;
    BPGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(BPGB_ERR_UNSUPPORTED, "device index >= 64");
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
        ptrs[dev] = static_cast<unsigned char *>(p);
    }
    *out = ptrs[dev];
    return BPGB_OK;
}

}  // namespace
}  // namespace bpgb

using namespace bpgb;

extern "C" int bpgb_backproject_noalloc(const float *d_H, uint32_t T, uint32_t h_pitch,
                                        const bpgb_pair *d_pairs, uint64_t num_lasers,
                                        uint64_t num_spads, int confocal,
                                        const uint32_t *voxels_per_side,
                                        const float *volume_zero_pos, const float *voxel_inc,
                                        float t0, float deltaT, float *d_volume, void *stream) {
    clear_error();
    if (!d_H || !d_pairs || !d_volume || !voxels_per_side || !volume_zero_pos || !voxel_inc)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    if (T == 0 || num_lasers == 0 || num_spads < 2 || (confocal && num_lasers != 1))
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "need T > 0, num_spads >= 2 and num_lasers >= 1 (1 when confocal)");
    const uint32_t pitch = h_pitch ? h_pitch : T;
    if (pitch < T || (pitch * 4ull) % 16 || ((uintptr_t)d_H) % 16)
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "H must be 16-byte aligned with a row pitch that is a multiple of 4");
    if (!std::isfinite(t0) || !(deltaT > 0.0f) || !std::isfinite(deltaT))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "t0 / deltaT must be finite, deltaT > 0");
    const uint64_t P = num_lasers * num_spads;
    if (P >= (1ull << 31) || T >= (1u << 30))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "P or T too large for TMA coordinates");
    const uint64_t tab_bytes = (num_spads + num_lasers) * sizeof(float4);
    if (kNoAllocDiagBytes + tab_bytes > kNoAllocScratchBytes)
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         "lasers + SPADs need " + std::to_string(kNoAllocDiagBytes + tab_bytes) +
                             " bytes of scratch; the no-alloc limit is " +
                             std::to_string(kNoAllocScratchBytes) + " bytes");
    Volume vol{};
    for (int k = 0; k < 3; k++) {
        vol.n[k] = voxels_per_side[k];
        vol.zero[k] = volume_zero_pos[k];
        if (!std::isfinite(vol.zero[k]))
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "volume_zero_pos is not finite");
    }
    for (int k = 0; k < 9; k++) {
        vol.inc[k] = voxel_inc[k];
        if (!std::isfinite(vol.inc[k]))
            return set_error(BPGB_ERR_INVALID_ARGUMENT, "voxel_inc is not finite");
    }
    if (vol.count() == 0) return BPGB_OK;
    double u[3][3], hd[3];
    if (!volume_frame(vol, u, hd))
        return set_error(BPGB_ERR_UNSUPPORTED, "voxel basis is not orthogonal");
    if (!encode_fn()) return set_error(BPGB_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    int sms = 0;
    int st = require_device(&sms);
    if (st) return st;
    unsigned char *scratch = nullptr;
    st = noalloc_scratch_ptr(&scratch);
    if (st) return st;

    // Launch arguments: the default tile preset of the FAST kernel, FP32 rows.
    const FastConfig cfg = fast_preset(-1, BPGB_DTYPE_F32);
    FastArgs a;
    std::string why;
    st = fast_args(a, cfg, vol, hd, confocal != 0, deltaT, t0, num_lasers, num_spads, T, 4, false,
                   0, 0, &why);
    if (st) return set_error(st, why);

    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *diag = reinterpret_cast<unsigned long long *>(scratch);
    float4 *tab = reinterpret_cast<float4 *>(scratch + kNoAllocDiagBytes);
    // The array keeps the previous call's contents: the counters must start at zero.
    BPGB_CUDA_TRY(cudaMemsetAsync(diag, 0, kNoAllocDiagBytes, s));
    // Tables in FP64 from the caller's device pair list (the kernel a plan uses); its
    // checks land in diag[2..4]: pairs out of the stated order, non-finite values, SPADs
    // off the planar wall.
    st = launch_tables(d_pairs, vol, u, (double)deltaT, (double)t0, num_lasers, num_spads,
                       confocal != 0, cfg.kaxis, tab, diag + 2, sms, s);
    if (st) return st;
    // A pair list with non-finite values or another order never reaches the window
    // arithmetic of the main kernel.
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    BPGB_CUDA_TRY(cudaMemcpyAsync(h, diag, sizeof(h), cudaMemcpyDeviceToHost, s));
    BPGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h[3]) return set_error(BPGB_ERR_INVALID_ARGUMENT, std::to_string(h[3]) + " non-finite pair values");
    if (h[2])
        return set_error(BPGB_ERR_INVALID_ARGUMENT,
                         std::to_string(h[2]) + " pairs break the stated lasers x SPADs order");

    // The kernel variant a plan on these pairs runs (the planar-wall form when every SPAD
    // lies on one plane across the voxel lines; the 8-warp build when the preset has 8
    // consumer warps), selected before its occupancy sets the pair splits, as in a plan.
    a.planar = (h[4] == 0 && cfg.k == 8) ? 1 : 0;
    const uint32_t threads = fast_threads(cfg);
    const uint32_t smem = fast_smem(a);
    void *kern = select_kernel(BPGB_DTYPE_F32, false, false, cfg.k, a.planar != 0,
                               cfg.consumer_warps() == 8);
    if (!kern) return set_error(BPGB_ERR_UNSUPPORTED, "default tile preset not built for FP32 rows");
    st = reserve_dynamic_smem(kern, smem);
    if (st) return st;
    int occ = 0;
    BPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, (int)threads, smem));
    if (occ < 1) return set_error(BPGB_ERR_UNSUPPORTED, "fast kernel does not fit on an SM");
    const uint64_t ntiles = (uint64_t)a.tiles[0] * a.tiles[1] * a.tiles[2];
    const uint64_t items = a.L * a.nchunks;
    uint64_t splits = 1;
    const uint64_t want = 2ull * sms * occ;
    if (ntiles < want) splits = (want + ntiles - 1) / ntiles;
    // partial sums must fit next to the tables: fewer splits, never an error
    const uint64_t part_off = (kNoAllocDiagBytes + tab_bytes + 255) / 256 * 256;
    const uint64_t part_room = kNoAllocScratchBytes - std::min<uint64_t>(kNoAllocScratchBytes, part_off);
    const uint64_t max_splits = part_room / (a.nvox * sizeof(float));
    splits = std::max<uint64_t>(1, std::min<uint64_t>({splits, items, max_splits}));
    if (ntiles * splits >= (1ull << 31)) return set_error(BPGB_ERR_UNSUPPORTED, "grid too large");
    a.splits = (uint32_t)splits;
    float *partial = reinterpret_cast<float *>(scratch + part_off);

    CUtensorMap map;
    st = encode_rows(&map, BPGB_DTYPE_F32, d_H, T, P, pitch, a.BW);
    if (st) return st;
    void *target = a.splits > 1 ? (void *)partial : (void *)d_volume;
    const float4 *spads = tab;
    const float4 *lasers = tab + num_spads;
    void *args[] = {(void *)&map, (void *)&spads, (void *)&lasers, (void *)&target, (void *)&diag,
                    (void *)&a};
    BPGB_CUDA_TRY(cudaLaunchKernel(kern, dim3((unsigned)(ntiles * splits)), dim3(threads), args, smem, s));
    count_launches(1);
    if (a.splits > 1) {
        const unsigned blocks = (unsigned)std::min<uint64_t>((a.nvox + 255) / 256, 152ull * 8);
        reduce_splits_kernel<false, false><<<blocks, 256, 0, s>>>(partial, d_volume, a.nvox,
                                                                 a.splits, 1.0f);
        count_launches(1);
        BPGB_CUDA_TRY(cudaGetLastError());
    }
    BPGB_CUDA_TRY(cudaMemcpyAsync(h, diag, sizeof(h), cudaMemcpyDeviceToHost, s));
    BPGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h[0]) return set_error(BPGB_ERR_TIMEOUT, std::to_string(h[0]) + " device waits timed out");
    return BPGB_OK;
}
