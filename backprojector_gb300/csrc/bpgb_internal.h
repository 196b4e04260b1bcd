// Internal declarations shared by the host-side translation units of libbpgb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "backprojector_gb300.h"

namespace bpgb {

// ---- errors -----------------------------------------------------------------
int set_error(int status, const std::string &msg);  // records msg, returns status
int cuda_error(cudaError_t e, const char *what);    // maps a CUDA error to a status
void clear_error();
void count_launches(uint64_t n);

#define BPGB_CUDA_TRY(expr)                                   \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return ::bpgb::cuda_error(e_, #expr); \
    } while (0)

// Checks that a GB300-class device (compute capability 10.x) is current.
int require_device(int *sm_count = nullptr);

// cuTensorMapEncodeTiled from the driver (looked up once, no libcuda link needed), or
// null when the driver does not provide it.
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion,
                                   CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();

// Raises (never lowers) a kernel's dynamic shared memory limit on the current device to
// at least `bytes`.  Plans and batches that share a kernel function stay launchable
// whatever order they were created in.
int reserve_dynamic_smem(const void *kernel, uint32_t bytes);

// ---- volume description -------------------------------------------------------
struct Volume {
    uint32_t n[3];
    float zero[3];
    float inc[9];  // rows: x step, y step, z step
    uint64_t count() const { return (uint64_t)n[0] * n[1] * n[2]; }
};

struct BinParams {
    float t0;
    float dT;
    uint32_t T;
};

// ---- exact kernels (bp_exact.cu) ----------------------------------------------
// H rows of `pitch` elements, float or interleaved complex64 (is_complex).
int launch_exact(const void *d_H, bool is_complex, uint64_t pitch, const bpgb_pair *d_pairs,
                 uint64_t P, const Volume &vol, const BinParams &bp, void *d_out,
                 cudaStream_t stream);
int launch_exact_bins(const bpgb_pair *d_pairs, uint64_t P, const Volume &vol,
                      const BinParams &bp, const int64_t *d_ids, int64_t n, int32_t *d_bins,
                      cudaStream_t stream);

// ---- geometry analysis (plan.cpp) ---------------------------------------------
enum Geometry { GEOM_GENERIC = 0, GEOM_SINGLE_LASER = 1, GEOM_EXHAUSTIVE = 2, GEOM_CONFOCAL = 3 };

struct Factorization {
    Geometry geom = GEOM_GENERIC;
    uint64_t L = 0, S = 0;  // pairs p = l * S + s
};
Factorization factorize_pairs(const bpgb_pair *pairs, uint64_t P);

// Orthonormal frame of the voxel basis: rows u[0..2] and the step lengths h[0..2].
// Returns false when the basis is not orthogonal (then only EXACT applies).
bool volume_frame(const Volume &vol, double u[3][3], double h[3]);

// Every pair value, the volume origin / steps, t0 and deltaT are finite (deltaT != 0);
// otherwise *why names the first offender.
bool finite_geometry(const bpgb_pair *pairs, uint64_t P, const Volume &vol,
                     const BinParams &bp, std::string *why);

// ---- fast kernels (bp_fast.cu) ------------------------------------------------
struct FastConfig {
    // lane layout inside a warp (product 32), voxels per thread (k) on a line along
    // axis `kaxis`, consumer warp layout
    uint32_t lx, ly, lz, k, wx, wy, wz, kaxis;
    uint32_t chunk;   // SPAD rows per pipeline stage and tile (<= 64 / groups)
    uint32_t stages;  // pipeline depth
    uint32_t groups = 1;  // tiles per CTA, each with its own wx x wy x wz consumer warps
    uint32_t tile(int a) const {
        const uint32_t l = a == 0 ? lx : (a == 1 ? ly : lz);
        const uint32_t w = a == 0 ? wx : (a == 1 ? wy : wz);
        return l * w * ((uint32_t)a == kaxis ? k : 1);
    }
    uint32_t consumer_warps() const { return wx * wy * wz; }  // per tile
    uint32_t cta_consumer_warps() const { return wx * wy * wz * groups; }
};

// Tile presets; index -1 selects the tuned default for the geometry.
FastConfig fast_preset(int index, int dtype);
int fast_preset_count();

struct FastPlan;  // opaque, defined in bp_fast.cu
// Tables are built on the GPU in FP64 from the plan's device pair list d_pairs (the
// host list was already factorised into fz).
int fast_plan_build(FastPlan **out, const bpgb_pair *d_pairs, uint64_t P,
                    const Factorization &fz, const Volume &vol, const BinParams &bp,
                    const bpgb_options &opt, int sm_count, std::string *why_not);
int fast_plan_execute(FastPlan *fp, const void *d_H, void *d_out, cudaStream_t stream);
int fast_plan_dump_bins(FastPlan *fp, const int64_t *d_ids, int64_t n, int32_t *d_bins,
                        cudaStream_t stream);
int fast_plan_execute_tiles(FastPlan *fp, const void *d_H, void *d_out, const uint32_t *d_list,
                            const uint32_t *d_count, uint32_t max_tiles, cudaStream_t stream);
int fast_plan_select_tiles(FastPlan *fp, const float *d_score, const uint32_t *block_dims,
                           uint32_t block_size, float threshold, uint32_t *d_list,
                           uint32_t *d_count, cudaStream_t stream);
int fast_plan_select_tiles_topk(FastPlan *fp, const float *d_score, const uint32_t *block_dims,
                                uint32_t block_size, uint32_t k, uint32_t *d_list,
                                uint32_t *d_count, cudaStream_t stream);
void fast_plan_info(const FastPlan *fp, bpgb_plan_info *info);
int fast_plan_tables(const FastPlan *fp, float *host_out, uint64_t capacity, uint64_t *count);
int fast_plan_check(FastPlan *fp, uint64_t *violations, uint64_t *timeouts);
void fast_plan_free(FastPlan *fp);
int wait_timeout_probe(uint32_t limit, int *timed_out);

// ---- phasor (phasor.cu) -------------------------------------------------------
int launch_phasor_pulse(const float *d_H, uint64_t rows, uint32_t T, uint32_t in_pitch,
                        const float *h_taps, int K, float *d_out, uint32_t out_pitch,
                        cudaStream_t stream);

// ---- geometry kernels (geometry.cu) -------------------------------------------
int launch_pairs_fp64(const float *d_laser_grid, uint32_t lx, uint32_t ly,
                      const float *d_camera_grid, uint32_t cx, uint32_t cy,
                      const double *laser_pos, const double *camera_pos, int confocal,
                      bpgb_pair *d_out, cudaStream_t stream);

// ---- device memory cache for the host-buffer entry points ----------------------
// Grow-only per-thread buffers reused across calls (avoids cudaMalloc per call).
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t need);
    ~DeviceBuffer();
};

}  // namespace bpgb
