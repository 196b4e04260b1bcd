/*
 * backprojector_gb300 -- C ABI of the GB300 (sm_103a) NLOS backprojection engine.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an int
 * status (0 = ok, negative = error; see bpgb_status) and never exits the process.
 * bpgb_last_error() returns a message for the last failure on the calling thread.
 *
 * Reference interfaces replaced (mjgalindo/backprojector):
 *   bpgb_backproject_f32  <- call_cuda_backprojection          backproject_cuda.hpp:19-28
 *                            (implementation backproject_cuda.cu:370-500)
 *   bpgb_backproject_c64  <- call_cuda_complex_backprojection  backproject_cuda.hpp:41-49
 *                            (implementation backproject_cuda.cu:671-801)
 *   bpgb_pair             <- struct CameraLaserPair            backproject_cuda.hpp:9-13
 *   bpgb_plan_*           <- the launch policy of the same launchers, split into a
 *                            reusable plan (geometry analysed once) and an asynchronous,
 *                            stream-ordered execute on device buffers.
 *   bpgb_phasor_pulse     <- bp::phasor_pulse                  backproject.hpp:430-479
 *   bpgb_precompute_pairs <- bp::precompute_distances          backproject.hpp:356-418
 *   bpgb_volume_basis     <- volume basis / voxel_inc          backproject.hpp:820-839
 *   bpgb_time_limits      <- bp::get_time_limits               backproject.hpp:617-674
 *   bpgb_backproject_capture / bpgb_phasor_capture
 *                         <- bp::backproject / bp::phasor_reconstruction
 *                            backproject.hpp:762-909 / 932-1039 (GPU, Naive access)
 *
 * Threading: every call is safe from several host threads on distinct plans and
 * buffers.  A plan must not be executed concurrently with itself.
 */
#ifndef BACKPROJECTOR_GB300_H
#define BACKPROJECTOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BPGB_ABI_VERSION 2

/* One (laser point, SPAD point) pair with its origin-to-wall legs.  Byte layout is the
 * reference's CameraLaserPair: camera point first, 32 bytes. */
typedef struct bpgb_pair {
    float camera_point[3];
    float laser_point[3];
    float camera_wall;
    float laser_wall;
} bpgb_pair;

typedef enum bpgb_status {
    BPGB_OK = 0,
    BPGB_ERR_INVALID_ARGUMENT = -1, /* shapes, NaN geometry, null pointers */
    BPGB_ERR_CUDA = -2,             /* a CUDA runtime call or launch failed */
    BPGB_ERR_OUT_OF_MEMORY = -3,    /* device allocation failed */
    BPGB_ERR_TIMEOUT = -4,          /* a bounded device-side wait gave up */
    BPGB_ERR_UNSUPPORTED = -5,      /* valid request the selected algorithm cannot serve */
    BPGB_ERR_NO_DEVICE = -6,        /* no CUDA device of compute capability 10.3 */
    BPGB_ERR_WINDOW = -7            /* checked mode saw a bin outside its staged window */
} bpgb_status;

/* Storage type of the transient rows H[pair, time]. */
typedef enum bpgb_dtype {
    BPGB_DTYPE_F32 = 0,
    BPGB_DTYPE_F16 = 1,
    BPGB_DTYPE_BF16 = 2,
    BPGB_DTYPE_C64 = 3, /* interleaved (re, im) float pairs */
    BPGB_DTYPE_C32 = 4  /* interleaved (re, im) FP16 pairs with a per-capture scale (FAST
                           only; the volume is complex64).  Half the bytes of complex64:
                           twice the rows per pipeline stage for the wide windows of
                           phasor-field captures. */
} bpgb_dtype;

typedef enum bpgb_algo {
    BPGB_ALGO_AUTO = 0,  /* FAST when the geometry allows it, else EXACT */
    BPGB_ALGO_EXACT = 1, /* the reference's FP32 expression: bin indices bit-identical */
    BPGB_ALGO_FAST = 2   /* factored legs, TMA-staged windows, sqrt.approx */
} bpgb_algo;

typedef enum bpgb_accum {
    BPGB_ACCUM_F32 = 0,  /* plain FP32 running sums */
    BPGB_ACCUM_KAHAN = 1 /* FP32 chunk sums folded with Kahan compensation */
} bpgb_accum;

typedef struct bpgb_options {
    int32_t algo;        /* bpgb_algo */
    int32_t h_dtype;     /* bpgb_dtype */
    int32_t accum;       /* bpgb_accum */
    uint32_t h_pitch;    /* elements between consecutive H rows (0 = T) */
    float h_scale;       /* result multiplier (FP16/BF16 per-capture scale; 0 = 1) */
    int32_t tile;        /* tile preset index (-1 = tuned default); 10-12: small tiles for
                            block-sparse passes, 13: four 8^3 tiles per CTA (real rows,
                            plain sums) */
    int32_t pair_splits; /* CTAs sharing one voxel tile over disjoint pair ranges (0 = auto) */
    int32_t checked;     /* 1 = clamp and count out-of-window bins (tests) */
    uint32_t spin_limit; /* bounded mbarrier waits: polls before giving up (0 = default) */
    int32_t chunk;       /* FAST: SPAD rows per pipeline stage, 1..64 (0 = from the preset;
                            preset 13: per tile, a power of two up to 32) */
    int32_t stages;      /* FAST: pipeline depth, 2..8 (0 = from the preset) */
    int32_t unfactored;  /* FAST, lasers x SPADs captures: 0 = per-voxel laser and SPAD legs
                            computed once per block and reused across the other grid
                            (default where it applies), 1 = the SPAD leg per pair */
    int32_t reserved[4];
} bpgb_options;

/* Read-only description of a plan, for tests, the bench and the autotuner. */
typedef struct bpgb_plan_info {
    int32_t algo;        /* algorithm selected (EXACT or FAST) */
    int32_t geometry;    /* 0 generic, 1 single laser, 2 exhaustive (L x S), 3 confocal */
    uint64_t num_lasers; /* L of the factorisation (P when generic) */
    uint64_t num_spads;  /* S of the factorisation (1 when generic) */
    uint32_t tile[3];    /* voxels per CTA tile along x, y, z */
    uint32_t window;     /* staged time bins per pair and tile (FAST) */
    uint32_t chunk;      /* pairs per pipeline stage (FAST) */
    uint32_t stages;     /* pipeline depth (FAST) */
    uint32_t pair_splits;
    uint32_t grid;       /* CTAs per execute */
    uint32_t threads;    /* threads per CTA */
    uint32_t smem_bytes; /* dynamic shared memory per CTA */
    uint64_t scratch_bytes; /* device scratch held by the plan */
    uint64_t updates;    /* voxel x pair updates per execute */
    uint32_t factored;   /* 1 = lasers x SPADs legs factored (FAST, exhaustive captures) */
    uint32_t reserved;
} bpgb_plan_info;

typedef struct bpgb_plan_s *bpgb_plan;

/* ---- library ----------------------------------------------------------- */
int bpgb_abi_version(void);
const char *bpgb_status_string(int status);
const char *bpgb_last_error(void);
void bpgb_options_default(bpgb_options *opt);
/* Number of kernel launches this process made through the library so far. */
uint64_t bpgb_launch_count(void);

/* ---- drop-in host-buffer calls ------------------------------------------
 * Same arguments and meaning as the reference: caller-owned HOST buffers,
 * transient_size = P * T elements, the voxel volume [Nx, Ny, Nz] (x slowest) is
 * OVERWRITTEN, the call is synchronous on the current device.  Unlike the reference,
 * every pair is used (it skips the last P mod blockDim pairs) and every voxel is
 * visited exactly once for any N (its voxel cursor wraps and recomputes some voxels
 * when N is not a multiple of 16, backproject_cuda.cu:65-80).
 * Algorithm as set by bpgb_set_dropin_algo / BPGB_ALGO (below; default ALGO_AUTO), FP32
 * accumulation.  Replaces backproject_cuda.cu:370-500 / 671-801. */
int bpgb_backproject_f32(const float *transient_chunk, uint64_t transient_size, uint32_t T,
                         const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                         float *voxel_volume, const uint32_t *voxels_per_side,
                         const float *volume_zero_pos, const float *voxel_inc, float t0,
                         float deltaT);
/* transient_chunk and voxel_volume hold interleaved complex64 (re, im). */
int bpgb_backproject_c64(const float *transient_chunk, uint64_t transient_size, uint32_t T,
                         const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                         float *voxel_volume, const uint32_t *voxels_per_side,
                         const float *volume_zero_pos, const float *voxel_inc, float t0,
                         float deltaT);
/* Algorithm of bpgb_backproject_f32 / _c64 (and so of the call_cuda_* C++ drop-in):
 * BPGB_ALGO_AUTO (default: FAST where the pair list factors, else EXACT), BPGB_ALGO_EXACT
 * (the reference kernel's FP32 expression: bins bit-identical to call_cuda_backprojection)
 * or BPGB_ALGO_FAST.  The environment variable BPGB_ALGO=exact|fast|auto sets the initial
 * value, read at the first drop-in call; bpgb_set_dropin_algo overrides it process-wide. */
int bpgb_set_dropin_algo(int algo);
int bpgb_get_dropin_algo(void);
/* As bpgb_backproject_f32/_c64 with explicit options (algo, accumulation). */
int bpgb_backproject_host(const void *transient_chunk, uint64_t transient_size, uint32_t T,
                          const bpgb_pair *scanned_pairs, uint64_t num_pairs,
                          void *voxel_volume, const uint32_t *voxels_per_side,
                          const float *volume_zero_pos, const float *voxel_inc, float t0,
                          float deltaT, const bpgb_options *opt);

/* ---- plans on device buffers --------------------------------------------
 * host_pairs: the pair list on the host (analysed once; copied to the device).
 * execute: d_H is a device array [P, h_pitch] of opt->h_dtype; d_volume is a device
 * float (or interleaved complex64 for C64) array [Nx, Ny, Nz] that is overwritten.
 * Asynchronous on `stream` (a cudaStream_t, NULL = legacy default stream); allocates
 * nothing, so it can be captured in a CUDA graph. */
int bpgb_plan_create(bpgb_plan *plan, const bpgb_pair *host_pairs, uint64_t num_pairs,
                     uint32_t T, const uint32_t *voxels_per_side,
                     const float *volume_zero_pos, const float *voxel_inc, float t0,
                     float deltaT, const bpgb_options *opt);
int bpgb_plan_execute(bpgb_plan plan, const void *d_H, void *d_volume, void *stream);
/* Block-sparse form of bpgb_plan_execute (FAST plans): computes only the voxel tiles
 * listed in device memory, d_tile_list[0 .. *d_tile_count), and leaves every other voxel
 * of d_volume untouched.  max_tiles bounds *d_tile_count and sets the launch size
 * (max_tiles x pair_splits CTAs, or ceil(max_tiles / 4) x pair_splits with tile preset
 * 13's four tiles per CTA; those past the count exit at once; list entries outside the
 * volume are skipped), so the call reads no device value on the host and can be captured
 * in a CUDA graph.  With pair_splits > 1
 * each listed tile's pairs are split over that many CTAs and a second kernel adds the
 * partial sums in split order, exactly as bpgb_plan_execute does, so the listed voxels
 * equal the full execute's bit for bit.  Tile ids follow the plan's tile grid
 * (bpgb_plan_info.tile voxels per tile; id = (ty * tiles_x + tx) * tiles_z + tz). */
int bpgb_plan_execute_tiles(bpgb_plan plan, const void *d_H, void *d_volume,
                            const uint32_t *d_tile_list, const uint32_t *d_tile_count,
                            uint32_t max_tiles, void *stream);
/* Fills the tile list for bpgb_plan_execute_tiles from a score grid of
 * block_size^3-voxel blocks (float [bx, by, bz], x slowest, covering the volume): a tile
 * is listed when any block it overlaps scores above `threshold`.  Zeroes *d_tile_count
 * first (stream-ordered). */
int bpgb_plan_select_tiles(bpgb_plan plan, const float *d_block_score,
                           const uint32_t *block_dims, uint32_t block_size, float threshold,
                           uint32_t *d_tile_list, uint32_t *d_tile_count, void *stream);
/* Budgeted form of bpgb_plan_select_tiles: lists the tiles overlapping the k
 * highest-scoring blocks (blocks tied with the k-th score included; scores are taken as
 * non-negative, NaN as 0).  The k-th score is found on the device (radix selection, one
 * CTA) and kept in the plan, so the call reads nothing on the host and can be captured
 * in a CUDA graph; it zeroes *d_tile_count first and lists nothing when k = 0.  A plan
 * must not run two selections concurrently. */
int bpgb_plan_select_tiles_topk(bpgb_plan plan, const float *d_block_score,
                                const uint32_t *block_dims, uint32_t block_size, uint32_t k,
                                uint32_t *d_tile_list, uint32_t *d_tile_count, void *stream);
/* Synchronises the plan's last stream and reports device-side diagnostics: returns
 * BPGB_ERR_TIMEOUT if a bounded wait gave up, BPGB_ERR_WINDOW if checked mode counted
 * out-of-window bins (count in *violations when non-null), else BPGB_OK. */
int bpgb_plan_check(bpgb_plan plan, uint64_t *violations);
int bpgb_plan_get_info(bpgb_plan plan, bpgb_plan_info *info);
/* Bin indices the plan's algorithm uses for voxels h_voxel_ids[0..n) and every pair:
 * d_bins[i * P + p] (int32, -1 = outside [0, T)).  For parity measurement only. */
int bpgb_plan_dump_bins(bpgb_plan plan, const int64_t *h_voxel_ids, int64_t n,
                        int32_t *d_bins, void *stream);
/* The FAST plan's FP32 tables, built on the GPU in FP64 from the pair list (the values
 * precompute_distances keeps in double, backproject.hpp:356-418, plus the volume frame):
 * num_spads SPAD entries {x, y, z, camera_wall / deltaT} ((camera_wall + laser_wall) /
 * deltaT when confocal), then num_lasers laser entries {x, y, z, laser_wall / deltaT -
 * t0 / deltaT}, positions in the voxel basis' orthonormal frame relative to
 * volume_zero_pos (metres).  Copies min(capacity, count) entries of 4 floats to host_out
 * and the count to *num_entries.  For inspection and tests; BPGB_ERR_UNSUPPORTED for
 * EXACT plans. */
int bpgb_plan_get_tables(bpgb_plan plan, float *host_out, uint64_t capacity,
                         uint64_t *num_entries);
int bpgb_plan_destroy(bpgb_plan plan);

/* ---- FP64 evaluation of listed voxels (measurement) ----------------------------
 * The reference kernel's quantity (backproject_cuda.cu:117-175) in double for the voxels
 * d_voxel_ids[0..n) (linear ids, x slowest): voxel position, both legs, the bin
 * round((d - t0) / deltaT) (half away from zero, kept in [0, T-1]) and the sum over
 * pairs in pair order, every operation separately rounded.  For measuring the FP32
 * paths' error on the GPU (the bench, tests); not a reconstruction path (one thread per
 * voxel, FP64 pipes).  d_H: device rows [P, h_pitch] of float, or interleaved complex64
 * when is_complex (h_pitch 0 = T, in elements); d_pairs: device pair list; d_out: device
 * double[n] (complex: [n][2]).  Asynchronous on `stream`. */
int bpgb_eval_f64_voxels(const void *d_H, int is_complex, uint32_t T, uint32_t h_pitch,
                         const bpgb_pair *d_pairs, uint64_t num_pairs,
                         const uint32_t *voxels_per_side, const float *volume_zero_pos,
                         const float *voxel_inc, float t0, float deltaT,
                         const int64_t *d_voxel_ids, int64_t n, double *d_out, void *stream);

/* ---- allocation-free backprojection ----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory
 * when they reconstruct: services running under a fixed, pre-sized memory pool,
 * host applications whose GPU allocator belongs to another framework, code that must
 * not call cudaMalloc / cudaFree after start-up.  Computes the same volume as a
 * FAST-algorithm plan (FP32 rows, FP32 sums) without allocating anything on the device
 * or the host heap: its working memory (SPAD / laser tables built on the GPU from
 * d_pairs, diagnostic counters, per-split partial sums) is one static device array of
 * BPGB_NOALLOC_SCRATCH_BYTES that every GPU which loads this library holds until the
 * process exits.
 *   d_H       device FP32 rows [P, h_pitch] (h_pitch 0 = T), 16-byte aligned, h_pitch a
 *             multiple of 4; P = num_lasers * num_spads
 *   d_pairs   device pair list in the order p = l * num_spads + s (precompute_distances
 *             order), or confocal (num_lasers = 1, laser point = camera point)
 *   d_volume  device float [Nx, Ny, Nz], overwritten
 * Lists whose tables need more than the array (16 * (num_lasers + num_spads) + 256
 * bytes > BPGB_NOALLOC_SCRATCH_BYTES) are rejected with BPGB_ERR_INVALID_ARGUMENT; for
 * large volumes it uses fewer pair splits so the partial sums fit.  The call is
 * synchronous on `stream`.  The first call on a device resolves the array's device
 * address (cudaGetSymbolAddress) for that device: make it before any stream capture.
 * Every call shares the one array and overwrites it, so calls that overlap on the GPU
 * (other threads, other streams) race: serialise them. */
#define BPGB_NOALLOC_SCRATCH_BYTES (16u << 20)
int bpgb_backproject_noalloc(const float *d_H, uint32_t T, uint32_t h_pitch,
                             const bpgb_pair *d_pairs, uint64_t num_lasers, uint64_t num_spads,
                             int confocal, const uint32_t *voxels_per_side,
                             const float *volume_zero_pos, const float *voxel_inc, float t0,
                             float deltaT, float *d_volume, void *stream);

/* ---- batches: many captures in persistent launches ------------------------------
 * No counterpart in the reference (it reconstructs one capture per call and relaunches
 * a 16^3 grid per 4096 voxels).  A batch holds the geometry of n captures of uneven pair
 * grids, T and volumes.  Their rows are packed into ONE device buffer
 * [total_rows, pitch] (capture c starts at row_offsets[c]; bins T_c..pitch-1 must be
 * zero) of opt->h_dtype (FP32 or FP16; per-capture h_scale multiplies the result), and
 * their volumes into one float buffer (capture c at voxel_offsets[c]).  execute runs
 * every work unit -- (capture, voxel tile, pair range) -- in persistent kernels, longest
 * units first, each CTA taking the next unit from a device work counter that the launch
 * re-arms when it ends: one launch for the captures with per-pair legs, one for the
 * lasers x SPADs captures with factored legs (opt->unfactored = 1: all per pair), then one
 * reduction per capture whose tiles were split over pair ranges (opt->pair_splits > 0
 * fixes the ranges per capture; 0 chooses them from each unit's length against a CTA's
 * share of its launch).  graph_launch captures these launches in a CUDA graph once per
 * (d_H, d_volumes) pair and replays it.  Executes of ONE batch must not overlap
 * (stream-order them): they share the work counters and the partial-sum scratch.  Each
 * capture's pairs must factor as lasers x SPADs or be confocal. */
typedef struct bpgb_capture_geometry {
    const bpgb_pair *pairs; /* host pair list of the capture */
    uint64_t num_pairs;
    uint32_t T;
    uint32_t voxels_per_side[3];
    float volume_zero_pos[3];
    float voxel_inc[9];
    float t0, deltaT;
    float h_scale; /* result multiplier for this capture (FP16 per-capture scale); 0 = 1 */
} bpgb_capture_geometry;

typedef struct bpgb_batch_info {
    uint32_t captures;
    uint32_t pitch;       /* elements per packed row */
    uint64_t total_rows;  /* rows of the packed H */
    uint64_t total_voxels;
    uint32_t work_units;  /* (capture, voxel tile, pair range) units over all captures */
    uint32_t grid;        /* persistent CTAs of the larger launch */
    uint32_t stages, chunk, smem_bytes; /* the per-pair launch's ring (else the factored) */
    uint64_t updates;     /* voxel x pair updates per execute */
    int32_t planar;       /* the planar-wall kernel variant runs */
} bpgb_batch_info;

typedef struct bpgb_batch_s *bpgb_batch;

int bpgb_batch_create(bpgb_batch *batch, const bpgb_capture_geometry *captures, uint32_t n,
                      const bpgb_options *opt);
/* row_offsets / voxel_offsets: n entries each (either may be NULL). */
int bpgb_batch_layout(bpgb_batch batch, uint64_t *row_offsets, uint64_t *voxel_offsets);
int bpgb_batch_get_info(bpgb_batch batch, bpgb_batch_info *info);
int bpgb_batch_execute(bpgb_batch batch, const void *d_H, float *d_volumes, void *stream);
int bpgb_batch_graph_launch(bpgb_batch batch, const void *d_H, float *d_volumes, void *stream);
/* Synchronises and reports device diagnostics like bpgb_plan_check. */
int bpgb_batch_check(bpgb_batch batch, uint64_t *violations);
int bpgb_batch_destroy(bpgb_batch batch);

/* ---- FP16 / BF16 row storage -------------------------------------------------------
 * *d_max (device float) = max |H| over rows x T (NaN counts as +inf); rows of `pitch`.
 * bpgb_rows_to_half: d_out[r][t] = H[r][t] / s as FP16 or BF16 (dtype), bins
 * T..out_pitch-1 zero, with s = scale, or s = *d_absmax / target read on the device when
 * d_absmax is non-null (so a capture is scaled without a host round trip).  A FAST plan
 * then either takes h_scale = s, or runs with h_scale = 1 and bpgb_volume_scale
 * (same s arguments) multiplies the volume back. */
int bpgb_rows_absmax(const float *d_H, uint64_t rows, uint32_t T, uint32_t pitch,
                     float *d_max, void *stream);
int bpgb_rows_to_half(const float *d_H, uint64_t rows, uint32_t T, uint32_t in_pitch, float scale,
                      const float *d_absmax, float target, int dtype, void *d_out,
                      uint32_t out_pitch, void *stream);
int bpgb_volume_scale(float *d_volume, uint64_t n, float scale, const float *d_absmax,
                      float target, void *stream);

/* ---- learned octree: block scores, fill, occupancy CNN ---------------------------
 * Replace the reference's threshold octree (octree_volume.hpp:18-198,
 * backproject.hpp:264-335; GPU backproject_cuda.cu:183-367, 503-669, which prints "NOT
 * WORKING YET"): a coarse dense pass feeds a small 3D CNN that scores 8^3-voxel blocks
 * of the fine volume; bpgb_plan_select_tiles + bpgb_plan_execute_tiles run the fine
 * pass on the scored blocks only.  Volumes are float [n0, n1, n2], x slowest. */

/* out[b] = max of d_volume over block b (block_size^3 voxels, edge blocks clipped);
 * out is float [ceil(n0/bs), ceil(n1/bs), ceil(n2/bs)]. */
int bpgb_block_max(const float *d_volume, const uint32_t *voxels_per_side, uint32_t block_size,
                   float *d_out, void *stream);
/* d_out[v] = sum over v's in-volume face neighbours u of (vol[v] - vol[u]): the negated
 * 7-point Laplacian filter (positive at local maxima, the usual sharpening of
 * unfiltered backprojections).  d_out must not alias d_volume. */
int bpgb_laplacian7(const float *d_volume, const uint32_t *voxels_per_side, float *d_out,
                    void *stream);
/* d_out[i] = |d_in[i]| for n interleaved complex64 values (block scores of phasor
 * volumes). */
int bpgb_complex_abs(const float *d_in, uint64_t n, float *d_out, void *stream);
/* d_fine = trilinear interpolation of d_coarse, both grids spanning one box with spacing
 * size / (n - 1) (the reference's voxel_inc, backproject.hpp:834-839). */
int bpgb_upsample_trilinear(const float *d_coarse, const uint32_t *coarse_dims, float *d_fine,
                            const uint32_t *fine_dims, void *stream);
/* Per-block predictor of the trilinear fill's error: for each block_size^3 block of the
 * fine grid (float [ceil(f/bs)...], x slowest), the mean over samples^3 evenly spread
 * voxels of (fill_hi - fill_lo)^2, where fill_* is the trilinear interpolation of two
 * coarse passes over the same box (d_coarse_lo coarser than d_coarse_hi).  When d_logits
 * (one per block) is given, blocks with logit >= logit_lo score +inf, so that
 * bpgb_plan_select_tiles_topk takes the occupancy model's blocks first. */
int bpgb_block_detail(const float *d_coarse_lo, const uint32_t *lo_dims, const float *d_coarse_hi,
                      const uint32_t *hi_dims, const uint32_t *fine_dims, uint32_t block_size,
                      uint32_t samples, const float *d_logits, float logit_lo, float *d_score,
                      void *stream);

/* Occupancy CNN kernels: 3x3x3 convolutions, zero padding, BF16 activations and weights,
 * FP32 accumulation on the tensor cores (mma.sync m16n8k16).  Activations are
 * channels-last BF16 [batch * n0 * n1 * n2][stride].  A layer with cin inputs has
 * K = 27 cin + 1 GEMM rows padded to bpgb_cnn_kp(cin): row t * cin + c = tap t
 * (offsets t/9-1, t/3%3-1, t%3-1 along x, y, z), input channel c; row 27 cin = bias.
 * Weights: FP32 master W[kp][cout]; packed BF16 Wt[np][kp] (np = cout padded to 8/16)
 * and, for the backward-data pass, Wb[np_back][kp(cout)] (taps flipped, channels
 * transposed, no bias) from bpgb_cnn_pack_weights.
 * conv3d: Y = act(conv(X, W)) with act = ReLU when relu != 0, then, when d_mask is set,
 * Y[v][c] = 0 wherever mask[v][c] <= 0 (ReLU backward); d_Y BF16 [V][np] and/or d_Yf =
 * channel 0 in FP32 [V].  (cin, np) in {(1,16), (2,16), (16,16), (16,8)}. */
uint32_t bpgb_cnn_kp(uint32_t cin);
int bpgb_cnn_conv3d(const void *d_X, uint32_t cin, uint32_t x_stride, const uint32_t *dims,
                    uint32_t batch, const void *d_Wt, uint32_t np, int relu, const void *d_mask,
                    uint32_t mask_stride, void *d_Y, float *d_Yf, void *stream);
/* dW[kp][cout] (FP32) = sum over voxels of im2col(X) x dY (dY BF16 [V][np]); partial
 * sums per 2048 voxels in d_scratch, reduced in a fixed order (deterministic). */
uint64_t bpgb_cnn_wgrad_scratch_bytes(uint32_t cin, uint32_t np, const uint32_t *dims,
                                      uint32_t batch);
int bpgb_cnn_conv3d_wgrad(const void *d_X, uint32_t cin, uint32_t x_stride, const uint32_t *dims,
                          uint32_t batch, const void *d_dY, uint32_t np, uint32_t cout,
                          float *d_scratch, uint64_t scratch_bytes, float *d_dW, void *stream);
int bpgb_cnn_pack_weights(const float *d_W, uint32_t cin, uint32_t cout, uint32_t np,
                          void *d_Wt, uint32_t np_back, void *d_Wb, void *stream);
/* BCE with logits: dZ[v][0..7] = (w (sigmoid(z) - y) scale, 0, ..., 0) BF16 (16-byte rows),
 * w = pos_weight where y = 1; d_loss (optional) = w (softplus(z) - y z) scale per v. */
int bpgb_cnn_bce_grad(const float *d_logits, const uint8_t *d_labels, uint64_t n,
                      float pos_weight, float scale, void *d_dZ, float *d_loss, void *stream);
/* Adam (bias-corrected, step >= 1) on FP32 parameters. */
int bpgb_cnn_adam(float *d_p, const float *d_g, float *d_m, float *d_v, uint64_t n, float lr,
                  float beta1, float beta2, float eps, uint32_t step, void *stream);
/* d_X (BF16 [batch * n0 n1 n2]) = each sample of d_coarse divided by its maximum. */
int bpgb_cnn_normalize(const float *d_coarse, const uint32_t *dims, uint32_t batch, void *d_X,
                       void *stream);
/* Two input channels per voxel, d_X BF16 [batch * n0 n1 n2][2]: the sample divided by
 * its maximum, and its negated 7-point Laplacian (as bpgb_laplacian7) divided by its
 * largest magnitude.  d_scratch (2 x batch floats, overwritten) lets the maxima be
 * reduced across the whole GPU; NULL reduces each sample in one CTA (slower). */
int bpgb_cnn_features(const float *d_coarse, const uint32_t *dims, uint32_t batch, void *d_X,
                      float *d_scratch, void *stream);

/* ---- occupancy CNN on the tcgen05 tensor cores (the training step) ------------------
 * Line-planes tensors: volumes of dims = {n0, n1, 32} (n1 a multiple of 8) per sample,
 * rows of 16 bytes holding 8 BF16 channels (1 plane for <= 8 channels, 2 for <= 16),
 *   row(s, x', y', h, z') = (((s (n0+2) + x') (n1+2) + y') planes + h) (32 + 2 zpad) + z'
 * with x' = x + 1, y' = y + 1, z' = z + zpad, and zero lines after the last sample.  The
 * caller allocates bpgb_cnn_lp_bytes and clears the buffer once: padding rows must stay
 * zero, and the kernels write interior rows only.  Forward inputs (activations) use
 * zpad = 0, backward inputs (gradients) zpad = 1.  Weights are the FP32 masters [KP][COUT]
 * of bpgb_cnn_conv3d (row t cin + ci, bias row 27 cin), packed per call site into
 * tensor-core images of bpgb_cnn_tc_weight_bytes(input channels). */
uint64_t bpgb_cnn_lp_bytes(uint32_t channels, uint32_t zpad, const uint32_t *dims,
                           uint32_t batch);
uint64_t bpgb_cnn_tc_weight_bytes(uint32_t in_channels);
/* Interior rows from / to channels-last BF16 [V][x_stride] (V = batch n0 n1 32). */
int bpgb_cnn_lp_pack(const void *d_X, uint32_t channels, uint32_t x_stride, const uint32_t *dims,
                     uint32_t batch, uint32_t zpad, void *d_lp, void *stream);
int bpgb_cnn_lp_unpack(const void *d_lp, uint32_t channels, uint32_t zpad, const uint32_t *dims,
                       uint32_t batch, void *d_X, void *stream);
/* Forward image (cin inputs) into d_Wf; backward-data image (cout inputs, taps flipped,
 * channels transposed) into d_Wb when non-null. */
int bpgb_cnn_tc_pack_weights(const float *d_W, uint32_t cin, uint32_t cout, void *d_Wf,
                             void *d_Wb, void *stream);
/* bpgb_cnn_tc_pack_weights for `layers` (<= 8) layers in one launch: host arrays of the
 * layers' masters, channel counts and image pointers (d_Wb or its entries may be null). */
int bpgb_cnn_tc_pack_layers(const float *const *d_W, const uint32_t *cin, const uint32_t *cout,
                            void *const *d_Wf, void *const *d_Wb, uint32_t layers, void *stream);
/* 3x3x3 convolution, zero padding: Y = act(conv(X) + bias) on the tensor cores.  d_bias
 * (out_channels FP32, or null), relu, d_mask (an activation-layout tensor of out_channels:
 * outputs where mask <= 0 are zeroed -- the ReLU derivative of the backward pass), d_Y
 * (out_channels, out_zpad) and/or d_Yf (channel 0 as FP32 [V]). */
int bpgb_cnn_tc_conv3d(const void *d_X, uint32_t in_channels, uint32_t in_zpad,
                       const uint32_t *dims, uint32_t batch, const void *d_W, const float *d_bias,
                       uint32_t out_channels, int relu, const void *d_mask, void *d_Y,
                       uint32_t out_zpad, float *d_Yf, void *stream);
/* dW [bpgb_cnn_kp(in_channels)][out_channels] (FP32, bias row 27 in_channels, padding rows
 * zero) of activation d_X (zpad 0) and output gradient d_dY (zpad 1). */
uint64_t bpgb_cnn_tc_wgrad_scratch_bytes(uint32_t in_channels, const uint32_t *dims,
                                         uint32_t batch);
int bpgb_cnn_tc_conv3d_wgrad(const void *d_X, uint32_t in_channels, const void *d_dY,
                             uint32_t out_channels, const uint32_t *dims, uint32_t batch,
                             float *d_scratch, uint64_t scratch_bytes, float *d_dW, void *stream);
/* bpgb_cnn_bce_grad writing dZ as a single-plane gradient (zpad 1); logits and labels [V]. */
int bpgb_cnn_tc_bce_grad(const float *d_logits, const uint8_t *d_labels, const uint32_t *dims,
                         uint32_t batch, float pos_weight, float scale, void *d_dZ, float *d_loss,
                         void *stream);
/* Synchronises the device and reads the tensor-core kernels' timeout bits (0 = none);
 * clears them when reset != 0. */
int bpgb_cnn_tc_status(uint32_t *status, int reset);

/* ---- learned octree as one native object --------------------------------------------
 * Replaces the reference's octree entry (call_cuda_octree_backprojection,
 * backproject_cuda.hpp:30-39, whose GPU implementation backproject_cuda.cu:503-669 prints
 * "NOT WORKING YET"; the CPU threshold octree backproject.hpp:264-335).  Per reconstruct,
 * on `stream`: (FP16 mode) scale and store the rows as FP16 on the device; the FAST pass
 * on the 8x coarser grid over the same box; the occupancy CNN (weights from an .npz written
 * by backprojector_gb300.octree_train: w0..w3 [kp][cout] FP32, in_channels, p_lo); the
 * trilinear fill of the whole volume; a full-resolution pass over the 8^3 blocks scoring
 * p >= p_lo (tile list, pair splits); the FP16 scale undone.  voxels_per_side must be
 * multiples of 8 (>= 16); d_H holds FP32 rows of pitch T.  opt: h_dtype F32 or F16
 * (opt = NULL: FP16 rows), tile (-1: 8^3 tiles), pair_splits (0: 8), chunk, stages.  p_lo <= 0
 * takes the weights file's.  Buffers are allocated at create; reconstruct allocates
 * nothing and reads no device value on the host. */
typedef struct bpgb_octree_info {
    uint32_t fine[3], coarse[3], tile[3];
    uint32_t tiles;        /* fine tiles in the volume */
    uint32_t in_channels;  /* CNN input channels (1 or 2) */
    uint32_t pair_splits;
    int32_t h_dtype;
    float p_lo;
    uint64_t scratch_bytes; /* device memory held */
} bpgb_octree_info;

typedef struct bpgb_octree_s *bpgb_octree;

int bpgb_octree_create(bpgb_octree *octree, const bpgb_pair *host_pairs, uint64_t num_pairs,
                       uint32_t T, const uint32_t *voxels_per_side, const float *volume_zero_pos,
                       const float *voxel_inc, float t0, float deltaT, const char *weights_path,
                       float p_lo, const bpgb_options *opt);
int bpgb_octree_reconstruct(bpgb_octree octree, const float *d_H, float *d_volume, void *stream);
/* Synchronous form on host buffers (H [P][T] FP32, volume [Nx, Ny, Nz]); the first call
 * allocates the device copies, later calls reuse them. */
int bpgb_octree_reconstruct_host(bpgb_octree octree, const float *h_H, float *h_volume);
/* Synchronises the last reconstruct's stream; *tiles = fine tiles it computed. */
int bpgb_octree_selected(bpgb_octree octree, uint32_t *tiles);
int bpgb_octree_get_info(bpgb_octree octree, bpgb_octree_info *info);
int bpgb_octree_destroy(bpgb_octree octree);

/* ---- autotuner -------------------------------------------------------------------
 * No counterpart in the reference (its launch shape is fixed: 16^3 voxels per launch,
 * the largest power-of-two block not above the pair count).  Times FAST configurations
 * on the caller's device buffers (contents are read, results are overwritten) on
 * `stream`, in three stages: every tile preset at its own chunk and depth; chunk
 * {16,32,64} x depth {2,3,4} on the two fastest presets; pair splits {1,2,4} on the
 * winner (plans only).  The winner is re-run with bin-window checking; a candidate
 * that puts any bin outside its window is never chosen.  On return opt->tile, chunk,
 * stages and pair_splits hold the choice (and opt->algo = FAST for plans); the other
 * fields of *opt (row type, accumulation, pitch, scale) are inputs.  Choices are cached
 * per device and workload shape for the life of the process (a cache hit times
 * nothing); bpgb_tune_cache_save / _load persist the cache as a text file. */
typedef struct bpgb_tune_report {
    uint32_t candidates; /* configurations timed (0 on a cache hit) */
    uint32_t cache_hit;
    float default_ms;    /* the untuned first preset at its own chunk/depth (-1: not run) */
    float best_ms;       /* the choice, ms per execute */
    int32_t tile, chunk, stages, pair_splits;
} bpgb_tune_report;

int bpgb_plan_autotune(const bpgb_pair *host_pairs, uint64_t num_pairs, uint32_t T,
                       const uint32_t *voxels_per_side, const float *volume_zero_pos,
                       const float *voxel_inc, float t0, float deltaT, const void *d_H,
                       void *d_volume, bpgb_options *opt, bpgb_tune_report *report,
                       void *stream);
int bpgb_batch_autotune(const bpgb_capture_geometry *captures, uint32_t n, const void *d_H,
                        float *d_volumes, bpgb_options *opt, bpgb_tune_report *report,
                        void *stream);
int bpgb_tune_cache_save(const char *path);
/* Merges the file's entries into the cache; a missing file is not an error. */
int bpgb_tune_cache_load(const char *path);
int bpgb_tune_cache_clear(void);
int bpgb_tune_cache_size(void);

/* Failure-path probe: a one-warp kernel waits, with the pipeline's bounded wait, on an
 * mbarrier that nothing arrives on.  Returns BPGB_ERR_TIMEOUT once `spin_limit` polls ran
 * out (the device stays usable), so callers and tests can check the timeout path. */
int bpgb_diag_wait_timeout(uint32_t spin_limit);

/* Measured per-SM, per-clock throughput on the current device of: rates[0] rsqrt.approx
 * results (XU pipe), rates[1] FP32 lanes of packed FP32x2 FMAs, rates[2] conflict-free
 * 32-bit shared-memory loads.  The roofline of the FAST update is derived from these. */
int bpgb_diag_pipe_rates(double *rates);
/* MUFU (special-function unit) results per SM per clock, measured one operation at a
 * time on the current device: rates[0] rsqrt.approx with 8 independent chains per
 * thread, [1] rsqrt.approx with 16, [2] ex2.approx, [3] sqrt.approx, [4] rcp.approx,
 * [5] sin.approx (the first n of them).  For the roofline of the FAST kernel, whose
 * update costs one rsqrt. */
int bpgb_diag_mufu_rates(double *rates, int n);

/* Known-answer probe of the tensor-core path (tcgen05.mma kind::f16, BF16 operands, FP32
 * accumulate): one CTA copies the 48 KB host image `h_image` into shared memory, issues
 * params[9] MMAs (K = 16 each) whose descriptors are built from params = {a_off, a_lbo,
 * a_sbo, a_kstep, b_off, b_lbo, b_sbo, b_kstep, idesc, nk, ncols} (byte offsets into the
 * image; MMA k adds k * kstep to the start), and writes the accumulator's 128 lanes x
 * ncols FP32 columns to h_out (row-major).  Every stride combination is checked to stay
 * inside the CTA's 96 KB of shared memory before the launch.  *h_status: bit 0 = the
 * commit wait ran out.  Pins the descriptor and accumulator layouts the CNN kernels use. */
int bpgb_diag_umma_probe(const void *h_image, uint32_t image_bytes, const uint32_t *params,
                         float *h_out, uint32_t *h_status);
/* Cycles per tcgen05.mma (BF16, K = 16) issued back to back by one thread on each SM over
 * independent accumulators, operands in shared memory: cycles[0] M128 N48 MN-major, [1]
 * M64 N48 MN-major, [2] M128 N48 K-major, [3] M128 N96, [4] M128 N128, [5] M128 N256
 * (K-major) -- the first n of them.  The issue floor of the CNN kernels' small MMAs. */
int bpgb_diag_umma_issue_rates(double *cycles, int n);

/* ---- phasor pulse --------------------------------------------------------
 * d_out[r, t] = sum_k d_H[r, t + k - K/2] * (cos_k, sin_k), read index in (0, T), with
 * K = int(times * wavelength / deltaT) taps built as the reference does (FP64 Gaussian
 * and phase, rounded to FP32).  d_H: float [rows, in_pitch]; d_out: interleaved
 * complex64 [rows, out_pitch].  Asynchronous on stream; the first call for a given
 * (wavelength, deltaT, times) on a device uploads the taps once (a small synchronous
 * allocation kept until exit), later calls allocate nothing. */
int bpgb_phasor_pulse(const float *d_H, uint64_t rows, uint32_t T, uint32_t in_pitch,
                      float wavelength, float deltaT, uint32_t times, float *d_out,
                      uint32_t out_pitch, void *stream);
/* The K taps (cos then sin, 2*K floats) of the pulse; returns K (taps may be NULL). */
int bpgb_phasor_taps(float wavelength, float deltaT, uint32_t times, float *taps, int cap);

/* ---- geometry ------------------------------------------------------------
 * Pair list and wall legs computed on the GPU in FP64 (rounded to FP32 fields).
 * Grids are host arrays [gx, gy, 3] row-major.  confocal != 0: P = cx*cy and the
 * laser point is the camera point.  out_pairs: host array of P pairs. */
int bpgb_precompute_pairs(const float *laser_position, const float *laser_grid, uint32_t lx,
                          uint32_t ly, const float *camera_position, const float *camera_grid,
                          uint32_t cx, uint32_t cy, int confocal, bpgb_pair *out_pairs);
/* zero = position - size/2; inc rows = axis * size / (n - 1) with axes x, y, z (or the
 * wall-aligned basis y = -normal, x = y cross z, z = y cross x when wall_normal != 0). */
int bpgb_volume_basis(const float *volume_position, const float *volume_size,
                      const uint32_t *voxels_per_side, const float *wall_normal,
                      float *volume_zero_pos, float *voxel_inc);
/* First and last time index any voxel can reach, +-100 bins, as fractional indices.
 * Bounds over every laser and camera grid point and the whole volume box (the reference,
 * backproject.hpp:617-674, takes corners only, which can miss the shortest paths). */
int bpgb_time_limits(const float *laser_position, const float *laser_grid, uint32_t lx,
                     uint32_t ly, const float *camera_position, const float *camera_grid,
                     uint32_t cx, uint32_t cy, const float *volume_position,
                     const float *volume_size, float t0, float deltaT, float *min_index,
                     float *max_index);
/* The reference's own bound (get_time_limits, backproject.hpp:617-674): distances
 * between the 4 corner points of each grid, the origins and the 8 corners of the volume
 * box, in FP64 per distance, summed in FP32, minus t0, over deltaT, padded by 100 bins.
 * Corners can miss the shortest paths through interior grid points, which the padding
 * usually covers.  The reference transposes the camera grid first in the row-major case
 * (:651-652); under xtensor's slicing rules that does not select the grid's corner
 * points, and xtensor is not available to reproduce it, so the grid's own 4 corners are
 * taken.  Selected in the capture calls by t0_mode + 4. */
int bpgb_time_limits_corners(const float *laser_position, const float *laser_grid, uint32_t lx,
                             uint32_t ly, const float *camera_position, const float *camera_grid,
                             uint32_t cx, uint32_t cy, const float *volume_position,
                             const float *volume_size, float t0, float deltaT, float *min_index,
                             float *max_index);

/* ---- time window on device-resident captures ------------------------------
 * The window bp::backproject / bp::phasor_reconstruction crop a capture to
 * (get_time_limits + get_transient_chunk, backproject.hpp:617-740): original bins
 * [*from, *from + *len) (from may be negative: zero-padded) and the chunk's t0 for
 * t0_mode 0 (dense, the reference's unfloored offset, :847), 1 (floored offset) or 2
 * (phasor: limits truncated to int, :962); adding 4 takes the limits from the reference's
 * corner bound (bpgb_time_limits_corners) instead of the bound over every grid point
 * (bpgb_time_limits).  bpgb_rows_crop copies that window of device
 * rows [rows][in_pitch] into [rows][out_pitch] (zeros outside [0, T) and past len) on
 * `stream`, so a device-resident capture is cropped without a host round trip; a plan
 * with T = len, h_pitch = out_pitch and t0 = *chunk_t0 then reproduces
 * bpgb_backproject_capture. */
int bpgb_capture_window(const float *camera_grid, uint32_t cx, uint32_t cy,
                        const float *laser_grid, uint32_t lx, uint32_t ly,
                        const float *camera_position, const float *laser_position, float t0,
                        float deltaT, int confocal, const float *volume_position,
                        const float *volume_size, int t0_mode, int64_t *from, uint32_t *len,
                        float *chunk_t0);
int bpgb_rows_crop(const float *d_in, uint64_t rows, uint32_t T, uint32_t in_pitch, int64_t from,
                   uint32_t len, float *d_out, uint32_t out_pitch, void *stream);

/* ---- whole reconstructions (host buffers) --------------------------------
 * bp::backproject / bp::phasor_reconstruction on the GPU: time-window crop, FP64 pair
 * precompute, basis, then the backprojection.  transient_data is row-major
 * [lx, ly, cx, cy, T] (exhaustive) or [cx, cy, T] (confocal).  t0_mode 0 keeps the
 * reference's fractional chunk offset (chunked_t0 = t0 + m*deltaT with m unfloored),
 * 1 uses the floored offset (no sub-bin shift); + 4 takes m from the reference's corner
 * bound (t0_mode 4: the reference's semantics, 5: its corners with the floored offset).
 * Output [Nx, Ny, Nz] float, or
 * interleaved complex64 for the phasor call. */
int bpgb_backproject_capture(const float *transient_data, uint32_t T,
                             const float *camera_grid, uint32_t cx, uint32_t cy,
                             const float *laser_grid, uint32_t lx, uint32_t ly,
                             const float *camera_position, const float *laser_position,
                             float t0, float deltaT, int confocal,
                             const float *volume_position, const float *volume_size,
                             const uint32_t *voxels_per_side, const float *wall_normal,
                             int t0_mode, const bpgb_options *opt, float *out_volume);
int bpgb_phasor_capture(const float *transient_data, uint32_t T, const float *camera_grid,
                        uint32_t cx, uint32_t cy, const float *laser_grid, uint32_t lx,
                        uint32_t ly, const float *camera_position, const float *laser_position,
                        float t0, float deltaT, int confocal, const float *volume_position,
                        const float *volume_size, const uint32_t *voxels_per_side,
                        const float *wall_normal, float wavelength, const bpgb_options *opt,
                        float *out_volume);

#ifdef __cplusplus
}
#endif

#endif /* BACKPROJECTOR_GB300_H */
