/*
 * CPU oracle for the NLOS backprojection hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library, and only as the checker (or as the timed CPU baseline of the
 * reference's OpenMP path).  The product path never calls it.
 *
 * Parity pins: the reference ships no tests or golden vectors.  The oracle is pinned
 * against outputs of the reference's own GPU kernel (backproject_cuda.cu built from its
 * sources for sm_103a and run on a GB300), committed as fixtures under tests/golden/.
 *
 * Restated functions (reference file:line):
 *   orc_bp_gpu_f64 / orc_bp_gpu_c64  -- cuda_backprojection_impl<FT> in FP64
 *        backproject_cuda.cu:117-175 (voxel position :144-148, pair loop :150-163,
 *        distance :25-46, bin window :155-159).
 *   orc_bp_gpu_f32emu               -- the same kernel with the reference's FP32
 *        arithmetic order (voxel position as an FMA chain, FP32 sums, IEEE division,
 *        round-half-away), used to reproduce its bin indices on the CPU.
 *   orc_bins_*                      -- per-(voxel, pair) bin indices of both forms.
 *   orc_bp_cpu_classic_{f32,c64}    -- classic_backprojection + accumulate_radiance
 *        backproject.hpp:75-96, 138-216 with OctreeVolume::position_at /
 *        voxel_size_at octree_volume.hpp:155-167 (grid step size/n, voxel-diagonal
 *        time window, FP64 distances truncated to FP32).
 *   orc_phasor_pulse                -- phasor_pulse backproject.hpp:430-479.
 *   orc_precompute_distances        -- precompute_distances backproject.hpp:356-418.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Layout-identical to CameraLaserPair (backproject_cuda.hpp:9-13): camera first. */
typedef struct {
    float camera_point[3];
    float laser_point[3];
    float camera_wall;
    float laser_wall;
} orc_pair;

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* FP64 restatement of the GPU kernel semantics.                              */
/* ------------------------------------------------------------------------- */

/* Voxel (ix,iy,iz) -> position zero + inc[0:3]*ix + inc[3:6]*iy + inc[6:9]*iz
 * (backproject_cuda.cu:144-148), evaluated in double. */
static inline void vox_pos_f64(const float *zero, const float *inc,
                               uint32_t ix, uint32_t iy, uint32_t iz, double *v)
{
    for (int k = 0; k < 3; k++)
        v[k] = (double)zero[k] + (double)inc[k] * ix + (double)inc[3 + k] * iy +
               (double)inc[6 + k] * iz;
}

static inline double dist3_f64(const float *p, const double *v)
{
    double dx = (double)p[0] - v[0], dy = (double)p[1] - v[1], dz = (double)p[2] - v[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

/* bin = round((lw + |l-v| + |v-c| + cw - t0) / dT); -1 when outside [0, T-1]
 * (backproject_cuda.cu:155-159 with a zero voxel footprint). */
static inline int64_t bin_f64(const orc_pair *pr, const double *v, double t0, double dT,
                              uint32_t T)
{
    double d = (double)pr->laser_wall + dist3_f64(pr->laser_point, v) +
               dist3_f64(pr->camera_point, v) + (double)pr->camera_wall;
    double b = round((d - t0) / dT);
    if (b < 0.0 || b > (double)T - 1.0) return -1;
    return (int64_t)b;
}

/* FP32 evaluation in the reference kernel's order.  The distance uses the
 * correctly-rounded FP32 value of the Euclidean norm; the reference calls norm3df,
 * whose result can differ by an ulp, so rare bins next to a .5 boundary differ. */
static inline void vox_pos_f32(const float *zero, const float *inc,
                               uint32_t ix, uint32_t iy, uint32_t iz, float *v)
{
    for (int k = 0; k < 3; k++) {
        float a = fmaf(inc[k], (float)ix, zero[k]);
        a = fmaf(inc[3 + k], (float)iy, a);
        v[k] = fmaf(inc[6 + k], (float)iz, a);
    }
}

static inline float norm_f32(float dx, float dy, float dz)
{
    double s = (double)dx * dx + (double)dy * dy + (double)dz * dz;
    return (float)sqrt(s);
}

static inline int64_t bin_f32emu(const orc_pair *pr, const float *v, float t0, float dT,
                                 uint32_t T)
{
    float lpv = norm_f32(pr->laser_point[0] - v[0], pr->laser_point[1] - v[1],
                         pr->laser_point[2] - v[2]);
    float vcp = norm_f32(v[0] - pr->camera_point[0], v[1] - pr->camera_point[1],
                         v[2] - pr->camera_point[2]);
    float total = pr->laser_wall + lpv;
    total = total + vcp;
    total = total + pr->camera_wall;
    float x = (total - t0 - 0.0f) / dT;
    float r = roundf(x);
    int32_t b = (int32_t)r;
    if (b < 0 || b > (int32_t)T - 1) return -1;
    return b;
}

/* Pairs kept by the reference: it loops i < P / blockDim (backproject_cuda.cu:150)
 * and drops the last P mod blockDim pairs.  block = 0 keeps every pair. */
static inline uint64_t kept_pairs(uint64_t P, uint32_t block)
{
    if (block == 0) return P;
    return (P / block) * block;
}

/* V[x,y,z] = sum_p H[p, bin(p, v)] in double.  out is double[Nx*Ny*Nz], x slowest.
 * voxel_list (optional, n_list entries of linear voxel ids) restricts the work to a
 * subset; then out has n_list entries. */
void orc_bp_gpu_f64(const float *H, uint64_t P, uint32_t T, const orc_pair *pairs,
                    const uint32_t *N, const float *zero, const float *inc, float t0,
                    float dT, uint32_t ref_block, const int64_t *voxel_list,
                    int64_t n_list, double *out)
{
    const uint64_t Pk = kept_pairs(P, ref_block);
    const int64_t nvox = voxel_list ? n_list : (int64_t)N[0] * N[1] * N[2];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < nvox; i++) {
        int64_t id = voxel_list ? voxel_list[i] : i;
        uint32_t iz = (uint32_t)(id % N[2]);
        uint32_t iy = (uint32_t)((id / N[2]) % N[1]);
        uint32_t ix = (uint32_t)(id / ((int64_t)N[1] * N[2]));
        double v[3];
        vox_pos_f64(zero, inc, ix, iy, iz, v);
        double acc = 0.0;
        for (uint64_t p = 0; p < Pk; p++) {
            int64_t b = bin_f64(&pairs[p], v, (double)t0, (double)dT, T);
            if (b >= 0) acc += (double)H[p * T + (uint64_t)b];
        }
        out[i] = acc;
    }
}

/* Complex64 input (interleaved re, im), complex128 output (interleaved). */
void orc_bp_gpu_c64(const float *H, uint64_t P, uint32_t T, const orc_pair *pairs,
                    const uint32_t *N, const float *zero, const float *inc, float t0,
                    float dT, uint32_t ref_block, const int64_t *voxel_list,
                    int64_t n_list, double *out)
{
    const uint64_t Pk = kept_pairs(P, ref_block);
    const int64_t nvox = voxel_list ? n_list : (int64_t)N[0] * N[1] * N[2];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < nvox; i++) {
        int64_t id = voxel_list ? voxel_list[i] : i;
        uint32_t iz = (uint32_t)(id % N[2]);
        uint32_t iy = (uint32_t)((id / N[2]) % N[1]);
        uint32_t ix = (uint32_t)(id / ((int64_t)N[1] * N[2]));
        double v[3];
        vox_pos_f64(zero, inc, ix, iy, iz, v);
        double re = 0.0, im = 0.0;
        for (uint64_t p = 0; p < Pk; p++) {
            int64_t b = bin_f64(&pairs[p], v, (double)t0, (double)dT, T);
            if (b >= 0) {
                re += (double)H[2 * (p * T + (uint64_t)b)];
                im += (double)H[2 * (p * T + (uint64_t)b) + 1];
            }
        }
        out[2 * i] = re;
        out[2 * i + 1] = im;
    }
}

/* The reference's FP32 bin arithmetic, accumulated in double (so the result does not
 * depend on summation order). */
void orc_bp_gpu_f32emu(const float *H, uint64_t P, uint32_t T, const orc_pair *pairs,
                       const uint32_t *N, const float *zero, const float *inc, float t0,
                       float dT, uint32_t ref_block, const int64_t *voxel_list,
                       int64_t n_list, double *out)
{
    const uint64_t Pk = kept_pairs(P, ref_block);
    const int64_t nvox = voxel_list ? n_list : (int64_t)N[0] * N[1] * N[2];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < nvox; i++) {
        int64_t id = voxel_list ? voxel_list[i] : i;
        uint32_t iz = (uint32_t)(id % N[2]);
        uint32_t iy = (uint32_t)((id / N[2]) % N[1]);
        uint32_t ix = (uint32_t)(id / ((int64_t)N[1] * N[2]));
        float v[3];
        vox_pos_f32(zero, inc, ix, iy, iz, v);
        double acc = 0.0;
        for (uint64_t p = 0; p < Pk; p++) {
            int64_t b = bin_f32emu(&pairs[p], v, t0, dT, T);
            if (b >= 0) acc += (double)H[p * T + (uint64_t)b];
        }
        out[i] = acc;
    }
}

/* Bin indices (int32, -1 = out of range) for every (voxel in list, pair):
 * out[i * P + p].  mode 0 = FP64, mode 1 = reference FP32 emulation. */
void orc_bins(uint64_t P, uint32_t T, const orc_pair *pairs, const uint32_t *N,
              const float *zero, const float *inc, float t0, float dT,
              const int64_t *voxel_list, int64_t n_list, int mode, int32_t *out)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < n_list; i++) {
        int64_t id = voxel_list[i];
        uint32_t iz = (uint32_t)(id % N[2]);
        uint32_t iy = (uint32_t)((id / N[2]) % N[1]);
        uint32_t ix = (uint32_t)(id / ((int64_t)N[1] * N[2]));
        if (mode == 0) {
            double v[3];
            vox_pos_f64(zero, inc, ix, iy, iz, v);
            for (uint64_t p = 0; p < P; p++)
                out[i * P + p] = (int32_t)bin_f64(&pairs[p], v, (double)t0, (double)dT, T);
        } else {
            float v[3];
            vox_pos_f32(zero, inc, ix, iy, iz, v);
            for (uint64_t p = 0; p < P; p++)
                out[i * P + p] = (int32_t)bin_f32emu(&pairs[p], v, t0, dT, T);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* The reference's OpenMP CPU path (the timed CPU baseline).                  */
/* ------------------------------------------------------------------------- */

/* Voxel position of the CPU path: zero_pos + index * (size / n), all FP32
 * (octree_volume.hpp:155-167 with depth -1). */
static inline void classic_pos(const float *vol_pos, const float *vol_size, const uint32_t *N,
                               uint64_t ix, uint64_t iy, uint64_t iz, float *v)
{
    const uint64_t idx[3] = {ix, iy, iz};
    for (int k = 0; k < 3; k++) {
        float zero = vol_pos[k] - vol_size[k] / 2.0f;
        float vs = vol_size[k] / (float)N[k];
        v[k] = zero + (float)idx[k] * vs;
    }
}

/* bp::distance (backproject.hpp:42-53) on FP32 points: the difference is an FP32
 * subtraction, stored in double, squared and summed in double. */
static inline double dist_ff_d(const float *a, const float *b)
{
    double t0 = (double)(a[0] - b[0]);
    double t1 = (double)(a[1] - b[1]);
    double t2 = (double)(a[2] - b[2]);
    return sqrt(t0 * t0 + t1 * t1 + t2 * t2);
}

/* Window [max(0, round((d - w/2 - t0)/dT)), min(T-1, round((d + w/2 - t0)/dT))) for one
 * pair (backproject.hpp:85-90).  Returns first/last through pointers. */
static inline void classic_window(const orc_pair *pr, const float *v, float t0, float dT,
                                  uint32_t T, float w, int *first, int *last)
{
    float wvw = (float)(dist_ff_d(pr->laser_point, v) + dist_ff_d(v, pr->camera_point));
    float total = pr->laser_wall + wvw;
    total = total + pr->camera_wall;
    int f = (int)roundf((total - w / 2.0f - t0) / dT);
    int l = (int)roundf((total + w / 2.0f - t0) / dT);
    *first = f > 0 ? f : 0;
    *last = l < (int)T - 1 ? l : (int)T - 1;
}

/* classic_backprojection (backproject.hpp:138-216) over the voxel list (or the whole
 * volume when voxel_list is NULL).  out is float[nvox]. */
void orc_bp_cpu_classic_f32(const float *H, uint64_t P, uint32_t T, const orc_pair *pairs,
                            const uint32_t *N, const float *vol_pos, const float *vol_size,
                            float t0, float dT, const int64_t *voxel_list, int64_t n_list,
                            float *out)
{
    float vs[3];
    for (int k = 0; k < 3; k++) vs[k] = vol_size[k] / (float)N[k];
    const float diag = sqrtf(vs[0] * vs[0] + vs[1] * vs[1] + vs[2] * vs[2]);
    const int64_t nvox = voxel_list ? n_list : (int64_t)N[0] * N[1] * N[2];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nvox; i++) {
        int64_t id = voxel_list ? voxel_list[i] : i;
        uint64_t iz = (uint64_t)(id % N[2]);
        uint64_t iy = (uint64_t)((id / N[2]) % N[1]);
        uint64_t ix = (uint64_t)(id / ((int64_t)N[1] * N[2]));
        float v[3];
        classic_pos(vol_pos, vol_size, N, ix, iy, iz, v);
        float acc = 0.0f;
        for (uint64_t p = 0; p < P; p++) {
            int first, last;
            classic_window(&pairs[p], v, t0, dT, T, diag, &first, &last);
            const float *row = H + p * T;
            for (int t = first; t < last; t++) acc += row[t];
        }
        out[i] = acc;
    }
}

void orc_bp_cpu_classic_c64(const float *H, uint64_t P, uint32_t T, const orc_pair *pairs,
                            const uint32_t *N, const float *vol_pos, const float *vol_size,
                            float t0, float dT, const int64_t *voxel_list, int64_t n_list,
                            float *out)
{
    float vs[3];
    for (int k = 0; k < 3; k++) vs[k] = vol_size[k] / (float)N[k];
    const float diag = sqrtf(vs[0] * vs[0] + vs[1] * vs[1] + vs[2] * vs[2]);
    const int64_t nvox = voxel_list ? n_list : (int64_t)N[0] * N[1] * N[2];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nvox; i++) {
        int64_t id = voxel_list ? voxel_list[i] : i;
        uint64_t iz = (uint64_t)(id % N[2]);
        uint64_t iy = (uint64_t)((id / N[2]) % N[1]);
        uint64_t ix = (uint64_t)(id / ((int64_t)N[1] * N[2]));
        float v[3];
        classic_pos(vol_pos, vol_size, N, ix, iy, iz, v);
        float re = 0.0f, im = 0.0f;
        for (uint64_t p = 0; p < P; p++) {
            int first, last;
            classic_window(&pairs[p], v, t0, dT, T, diag, &first, &last);
            const float *row = H + 2 * p * T;
            for (int t = first; t < last; t++) {
                re += row[2 * t];
                im += row[2 * t + 1];
            }
        }
        out[2 * i] = re;
        out[2 * i + 1] = im;
    }
}

/* ------------------------------------------------------------------------- */
/* Phasor pulse and pair precompute.                                          */
/* ------------------------------------------------------------------------- */

/* Pulse taps (cos, sin) as the reference builds them (backproject.hpp:433-451):
 * K = int(times*wl/dT), C = int(wl/dT), sigma = times*wl/6, t_k = dT*(k - K/2.0) for
 * k = 1..K, gaussian in double, cos/sin of 2*pi*k/C rounded to FP32, product in double
 * rounded to FP32.  Returns K; taps must hold 2*K floats (cos then sin). */
int orc_phasor_taps(float wavelength, float deltaT, uint32_t times, float *taps, int cap)
{
    int K = (int)((float)times * wavelength / deltaT);
    int C = (int)(wavelength / deltaT);
    float vsigma = ((float)times * wavelength) / 6.0f;
    /* 2 * vsigma * vsigma is an FP32 product in the reference expression. */
    const double denom = (double)(2.0f * vsigma * vsigma);
    if (K <= 0 || C <= 0) return K;
    if (taps == NULL || cap < K) return K;
    for (int k = 0; k < K; k++) {
        double kk = (double)(k + 1);
        double t = (double)deltaT * (kk - K / 2.0);
        double g = exp(-t * t / denom);
        double prog = 2.0 * M_PI * (1.0 / C * kk);
        float s = (float)sin(prog);
        float c = (float)cos(prog);
        taps[k] = (float)((double)c * g);
        taps[K + k] = (float)((double)s * g);
    }
    return K;
}

/* Hc[r, t] = sum_k H[r, t + k - K/2] * (cos_k, sin_k) over read indices in (0, T)
 * (backproject.hpp:459-476; read index 0 is excluded).  FP32 accumulation in tap order.
 * out is interleaved complex64 [rows, T]. */
void orc_phasor_pulse(const float *H, int64_t rows, int32_t T, float wavelength, float deltaT,
                      uint32_t times, float *out)
{
    int K = orc_phasor_taps(wavelength, deltaT, times, NULL, 0);
    if (K <= 0) {
        memset(out, 0, sizeof(float) * 2 * (size_t)rows * (size_t)T);
        return;
    }
    float *taps = (float *)malloc(sizeof(float) * 2 * (size_t)K);
    orc_phasor_taps(wavelength, deltaT, times, taps, K);
    const int half = K / 2;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; r++) {
        const float *row = H + r * T;
        for (int t = 0; t < T; t++) {
            float re = 0.0f, im = 0.0f;
            for (int k = 0; k < K; k++) {
                int ri = t + k - half;
                if (ri > 0 && ri < T) {
                    re += row[ri] * taps[k];
                    im += row[ri] * taps[K + k];
                }
            }
            out[2 * (r * T + t)] = re;
            out[2 * (r * T + t) + 1] = im;
        }
    }
    free(taps);
}

static inline float dist_ff(const float *a, const float *b)
{
    return (float)dist_ff_d(a, b);
}

/* precompute_distances (backproject.hpp:356-418).  Grids are row-major [gx, gy, 3].
 * confocal != 0: P = cx*cy, laser := camera point, both legs = |camera_pos - point|.
 * Otherwise P = lx*ly*cx*cy in order ((lx*Ly+ly)*Cx+cx)*Cy+cy. */
void orc_precompute_distances(const float *laser_pos, const float *laser_grid, uint32_t lx,
                              uint32_t ly, const float *camera_pos, const float *camera_grid,
                              uint32_t cx, uint32_t cy, int confocal, orc_pair *out)
{
    if (confocal) {
        for (uint32_t i = 0; i < cx; i++)
            for (uint32_t j = 0; j < cy; j++) {
                const float *c = camera_grid + 3 * ((uint64_t)i * cy + j);
                orc_pair *pr = &out[(uint64_t)i * cy + j];
                memcpy(pr->laser_point, c, 12);
                memcpy(pr->camera_point, c, 12);
                float w = dist_ff(camera_pos, c);
                pr->camera_wall = w;
                pr->laser_wall = w;
            }
        return;
    }
    const uint64_t S = (uint64_t)cx * cy;
    for (uint32_t a = 0; a < lx; a++)
        for (uint32_t b = 0; b < ly; b++) {
            const float *l = laser_grid + 3 * ((uint64_t)a * ly + b);
            float lw = dist_ff(laser_pos, l);
            for (uint32_t i = 0; i < cx; i++)
                for (uint32_t j = 0; j < cy; j++) {
                    const float *c = camera_grid + 3 * ((uint64_t)i * cy + j);
                    orc_pair *pr = &out[((uint64_t)a * ly + b) * S + (uint64_t)i * cy + j];
                    memcpy(pr->laser_point, l, 12);
                    memcpy(pr->camera_point, c, 12);
                    pr->camera_wall = dist_ff(camera_pos, c);
                    pr->laser_wall = lw;
                }
        }
}

/* ------------------------------------------------------------------------- */
/* Synthetic captures for the reference arm of the bench (not reference       */
/* algorithms): the scene renderer and Poisson noise of the synthetic         */
/* workloads, restated so that arm builds its inputs without the product      */
/* library.  Same arithmetic as the product's host renderer, so the captures  */
/* are identical bit for bit (tests/test_cpu.py checks it).                   */
/* ------------------------------------------------------------------------- */

/* H[p, b] += albedo / (|l - q|^2 |q - c|^2) for every scatterer q of pair p, b =
 * round((lw + |l - q| + |q - c| + cw - t0) / dT), in FP64, scatterers in order. */
void orc_synth_render(const orc_pair *pairs, uint64_t P, uint32_t T, float t0, float deltaT,
                      const float *points, const float *albedo, uint64_t n, float *out)
{
    const double dT = deltaT;
#pragma omp parallel
    {
        double *row = (double *)malloc(sizeof(double) * T);
#pragma omp for schedule(dynamic, 8)
        for (int64_t p = 0; p < (int64_t)P; p++) {
            for (uint32_t t = 0; t < T; t++) row[t] = 0.0;
            const orc_pair *pr = &pairs[p];
            for (uint64_t i = 0; i < n; i++) {
                const float *q = points + 3 * i;
                double a2 = 0.0, b2 = 0.0;
                for (int k = 0; k < 3; k++) {
                    const double da = (double)pr->laser_point[k] - q[k];
                    const double db = (double)q[k] - pr->camera_point[k];
                    a2 += da * da;
                    b2 += db * db;
                }
                const double d = (double)pr->laser_wall + sqrt(a2) + sqrt(b2) +
                                 (double)pr->camera_wall;
                const double b = round((d - (double)t0) / dT);
                if (b < 0.0 || b >= (double)T || a2 <= 0.0 || b2 <= 0.0) continue;
                row[(uint32_t)b] += (double)albedo[i] / (a2 * b2);
            }
            float *o = out + (uint64_t)p * T;
            for (uint32_t t = 0; t < T; t++) o[t] = (float)row[t];
        }
        free(row);
    }
}

static inline uint64_t orc_splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static inline double orc_uniform(uint64_t seed, uint64_t index, uint64_t draw)
{
    const uint64_t r = orc_splitmix64(seed ^ orc_splitmix64(index * 0x100000001B3ull + draw));
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static double orc_poisson_sample(double lam, uint64_t seed, uint64_t index)
{
    if (!(lam > 0.0)) return 0.0;
    if (lam < 30.0) {
        const double L = exp(-lam);
        double p = 1.0;
        uint64_t k = 0;
        do {
            p *= orc_uniform(seed, index, k);
            k++;
        } while (p > L && k < 1000);
        return (double)(k - 1);
    }
    const double u1 = orc_uniform(seed, index, 0), u2 = orc_uniform(seed, index, 1);
    const double z = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
    const double v = floor(lam + sqrt(lam) * z + 0.5);
    return v > 0.0 ? v : 0.0;
}

/* H := Poisson(H * peak / max(H)) per bin, counter-based draws (seed, bin index). */
void orc_synth_poisson(float *H, uint64_t n, float peak, uint64_t seed)
{
    if (!(peak > 0.0f) || n == 0) return;
    float mx = 0.0f;
#pragma omp parallel for reduction(max : mx)
    for (int64_t i = 0; i < (int64_t)n; i++) mx = H[i] > mx ? H[i] : mx;
    if (!(mx > 0.0f)) return;
    const double scale = (double)peak / (double)mx;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        H[i] = (float)orc_poisson_sample((double)H[i] * scale, seed, (uint64_t)i);
}

/* ------------------------------------------------------------------------- */
/* get_time_limits (backproject.hpp:617-674) with its corner semantics:       */
/* get_corner / get_nd_corners (:490-569), get_min_max_distances (:580-598),  */
/* bp::distance (:42-53).  Grid corner i: bit 1 -> last row, bit 0 -> last    */
/* column (mask & 1 << (ndim - 1 - dim)); volume corner i: bit (2 - k) adds   */
/* size[k] to position[k] - size[k] / 2.  The camera-grid transpose of the    */
/* row-major case (:651-652) is not reproduced (xtensor slicing semantics).   */
/* ------------------------------------------------------------------------- */
static double orc_ref_distance(const float *p1, const float *p2)
{
    double t[3];
    for (int i = 0; i < 3; i++) {
        t[i] = (double)p1[i] - (double)p2[i];
        t[i] = t[i] * t[i];
    }
    return sqrt(t[0] + t[1] + t[2]);
}

static void orc_minmax(const float *A, int na, const float *B, int nb, float *mn, float *mx)
{
    float lo = 3.402823466e+38f, hi = 0.0f;
    for (int i = 0; i < na; i++)
        for (int j = 0; j < nb; j++) {
            float d = (float)orc_ref_distance(A + 3 * i, B + 3 * j);
            lo = d < lo ? d : lo;
            hi = d > hi ? d : hi;
        }
    *mn = lo;
    *mx = hi;
}

void orc_time_limits_corners(const float *laser_pos, const float *laser_grid, uint32_t lx,
                             uint32_t ly, const float *camera_pos, const float *camera_grid,
                             uint32_t cx, uint32_t cy, const float *vol_pos,
                             const float *vol_size, float t0, float dT, float *out)
{
    float las[12], cam[12], vol[24];
    for (int i = 0; i < 4; i++) {
        uint32_t a = (i & 2) ? lx - 1 : 0, b = (i & 1) ? ly - 1 : 0;
        uint32_t c = (i & 2) ? cx - 1 : 0, d = (i & 1) ? cy - 1 : 0;
        for (int k = 0; k < 3; k++) {
            las[3 * i + k] = laser_grid[3 * ((uint64_t)a * ly + b) + k];
            cam[3 * i + k] = camera_grid[3 * ((uint64_t)c * cy + d) + k];
        }
    }
    for (int i = 0; i < 8; i++)
        for (int k = 0; k < 3; k++) {
            float lower = vol_pos[k] - vol_size[k] / 2.0f;
            float m = (i & (1 << (2 - k))) ? 1.0f : 0.0f;
            vol[3 * i + k] = lower + m * vol_size[k];
        }
    float a0, a1, b0, b1, c0, c1, d0, d1;
    orc_minmax(laser_pos, 1, las, 4, &a0, &a1);
    orc_minmax(camera_pos, 1, cam, 4, &b0, &b1);
    orc_minmax(vol, 8, las, 4, &c0, &c1);
    orc_minmax(vol, 8, cam, 4, &d0, &d1);
    float mn = a0 + b0 + c0 + d0, mx = a1 + b1 + c1 + d1;
    mn -= t0;
    mx -= t0;
    out[0] = mn / dT - 100;
    out[1] = mx / dT + 100;
}
