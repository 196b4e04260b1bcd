// Capture geometry: the pair list with its wall legs (FP64 on the GPU), the volume basis
// and the time window of the capture.
//
//   bpgb_precompute_pairs  <- precompute_distances  backproject.hpp:356-418
//   bpgb_volume_basis      <- volume basis / voxel_inc backproject.hpp:820-839
//   bpgb_time_limits       <- get_time_limits       backproject.hpp:617-674
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "bpgb_internal.h"

namespace bpgb {
namespace {

// bp::distance (backproject.hpp:42-53) on FP32 points: FP32 difference, squares and sum
// in double, sqrt in double.  Explicit _rn operations keep the GPU result identical to
// the CPU evaluation (no FMA contraction).
__device__ __forceinline__ double leg_fp64(const double *o, const float *pt) {
    const float o0 = (float)o[0], o1 = (float)o[1], o2 = (float)o[2];
    const double d0 = (double)(o0 - pt[0]);
    const double d1 = (double)(o1 - pt[1]);
    const double d2 = (double)(o2 - pt[2]);
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

struct PairArgs {
    uint32_t lx, ly, cx, cy;
    double laser_pos[3], camera_pos[3];
    int confocal;
};

__global__ void pairs_fp64_kernel(const float *__restrict__ lgrid, const float *__restrict__ cgrid,
                                  bpgb_pair *__restrict__ out, const PairArgs a) {
    const uint64_t S = (uint64_t)a.cx * a.cy;
    const uint64_t P = a.confocal ? S : (uint64_t)a.lx * a.ly * S;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P;
         p += (uint64_t)gridDim.x * blockDim.x) {
        bpgb_pair pr;
        const uint64_t s = a.confocal ? p : p % S;
        const float *c = cgrid + 3 * s;
        pr.camera_point[0] = c[0];
        pr.camera_point[1] = c[1];
        pr.camera_point[2] = c[2];
        const float cw = (float)leg_fp64(a.camera_pos, c);
        pr.camera_wall = cw;
        if (a.confocal) {
            pr.laser_point[0] = c[0];
            pr.laser_point[1] = c[1];
            pr.laser_point[2] = c[2];
            pr.laser_wall = cw;
        } else {
            const float *l = lgrid + 3 * (p / S);
            pr.laser_point[0] = l[0];
            pr.laser_point[1] = l[1];
            pr.laser_point[2] = l[2];
            pr.laser_wall = (float)leg_fp64(a.laser_pos, l);
        }
        out[p] = pr;
    }
}

}  // namespace

int launch_pairs_fp64(const float *d_laser_grid, uint32_t lx, uint32_t ly,
                      const float *d_camera_grid, uint32_t cx, uint32_t cy,
                      const double *laser_pos, const double *camera_pos, int confocal,
                      bpgb_pair *d_out, cudaStream_t stream) {
    PairArgs a{};
    a.lx = lx;
    a.ly = ly;
    a.cx = cx;
    a.cy = cy;
    for (int k = 0; k < 3; k++) {
        a.laser_pos[k] = laser_pos[k];
        a.camera_pos[k] = camera_pos[k];
    }
    a.confocal = confocal;
    const uint64_t P = confocal ? (uint64_t)cx * cy : (uint64_t)lx * ly * cx * cy;
    if (P == 0) return BPGB_OK;
    const unsigned blocks = (unsigned)std::min<uint64_t>((P + 255) / 256, 152ull * 32);
    pairs_fp64_kernel<<<blocks, 256, 0, stream>>>(d_laser_grid, d_camera_grid, d_out, a);
    count_launches(1);
    BPGB_CUDA_TRY(cudaGetLastError());
    return BPGB_OK;
}

}  // namespace bpgb

using namespace bpgb;

namespace {

bool finite_n(const float *p, int n) {
    for (int i = 0; i < n; i++)
        if (!std::isfinite(p[i])) return false;
    return true;
}

// Euclidean distance of two FP32 points with the reference's mixed precision.
float dist_ff(const float *a, const float *b) {
    const double d0 = (double)(a[0] - b[0]);
    const double d1 = (double)(a[1] - b[1]);
    const double d2 = (double)(a[2] - b[2]);
    return (float)std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

}  // namespace

extern "C" {

int bpgb_precompute_pairs(const float *laser_position, const float *laser_grid, uint32_t lx,
                          uint32_t ly, const float *camera_position, const float *camera_grid,
                          uint32_t cx, uint32_t cy, int confocal, bpgb_pair *out_pairs) {
    clear_error();
    if (!camera_position || !camera_grid || !out_pairs || (!confocal && (!laser_position || !laser_grid)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null geometry pointer");
    const uint64_t S = (uint64_t)cx * cy;
    const uint64_t L = confocal ? 0 : (uint64_t)lx * ly;
    const uint64_t P = confocal ? S : L * S;
    if (P == 0) return BPGB_OK;
    if (!finite_n(camera_grid, (int)std::min<uint64_t>(3 * S, 1u << 30)) ||
        !finite_n(camera_position, 3) || (!confocal && (!finite_n(laser_position, 3) ||
                                                        !finite_n(laser_grid, (int)(3 * L)))))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "non-finite grid or origin position");
    int st = require_device();
    if (st) return st;
    double lp[3] = {0, 0, 0}, cp[3];
    for (int k = 0; k < 3; k++) {
        cp[k] = camera_position[k];
        if (!confocal) lp[k] = laser_position[k];
    }
    float *d_l = nullptr, *d_c = nullptr;
    bpgb_pair *d_p = nullptr;
    cudaError_t e = cudaMalloc(&d_c, 3 * S * sizeof(float));
    if (e == cudaSuccess && L) e = cudaMalloc(&d_l, 3 * L * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_p, P * sizeof(bpgb_pair));
    if (e == cudaSuccess) e = cudaMemcpy(d_c, camera_grid, 3 * S * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && L)
        e = cudaMemcpy(d_l, laser_grid, 3 * L * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        st = launch_pairs_fp64(d_l, lx, ly, d_c, cx, cy, lp, cp, confocal, d_p, nullptr);
        if (!st) e = cudaMemcpy(out_pairs, d_p, P * sizeof(bpgb_pair), cudaMemcpyDeviceToHost);
    }
    cudaFree(d_l);
    cudaFree(d_c);
    cudaFree(d_p);
    if (st) return st;
    if (e != cudaSuccess) return cuda_error(e, "pair precompute");
    return BPGB_OK;
}

int bpgb_volume_basis(const float *volume_position, const float *volume_size,
                      const uint32_t *voxels_per_side, const float *wall_normal,
                      float *volume_zero_pos, float *voxel_inc) {
    clear_error();
    if (!volume_position || !volume_size || !voxels_per_side || !volume_zero_pos || !voxel_inc)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null argument");
    for (int k = 0; k < 3; k++)
        if (voxels_per_side[k] < 2)
            return set_error(BPGB_ERR_INVALID_ARGUMENT,
                             "voxels_per_side must be >= 2 (the step is size / (n - 1))");
    float x[3] = {1, 0, 0}, y[3] = {0, 1, 0}, z[3] = {0, 0, 1};
    if (wall_normal && (wall_normal[0] != 0.0f || wall_normal[1] != 0.0f || wall_normal[2] != 0.0f)) {
        for (int k = 0; k < 3; k++) y[k] = -wall_normal[k];
        auto cross = [](const float *a, const float *b, float *o) {
            o[0] = a[1] * b[2] - a[2] * b[1];
            o[1] = a[2] * b[0] - a[0] * b[2];
            o[2] = a[0] * b[1] - a[1] * b[0];
        };
        float nx[3], nz[3];
        cross(y, z, nx);
        std::memcpy(x, nx, 12);
        cross(y, x, nz);
        std::memcpy(z, nz, 12);
        for (float *v : {x, y, z}) {
            const float n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (!(n > 0.0f)) return set_error(BPGB_ERR_INVALID_ARGUMENT, "degenerate wall_normal");
            for (int k = 0; k < 3; k++) v[k] = v[k] / n;
        }
    }
    for (int k = 0; k < 3; k++) volume_zero_pos[k] = volume_position[k] - volume_size[k] / 2.0f;
    const float *axes[3] = {x, y, z};
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 3; k++)
            voxel_inc[3 * a + k] = (axes[a][k] * volume_size[k]) / (float)(voxels_per_side[k] - 1);
    return BPGB_OK;
}

int bpgb_time_limits(const float *laser_position, const float *laser_grid, uint32_t lx,
                     uint32_t ly, const float *camera_position, const float *camera_grid,
                     uint32_t cx, uint32_t cy, const float *volume_position,
                     const float *volume_size, float t0, float deltaT, float *min_index,
                     float *max_index) {
    // get_time_limits (backproject.hpp:617-674) takes the min / max path over the corners
    // of the laser grid, the camera grid and the volume, minus t0, in bins, padded by 100
    // bins.  Corners miss interior grid points (the shortest path usually runs through
    // the grid point nearest the volume), so this bound runs over every grid point and
    // the volume box instead: min = min_l(|lo - l| + dist(l, box)) + min_c(...), max the
    // same with the farthest box point.  Every bin a voxel reaches lies inside.
    clear_error();
    if (!laser_position || !laser_grid || !camera_position || !camera_grid || !volume_position ||
        !volume_size || !min_index || !max_index || lx == 0 || ly == 0 || cx == 0 || cy == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad time-limit arguments");
    if (!(deltaT > 0.0f)) return set_error(BPGB_ERR_INVALID_ARGUMENT, "deltaT must be > 0");
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = (double)volume_position[k] - (double)volume_size[k] / 2;
        hi[k] = (double)volume_position[k] + (double)volume_size[k] / 2;
    }
    auto legs = [&](const float *origin, const float *grid, uint64_t n, double &mn, double &mx) {
        mn = std::numeric_limits<double>::max();
        mx = 0.0;
        for (uint64_t i = 0; i < n; i++) {
            const float *g = grid + 3 * i;
            const double wall = dist_ff(origin, g);
            double a = 0.0, b = 0.0;
            for (int k = 0; k < 3; k++) {
                const double c = std::min(std::max((double)g[k], lo[k]), hi[k]);
                const double d = (double)g[k] - c;
                const double e = std::max(std::fabs((double)g[k] - lo[k]), std::fabs((double)g[k] - hi[k]));
                a += d * d;
                b += e * e;
            }
            mn = std::min(mn, wall + std::sqrt(a));
            mx = std::max(mx, wall + std::sqrt(b));
        }
    };
    double lmin, lmax, cmin, cmax;
    legs(laser_position, laser_grid, (uint64_t)lx * ly, lmin, lmax);
    legs(camera_position, camera_grid, (uint64_t)cx * cy, cmin, cmax);
    const float mn = (float)(lmin + cmin) - t0;
    const float mx = (float)(lmax + cmax) - t0;
    *min_index = mn / deltaT - 100;
    *max_index = mx / deltaT + 100;
    return BPGB_OK;
}

int bpgb_time_limits_corners(const float *laser_position, const float *laser_grid, uint32_t lx,
                             uint32_t ly, const float *camera_position, const float *camera_grid,
                             uint32_t cx, uint32_t cy, const float *volume_position,
                             const float *volume_size, float t0, float deltaT, float *min_index,
                             float *max_index) {
    // get_time_limits (backproject.hpp:617-674) as written: the 4 corner points of each
    // grid (get_nd_corners / get_corner, :490-547), the 8 corners of the volume box
    // position - size / 2 + {0, 1} size (:513-569), min / max of bp::distance (FP32
    // points, FP64 differences and sum, :42-53) between origin and grid corners and
    // between volume corners and grid corners (get_min_max_distances, :580-598, kept
    // in float), the four minima (maxima) summed in float, minus t0, over deltaT, padded
    // by 100 bins.  The reference transposes the camera grid in the row-major case
    // (:651-652), which under xtensor's slicing rules does not yield the grid's corner
    // points; the grid's 4 corners are used here.
    clear_error();
    if (!laser_position || !laser_grid || !camera_position || !camera_grid || !volume_position ||
        !volume_size || !min_index || !max_index || lx == 0 || ly == 0 || cx == 0 || cy == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "bad time-limit arguments");
    if (!(deltaT > 0.0f)) return set_error(BPGB_ERR_INVALID_ARGUMENT, "deltaT must be > 0");
    auto dist = [](const float *a, const float *b) {
        double t[3];
        for (int k = 0; k < 3; k++) {
            t[k] = (double)a[k] - (double)b[k];
            t[k] = t[k] * t[k];
        }
        return std::sqrt(t[0] + t[1] + t[2]);
    };
    // corner i of a [gx, gy, 3] grid: bit 1 of i selects the last row, bit 0 the last column
    auto grid_corners = [](const float *g, uint32_t gx, uint32_t gy, float out[4][3]) {
        for (int i = 0; i < 4; i++) {
            const uint32_t a = (i & 2) ? gx - 1 : 0, b = (i & 1) ? gy - 1 : 0;
            for (int k = 0; k < 3; k++) out[i][k] = g[3 * ((uint64_t)a * gy + b) + k];
        }
    };
    float las[4][3], cam[4][3], vol[8][3];
    grid_corners(laser_grid, lx, ly, las);
    grid_corners(camera_grid, cx, cy, cam);
    for (int i = 0; i < 8; i++)
        for (int k = 0; k < 3; k++) {
            const float lower = volume_position[k] - volume_size[k] / 2.0f;
            const float m = (i & (1 << (2 - k))) ? 1.0f : 0.0f;
            vol[i][k] = lower + m * volume_size[k];
        }
    auto minmax = [&](const float (*A)[3], int na, const float (*B)[3], int nb, float &mn, float &mx) {
        mn = std::numeric_limits<float>::max();
        mx = 0.0f;
        for (int i = 0; i < na; i++)
            for (int j = 0; j < nb; j++) {
                const float d = (float)dist(A[i], B[j]);
                mn = std::min(d, mn);
                mx = std::max(d, mx);
            }
    };
    float a0, a1, b0, b1, c0, c1, d0, d1;
    minmax((const float(*)[3])laser_position, 1, las, 4, a0, a1);
    minmax((const float(*)[3])camera_position, 1, cam, 4, b0, b1);
    minmax(vol, 8, las, 4, c0, c1);
    minmax(vol, 8, cam, 4, d0, d1);
    float mn = a0 + b0 + c0 + d0;
    float mx = a1 + b1 + c1 + d1;
    mn -= t0;
    mx -= t0;
    *min_index = mn / deltaT - 100;
    *max_index = mx / deltaT + 100;
    return BPGB_OK;
}

}  // extern "C"
