// Whole reconstructions from a capture on host buffers:
//   bpgb_backproject_capture <- bp::backproject            backproject.hpp:762-909
//   bpgb_phasor_capture      <- bp::phasor_reconstruction  backproject.hpp:932-1039
// (GPU compute, Naive volume access).  Steps, as in the reference:
//   1. time window [floor(m), ceil(M)) of the capture (get_time_limits, :617-674);
//   2. crop + zero-pad the transient rows to that window while copying them to the
//      device (get_transient_chunk, :689-740, done by one pitched copy);
//   3. pair list and wall legs in FP64 on the GPU (precompute_distances, :356-418);
//   4. volume basis (:820-839);
//   5. chunked t0: t0 + m * deltaT (dense, m unfloored, :847) or t0 + int(m) * deltaT
//      (phasor, :962, :1011);
//   6. phasor only: pulse convolution on the GPU (:1000);
//   7. backprojection through a plan.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bpgb_internal.h"

using namespace bpgb;

namespace {

struct Window {
    int64_t from;   // floor(m): first original bin of the chunk (may be negative)
    uint32_t len;   // chunk length T'
    float m;        // fractional first index from the time limits
    float M;        // fractional last index from the time limits
};

// corners: the reference's corner-point bound (bpgb_time_limits_corners) instead of the
// bound over every grid point (bpgb_time_limits).
int capture_window(const float *laser_grid, uint32_t lx, uint32_t ly, const float *camera_grid,
                   uint32_t cx, uint32_t cy, const float *camera_position,
                   const float *laser_position, float t0, float deltaT, int confocal,
                   const float *volume_position, const float *volume_size, Window *w,
                   bool corners = false) {
    float mn = 0, mx = 0;
    // Confocal captures illuminate the camera grid from the camera position: both legs
    // are |camera_position - c| (backproject.hpp:405-411).
    const float *lg = confocal ? camera_grid : laser_grid;
    const float *lp = confocal ? camera_position : laser_position;
    const uint32_t glx = confocal ? cx : lx, gly = confocal ? cy : ly;
    int st = (corners ? bpgb_time_limits_corners : bpgb_time_limits)(
        lp, lg, glx, gly, camera_position, camera_grid, cx, cy, volume_position, volume_size,
        t0, deltaT, &mn, &mx);
    if (st) return st;
    const double lo = std::floor((double)mn), hi = std::ceil((double)mx);
    if (!(hi > lo) || hi - lo > 1e8)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "degenerate capture time window");
    w->from = (int64_t)lo;
    w->len = (uint32_t)(hi - lo);
    w->m = mn;
    w->M = mx;
    return BPGB_OK;
}

// Copies rows [P, T] (host) into the device chunk [P, pitch] holding original bins
// [from, from + len), zero elsewhere.
int upload_chunk(const float *h, uint64_t P, uint32_t T, const Window &w, uint32_t pitch,
                 float *d, cudaStream_t s) {
    BPGB_CUDA_TRY(cudaMemsetAsync(d, 0, P * (size_t)pitch * sizeof(float), s));
    const int64_t src0 = std::max<int64_t>(0, w.from);
    const int64_t src1 = std::min<int64_t>((int64_t)T, w.from + (int64_t)w.len);
    if (src1 <= src0 || P == 0) return BPGB_OK;
    const int64_t dst0 = src0 - w.from;
    BPGB_CUDA_TRY(cudaMemcpy2DAsync(d + dst0, (size_t)pitch * sizeof(float), h + src0,
                                    (size_t)T * sizeof(float), (size_t)(src1 - src0) * sizeof(float),
                                    P, cudaMemcpyHostToDevice, s));
    return BPGB_OK;
}

struct Common {
    std::vector<bpgb_pair> pairs;
    float zero[3], inc[9];
    Window w;
    uint64_t P;
};

int prepare(const float *camera_grid, uint32_t cx, uint32_t cy, const float *laser_grid,
            uint32_t lx, uint32_t ly, const float *camera_position, const float *laser_position,
            float t0, float deltaT, int confocal, const float *volume_position,
            const float *volume_size, const uint32_t *voxels_per_side, const float *wall_normal,
            Common *c, bool corners = false) {
    if (!camera_grid || !camera_position || !volume_position || !volume_size || !voxels_per_side)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null capture argument");
    if (!confocal && (!laser_grid || !laser_position))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "exhaustive capture needs the laser grid");
    if (cx == 0 || cy == 0 || (!confocal && (lx == 0 || ly == 0)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "empty grid");
    const float zeros3[3] = {0, 0, 0};
    const float *lpos = laser_position ? laser_position : zeros3;
    int st = capture_window(laser_grid, lx, ly, camera_grid, cx, cy, camera_position, lpos, t0,
                            deltaT, confocal, volume_position, volume_size, &c->w, corners);
    if (st) return st;
    c->P = confocal ? (uint64_t)cx * cy : (uint64_t)lx * ly * cx * cy;
    c->pairs.resize(c->P);
    st = bpgb_precompute_pairs(lpos, laser_grid, lx, ly, camera_position, camera_grid, cx, cy,
                               confocal, c->pairs.data());
    if (st) return st;
    return bpgb_volume_basis(volume_position, volume_size, voxels_per_side, wall_normal, c->zero,
                             c->inc);
}

}  // namespace

extern "C" {

int bpgb_capture_window(const float *camera_grid, uint32_t cx, uint32_t cy,
                        const float *laser_grid, uint32_t lx, uint32_t ly,
                        const float *camera_position, const float *laser_position, float t0,
                        float deltaT, int confocal, const float *volume_position,
                        const float *volume_size, int t0_mode, int64_t *from, uint32_t *len,
                        float *chunk_t0) {
    clear_error();
    if (!camera_grid || !camera_position || !volume_position || !volume_size || !from || !len ||
        !chunk_t0 || (!confocal && (!laser_grid || !laser_position)))
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null capture argument");
    if ((t0_mode & ~4) < 0 || (t0_mode & ~4) > 2)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "t0_mode 0, 1 or 2, plus 4 for corner limits");
    const bool corners = (t0_mode & 4) != 0;
    t0_mode &= ~4;
    const float zeros3[3] = {0, 0, 0};
    Window w;
    int st = capture_window(laser_grid, lx, ly, camera_grid, cx, cy, camera_position,
                            laser_position ? laser_position : zeros3, t0, deltaT, confocal,
                            volume_position, volume_size, &w, corners);
    if (st) return st;
    if (t0_mode == 2) {  // phasor: int limits (backproject.hpp:962)
        const int mi = (int)w.m, Mi = (int)w.M;
        if (Mi <= mi) return set_error(BPGB_ERR_INVALID_ARGUMENT, "degenerate capture time window");
        *from = mi;
        *len = (uint32_t)(Mi - mi);
        *chunk_t0 = t0 + (float)mi * deltaT;
        return BPGB_OK;
    }
    *from = w.from;
    *len = w.len;
    *chunk_t0 = t0_mode == 0 ? t0 + w.m * deltaT : t0 + (float)w.from * deltaT;
    return BPGB_OK;
}

int bpgb_backproject_capture(const float *transient_data, uint32_t T,
                             const float *camera_grid, uint32_t cx, uint32_t cy,
                             const float *laser_grid, uint32_t lx, uint32_t ly,
                             const float *camera_position, const float *laser_position,
                             float t0, float deltaT, int confocal,
                             const float *volume_position, const float *volume_size,
                             const uint32_t *voxels_per_side, const float *wall_normal,
                             int t0_mode, const bpgb_options *opt, float *out_volume) {
    clear_error();
    if (!transient_data || !out_volume || T == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null transient data / output or T == 0");
    if ((t0_mode & ~4) < 0 || (t0_mode & ~4) > 1)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "t0_mode 0 or 1, plus 4 for corner limits");
    const bool corners = (t0_mode & 4) != 0;
    t0_mode &= ~4;
    int st = require_device();
    if (st) return st;
    Common c;
    st = prepare(camera_grid, cx, cy, laser_grid, lx, ly, camera_position, laser_position, t0,
                 deltaT, confocal, volume_position, volume_size, voxels_per_side, wall_normal, &c,
                 corners);
    if (st) return st;
    bpgb_options o;
    bpgb_options_default(&o);
    if (opt) o = *opt;
    if (o.h_dtype != BPGB_DTYPE_F32)
        return set_error(BPGB_ERR_UNSUPPORTED, "capture calls take FP32 transients");
    const uint32_t pitch = (c.w.len + 3) / 4 * 4;
    o.h_pitch = pitch;
    // chunked_t0 (backproject.hpp:847): the reference keeps the unfloored m.
    const float ct0 = t0_mode == 0 ? t0 + c.w.m * deltaT : t0 + (float)c.w.from * deltaT;
    bpgb_plan plan = nullptr;
    st = bpgb_plan_create(&plan, c.pairs.data(), c.P, c.w.len, voxels_per_side, c.zero, c.inc,
                          ct0, deltaT, &o);
    if (st) return st;
    const uint64_t nvox = (uint64_t)voxels_per_side[0] * voxels_per_side[1] * voxels_per_side[2];
    thread_local DeviceBuffer dH, dV;
    st = dH.reserve(std::max<size_t>(16, c.P * (size_t)pitch * 4));
    if (!st) st = dV.reserve(std::max<size_t>(16, nvox * 4));
    if (!st) st = upload_chunk(transient_data, c.P, T, c.w, pitch, (float *)dH.ptr, nullptr);
    if (!st) st = bpgb_plan_execute(plan, dH.ptr, dV.ptr, nullptr);
    if (!st) st = bpgb_plan_check(plan, nullptr);
    if (!st) {
        cudaError_t e = cudaMemcpy(out_volume, dV.ptr, nvox * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_error(e, "volume download");
    }
    const std::string keep = st ? std::string(bpgb_last_error()) : std::string();
    bpgb_plan_destroy(plan);
    if (st) set_error(st, keep);
    return st;
}

int bpgb_phasor_capture(const float *transient_data, uint32_t T, const float *camera_grid,
                        uint32_t cx, uint32_t cy, const float *laser_grid, uint32_t lx,
                        uint32_t ly, const float *camera_position, const float *laser_position,
                        float t0, float deltaT, int confocal, const float *volume_position,
                        const float *volume_size, const uint32_t *voxels_per_side,
                        const float *wall_normal, float wavelength, const bpgb_options *opt,
                        float *out_volume) {
    clear_error();
    if (!transient_data || !out_volume || T == 0)
        return set_error(BPGB_ERR_INVALID_ARGUMENT, "null transient data / output or T == 0");
    int st = require_device();
    if (st) return st;
    Common c;
    st = prepare(camera_grid, cx, cy, laser_grid, lx, ly, camera_position, laser_position, t0,
                 deltaT, confocal, volume_position, volume_size, voxels_per_side, wall_normal, &c);
    if (st) return st;
    // The phasor path stores the limits in ints (backproject.hpp:962), i.e. truncates.
    const int mi = (int)c.w.m, Mi = (int)c.w.M;
    if (Mi <= mi) return set_error(BPGB_ERR_INVALID_ARGUMENT, "degenerate capture time window");
    c.w.from = mi;
    c.w.len = (uint32_t)(Mi - mi);
    bpgb_options o;
    bpgb_options_default(&o);
    if (opt) o = *opt;
    o.h_dtype = BPGB_DTYPE_C64;
    const uint32_t pitch = (c.w.len + 1) / 2 * 2;
    o.h_pitch = pitch;
    const float ct0 = t0 + (float)mi * deltaT;
    bpgb_plan plan = nullptr;
    st = bpgb_plan_create(&plan, c.pairs.data(), c.P, c.w.len, voxels_per_side, c.zero, c.inc,
                          ct0, deltaT, &o);
    if (st) return st;
    const uint64_t nvox = (uint64_t)voxels_per_side[0] * voxels_per_side[1] * voxels_per_side[2];
    thread_local DeviceBuffer dR, dC, dV;
    st = dR.reserve(std::max<size_t>(16, c.P * (size_t)pitch * 4));
    if (!st) st = dC.reserve(std::max<size_t>(16, c.P * (size_t)pitch * 8));
    if (!st) st = dV.reserve(std::max<size_t>(16, nvox * 8));
    if (!st) st = upload_chunk(transient_data, c.P, T, c.w, pitch, (float *)dR.ptr, nullptr);
    if (!st)
        st = bpgb_phasor_pulse((const float *)dR.ptr, c.P, c.w.len, pitch, wavelength, deltaT, 4,
                               (float *)dC.ptr, pitch, nullptr);
    if (!st) st = bpgb_plan_execute(plan, dC.ptr, dV.ptr, nullptr);
    if (!st) st = bpgb_plan_check(plan, nullptr);
    if (!st) {
        cudaError_t e = cudaMemcpy(out_volume, dV.ptr, nvox * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_error(e, "volume download");
    }
    const std::string keep = st ? std::string(bpgb_last_error()) : std::string();
    bpgb_plan_destroy(plan);
    if (st) set_error(st, keep);
    return st;
}

}  // extern "C"
