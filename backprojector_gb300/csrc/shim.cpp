// C++ drop-in entry points with the reference's signatures (backproject_cuda.hpp:19-49),
// implemented over the C ABI.  Non-zero status -> std::runtime_error.
#include <stdexcept>
#include <string>

#include "backproject_cuda_gb300.hpp"
#include "backprojector_gb300.h"

static_assert(sizeof(CameraLaserPair) == sizeof(bpgb_pair), "pair layout");
static_assert(sizeof(std::complex<float>) == 8, "complex64 layout");

namespace {
void raise_on(int st, const char *what) {
    if (st != BPGB_OK)
        throw std::runtime_error(std::string(what) + ": " + bpgb_status_string(st) + ": " +
                                 bpgb_last_error());
}
}  // namespace

void call_cuda_backprojection(const float *transient_chunk, uint32_t transient_size, uint32_t T,
                              const std::vector<CameraLaserPair> scanned_pairs,
                              float *voxel_volume, const uint32_t *voxels_per_side,
                              const float *volume_zero_pos, const float *voxel_inc, float t0,
                              float deltaT) {
    raise_on(bpgb_backproject_f32(transient_chunk, transient_size, T,
                                  reinterpret_cast<const bpgb_pair *>(scanned_pairs.data()),
                                  scanned_pairs.size(), voxel_volume, voxels_per_side,
                                  volume_zero_pos, voxel_inc, t0, deltaT),
             "call_cuda_backprojection");
}

void call_cuda_octree_backprojection(const float *transient_chunk, uint32_t transient_size,
                                     uint32_t T,
                                     const std::vector<CameraLaserPair> scanned_pairs,
                                     float *voxel_volume, const uint32_t *voxels_per_side,
                                     const float *volume_zero_pos, const float *voxel_inc,
                                     float t0, float deltaT) {
    raise_on(bpgb_backproject_f32(transient_chunk, transient_size, T,
                                  reinterpret_cast<const bpgb_pair *>(scanned_pairs.data()),
                                  scanned_pairs.size(), voxel_volume, voxels_per_side,
                                  volume_zero_pos, voxel_inc, t0, deltaT),
             "call_cuda_octree_backprojection");
}

void call_cuda_complex_backprojection(const std::complex<float> *transient_chunk,
                                      uint32_t transient_size, uint32_t T,
                                      const std::vector<CameraLaserPair> scanned_pairs,
                                      std::complex<float> *voxel_volume,
                                      const uint32_t *voxels_per_side,
                                      const float *volume_zero_pos, const float *voxel_inc,
                                      float t0, float deltaT) {
    raise_on(bpgb_backproject_c64(reinterpret_cast<const float *>(transient_chunk),
                                  transient_size, T,
                                  reinterpret_cast<const bpgb_pair *>(scanned_pairs.data()),
                                  scanned_pairs.size(), reinterpret_cast<float *>(voxel_volume),
                                  voxels_per_side, volume_zero_pos, voxel_inc, t0, deltaT),
             "call_cuda_complex_backprojection");
}
