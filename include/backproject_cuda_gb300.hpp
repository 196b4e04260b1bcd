/*
 * C++ drop-in for the reference's CUDA API header (backproject_cuda.hpp:1-51).
 *
 * Same struct and the same three signatures, so code written against the reference
 * (bp::backproject, main.cpp, nlosbpy) links against libbpgb300 unchanged.  Behaviour
 * differences, all deliberate:
 *   - errors throw std::runtime_error (the reference prints and calls exit(1));
 *   - every pair is used and every voxel visited (the reference drops P mod blockDim
 *     pairs and skips voxels when N is not a multiple of 16);
 *   - call_cuda_octree_backprojection computes the dense volume (the reference's GPU
 *     octree prints "NOT WORKING YET" and depends on environment variables).
 */
#ifndef BACKPROJECT_CUDA_GB300_HPP
#define BACKPROJECT_CUDA_GB300_HPP

#include <inttypes.h>

#include <array>
#include <complex>
#include <vector>

struct CameraLaserPair {
    float camera_point[3], laser_point[3];
    float camera_wall, laser_wall;
};

/* call_cuda_backprojection, backproject_cuda.hpp:19-28 */
void call_cuda_backprojection(const float *transient_chunk, uint32_t transient_size, uint32_t T,
                              const std::vector<CameraLaserPair> scanned_pairs,
                              float *voxel_volume, const uint32_t *voxels_per_side,
                              const float *volume_zero_pos, const float *voxel_inc, float t0,
                              float deltaT);

/* call_cuda_octree_backprojection, backproject_cuda.hpp:30-39 */
void call_cuda_octree_backprojection(const float *transient_chunk, uint32_t transient_size,
                                     uint32_t T,
                                     const std::vector<CameraLaserPair> scanned_pairs,
                                     float *voxel_volume, const uint32_t *voxels_per_side,
                                     const float *volume_zero_pos, const float *voxel_inc,
                                     float t0, float deltaT);

/* call_cuda_complex_backprojection, backproject_cuda.hpp:41-49 */
void call_cuda_complex_backprojection(const std::complex<float> *transient_chunk,
                                      uint32_t transient_size, uint32_t T,
                                      const std::vector<CameraLaserPair> scanned_pairs,
                                      std::complex<float> *voxel_volume,
                                      const uint32_t *voxels_per_side,
                                      const float *volume_zero_pos, const float *voxel_inc,
                                      float t0, float deltaT);

#endif
