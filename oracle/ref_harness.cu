// Loader for the reference kernel -- TEST INFRASTRUCTURE ONLY.
//
// The reference's own kernel, cuda_backprojection_impl<float | cuComplex>
// (backproject_cuda.cu:117-175), is compiled from its unmodified sources into
// oracle/_ref/backproject_cuda_ref.cubin (see backprojector_gb300/build.py).  Its host
// launcher in the same file is x86 code built against thrust, so this file restates the
// launcher's policy (backproject_cuda.cu:380-499 / 681-800) with the driver API:
//   block = min(cudaOccupancyMaxPotentialBlockSize(kernel, dyn smem = sizeof(FT)), P, 256)
//   grid = 16 x 16 x 16, per-block voxel cursors initialised to the block coordinates,
//   ceil(max(N) / 16)^3 launches with a device synchronise after each,
//   dynamic shared memory = block * sizeof(FT), footprint 0, output copied in and out.
// Used only to generate golden fixtures and to time the reference kernel on the GPU.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

namespace {

const char *kFloatKernel =
    "_Z24cuda_backprojection_implIfEvPT_PjS2_P15CameraLaserPairS1_PfS5_S5_S5_S5_S2_S2_";
const char *kComplexKernel =
    "_Z24cuda_backprojection_implI6float2EvPT_PjS3_P15CameraLaserPairS2_PfS6_S6_S6_S6_S3_S3_";

template <typename T>
int dev_copy(T **d, const T *h, size_t n) {
    if (cudaMalloc((void **)d, n * sizeof(T)) != cudaSuccess) return -3;
    if (h && cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return -2;
    return 0;
}

}  // namespace

extern "C" int bpref_backproject(const char *cubin_path, int is_complex, const float *H,
                                 uint64_t P, uint32_t T, const void *pairs, float *volume,
                                 const uint32_t *N, const float *zero, const float *inc,
                                 float t0, float deltaT, int *block_out, double *ms_out) {
    // The reference indexes H with 32-bit arithmetic (pair * T + bin) and needs P > 0.
    if (P == 0 || P * (uint64_t)T >= (1ull << 32) || (uint64_t)N[0] * N[1] * N[2] >= (1ull << 32))
        return -1;
    if (cudaFree(0) != cudaSuccess) return -6;
    CUmodule mod;
    if (cuModuleLoad(&mod, cubin_path) != CUDA_SUCCESS) return -10;
    CUfunction f;
    if (cuModuleGetFunction(&f, mod, is_complex ? kComplexKernel : kFloatKernel) != CUDA_SUCCESS) {
        cuModuleUnload(mod);
        return -11;
    }
    const size_t fsz = is_complex ? 8 : 4;
    int min_grid = 0, block = 0;
    if (cuOccupancyMaxPotentialBlockSize(&min_grid, &block, f, nullptr, fsz, 0) != CUDA_SUCCESS) {
        cuModuleUnload(mod);
        return -12;
    }
    block = (int)std::min<uint64_t>(std::min<uint64_t>((uint64_t)block, P), 256);
    if (block_out) *block_out = block;
    const uint32_t G = 16;
    std::vector<uint32_t> cursors(G * G * G * 3);
    for (uint32_t x = 0; x < G; x++)
        for (uint32_t y = 0; y < G; y++)
            for (uint32_t z = 0; z < G; z++) {
                const uint32_t b = (x * G * G + y * G + z) * 3;
                cursors[b] = x;
                cursors[b + 1] = y;
                cursors[b + 2] = z;
            }
    const uint64_t nvox = (uint64_t)N[0] * N[1] * N[2];
    const uint32_t num_pairs = (uint32_t)P;
    const float footprint = 0.0f;
    float *dH = nullptr, *dV = nullptr, *dz = nullptr, *di = nullptr, *dt0 = nullptr,
          *ddT = nullptr, *dfp = nullptr;
    uint32_t *dTn = nullptr, *dP = nullptr, *dN = nullptr, *dcur = nullptr;
    void *dpairs = nullptr;
    int st = 0;
    st = st ? st : dev_copy(&dH, H, P * T * (is_complex ? 2 : 1));
    st = st ? st : dev_copy(&dV, volume, nvox * (is_complex ? 2 : 1));
    st = st ? st : dev_copy(&dz, zero, 3);
    st = st ? st : dev_copy(&di, inc, 9);
    st = st ? st : dev_copy(&dt0, &t0, 1);
    st = st ? st : dev_copy(&ddT, &deltaT, 1);
    st = st ? st : dev_copy(&dfp, &footprint, 1);
    st = st ? st : dev_copy(&dTn, &T, 1);
    st = st ? st : dev_copy(&dP, &num_pairs, 1);
    st = st ? st : dev_copy(&dN, N, 3);
    st = st ? st : dev_copy(&dcur, cursors.data(), cursors.size());
    if (!st) {
        if (cudaMalloc(&dpairs, P * 32) != cudaSuccess ||
            cudaMemcpy(dpairs, pairs, P * 32, cudaMemcpyHostToDevice) != cudaSuccess)
            st = -2;
    }
    if (!st) {
        const uint32_t maxn = std::max(std::max(N[0], N[1]), N[2]);
        uint32_t runs = (uint32_t)std::ceil(maxn / (float)G);
        runs = runs * runs * runs;
        void *args[] = {&dH, &dTn, &dP, &dpairs, &dV, &dz, &di, &dt0, &ddT, &dfp, &dN, &dcur};
        const auto t_start = std::chrono::steady_clock::now();
        for (uint32_t r = 0; r < runs && !st; r++) {
            if (cuLaunchKernel(f, G, G, G, block, 1, 1, block * fsz, nullptr, args, nullptr) !=
                CUDA_SUCCESS)
                st = -13;
            else if (cuCtxSynchronize() != CUDA_SUCCESS)
                st = -14;
        }
        const auto t_end = std::chrono::steady_clock::now();
        if (ms_out) ms_out[0] = std::chrono::duration<double, std::milli>(t_end - t_start).count();
    }
    if (!st && cudaMemcpy(volume, dV, nvox * fsz, cudaMemcpyDeviceToHost) != cudaSuccess) st = -2;
    cudaFree(dH);
    cudaFree(dV);
    cudaFree(dz);
    cudaFree(di);
    cudaFree(dt0);
    cudaFree(ddT);
    cudaFree(dfp);
    cudaFree(dTn);
    cudaFree(dP);
    cudaFree(dN);
    cudaFree(dcur);
    cudaFree(dpairs);
    cuModuleUnload(mod);
    return st;
}
