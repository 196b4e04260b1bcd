// A caller written against the reference's CUDA API header (backproject_cuda.hpp:19-49),
// compiled against include/backproject_cuda_gb300.hpp and linked with libbpgb300: the
// shape of code in bp::backproject (backproject.hpp:883, 894) and
// bp::phasor_reconstruction (:1027), which pass a std::vector<CameraLaserPair> and
// caller-owned host buffers.
//
//   dropin_caller <input.bin> <output.bin>
//
// input.bin (little endian): "BPIN", u32 complex, u32 T, u32 P, u32 N[3], f32 zero[3],
// f32 inc[9], f32 t0, f32 deltaT, then H (P * T floats, or P * T complex64) and P pairs
// (32 bytes each).  output.bin: the volume (N[0] * N[1] * N[2] floats or complex64).
// Exit status: 0 ok, 2 bad input, 3 the call threw; after a successful call it also
// checks that a malformed call (transient_size != P * T) throws std::runtime_error.
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "backproject_cuda_gb300.hpp"

namespace {
template <typename T>
bool read(FILE *f, T *dst, size_t n) {
    return std::fread(dst, sizeof(T), n, f) == n;
}
}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    char magic[4];
    uint32_t cplx = 0, T = 0, P = 0, N[3];
    float zero[3], inc[9], t0 = 0, dT = 0;
    bool ok = read(f, magic, 4) && std::memcmp(magic, "BPIN", 4) == 0 && read(f, &cplx, 1) &&
              read(f, &T, 1) && read(f, &P, 1) && read(f, N, 3) && read(f, zero, 3) &&
              read(f, inc, 9) && read(f, &t0, 1) && read(f, &dT, 1);
    if (!ok) return 2;
    const size_t nh = (size_t)P * T, nv = (size_t)N[0] * N[1] * N[2];
    std::vector<float> H(nh * (cplx ? 2 : 1));
    std::vector<CameraLaserPair> pairs(P);
    ok = read(f, H.data(), H.size()) && read(f, pairs.data(), P);
    std::fclose(f);
    if (!ok) return 2;

    std::vector<float> vol(nv * (cplx ? 2 : 1), -1.0f);
    try {
        if (cplx)
            call_cuda_complex_backprojection(
                reinterpret_cast<const std::complex<float> *>(H.data()), (uint32_t)nh, T, pairs,
                reinterpret_cast<std::complex<float> *>(vol.data()), N, zero, inc, t0, dT);
        else
            call_cuda_backprojection(H.data(), (uint32_t)nh, T, pairs, vol.data(), N, zero, inc, t0,
                                     dT);
    } catch (const std::runtime_error &e) {
        std::fprintf(stderr, "call threw: %s\n", e.what());
        return 3;
    }
    FILE *o = std::fopen(argv[2], "wb");
    if (!o || std::fwrite(vol.data(), sizeof(float), vol.size(), o) != vol.size()) return 2;
    std::fclose(o);

    // The reference prints and exits on a bad call; this drop-in throws instead.
    bool threw = false;
    try {
        call_cuda_backprojection(H.data(), (uint32_t)nh + 1, T, pairs, vol.data(), N, zero, inc,
                                 t0, dT);
    } catch (const std::runtime_error &) {
        threw = true;
    }
    if (!threw) {
        std::fprintf(stderr, "malformed call did not throw\n");
        return 4;
    }
    std::printf("ok\n");
    return 0;
}
