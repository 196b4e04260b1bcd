// bpgb_backprojector: the command-line reconstruction tool (the reference's main.cpp:27-189)
// over this library's C ABI.  The reference reads Zaragoza-format HDF5 datasets and writes
// HDF5; libhdf5 is not part of this build, so the dataset arrives as an uncompressed .npz
// with the same arrays and the volume leaves as a float32 .npy:
//
//   data                    float32 [lx, ly, cx, cy, T]  ([cx, cy, T] confocal); with a
//                           bounce axis before T ([..., B, T]) plus `bounces` (int [B], the
//                           bounce number of each slice) the slices 3..max-bounce are summed
//   camera_grid_positions   float32 [cx, cy, 3]
//   laser_grid_positions    float32 [lx, ly, 3] (ignored when confocal)
//   camera_position, laser_position   float32 [3]
//   t0, deltat              scalars
//   is_confocal             scalar (0 / 1), optional (default 0)
//   hidden_volume_position  float32 [3];  hidden_volume_size  float32 [3] or scalar
//
// Flags follow the reference: -b/--max-bounce, -r/--voxel-resolution X Y Z (equal values are
// scaled to the volume's aspect, main.cpp:128-131), -c/--volume-position, -s/--volume-size,
// -d/--volume-direction (not implemented in the reference either: ignored), -o/--output,
// --cpu (rejected: this engine has no CPU path), --octree (the learned octree, weights from
// --weights), --phasor with -w/--wavelength (the magnitude of the complex volume is saved,
// main.cpp:162-166).  Extra: --t0-mode 0|1 (0 keeps the reference's fractional time-window
// offset, 1 floors it), --fp16 (octree: FP16 rows).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "backprojector_gb300.h"
#include "npy.h"

using bpgb::NpyArray;

namespace {

int usage(const char *msg) {
    if (msg) std::fprintf(stderr, "error: %s\n\n", msg);
    std::fprintf(stderr,
                 "usage: bpgb_backprojector DATASET.npz [-b N] [-r X Y Z] [-c X Y Z] [-s X Y Z]\n"
                 "                          [-d X Y Z] [-o OUT.npy] [--cpu] [--octree [--weights W.npz]]\n"
                 "                          [--phasor] [-w WAVELENGTH] [--t0-mode 0|1] [--fp16]\n"
                 "Takes an NLOS dataset (.npz) and writes an unfiltered backprojection volume (.npy).\n");
    return msg ? 2 : 0;
}

bool vec3(int &i, int argc, char **argv, float *v) {
    if (i + 3 >= argc) return false;
    for (int k = 0; k < 3; k++) {
        char *end = nullptr;
        v[k] = std::strtof(argv[++i], &end);
        if (!end || *end) return false;
    }
    return true;
}

int fail(const std::string &m) {
    std::fprintf(stderr, "error: %s\n", m.c_str());
    return 1;
}

std::string lib_error(int st) {
    return std::string(bpgb_status_string(st)) + ": " + bpgb_last_error();
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) return usage("a dataset file is required");
    std::string file, outfile, weights;
    int max_bounce = 3, t0_mode = 0;
    float res[3] = {32, 32, 32}, pos[3] = {NAN, NAN, NAN}, size[3] = {NAN, NAN, NAN}, dir[3];
    float wavelength = 0.005f;
    bool use_cpu = false, use_octree = false, use_phasor = false, fp16 = false;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto next = [&](const char *what) -> const char * {
            if (i + 1 >= argc) {
                usage((std::string(what) + " needs a value").c_str());
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help") return usage(nullptr);
        if (a == "-b" || a == "--max-bounce") {
            max_bounce = std::atoi(next("-b"));
        } else if (a == "-r" || a == "--voxel-resolution") {
            if (!vec3(i, argc, argv, res)) return usage("-r takes three numbers");
        } else if (a == "-c" || a == "--volume-position") {
            if (!vec3(i, argc, argv, pos)) return usage("-c takes three numbers");
        } else if (a == "-s" || a == "--volume-size") {
            if (!vec3(i, argc, argv, size)) return usage("-s takes three numbers");
        } else if (a == "-d" || a == "--volume-direction") {
            if (!vec3(i, argc, argv, dir)) return usage("-d takes three numbers");
            std::fprintf(stderr, "warning: --volume-direction is not implemented; ignored\n");
        } else if (a == "-o" || a == "--output") {
            outfile = next("-o");
        } else if (a == "--cpu") {
            use_cpu = true;
        } else if (a == "--octree") {
            use_octree = true;
        } else if (a == "--phasor") {
            use_phasor = true;
        } else if (a == "-w" || a == "--wl" || a == "--wavelength") {
            wavelength = std::strtof(next("-w"), nullptr);
        } else if (a == "--weights") {
            weights = next("--weights");
        } else if (a == "--t0-mode") {
            t0_mode = std::atoi(next("--t0-mode"));
        } else if (a == "--fp16") {
            fp16 = true;
        } else if (!a.empty() && a[0] == '-') {
            return usage(("unknown flag " + a).c_str());
        } else if (file.empty()) {
            file = a;
        } else {
            return usage(("unexpected argument " + a).c_str());
        }
    }
    if (file.empty()) return usage("a dataset file is required");
    if (use_cpu) return fail("--cpu: this engine has no CPU path (GB300 only)");
    if (use_octree && use_phasor) return fail("--octree and --phasor together are not supported");
    if (max_bounce < 3) return fail("--max-bounce counts from 3");

    std::map<std::string, NpyArray> ds;
    std::string why;
    if (!bpgb::npz_load(file, &ds, &why)) return fail(why);
    for (const char *k : {"data", "camera_grid_positions", "camera_position", "t0", "deltat",
                          "hidden_volume_position", "hidden_volume_size"})
        if (!ds.count(k)) return fail(file + ": missing array '" + k + "'");
    const bool confocal = ds.count("is_confocal") && ds["is_confocal"].at(0) != 0.0;
    if (!confocal)
        for (const char *k : {"laser_grid_positions", "laser_position"})
            if (!ds.count(k)) return fail(file + ": missing array '" + k + "'");
    const NpyArray &cg = ds["camera_grid_positions"];
    if (cg.shape.size() != 3 || cg.shape[2] != 3) return fail("camera_grid_positions must be [cx, cy, 3]");
    const uint32_t cx = (uint32_t)cg.shape[0], cy = (uint32_t)cg.shape[1];
    uint32_t lx = 1, ly = 1;
    std::vector<float> lgrid, lpos(3, 0.0f);
    if (!confocal) {
        const NpyArray &lg = ds["laser_grid_positions"];
        if (lg.shape.size() != 3 || lg.shape[2] != 3) return fail("laser_grid_positions must be [lx, ly, 3]");
        lx = (uint32_t)lg.shape[0];
        ly = (uint32_t)lg.shape[1];
        lgrid = lg.as_float();
        lpos = ds["laser_position"].as_float();
    }
    const std::vector<float> cgrid = cg.as_float(), cpos = ds["camera_position"].as_float();
    if (cpos.size() != 3 || lpos.size() != 3) return fail("positions must have 3 components");
    const float t0 = (float)ds["t0"].at(0), deltaT = (float)ds["deltat"].at(0);

    // transient data, bounce slices summed
    const NpyArray &d = ds["data"];
    const size_t grid_dims = confocal ? 2 : 4;
    const uint64_t P = confocal ? (uint64_t)cx * cy : (uint64_t)lx * ly * cx * cy;
    std::vector<uint64_t> want(confocal ? std::vector<uint64_t>{cx, cy}
                                        : std::vector<uint64_t>{lx, ly, cx, cy});
    bool bounce_axis = d.shape.size() == grid_dims + 2;
    if (d.shape.size() != grid_dims + 1 && !bounce_axis)
        return fail("data must be [lx, ly, cx, cy, T] ([cx, cy, T] confocal), optionally with a "
                    "bounce axis before T");
    for (size_t k = 0; k < grid_dims; k++)
        if (d.shape[k] != want[k]) return fail("data's grid dimensions do not match the grids");
    const uint32_t T = (uint32_t)d.shape.back();
    std::vector<float> H((size_t)P * T, 0.0f);
    if (!bounce_axis) {
        H = d.as_float();
    } else {
        const uint64_t B = d.shape[grid_dims];
        if (!ds.count("bounces") || ds["bounces"].count() != B)
            return fail("a bounce axis needs 'bounces' with one bounce number per slice");
        const std::vector<float> all = d.as_float();
        for (uint64_t b = 0; b < B; b++) {
            const double id = ds["bounces"].at(b);
            if (id < 3 || id > max_bounce) continue;
            for (uint64_t p = 0; p < P; p++)
                for (uint32_t t = 0; t < T; t++) H[p * T + t] += all[(p * B + b) * T + t];
        }
    }

    // volume: dataset defaults, resolution scaled to the aspect when all three are equal
    const std::vector<float> dpos = ds["hidden_volume_position"].as_float();
    const std::vector<float> dsize = ds["hidden_volume_size"].as_float();
    for (int k = 0; k < 3; k++) {
        if (std::isnan(pos[k])) pos[k] = dpos.size() == 3 ? dpos[k] : dpos[0];
        if (std::isnan(size[k])) size[k] = dsize.size() == 3 ? dsize[k] : dsize[0];
    }
    uint32_t n[3];
    if (res[0] == res[1] && res[1] == res[2]) {
        const float mx = std::fmax(size[0], std::fmax(size[1], size[2]));
        for (int k = 0; k < 3; k++) n[k] = (uint32_t)(res[k] * size[k] / mx);
    } else {
        for (int k = 0; k < 3; k++) n[k] = (uint32_t)res[k];
    }
    for (int k = 0; k < 3; k++)
        if (n[k] == 0) return fail("voxel resolution is zero along an axis");
    const uint64_t nvox = (uint64_t)n[0] * n[1] * n[2];
    std::vector<float> vol(nvox);

    int st = 0;
    if (use_phasor) {
        std::vector<float> cvol(2 * nvox);
        st = bpgb_phasor_capture(H.data(), T, cgrid.data(), cx, cy, confocal ? nullptr : lgrid.data(),
                                 lx, ly, cpos.data(), lpos.data(), t0, deltaT, confocal ? 1 : 0, pos,
                                 size, n, nullptr, wavelength, nullptr, cvol.data());
        for (uint64_t i = 0; i < nvox; i++) vol[i] = std::hypot(cvol[2 * i], cvol[2 * i + 1]);
    } else if (use_octree) {
        if (weights.empty()) {
            const char *env = std::getenv("BPGB_OCTREE_WEIGHTS");
            if (!env) return fail("--octree needs --weights W.npz (or BPGB_OCTREE_WEIGHTS)");
            weights = env;
        }
        std::vector<bpgb_pair> pairs(P);
        st = bpgb_precompute_pairs(lpos.data(), confocal ? cgrid.data() : lgrid.data(),
                                   confocal ? cx : lx, confocal ? cy : ly, cpos.data(), cgrid.data(),
                                   cx, cy, confocal ? 1 : 0, pairs.data());
        float zero[3], inc[9];
        if (st == 0) st = bpgb_volume_basis(pos, size, n, nullptr, zero, inc);
        bpgb_octree oc = nullptr;
        bpgb_options o;
        bpgb_options_default(&o);
        o.h_dtype = fp16 ? BPGB_DTYPE_F16 : BPGB_DTYPE_F32;
        if (st == 0)
            st = bpgb_octree_create(&oc, pairs.data(), P, T, n, zero, inc, t0, deltaT,
                                    weights.c_str(), 0.0f, &o);
        if (st == 0) st = bpgb_octree_reconstruct_host(oc, H.data(), vol.data());
        uint32_t sel = 0;
        bpgb_octree_info info;
        if (st == 0 && bpgb_octree_selected(oc, &sel) == 0 && bpgb_octree_get_info(oc, &info) == 0)
            std::printf("octree: %u of %u tiles at full resolution\n", sel, info.tiles);
        if (oc) bpgb_octree_destroy(oc);
    } else {
        st = bpgb_backproject_capture(H.data(), T, cgrid.data(), cx, cy,
                                      confocal ? nullptr : lgrid.data(), lx, ly, cpos.data(),
                                      lpos.data(), t0, deltaT, confocal ? 1 : 0, pos, size, n,
                                      nullptr, t0_mode, nullptr, vol.data());
    }
    if (st) return fail(lib_error(st));
    if (outfile.empty()) {
        const size_t dot = file.rfind(".npz");
        outfile = (dot == std::string::npos ? file : file.substr(0, dot)) + "_recon.npy";
    }
    if (!bpgb::npy_save_f32(outfile, vol.data(), {n[0], n[1], n[2]}, &why)) return fail(why);
    std::printf("Backprojected to %s\n", outfile.c_str());
    return 0;
}
