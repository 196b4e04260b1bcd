// Python module `nlosbpy` with the reference binding's functions and keyword arguments
// (nlosbpy.cpp:15-120): backproject(...) -> float32 [Nx, Ny, Nz] and
// phasor(...) -> complex64 [Nx, Ny, Nz], on the GPU through the C ABI.
//
// Layouts: assume_row_major=True takes transient data [lx, ly, cx, cy, T] (exhaustive) or
// [cx, cy, T] (confocal) and grids [gx, gy, 3].  assume_row_major=False (the reference's
// default) takes the same arrays with all axes reversed ([T, cy, cx, ly, lx], grids
// [3, gy, gx]) and transposes them.  use_cpu=True raises: this engine has no CPU path.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "backprojector_gb300.h"

namespace py = pybind11;
using namespace pybind11::literals;

namespace {

using farr = py::array_t<float, py::array::c_style | py::array::forcecast>;
using uarr = py::array_t<uint32_t, py::array::c_style | py::array::forcecast>;

void check(int st, const char *what) {
    if (st != BPGB_OK)
        throw std::runtime_error(std::string(what) + ": " + bpgb_status_string(st) + ": " +
                                 bpgb_last_error());
}

// Reverses the axes of a column-major array into a C-contiguous row-major copy.
farr to_row_major(const py::array &a, bool row_major) {
    if (row_major) return farr::ensure(a);
    py::object t = a.attr("transpose")();
    return farr::ensure(py::module_::import("numpy").attr("ascontiguousarray")(t, "dtype"_a = "float32"));
}

std::vector<float> vec3(const py::array &a, const char *name) {
    farr f = farr::ensure(a);
    if (!f || f.size() != 3) throw std::invalid_argument(std::string(name) + " must have 3 entries");
    return std::vector<float>(f.data(), f.data() + 3);
}

struct Capture {
    farr data, cgrid, lgrid;
    uint32_t T = 0, cx = 0, cy = 0, lx = 0, ly = 0;
};

Capture read_capture(const py::array &transient_data, const py::array &camera_grid_positions,
                     const py::array &laser_grid_positions, bool is_confocal, bool row_major) {
    Capture c;
    c.data = to_row_major(transient_data, row_major);
    c.cgrid = to_row_major(camera_grid_positions, row_major);
    c.lgrid = to_row_major(laser_grid_positions, row_major);
    if (c.cgrid.ndim() != 3 || c.cgrid.shape(2) != 3)
        throw std::invalid_argument("camera_grid_positions must be [cx, cy, 3] (row-major)");
    c.cx = (uint32_t)c.cgrid.shape(0);
    c.cy = (uint32_t)c.cgrid.shape(1);
    if (is_confocal) {
        if (c.data.ndim() != 3 || (uint32_t)c.data.shape(0) != c.cx ||
            (uint32_t)c.data.shape(1) != c.cy)
            throw std::invalid_argument("confocal transient_data must be [cx, cy, T]");
        c.T = (uint32_t)c.data.shape(2);
        c.lx = c.cx;
        c.ly = c.cy;
    } else {
        if (c.lgrid.ndim() != 3 || c.lgrid.shape(2) != 3)
            throw std::invalid_argument("laser_grid_positions must be [lx, ly, 3] (row-major)");
        c.lx = (uint32_t)c.lgrid.shape(0);
        c.ly = (uint32_t)c.lgrid.shape(1);
        if (c.data.ndim() != 5 || (uint32_t)c.data.shape(0) != c.lx ||
            (uint32_t)c.data.shape(1) != c.ly || (uint32_t)c.data.shape(2) != c.cx ||
            (uint32_t)c.data.shape(3) != c.cy)
            throw std::invalid_argument("transient_data must be [lx, ly, cx, cy, T]");
        c.T = (uint32_t)c.data.shape(4);
    }
    return c;
}

py::array backproject(const py::array &transient_data, const py::array &camera_grid_positions,
                      const py::array &laser_grid_positions, const py::array &camera_position,
                      const py::array &laser_position, float t0, float deltaT, bool is_confocal,
                      const py::array &volume_position, const py::array &volume_size,
                      const py::array &voxels_per_side, const py::array &wall_normal,
                      bool assume_row_major, bool use_cpu) {
    if (use_cpu)
        throw std::invalid_argument("use_cpu=True: this engine runs on the GPU only");
    Capture c = read_capture(transient_data, camera_grid_positions, laser_grid_positions,
                             is_confocal, assume_row_major);
    const auto cp = vec3(camera_position, "camera_position");
    const auto lp = vec3(laser_position, "laser_position");
    const auto vp = vec3(volume_position, "volume_position");
    const auto vs = vec3(volume_size, "volume_size");
    const auto wn = vec3(wall_normal, "wall_normal");
    uarr n = uarr::ensure(voxels_per_side);
    if (!n || n.size() != 3) throw std::invalid_argument("voxels_per_side must have 3 entries");
    py::array_t<float> out({(py::ssize_t)n.data()[0], (py::ssize_t)n.data()[1], (py::ssize_t)n.data()[2]});
    int st;
    {
        py::gil_scoped_release nogil;
        st = bpgb_backproject_capture(c.data.data(), c.T, c.cgrid.data(), c.cx, c.cy,
                                      c.lgrid.data(), c.lx, c.ly, cp.data(), lp.data(), t0,
                                      deltaT, is_confocal ? 1 : 0, vp.data(), vs.data(), n.data(),
                                      wn.data(), 0, nullptr, out.mutable_data());
    }
    check(st, "backproject");
    return out;
}

py::array phasor(const py::array &transient_data, const py::array &camera_grid_positions,
                 const py::array &laser_grid_positions, const py::array &camera_position,
                 const py::array &laser_position, float t0, float deltaT, bool is_confocal,
                 const py::array &volume_position, const py::array &volume_size,
                 const py::array &voxels_per_side, float wavelength, bool assume_row_major,
                 bool use_cpu) {
    if (use_cpu)
        throw std::invalid_argument("use_cpu=True: this engine runs on the GPU only");
    Capture c = read_capture(transient_data, camera_grid_positions, laser_grid_positions,
                             is_confocal, assume_row_major);
    const auto cp = vec3(camera_position, "camera_position");
    const auto lp = vec3(laser_position, "laser_position");
    const auto vp = vec3(volume_position, "volume_position");
    const auto vs = vec3(volume_size, "volume_size");
    uarr n = uarr::ensure(voxels_per_side);
    if (!n || n.size() != 3) throw std::invalid_argument("voxels_per_side must have 3 entries");
    py::array_t<std::complex<float>> out(
        {(py::ssize_t)n.data()[0], (py::ssize_t)n.data()[1], (py::ssize_t)n.data()[2]});
    const float zeros[3] = {0, 0, 0};
    int st;
    {
        py::gil_scoped_release nogil;
        st = bpgb_phasor_capture(c.data.data(), c.T, c.cgrid.data(), c.cx, c.cy, c.lgrid.data(),
                                 c.lx, c.ly, cp.data(), lp.data(), t0, deltaT,
                                 is_confocal ? 1 : 0, vp.data(), vs.data(), n.data(), zeros,
                                 wavelength, nullptr, reinterpret_cast<float *>(out.mutable_data()));
    }
    check(st, "phasor");
    return out;
}

}  // namespace

PYBIND11_MODULE(nlosbpy, m) {
    m.doc() = "GB300 NLOS backprojection and phasor-field reconstruction (drop-in for nlosbpy)";
    m.def("backproject", &backproject,
          "Backprojects a transient capture to get an unfiltered volume.", "transient_data"_a,
          "camera_grid_positions"_a, "laser_grid_positions"_a, "camera_position"_a,
          "laser_position"_a, "t0"_a, "deltaT"_a, "is_confocal"_a, "volume_position"_a,
          "volume_size"_a, "voxels_per_side"_a, "wall_normal"_a, "assume_row_major"_a = false,
          "use_cpu"_a = false);
    m.def("phasor", &phasor, "Reconstruct a transient capture using phasor fields.",
          "transient_data"_a, "camera_grid_positions"_a, "laser_grid_positions"_a,
          "camera_position"_a, "laser_position"_a, "t0"_a, "deltaT"_a, "is_confocal"_a,
          "volume_position"_a, "volume_size"_a, "voxels_per_side"_a, "wavelength"_a,
          "assume_row_major"_a = false, "use_cpu"_a = false);
}
