"""CPU oracle for the backprojection hot path -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker (or as the timed restatement of the reference's OpenMP CPU path).  The product
package never imports it.

Parity pins (the reference has no tests or golden vectors of its own): the committed
fixtures under tests/golden/ hold outputs of the reference's unmodified kernel
(backproject_cuda.cu, built from its sources for sm_103a and run on a GB300 through
oracle/ref_harness.cu), generated by tests/golden/make_golden.py.

C restatements live in oracle.c (each function cites the reference file:line it
follows); this module wraps them with numpy and adds the parity metrics.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_CUBIN = HERE / "_ref" / "backproject_cuda_ref.cubin"
REF_LIB = HERE / "_ref" / "libbpref.so"

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_U32 = C.POINTER(C.c_uint32)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_P = C.c_void_p

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            import sys

            sys.path.insert(0, str(HERE.parent))
            from backprojector_gb300 import build

            build.build_oracle()
        L = C.CDLL(str(LIB))
        common = [_F, C.c_uint64, C.c_uint32, _P, _U32, _F, _F, C.c_float, C.c_float, C.c_uint32,
                  _I64, C.c_int64, _D]
        for name in ("orc_bp_gpu_f64", "orc_bp_gpu_c64", "orc_bp_gpu_f32emu"):
            getattr(L, name).argtypes = common
            getattr(L, name).restype = None
        L.orc_bins.argtypes = [C.c_uint64, C.c_uint32, _P, _U32, _F, _F, C.c_float, C.c_float, _I64,
                               C.c_int64, C.c_int, _I32]
        L.orc_bins.restype = None
        for name in ("orc_bp_cpu_classic_f32", "orc_bp_cpu_classic_c64"):
            getattr(L, name).argtypes = [_F, C.c_uint64, C.c_uint32, _P, _U32, _F, _F, C.c_float,
                                         C.c_float, _I64, C.c_int64, _F]
            getattr(L, name).restype = None
        L.orc_phasor_taps.argtypes = [C.c_float, C.c_float, C.c_uint32, _F, C.c_int]
        L.orc_phasor_taps.restype = C.c_int
        L.orc_phasor_pulse.argtypes = [_F, C.c_int64, C.c_int32, C.c_float, C.c_float, C.c_uint32, _F]
        L.orc_phasor_pulse.restype = None
        L.orc_precompute_distances.argtypes = [_F, _F, C.c_uint32, C.c_uint32, _F, _F, C.c_uint32,
                                               C.c_uint32, C.c_int, _P]
        L.orc_precompute_distances.restype = None
        L.orc_synth_render.argtypes = [_P, C.c_uint64, C.c_uint32, C.c_float, C.c_float, _F, _F,
                                       C.c_uint64, _F]
        L.orc_synth_render.restype = None
        L.orc_synth_poisson.argtypes = [_F, C.c_uint64, C.c_float, C.c_uint64]
        L.orc_synth_poisson.restype = None
        L.orc_time_limits_corners.argtypes = [_F, _F, C.c_uint32, C.c_uint32, _F, _F, C.c_uint32,
                                              C.c_uint32, _F, _F, C.c_float, C.c_float, _F]
        L.orc_time_limits_corners.restype = None
        L.orc_num_threads.argtypes = []
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _fp(a):
    return a.ctypes.data_as(_F)


def _ids(voxels):
    if voxels is None:
        return None, 0
    v = np.ascontiguousarray(np.asarray(voxels, dtype=np.int64))
    return v, len(v)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def _gpu_call(name, H, pairs, N, zero, inc, t0, dT, ref_block, voxels, cplx):
    Hc = np.ascontiguousarray(H)
    if cplx:
        Hc = np.ascontiguousarray(Hc.astype(np.complex64)).view(np.float32)
        T = Hc.shape[-1] // 2
    else:
        Hc = _f32(Hc)
        T = Hc.shape[-1]
    n = np.ascontiguousarray(np.asarray(N, dtype=np.uint32))
    ids, nl = _ids(voxels)
    nout = nl if ids is not None else int(np.prod(n.astype(np.int64)))
    out = np.zeros(nout * (2 if cplx else 1), np.float64)
    getattr(lib(), name)(_fp(Hc), len(pairs), T, C.c_void_p(pairs.ctypes.data),
                         n.ctypes.data_as(_U32), _fp(_f32(zero)), _fp(_f32(inc)), t0, dT,
                         ref_block, ids.ctypes.data_as(_I64) if ids is not None else None, nl,
                         out.ctypes.data_as(_D))
    if cplx:
        out = out.view(np.complex128)
    return out if ids is not None else out.reshape(tuple(int(x) for x in n))


def bp_gpu_f64(H, pairs, N, zero, inc, t0, dT, ref_block=0, voxels=None):
    """FP64 restatement of cuda_backprojection_impl<float> (backproject_cuda.cu:117-175)."""
    return _gpu_call("orc_bp_gpu_f64", H, pairs, N, zero, inc, t0, dT, ref_block, voxels, False)


def bp_gpu_c64(H, pairs, N, zero, inc, t0, dT, ref_block=0, voxels=None):
    """FP64 restatement of cuda_backprojection_impl<cuComplex>; complex128 result."""
    return _gpu_call("orc_bp_gpu_c64", H, pairs, N, zero, inc, t0, dT, ref_block, voxels, True)


def bp_gpu_f32emu(H, pairs, N, zero, inc, t0, dT, ref_block=0, voxels=None):
    """The reference kernel's FP32 bin arithmetic, sums in FP64."""
    return _gpu_call("orc_bp_gpu_f32emu", H, pairs, N, zero, inc, t0, dT, ref_block, voxels, False)


def bins(pairs, T, N, zero, inc, t0, dT, voxels, mode=0) -> np.ndarray:
    """int32 [len(voxels), P] bin indices (-1 = out of range); mode 0 FP64, 1 FP32 emulation."""
    ids, nl = _ids(voxels)
    n = np.ascontiguousarray(np.asarray(N, dtype=np.uint32))
    out = np.zeros((nl, len(pairs)), np.int32)
    lib().orc_bins(len(pairs), T, C.c_void_p(pairs.ctypes.data), n.ctypes.data_as(_U32),
                   _fp(_f32(zero)), _fp(_f32(inc)), t0, dT, ids.ctypes.data_as(_I64), nl, mode,
                   out.ctypes.data_as(_I32))
    return out


def classic(H, pairs, N, volume_position, volume_size, t0, dT, voxels=None):
    """classic_backprojection (backproject.hpp:138-216): the reference's CPU path."""
    cplx = np.iscomplexobj(H)
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.complex64 if cplx else np.float32))
    T = Hc.shape[-1]
    Hf = Hc.view(np.float32) if cplx else Hc
    n = np.ascontiguousarray(np.asarray(N, dtype=np.uint32))
    ids, nl = _ids(voxels)
    nout = nl if ids is not None else int(np.prod(n.astype(np.int64)))
    out = np.zeros(nout * (2 if cplx else 1), np.float32)
    fn = lib().orc_bp_cpu_classic_c64 if cplx else lib().orc_bp_cpu_classic_f32
    fn(_fp(Hf), len(pairs), T, C.c_void_p(pairs.ctypes.data), n.ctypes.data_as(_U32),
       _fp(_f32(volume_position)), _fp(_f32(volume_size)), t0, dT,
       ids.ctypes.data_as(_I64) if ids is not None else None, nl, _fp(out))
    if cplx:
        out = out.view(np.complex64)
    return out if ids is not None else out.reshape(tuple(int(x) for x in n))


def phasor_taps(wavelength, deltaT, times=4) -> np.ndarray:
    K = lib().orc_phasor_taps(wavelength, deltaT, times, None, 0)
    if K <= 0:
        return np.zeros((2, 0), np.float32)
    t = np.zeros(2 * K, np.float32)
    lib().orc_phasor_taps(wavelength, deltaT, times, _fp(t), K)
    return t.reshape(2, K)


def phasor_pulse(H, wavelength, deltaT, times=4) -> np.ndarray:
    """phasor_pulse (backproject.hpp:430-479): complex64 [..., T]."""
    Hc = _f32(H)
    T = Hc.shape[-1]
    rows = Hc.size // T
    out = np.zeros(Hc.shape, np.complex64)
    lib().orc_phasor_pulse(_fp(Hc), rows, T, wavelength, deltaT, times, _fp(out.view(np.float32)))
    return out


def precompute_distances(laser_position, laser_grid, camera_position, camera_grid, confocal=False):
    from backprojector_gb300.capi import PAIR_DTYPE

    cg = _f32(camera_grid)
    lg = _f32(laser_grid) if laser_grid is not None else cg
    cx, cy = cg.shape[:2]
    lx, ly = lg.shape[:2]
    P = cx * cy if confocal else lx * ly * cx * cy
    out = np.zeros(P, PAIR_DTYPE)
    lib().orc_precompute_distances(_fp(_f32(laser_position)), _fp(lg), lx, ly,
                                   _fp(_f32(camera_position)), _fp(cg), cx, cy, 1 if confocal else 0,
                                   C.c_void_p(out.ctypes.data))
    return out


# ---------------------------------------------------------------- emulation of the launcher

def reference_visited(N) -> np.ndarray:
    """Voxels the reference launcher writes (backproject_cuda.cu:48-85, 423-478): a 16^3 grid
    of voxel cursors advanced by (z += 16, wrap z % Nz then y += 16, wrap y % Ny then
    x += 16) over ceil(max N / 16)^3 launches.  Voxels never visited keep the input value."""
    N = [int(v) for v in N]
    G = 16
    runs = int(np.ceil(max(N) / G)) ** 3
    x, y, z = np.meshgrid(np.arange(G), np.arange(G), np.arange(G), indexing="ij")
    x, y, z = x.ravel().copy(), y.ravel().copy(), z.ravel().copy()
    seen = np.zeros(N, bool)
    for _ in range(runs):
        ok = (x < N[0]) & (y < N[1]) & (z < N[2])
        seen[x[ok], y[ok], z[ok]] = True
        # cursors of blocks that returned early are still advanced by thread 0 before
        # the range check (advance_block runs first)
        nz = z + G
        wrap_z = nz >= N[2]
        nz = np.where(wrap_z, nz % N[2], nz)
        ny = np.where(wrap_z, y + G, y)
        wrap_y = wrap_z & (ny >= N[1])
        ny = np.where(wrap_y, ny % N[1], ny)
        nx = np.where(wrap_y, x + G, x)
        x, y, z = nx, ny, nz
    return seen


# ---------------------------------------------------------------- reference kernel on a GPU

def reference_gpu(H, pairs, N, zero, inc, t0, dT, volume_init=None):
    """Runs the reference's own kernel (cubin built from backproject_cuda.cu) through
    ref_harness.cu.  Returns (volume, blockDim used, launch-loop milliseconds)."""
    if not REF_LIB.exists() or not REF_CUBIN.exists():
        raise RuntimeError("reference kernel not built (oracle/_ref)")
    L = C.CDLL(str(REF_LIB))
    L.bpref_backproject.restype = C.c_int
    L.bpref_backproject.argtypes = [C.c_char_p, C.c_int, _F, C.c_uint64, C.c_uint32, _P, _F, _U32,
                                    _F, _F, C.c_float, C.c_float, C.POINTER(C.c_int), _D]
    cplx = np.iscomplexobj(H)
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.complex64 if cplx else np.float32))
    T = Hc.shape[-1]
    n = np.ascontiguousarray(np.asarray(N, dtype=np.uint32))
    shape = tuple(int(v) for v in n)
    vol = np.zeros(shape, np.complex64 if cplx else np.float32)
    if volume_init is not None:
        vol[...] = volume_init
    blk = C.c_int(0)
    ms = C.c_double(0)
    st = L.bpref_backproject(str(REF_CUBIN).encode(), 1 if cplx else 0,
                             _fp(Hc.view(np.float32) if cplx else Hc), len(pairs), T,
                             C.c_void_p(pairs.ctypes.data),
                             _fp(vol.view(np.float32) if cplx else vol), n.ctypes.data_as(_U32),
                             _fp(_f32(zero)), _fp(_f32(inc)), t0, dT, C.byref(blk), C.byref(ms))
    if st != 0:
        raise RuntimeError(f"reference harness failed with status {st}")
    return vol, blk.value, ms.value


# ---------------------------------------------------------------- parity metrics

def rel_l2(x, ref) -> float:
    x = np.asarray(x, np.complex128 if np.iscomplexobj(x) or np.iscomplexobj(ref) else np.float64)
    ref = np.asarray(ref, x.dtype)
    den = np.linalg.norm(ref.ravel())
    return float(np.linalg.norm((x - ref).ravel()) / (den if den > 0 else 1.0))


def linf_rel(x, ref) -> float:
    x = np.asarray(x, np.complex128 if np.iscomplexobj(x) or np.iscomplexobj(ref) else np.float64)
    ref = np.asarray(ref, x.dtype)
    den = np.abs(ref).max()
    return float(np.abs(x - ref).max() / (den if den > 0 else 1.0))


def misbinned_fraction(bins_a, bins_b) -> float:
    """Fraction of (voxel, pair) updates whose bin (or in/out-of-range state) differs."""
    a, b = np.asarray(bins_a), np.asarray(bins_b)
    return float(np.mean(a != b))


# ---------------------------------------------------------------- synthetic captures

class SynthBackend:
    """Host functions of a synthetic capture (volume basis, renderer, noise) without the
    product library, for the bench's reference arm: the basis in FP32 numpy in the
    product's operation order, the renderer and noise in oracle.c.  Identical captures
    to the product's own (tests/test_cpu.py)."""

    @staticmethod
    def volume_basis(volume_position, volume_size, voxels_per_side):
        pos = np.asarray(volume_position, np.float32)
        size = np.asarray(volume_size, np.float32)
        n = np.asarray(voxels_per_side, np.uint32)
        zero = (pos - size / np.float32(2.0)).astype(np.float32)
        inc = np.zeros(9, np.float32)
        for a in range(3):
            for k in range(3):
                ax = np.float32(1.0 if a == k else 0.0)
                inc[3 * a + k] = (ax * size[k]) / np.float32(int(n[k]) - 1)
        return zero, inc

    @staticmethod
    def render(pairs, T, t0, deltaT, points, albedo):
        pts = np.ascontiguousarray(points, np.float32)
        alb = np.ascontiguousarray(albedo, np.float32)
        out = np.zeros((len(pairs), T), np.float32)
        lib().orc_synth_render(C.c_void_p(pairs.ctypes.data), len(pairs), T, t0, deltaT,
                               _fp(pts), _fp(alb), len(alb), _fp(out))
        return out

    @staticmethod
    def poisson(H, peak, seed):
        lib().orc_synth_poisson(_fp(H), H.size, peak, seed)
        return H


def time_limits_corners(laser_position, laser_grid, camera_position, camera_grid,
                        volume_position, volume_size, t0, deltaT):
    """get_time_limits (backproject.hpp:617-674) with its corner bound: (min, max) bins."""
    lg, cg = _f32(laser_grid), _f32(camera_grid)
    out = np.zeros(2, np.float32)
    lib().orc_time_limits_corners(_fp(_f32(laser_position)), _fp(lg), lg.shape[0], lg.shape[1],
                                  _fp(_f32(camera_position)), _fp(cg), cg.shape[0], cg.shape[1],
                                  _fp(_f32(volume_position)), _fp(_f32(volume_size)), t0, deltaT,
                                  _fp(out))
    return float(out[0]), float(out[1])
