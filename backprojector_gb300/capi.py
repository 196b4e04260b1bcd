"""ctypes binding of the C ABI (include/backprojector_gb300.h, include/bpgb_synth.h).

The shared library is built in-tree by `backprojector_gb300.build` (or
`__graft_entry__.build()`); importing a function that needs it raises when it is
missing -- there is no Python or CPU fallback for any compute call.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libbpgb300.so"

# Status codes (bpgb_status)
OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_CUDA = -2
ERR_OUT_OF_MEMORY = -3
ERR_TIMEOUT = -4
ERR_UNSUPPORTED = -5
ERR_NO_DEVICE = -6
ERR_WINDOW = -7

ABI_VERSION = 2  # BPGB_ABI_VERSION of the structures mirrored below
DTYPE_F32, DTYPE_F16, DTYPE_BF16, DTYPE_C64, DTYPE_C32 = 0, 1, 2, 3, 4
ALGO_AUTO, ALGO_EXACT, ALGO_FAST = 0, 1, 2
ACCUM_F32, ACCUM_KAHAN = 0, 1
GEOMETRY_NAMES = {0: "generic", 1: "single_laser", 2: "exhaustive", 3: "confocal"}

# numpy view of bpgb_pair / CameraLaserPair (camera first, 32 bytes)
PAIR_DTYPE = np.dtype([("camera_point", "<f4", (3,)), ("laser_point", "<f4", (3,)),
                       ("camera_wall", "<f4"), ("laser_wall", "<f4")])
assert PAIR_DTYPE.itemsize == 32


class Options(C.Structure):
    _fields_ = [("algo", C.c_int32), ("h_dtype", C.c_int32), ("accum", C.c_int32),
                ("h_pitch", C.c_uint32), ("h_scale", C.c_float), ("tile", C.c_int32),
                ("pair_splits", C.c_int32), ("checked", C.c_int32), ("spin_limit", C.c_uint32),
                ("chunk", C.c_int32), ("stages", C.c_int32), ("unfactored", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class PlanInfo(C.Structure):
    _fields_ = [("algo", C.c_int32), ("geometry", C.c_int32), ("num_lasers", C.c_uint64),
                ("num_spads", C.c_uint64), ("tile", C.c_uint32 * 3), ("window", C.c_uint32),
                ("chunk", C.c_uint32), ("stages", C.c_uint32), ("pair_splits", C.c_uint32),
                ("grid", C.c_uint32), ("threads", C.c_uint32), ("smem_bytes", C.c_uint32),
                ("scratch_bytes", C.c_uint64), ("updates", C.c_uint64),
                ("factored", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}
        d["tile"] = list(self.tile)
        d["algo"] = {1: "exact", 2: "fast"}.get(self.algo, str(self.algo))
        d["geometry"] = GEOMETRY_NAMES.get(self.geometry, str(self.geometry))
        return d


class CaptureGeometry(C.Structure):
    _fields_ = [("pairs", C.c_void_p), ("num_pairs", C.c_uint64), ("T", C.c_uint32),
                ("voxels_per_side", C.c_uint32 * 3), ("volume_zero_pos", C.c_float * 3),
                ("voxel_inc", C.c_float * 9), ("t0", C.c_float), ("deltaT", C.c_float),
                ("h_scale", C.c_float)]


class BatchInfo(C.Structure):
    _fields_ = [("captures", C.c_uint32), ("pitch", C.c_uint32), ("total_rows", C.c_uint64),
                ("total_voxels", C.c_uint64), ("work_units", C.c_uint32), ("grid", C.c_uint32),
                ("stages", C.c_uint32), ("chunk", C.c_uint32), ("smem_bytes", C.c_uint32),
                ("updates", C.c_uint64), ("planar", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneReport(C.Structure):
    _fields_ = [("candidates", C.c_uint32), ("cache_hit", C.c_uint32), ("default_ms", C.c_float),
                ("best_ms", C.c_float), ("tile", C.c_int32), ("chunk", C.c_int32),
                ("stages", C.c_int32), ("pair_splits", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class OctreeInfo(C.Structure):
    _fields_ = [("fine", C.c_uint32 * 3), ("coarse", C.c_uint32 * 3), ("tile", C.c_uint32 * 3),
                ("tiles", C.c_uint32), ("in_channels", C.c_uint32), ("pair_splits", C.c_uint32),
                ("h_dtype", C.c_int32), ("p_lo", C.c_float), ("scratch_bytes", C.c_uint64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        for k in ("fine", "coarse", "tile"):
            d[k] = list(d[k])
        return d


class BackprojectorError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U32 = C.POINTER(C.c_uint32)

# name -> (restype, argtypes); every exported symbol of include/*.h
SIGNATURES: dict[str, tuple] = {
    "bpgb_abi_version": (C.c_int, []),
    "bpgb_status_string": (C.c_char_p, [C.c_int]),
    "bpgb_last_error": (C.c_char_p, []),
    "bpgb_options_default": (None, [C.POINTER(Options)]),
    "bpgb_launch_count": (C.c_uint64, []),
    "bpgb_backproject_f32": (C.c_int, [_P, C.c_uint64, C.c_uint32, _P, C.c_uint64, _P, _U32, _F,
                                       _F, C.c_float, C.c_float]),
    "bpgb_backproject_c64": (C.c_int, [_P, C.c_uint64, C.c_uint32, _P, C.c_uint64, _P, _U32, _F,
                                       _F, C.c_float, C.c_float]),
    "bpgb_backproject_host": (C.c_int, [_P, C.c_uint64, C.c_uint32, _P, C.c_uint64, _P, _U32, _F,
                                        _F, C.c_float, C.c_float, C.POINTER(Options)]),
    "bpgb_plan_create": (C.c_int, [C.POINTER(_P), _P, C.c_uint64, C.c_uint32, _U32, _F, _F,
                                   C.c_float, C.c_float, C.POINTER(Options)]),
    "bpgb_plan_execute": (C.c_int, [_P, _P, _P, _P]),
    "bpgb_plan_check": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "bpgb_plan_get_info": (C.c_int, [_P, C.POINTER(PlanInfo)]),
    "bpgb_plan_dump_bins": (C.c_int, [_P, C.POINTER(C.c_int64), C.c_int64, _P, _P]),
    "bpgb_eval_f64_voxels": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_uint32, _P, C.c_uint64, _P,
                                       _P, _P, C.c_float, C.c_float, _P, C.c_int64, _P, _P]),
    "bpgb_block_detail": (C.c_int, [_P, _U32, _P, _U32, _U32, C.c_uint32, C.c_uint32, _P,
                                    C.c_float, _P, _P]),
    "bpgb_plan_select_tiles_topk": (C.c_int, [_P, _P, _U32, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "bpgb_diag_mufu_rates": (C.c_int, [C.POINTER(C.c_double), C.c_int]),
    "bpgb_diag_umma_probe": (C.c_int, [_P, C.c_uint32, _U32, _F, _U32]),
    "bpgb_diag_umma_issue_rates": (C.c_int, [C.POINTER(C.c_double), C.c_int]),
    "bpgb_set_dropin_algo": (C.c_int, [C.c_int]),
    "bpgb_get_dropin_algo": (C.c_int, []),
    "bpgb_plan_get_tables": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "bpgb_plan_destroy": (C.c_int, [_P]),
    "bpgb_diag_wait_timeout": (C.c_int, [C.c_uint32]),
    "bpgb_diag_pipe_rates": (C.c_int, [C.POINTER(C.c_double)]),
    "bpgb_backproject_noalloc": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, C.c_uint64, C.c_uint64,
                                           C.c_int, _U32, _F, _F, C.c_float, C.c_float, _P, _P]),
    "bpgb_phasor_pulse": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, C.c_float,
                                    C.c_uint32, _P, C.c_uint32, _P]),
    "bpgb_phasor_taps": (C.c_int, [C.c_float, C.c_float, C.c_uint32, _F, C.c_int]),
    "bpgb_precompute_pairs": (C.c_int, [_F, _F, C.c_uint32, C.c_uint32, _F, _F, C.c_uint32,
                                        C.c_uint32, C.c_int, _P]),
    "bpgb_volume_basis": (C.c_int, [_F, _F, _U32, _F, _F, _F]),
    "bpgb_time_limits": (C.c_int, [_F, _F, C.c_uint32, C.c_uint32, _F, _F, C.c_uint32,
                                   C.c_uint32, _F, _F, C.c_float, C.c_float, _F, _F]),
    "bpgb_time_limits_corners": (C.c_int, [_F, _F, C.c_uint32, C.c_uint32, _F, _F, C.c_uint32,
                                   C.c_uint32, _F, _F, C.c_float, C.c_float, _F, _F]),
    "bpgb_backproject_capture": (C.c_int, [_F, C.c_uint32, _F, C.c_uint32, C.c_uint32, _F,
                                           C.c_uint32, C.c_uint32, _F, _F, C.c_float, C.c_float,
                                           C.c_int, _F, _F, _U32, _F, C.c_int,
                                           C.POINTER(Options), _F]),
    "bpgb_phasor_capture": (C.c_int, [_F, C.c_uint32, _F, C.c_uint32, C.c_uint32, _F, C.c_uint32,
                                      C.c_uint32, _F, _F, C.c_float, C.c_float, C.c_int, _F, _F,
                                      _U32, _F, C.c_float, C.POINTER(Options), _F]),
    "bpgb_synth_render": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_float, C.c_float, _F, _F,
                                    C.c_uint64, _F]),
    "bpgb_synth_poisson": (C.c_int, [_F, C.c_uint64, C.c_float, C.c_uint64]),
    "bpgb_batch_create": (C.c_int, [C.POINTER(_P), C.POINTER(CaptureGeometry), C.c_uint32,
                                    C.POINTER(Options)]),
    "bpgb_batch_layout": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "bpgb_batch_get_info": (C.c_int, [_P, C.POINTER(BatchInfo)]),
    "bpgb_batch_execute": (C.c_int, [_P, _P, _P, _P]),
    "bpgb_batch_graph_launch": (C.c_int, [_P, _P, _P, _P]),
    "bpgb_batch_check": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "bpgb_batch_destroy": (C.c_int, [_P]),
    "bpgb_plan_autotune": (C.c_int, [_P, C.c_uint64, C.c_uint32, _U32, _F, _F, C.c_float, C.c_float,
                                     _P, _P, C.POINTER(Options), C.POINTER(TuneReport), _P]),
    "bpgb_batch_autotune": (C.c_int, [C.POINTER(CaptureGeometry), C.c_uint32, _P, _P,
                                      C.POINTER(Options), C.POINTER(TuneReport), _P]),
    "bpgb_tune_cache_save": (C.c_int, [C.c_char_p]),
    "bpgb_tune_cache_load": (C.c_int, [C.c_char_p]),
    "bpgb_tune_cache_clear": (C.c_int, []),
    "bpgb_tune_cache_size": (C.c_int, []),
    "bpgb_plan_execute_tiles": (C.c_int, [_P, _P, _P, _P, _P, C.c_uint32, _P]),
    "bpgb_plan_select_tiles": (C.c_int, [_P, _P, _U32, C.c_uint32, C.c_float, _P, _P, _P]),
    "bpgb_synth_render_device": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_float, C.c_float, _P,
                                           _P, C.c_uint64, _P, C.c_uint32, _P]),
    "bpgb_block_max": (C.c_int, [_P, _U32, C.c_uint32, _P, _P]),
    "bpgb_upsample_trilinear": (C.c_int, [_P, _U32, _P, _U32, _P]),
    "bpgb_laplacian7": (C.c_int, [_P, _U32, _P, _P]),
    "bpgb_complex_abs": (C.c_int, [_P, C.c_uint64, _P, _P]),
    "bpgb_capture_window": (C.c_int, [_F, C.c_uint32, C.c_uint32, _F, C.c_uint32, C.c_uint32, _F,
                                      _F, C.c_float, C.c_float, C.c_int, _F, _F, C.c_int,
                                      C.POINTER(C.c_int64), C.POINTER(C.c_uint32), _F]),
    "bpgb_rows_crop": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int64, C.c_uint32,
                                 _P, C.c_uint32, _P]),
    "bpgb_octree_create": (C.c_int, [C.POINTER(_P), _P, C.c_uint64, C.c_uint32, _U32, _F, _F,
                                     C.c_float, C.c_float, C.c_char_p, C.c_float,
                                     C.POINTER(Options)]),
    "bpgb_octree_reconstruct": (C.c_int, [_P, _P, _P, _P]),
    "bpgb_octree_reconstruct_host": (C.c_int, [_P, _P, _P]),
    "bpgb_octree_selected": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "bpgb_octree_get_info": (C.c_int, [_P, C.POINTER(OctreeInfo)]),
    "bpgb_octree_destroy": (C.c_int, [_P]),
    "bpgb_rows_absmax": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, _P, _P]),
    "bpgb_rows_to_half": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, _P,
                                    C.c_float, C.c_int, _P, C.c_uint32, _P]),
    "bpgb_volume_scale": (C.c_int, [_P, C.c_uint64, C.c_float, _P, C.c_float, _P]),
    "bpgb_cnn_kp": (C.c_uint32, [C.c_uint32]),
    "bpgb_cnn_conv3d": (C.c_int, [_P, C.c_uint32, C.c_uint32, _U32, C.c_uint32, _P, C.c_uint32,
                                  C.c_int, _P, C.c_uint32, _P, _P, _P]),
    "bpgb_cnn_wgrad_scratch_bytes": (C.c_uint64, [C.c_uint32, C.c_uint32, _U32, C.c_uint32]),
    "bpgb_cnn_conv3d_wgrad": (C.c_int, [_P, C.c_uint32, C.c_uint32, _U32, C.c_uint32, _P,
                                        C.c_uint32, C.c_uint32, _P, C.c_uint64, _P, _P]),
    "bpgb_cnn_pack_weights": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P, C.c_uint32,
                                        _P, _P]),
    "bpgb_cnn_bce_grad": (C.c_int, [_P, _P, C.c_uint64, C.c_float, C.c_float, _P, _P, _P]),
    "bpgb_cnn_adam": (C.c_int, [_P, _P, _P, _P, C.c_uint64, C.c_float, C.c_float, C.c_float,
                                C.c_float, C.c_uint32, _P]),
    "bpgb_cnn_normalize": (C.c_int, [_P, _U32, C.c_uint32, _P, _P]),
    "bpgb_cnn_features": (C.c_int, [_P, _U32, C.c_uint32, _P, _P, _P]),
    "bpgb_cnn_lp_bytes": (C.c_uint64, [C.c_uint32, C.c_uint32, _U32, C.c_uint32]),
    "bpgb_cnn_tc_weight_bytes": (C.c_uint64, [C.c_uint32]),
    "bpgb_cnn_lp_pack": (C.c_int, [_P, C.c_uint32, C.c_uint32, _U32, C.c_uint32, C.c_uint32, _P,
                                   _P]),
    "bpgb_cnn_lp_unpack": (C.c_int, [_P, C.c_uint32, C.c_uint32, _U32, C.c_uint32, _P, _P]),
    "bpgb_cnn_tc_pack_weights": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "bpgb_cnn_tc_pack_layers": (C.c_int, [C.POINTER(C.c_void_p), _U32, _U32,
                                          C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                          C.c_uint32, _P]),
    "bpgb_cnn_tc_conv3d": (C.c_int, [_P, C.c_uint32, C.c_uint32, _U32, C.c_uint32, _P, _P,
                                     C.c_uint32, C.c_int, _P, _P, C.c_uint32, _P, _P]),
    "bpgb_cnn_tc_wgrad_scratch_bytes": (C.c_uint64, [C.c_uint32, _U32, C.c_uint32]),
    "bpgb_cnn_tc_conv3d_wgrad": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32, _U32, C.c_uint32, _P,
                                           C.c_uint64, _P, _P]),
    "bpgb_cnn_tc_bce_grad": (C.c_int, [_P, _P, _U32, C.c_uint32, C.c_float, C.c_float, _P, _P,
                                       _P]),
    "bpgb_cnn_tc_status": (C.c_int, [_U32, C.c_int]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded libbpgb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA extension first "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(str(LIB_PATH))
        L.bpgb_abi_version.restype = C.c_int
        if L.bpgb_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{LIB_PATH} has ABI {L.bpgb_abi_version()}, these bindings "
                               f"{ABI_VERSION}: rebuild the extension")
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str) -> None:
    if status != OK:
        L = lib()
        msg = L.bpgb_last_error().decode(errors="replace")
        name = L.bpgb_status_string(status).decode()
        raise BackprojectorError(status, f"{what}: {name} ({status}): {msg}")


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)


def u32ptr(a: np.ndarray):
    return a.ctypes.data_as(_U32)


def vptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def f32(a, shape=None) -> np.ndarray:
    out = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None and out.shape != tuple(shape):
        out = out.reshape(shape)
    return out


def options(**kw) -> Options:
    o = Options()
    lib().bpgb_options_default(C.byref(o))
    for k, v in kw.items():
        if v is None:
            continue
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


def pipe_rates() -> dict:
    """Measured per-SM per-clock rates: rsqrt results, FP32 lanes (packed FMA), shared loads."""
    r = (C.c_double * 3)()
    check(lib().bpgb_diag_pipe_rates(r), "bpgb_diag_pipe_rates")
    return {"rsqrt_per_sm_clk": r[0], "fp32_lanes_per_sm_clk": r[1], "lds_per_sm_clk": r[2]}


def mufu_rates() -> dict:
    """MUFU results per SM per clock, per operation (bpgb_diag_mufu_rates)."""
    r = (C.c_double * 6)()
    check(lib().bpgb_diag_mufu_rates(r, 6), "bpgb_diag_mufu_rates")
    return dict(zip(("rsqrt_8_chains", "rsqrt_16_chains", "ex2", "sqrt", "rcp", "sin"), list(r)))


def umma_issue_rates() -> dict:
    """Cycles per tcgen05.mma by shape, one issuing thread per SM (bpgb_diag_umma_issue_rates)."""
    r = (C.c_double * 6)()
    check(lib().bpgb_diag_umma_issue_rates(r, 6), "bpgb_diag_umma_issue_rates")
    keys = ("m128_n48_mn", "m64_n48_mn", "m128_n48_k", "m128_n96_k", "m128_n128_k", "m128_n256_k")
    return dict(zip(keys, list(r)))


def umma_probe(image: np.ndarray, params, ncols: int):
    """Run bpgb_diag_umma_probe: image (<= 48 KB of bytes), params = (a_off, a_lbo, a_sbo,
    a_kstep, b_off, b_lbo, b_sbo, b_kstep, idesc, nk); returns (accumulator [128, ncols]
    FP32, status)."""
    img = np.ascontiguousarray(image).view(np.uint8).reshape(-1)
    prm = np.asarray(list(params) + [ncols], dtype=np.uint32)
    out = np.empty((128, ncols), np.float32)
    st = np.zeros(1, np.uint32)
    check(lib().bpgb_diag_umma_probe(img.ctypes.data, img.nbytes, u32ptr(prm), fptr(out),
                                     u32ptr(st)), "bpgb_diag_umma_probe")
    return out, int(st[0])


def launch_count() -> int:
    return int(lib().bpgb_launch_count())


# ---------------------------------------------------------------- host helpers (no GPU)

def volume_basis(volume_position, volume_size, voxels_per_side, wall_normal=(0, 0, 0)):
    """(volume_zero_pos[3], voxel_inc[9]) as the reference computes them."""
    pos, size, wn = f32(volume_position), f32(volume_size), f32(wall_normal)
    n = np.ascontiguousarray(np.asarray(voxels_per_side, dtype=np.uint32))
    zero = np.zeros(3, np.float32)
    inc = np.zeros(9, np.float32)
    check(lib().bpgb_volume_basis(fptr(pos), fptr(size), u32ptr(n), fptr(wn), fptr(zero), fptr(inc)),
          "bpgb_volume_basis")
    return zero, inc


def time_limits(laser_position, laser_grid, camera_position, camera_grid, volume_position,
                volume_size, t0, deltaT, corners: bool = False):
    """(min, max) fractional bin limits: over every grid point (default) or the
    reference's corner bound (corners=True, bpgb_time_limits_corners)."""
    lg, cg = f32(laser_grid), f32(camera_grid)
    mn, mx = C.c_float(), C.c_float()
    name = "bpgb_time_limits_corners" if corners else "bpgb_time_limits"
    check(getattr(lib(), name)(fptr(f32(laser_position)), fptr(lg), lg.shape[0], lg.shape[1],
                               fptr(f32(camera_position)), fptr(cg), cg.shape[0], cg.shape[1],
                               fptr(f32(volume_position)), fptr(f32(volume_size)), t0, deltaT,
                               C.byref(mn), C.byref(mx)), name)
    return mn.value, mx.value


def phasor_taps(wavelength: float, deltaT: float, times: int = 4) -> np.ndarray:
    """(2, K) array: cos taps then sin taps."""
    K = lib().bpgb_phasor_taps(wavelength, deltaT, times, None, 0)
    if K <= 0:
        return np.zeros((2, 0), np.float32)
    taps = np.zeros(2 * K, np.float32)
    lib().bpgb_phasor_taps(wavelength, deltaT, times, fptr(taps), K)
    return taps.reshape(2, K)


def synth_render(pairs: np.ndarray, T: int, t0: float, deltaT: float, points, albedo) -> np.ndarray:
    pts, alb = f32(points), f32(albedo)
    out = np.empty((len(pairs), T), np.float32)
    check(lib().bpgb_synth_render(vptr(pairs), len(pairs), T, t0, deltaT, fptr(pts), fptr(alb),
                                  len(alb), fptr(out)), "bpgb_synth_render")
    return out


def synth_poisson(H: np.ndarray, peak: float, seed: int) -> np.ndarray:
    assert H.dtype == np.float32 and H.flags.c_contiguous
    check(lib().bpgb_synth_poisson(fptr(H), H.size, peak, seed), "bpgb_synth_poisson")
    return H


# ---------------------------------------------------------------- GPU calls (host buffers)

def backproject_host(H: np.ndarray, pairs: np.ndarray, voxels_per_side, zero, inc, t0: float,
                     deltaT: float, **opt) -> np.ndarray:
    """bpgb_backproject_host: H [P, T] float32 (or complex64) on the host."""
    P = len(pairs)
    cplx = np.iscomplexobj(H)
    Hc = np.ascontiguousarray(H, dtype=np.complex64 if cplx else None)
    T = Hc.shape[-1]
    n = np.ascontiguousarray(np.asarray(voxels_per_side, dtype=np.uint32))
    out = np.zeros(tuple(int(x) for x in n), np.complex64 if cplx else np.float32)
    if "h_dtype" not in opt:
        opt["h_dtype"] = DTYPE_C64 if cplx else DTYPE_F32
    o = options(**opt)
    check(lib().bpgb_backproject_host(vptr(Hc), P * T, T, vptr(pairs), P, vptr(out), u32ptr(n),
                                      fptr(f32(zero)), fptr(f32(inc)), t0, deltaT, C.byref(o)),
          "bpgb_backproject_host")
    return out


def precompute_pairs(laser_position, laser_grid, camera_position, camera_grid, confocal=False):
    cg = f32(camera_grid)
    cx, cy = cg.shape[0], cg.shape[1]
    if confocal:
        lg = cg
        lx = ly = 0
        P = cx * cy
    else:
        lg = f32(laser_grid)
        lx, ly = lg.shape[0], lg.shape[1]
        P = lx * ly * cx * cy
    out = np.zeros(P, PAIR_DTYPE)
    check(lib().bpgb_precompute_pairs(fptr(f32(laser_position)), fptr(lg), lx, ly,
                                      fptr(f32(camera_position)), fptr(cg), cx, cy,
                                      1 if confocal else 0, vptr(out)), "bpgb_precompute_pairs")
    return out


# ---------------------------------------------------------------- plans (device buffers)

def _ptr(x) -> C.c_void_p:
    """Device pointer of a torch tensor or an int address."""
    if x is None:
        return C.c_void_p(0)
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(int(x))


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Plan:
    """bpgb_plan: geometry analysed once, execute() on device buffers (async)."""

    def __init__(self, pairs: np.ndarray, T: int, voxels_per_side, zero, inc, t0: float,
                 deltaT: float, **opt):
        self._pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
        self.n = tuple(int(v) for v in voxels_per_side)
        n = np.asarray(self.n, dtype=np.uint32)
        self.T = int(T)
        self.opt = options(**opt)
        h = C.c_void_p()
        check(lib().bpgb_plan_create(C.byref(h), vptr(self._pairs), len(self._pairs), self.T,
                                     u32ptr(n), fptr(f32(zero)), fptr(f32(inc)), t0, deltaT,
                                     C.byref(self.opt)), "bpgb_plan_create")
        self.handle = h

    @property
    def num_pairs(self) -> int:
        return len(self._pairs)

    def info(self) -> dict:
        i = PlanInfo()
        check(lib().bpgb_plan_get_info(self.handle, C.byref(i)), "bpgb_plan_get_info")
        return i.as_dict()

    def execute(self, d_H, d_volume, stream=None) -> None:
        check(lib().bpgb_plan_execute(self.handle, _ptr(d_H), _ptr(d_volume), _stream_ptr(stream)),
              "bpgb_plan_execute")

    def check(self) -> int:
        v = C.c_uint64()
        check(lib().bpgb_plan_check(self.handle, C.byref(v)), "bpgb_plan_check")
        return int(v.value)

    def check_status(self) -> tuple[int, int]:
        """(status, violations) without raising."""
        v = C.c_uint64()
        st = lib().bpgb_plan_check(self.handle, C.byref(v))
        return st, int(v.value)

    def execute_tiles(self, d_H, d_volume, d_tile_list, d_tile_count, max_tiles: int,
                      stream=None) -> None:
        check(lib().bpgb_plan_execute_tiles(self.handle, _ptr(d_H), _ptr(d_volume),
                                            _ptr(d_tile_list), _ptr(d_tile_count), int(max_tiles),
                                            _stream_ptr(stream)), "bpgb_plan_execute_tiles")

    def select_tiles(self, d_score, block_dims, block_size: int, threshold: float, d_tile_list,
                     d_tile_count, stream=None) -> None:
        bd = np.asarray([int(v) for v in block_dims], np.uint32)
        check(lib().bpgb_plan_select_tiles(self.handle, _ptr(d_score), u32ptr(bd), int(block_size),
                                           float(threshold), _ptr(d_tile_list),
                                           _ptr(d_tile_count), _stream_ptr(stream)),
              "bpgb_plan_select_tiles")

    def select_tiles_topk(self, d_score, block_dims, block_size: int, k: int, d_tile_list,
                          d_tile_count, stream=None) -> None:
        check(lib().bpgb_plan_select_tiles_topk(self.handle, _ptr(d_score),
                                                u32ptr(_dims(block_dims)), block_size, int(k),
                                                _ptr(d_tile_list), _ptr(d_tile_count),
                                                _stream_ptr(stream)),
              "bpgb_plan_select_tiles_topk")

    def dump_bins(self, voxel_ids, d_bins, stream=None) -> None:
        ids = np.ascontiguousarray(np.asarray(voxel_ids, dtype=np.int64))
        check(lib().bpgb_plan_dump_bins(self.handle, ids.ctypes.data_as(C.POINTER(C.c_int64)),
                                        len(ids), _ptr(d_bins), _stream_ptr(stream)),
              "bpgb_plan_dump_bins")

    def tables(self) -> np.ndarray:
        """The FAST plan's tables as float32 [S + L, 4] (SPAD entries, then lasers)."""
        n = C.c_uint64(0)
        check(lib().bpgb_plan_get_tables(self.handle, None, 0, C.byref(n)), "bpgb_plan_get_tables")
        out = np.zeros((int(n.value), 4), np.float32)
        check(lib().bpgb_plan_get_tables(self.handle, out.ctypes.data_as(C.c_void_p), n.value,
                                         C.byref(n)), "bpgb_plan_get_tables")
        return out

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().bpgb_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def eval_f64_voxels(d_H, T: int, d_pairs, num_pairs: int, voxels_per_side, zero, inc,
                    t0: float, deltaT: float, d_voxel_ids, d_out, h_pitch: int = 0,
                    is_complex: bool = False, stream=None) -> None:
    """FP64 values of the listed voxels (device int64 ids -> device float64 out)."""
    check(lib().bpgb_eval_f64_voxels(_ptr(d_H), 1 if is_complex else 0, T, h_pitch, _ptr(d_pairs),
                                     num_pairs, u32ptr(_dims(voxels_per_side)), fptr(f32(zero)),
                                     fptr(f32(inc)), t0, deltaT, _ptr(d_voxel_ids),
                                     int(d_voxel_ids.numel()), _ptr(d_out), _stream_ptr(stream)),
          "bpgb_eval_f64_voxels")


def phasor_pulse_device(d_H, rows: int, T: int, in_pitch: int, wavelength: float, deltaT: float,
                        d_out, out_pitch: int, times: int = 4, stream=None) -> None:
    check(lib().bpgb_phasor_pulse(_ptr(d_H), rows, T, in_pitch, wavelength, deltaT, times,
                                  _ptr(d_out), out_pitch, _stream_ptr(stream)), "bpgb_phasor_pulse")


class Batch:
    """bpgb_batch: many captures (list of dicts or Capture-like objects with pairs, T,
    voxels_per_side, zero, inc, t0, deltaT and optional h_scale) in persistent launches
    (one per kind of capture) captured together in one CUDA graph.

    Device buffers: H packed [total_rows, pitch] (capture c at rows row_offsets[c], bins
    >= its T zero) and volumes packed [total_voxels] (capture c at voxel_offsets[c])."""

    def __init__(self, captures, **opt):
        geo, self._pairs = _capture_geometry_array(captures)
        self.opt = options(**opt)
        h = C.c_void_p()
        check(lib().bpgb_batch_create(C.byref(h), geo, len(captures), C.byref(self.opt)),
              "bpgb_batch_create")
        self.handle = h
        self.n = len(captures)
        rows = (C.c_uint64 * self.n)()
        vox = (C.c_uint64 * self.n)()
        check(lib().bpgb_batch_layout(h, rows, vox), "bpgb_batch_layout")
        self.row_offsets = [int(v) for v in rows]
        self.voxel_offsets = [int(v) for v in vox]

    def info(self) -> dict:
        i = BatchInfo()
        check(lib().bpgb_batch_get_info(self.handle, C.byref(i)), "bpgb_batch_get_info")
        return i.as_dict()

    def execute(self, d_H, d_volumes, stream=None) -> None:
        check(lib().bpgb_batch_execute(self.handle, _ptr(d_H), _ptr(d_volumes), _stream_ptr(stream)),
              "bpgb_batch_execute")

    def graph_launch(self, d_H, d_volumes, stream=None) -> None:
        check(lib().bpgb_batch_graph_launch(self.handle, _ptr(d_H), _ptr(d_volumes),
                                            _stream_ptr(stream)), "bpgb_batch_graph_launch")

    def check(self) -> int:
        v = C.c_uint64()
        check(lib().bpgb_batch_check(self.handle, C.byref(v)), "bpgb_batch_check")
        return int(v.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().bpgb_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---------------------------------------------------------------- autotuner

TUNED_KEYS = ("tile", "chunk", "stages", "pair_splits")


def _capture_geometry_array(captures):
    keep = [np.ascontiguousarray(c["pairs"], dtype=PAIR_DTYPE) for c in captures]
    geo = (CaptureGeometry * len(captures))()
    for i, c in enumerate(captures):
        g = geo[i]
        g.pairs = keep[i].ctypes.data
        g.num_pairs = len(keep[i])
        g.T = int(c["T"])
        for k in range(3):
            g.voxels_per_side[k] = int(c["voxels_per_side"][k])
            g.volume_zero_pos[k] = float(c["zero"][k])
        for k in range(9):
            g.voxel_inc[k] = float(c["inc"][k])
        g.t0 = float(c["t0"])
        g.deltaT = float(c["deltaT"])
        g.h_scale = float(c.get("h_scale", 1.0))
    return geo, keep


def autotune_plan(pairs, T, voxels_per_side, zero, inc, t0, deltaT, d_H, d_volume, stream=None,
                  **opt) -> tuple[dict, dict]:
    """bpgb_plan_autotune: returns (tuned option overrides, report).  d_H holds the
    capture's rows (read), d_volume is overwritten."""
    pr = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
    n = np.asarray([int(v) for v in voxels_per_side], np.uint32)
    o = options(**opt)
    rep = TuneReport()
    check(lib().bpgb_plan_autotune(vptr(pr), len(pr), int(T), u32ptr(n), fptr(f32(zero)),
                                   fptr(f32(inc)), t0, deltaT, _ptr(d_H), _ptr(d_volume),
                                   C.byref(o), C.byref(rep), _stream_ptr(stream)),
          "bpgb_plan_autotune")
    tuned = {k: getattr(o, k) for k in TUNED_KEYS}
    tuned["algo"] = o.algo
    return tuned, rep.as_dict()


def autotune_batch(captures, d_H, d_volumes, stream=None, **opt) -> tuple[dict, dict]:
    """bpgb_batch_autotune over capture geometry dicts (as for Batch)."""
    geo, keep = _capture_geometry_array(captures)
    o = options(**opt)
    rep = TuneReport()
    check(lib().bpgb_batch_autotune(geo, len(captures), _ptr(d_H), _ptr(d_volumes), C.byref(o),
                                    C.byref(rep), _stream_ptr(stream)), "bpgb_batch_autotune")
    del keep
    return {k: getattr(o, k) for k in TUNED_KEYS[:3]}, rep.as_dict()


def tune_cache_save(path) -> None:
    check(lib().bpgb_tune_cache_save(str(path).encode()), "bpgb_tune_cache_save")


def tune_cache_load(path) -> None:
    check(lib().bpgb_tune_cache_load(str(path).encode()), "bpgb_tune_cache_load")


def tune_cache_clear() -> None:
    lib().bpgb_tune_cache_clear()


def tune_cache_size() -> int:
    return int(lib().bpgb_tune_cache_size())


# ---------------------------------------------------------------- octree / CNN kernels

def _dims(d) -> np.ndarray:
    return np.asarray([int(v) for v in d], np.uint32)


def synth_render_device(d_pairs, num_pairs: int, T: int, t0: float, deltaT: float, d_points,
                        d_albedo, num_points: int, d_out, pitch: int | None = None,
                        stream=None) -> None:
    check(lib().bpgb_synth_render_device(_ptr(d_pairs), int(num_pairs), int(T), float(t0),
                                         float(deltaT), _ptr(d_points), _ptr(d_albedo),
                                         int(num_points), _ptr(d_out), int(pitch or T),
                                         _stream_ptr(stream)), "bpgb_synth_render_device")


def block_max(d_volume, voxels_per_side, block_size: int, d_out, stream=None) -> None:
    check(lib().bpgb_block_max(_ptr(d_volume), u32ptr(_dims(voxels_per_side)), int(block_size),
                               _ptr(d_out), _stream_ptr(stream)), "bpgb_block_max")


def upsample_trilinear(d_coarse, coarse_dims, d_fine, fine_dims, stream=None) -> None:
    check(lib().bpgb_upsample_trilinear(_ptr(d_coarse), u32ptr(_dims(coarse_dims)), _ptr(d_fine),
                                        u32ptr(_dims(fine_dims)), _stream_ptr(stream)),
          "bpgb_upsample_trilinear")


def block_detail(d_coarse_lo, lo_dims, d_coarse_hi, hi_dims, fine_dims, block_size: int,
                 d_score, samples: int = 4, d_logits=None, logit_lo: float = 0.0,
                 stream=None) -> None:
    check(lib().bpgb_block_detail(_ptr(d_coarse_lo), u32ptr(_dims(lo_dims)), _ptr(d_coarse_hi),
                                  u32ptr(_dims(hi_dims)), u32ptr(_dims(fine_dims)), block_size,
                                  samples, _ptr(d_logits) if d_logits is not None else None,
                                  logit_lo, _ptr(d_score), _stream_ptr(stream)),
          "bpgb_block_detail")


def cnn_kp(cin: int) -> int:
    return int(lib().bpgb_cnn_kp(int(cin)))


def cnn_conv3d(d_X, cin: int, x_stride: int, dims, batch: int, d_Wt, np_: int, relu: bool,
               d_Y=None, d_Yf=None, d_mask=None, mask_stride: int = 0, stream=None) -> None:
    check(lib().bpgb_cnn_conv3d(_ptr(d_X), int(cin), int(x_stride), u32ptr(_dims(dims)), int(batch),
                                _ptr(d_Wt), int(np_), 1 if relu else 0, _ptr(d_mask),
                                int(mask_stride), _ptr(d_Y), _ptr(d_Yf), _stream_ptr(stream)),
          "bpgb_cnn_conv3d")


def cnn_wgrad_scratch_bytes(cin: int, np_: int, dims, batch: int) -> int:
    return int(lib().bpgb_cnn_wgrad_scratch_bytes(int(cin), int(np_), u32ptr(_dims(dims)),
                                                  int(batch)))


def cnn_conv3d_wgrad(d_X, cin: int, x_stride: int, dims, batch: int, d_dY, np_: int, cout: int,
                     d_scratch, scratch_bytes: int, d_dW, stream=None) -> None:
    check(lib().bpgb_cnn_conv3d_wgrad(_ptr(d_X), int(cin), int(x_stride), u32ptr(_dims(dims)),
                                      int(batch), _ptr(d_dY), int(np_), int(cout), _ptr(d_scratch),
                                      int(scratch_bytes), _ptr(d_dW), _stream_ptr(stream)),
          "bpgb_cnn_conv3d_wgrad")


def cnn_pack_weights(d_W, cin: int, cout: int, np_: int, d_Wt, np_back: int = 0, d_Wb=None,
                     stream=None) -> None:
    check(lib().bpgb_cnn_pack_weights(_ptr(d_W), int(cin), int(cout), int(np_), _ptr(d_Wt),
                                      int(np_back), _ptr(d_Wb), _stream_ptr(stream)),
          "bpgb_cnn_pack_weights")


def cnn_bce_grad(d_logits, d_labels, n: int, pos_weight: float, scale: float, d_dZ, d_loss=None,
                 stream=None) -> None:
    check(lib().bpgb_cnn_bce_grad(_ptr(d_logits), _ptr(d_labels), int(n), float(pos_weight),
                                  float(scale), _ptr(d_dZ), _ptr(d_loss), _stream_ptr(stream)),
          "bpgb_cnn_bce_grad")


def cnn_adam(d_p, d_g, d_m, d_v, n: int, lr: float, beta1: float, beta2: float, eps: float,
             step: int, stream=None) -> None:
    check(lib().bpgb_cnn_adam(_ptr(d_p), _ptr(d_g), _ptr(d_m), _ptr(d_v), int(n), float(lr),
                              float(beta1), float(beta2), float(eps), int(step),
                              _stream_ptr(stream)), "bpgb_cnn_adam")


def cnn_normalize(d_coarse, dims, batch: int, d_X, stream=None) -> None:
    check(lib().bpgb_cnn_normalize(_ptr(d_coarse), u32ptr(_dims(dims)), int(batch), _ptr(d_X),
                                   _stream_ptr(stream)), "bpgb_cnn_normalize")


def laplacian7(d_volume, voxels_per_side, d_out, stream=None) -> None:
    check(lib().bpgb_laplacian7(_ptr(d_volume), u32ptr(_dims(voxels_per_side)), _ptr(d_out),
                                _stream_ptr(stream)), "bpgb_laplacian7")


def cnn_features(d_coarse, dims, batch: int, d_X, d_scratch=None, stream=None) -> None:
    check(lib().bpgb_cnn_features(_ptr(d_coarse), u32ptr(_dims(dims)), int(batch), _ptr(d_X),
                                  _ptr(d_scratch), _stream_ptr(stream)), "bpgb_cnn_features")


# ---- occupancy CNN on the tcgen05 tensor cores (line-planes tensors)

def cnn_lp_bytes(channels: int, zpad: int, dims, batch: int) -> int:
    return int(lib().bpgb_cnn_lp_bytes(int(channels), int(zpad), u32ptr(_dims(dims)), int(batch)))


def cnn_tc_weight_bytes(in_channels: int) -> int:
    return int(lib().bpgb_cnn_tc_weight_bytes(int(in_channels)))


def cnn_lp_pack(d_X, channels: int, x_stride: int, dims, batch: int, zpad: int, d_lp,
                stream=None) -> None:
    check(lib().bpgb_cnn_lp_pack(_ptr(d_X), int(channels), int(x_stride), u32ptr(_dims(dims)),
                                 int(batch), int(zpad), _ptr(d_lp), _stream_ptr(stream)),
          "bpgb_cnn_lp_pack")


def cnn_lp_unpack(d_lp, channels: int, zpad: int, dims, batch: int, d_X, stream=None) -> None:
    check(lib().bpgb_cnn_lp_unpack(_ptr(d_lp), int(channels), int(zpad), u32ptr(_dims(dims)),
                                   int(batch), _ptr(d_X), _stream_ptr(stream)), "bpgb_cnn_lp_unpack")


def cnn_tc_pack_weights(d_W, cin: int, cout: int, d_Wf, d_Wb=None, stream=None) -> None:
    check(lib().bpgb_cnn_tc_pack_weights(_ptr(d_W), int(cin), int(cout), _ptr(d_Wf), _ptr(d_Wb),
                                         _stream_ptr(stream)), "bpgb_cnn_tc_pack_weights")


def cnn_tc_pack_layers(d_Ws, cins, couts, d_Wfs, d_Wbs, stream=None) -> None:
    """bpgb_cnn_tc_pack_layers: lists of masters, channel counts, images (None allowed in d_Wbs)."""
    L = len(d_Ws)
    W = (C.c_void_p * L)(*[_ptr(w) for w in d_Ws])
    F = (C.c_void_p * L)(*[_ptr(w) for w in d_Wfs])
    B = (C.c_void_p * L)(*[_ptr(w) if w is not None else None for w in d_Wbs])
    ci = np.asarray(cins, np.uint32)
    co = np.asarray(couts, np.uint32)
    check(lib().bpgb_cnn_tc_pack_layers(W, u32ptr(ci), u32ptr(co), F, B, L, _stream_ptr(stream)),
          "bpgb_cnn_tc_pack_layers")


def cnn_tc_conv3d(d_X, in_channels: int, in_zpad: int, dims, batch: int, d_W, d_bias,
                  out_channels: int, relu: bool, d_mask=None, d_Y=None, out_zpad: int = 0,
                  d_Yf=None, stream=None) -> None:
    check(lib().bpgb_cnn_tc_conv3d(_ptr(d_X), int(in_channels), int(in_zpad), u32ptr(_dims(dims)),
                                   int(batch), _ptr(d_W), _ptr(d_bias), int(out_channels),
                                   1 if relu else 0, _ptr(d_mask), _ptr(d_Y), int(out_zpad),
                                   _ptr(d_Yf), _stream_ptr(stream)), "bpgb_cnn_tc_conv3d")


def cnn_tc_wgrad_scratch_bytes(in_channels: int, dims, batch: int) -> int:
    return int(lib().bpgb_cnn_tc_wgrad_scratch_bytes(int(in_channels), u32ptr(_dims(dims)),
                                                     int(batch)))


def cnn_tc_conv3d_wgrad(d_X, in_channels: int, d_dY, out_channels: int, dims, batch: int,
                        d_scratch, scratch_bytes: int, d_dW, stream=None) -> None:
    check(lib().bpgb_cnn_tc_conv3d_wgrad(_ptr(d_X), int(in_channels), _ptr(d_dY),
                                         int(out_channels), u32ptr(_dims(dims)), int(batch),
                                         _ptr(d_scratch), int(scratch_bytes), _ptr(d_dW),
                                         _stream_ptr(stream)), "bpgb_cnn_tc_conv3d_wgrad")


def cnn_tc_bce_grad(d_logits, d_labels, dims, batch: int, pos_weight: float, scale: float, d_dZ,
                    d_loss=None, stream=None) -> None:
    check(lib().bpgb_cnn_tc_bce_grad(_ptr(d_logits), _ptr(d_labels), u32ptr(_dims(dims)),
                                     int(batch), float(pos_weight), float(scale), _ptr(d_dZ),
                                     _ptr(d_loss), _stream_ptr(stream)), "bpgb_cnn_tc_bce_grad")


def cnn_tc_status(reset: bool = True) -> int:
    """Synchronises; the tensor-core CNN kernels' timeout bits (0 = none)."""
    st = np.zeros(1, np.uint32)
    check(lib().bpgb_cnn_tc_status(u32ptr(st), 1 if reset else 0), "bpgb_cnn_tc_status")
    return int(st[0])


def rows_absmax(d_H, rows: int, T: int, pitch: int, d_max, stream=None) -> None:
    check(lib().bpgb_rows_absmax(_ptr(d_H), int(rows), int(T), int(pitch), _ptr(d_max),
                                 _stream_ptr(stream)), "bpgb_rows_absmax")


def rows_to_half(d_H, rows: int, T: int, in_pitch: int, dtype: int, d_out, out_pitch: int,
                 scale: float = 1.0, d_absmax=None, target: float = 0.0, stream=None) -> None:
    check(lib().bpgb_rows_to_half(_ptr(d_H), int(rows), int(T), int(in_pitch), float(scale),
                                  _ptr(d_absmax), float(target), int(dtype), _ptr(d_out),
                                  int(out_pitch), _stream_ptr(stream)), "bpgb_rows_to_half")


def volume_scale(d_volume, n: int, scale: float = 1.0, d_absmax=None, target: float = 0.0,
                 stream=None) -> None:
    check(lib().bpgb_volume_scale(_ptr(d_volume), int(n), float(scale), _ptr(d_absmax),
                                  float(target), _stream_ptr(stream)), "bpgb_volume_scale")


class NativeOctree:
    """bpgb_octree: the learned-octree reconstruction as one native object (weights from
    an .npz written by backprojector_gb300.octree_train)."""

    def __init__(self, pairs, T: int, voxels_per_side, zero, inc, t0: float, deltaT: float,
                 weights, p_lo: float = 0.0, **opt):
        self._pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
        n = np.asarray([int(v) for v in voxels_per_side], np.uint32)
        self.n = tuple(int(v) for v in n)
        self.opt = options(**opt)
        h = C.c_void_p()
        check(lib().bpgb_octree_create(C.byref(h), vptr(self._pairs), len(self._pairs), int(T),
                                       u32ptr(n), fptr(f32(zero)), fptr(f32(inc)), float(t0),
                                       float(deltaT), str(weights).encode(), float(p_lo),
                                       C.byref(self.opt)), "bpgb_octree_create")
        self.handle = h

    def reconstruct(self, d_H, d_volume, stream=None) -> None:
        check(lib().bpgb_octree_reconstruct(self.handle, _ptr(d_H), _ptr(d_volume),
                                            _stream_ptr(stream)), "bpgb_octree_reconstruct")

    def reconstruct_host(self, H: np.ndarray) -> np.ndarray:
        Hc = np.ascontiguousarray(H, dtype=np.float32)
        out = np.empty(self.n, np.float32)
        check(lib().bpgb_octree_reconstruct_host(self.handle, Hc.ctypes.data, out.ctypes.data),
              "bpgb_octree_reconstruct_host")
        return out

    def selected(self) -> int:
        v = C.c_uint32()
        check(lib().bpgb_octree_selected(self.handle, C.byref(v)), "bpgb_octree_selected")
        return int(v.value)

    def info(self) -> dict:
        i = OctreeInfo()
        check(lib().bpgb_octree_get_info(self.handle, C.byref(i)), "bpgb_octree_get_info")
        return i.as_dict()

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().bpgb_octree_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def capture_window(camera_grid, laser_grid, camera_position, laser_position, t0: float,
                   deltaT: float, confocal: bool, volume_position, volume_size,
                   t0_mode: int = 0) -> tuple[int, int, float]:
    """(from, len, chunk_t0) of bpgb_capture_window."""
    cg = f32(camera_grid)
    lg = f32(laser_grid) if laser_grid is not None else np.zeros(3, np.float32)
    fr, ln, ct = C.c_int64(), C.c_uint32(), C.c_float()
    check(lib().bpgb_capture_window(fptr(cg), cg.shape[0], cg.shape[1], fptr(lg),
                                    lg.shape[0] if lg.ndim == 3 else 1,
                                    lg.shape[1] if lg.ndim == 3 else 1, fptr(f32(camera_position)),
                                    fptr(f32(laser_position if laser_position is not None else
                                             np.zeros(3))), float(t0), float(deltaT),
                                    1 if confocal else 0, fptr(f32(volume_position)),
                                    fptr(f32(volume_size)), int(t0_mode), C.byref(fr), C.byref(ln),
                                    C.byref(ct)), "bpgb_capture_window")
    return int(fr.value), int(ln.value), float(ct.value)


def rows_crop(d_in, rows: int, T: int, in_pitch: int, from_: int, length: int, d_out,
              out_pitch: int, stream=None) -> None:
    check(lib().bpgb_rows_crop(_ptr(d_in), int(rows), int(T), int(in_pitch), int(from_),
                               int(length), _ptr(d_out), int(out_pitch), _stream_ptr(stream)),
          "bpgb_rows_crop")


def complex_abs(d_in, n: int, d_out, stream=None) -> None:
    check(lib().bpgb_complex_abs(_ptr(d_in), int(n), _ptr(d_out), _stream_ptr(stream)),
          "bpgb_complex_abs")
