"""Builds the native parts in-tree (no cmake, no pip install).

Outputs (git-ignored):
  backprojector_gb300/_lib/libbpgb300.so      kernels (sm_103a) + C ABI + host code
  backprojector_gb300/nlosbpy<EXT_SUFFIX>      pybind11 module over the C ABI
  oracle/_build/liboracle.so                   CPU oracle (test infrastructure)
  oracle/_ref/backproject_cuda_ref.cubin       reference kernel built from its sources,
                                               only where the reference sources exist
  oracle/_ref/libbpref.so                      loader for that cubin (test infrastructure)

Translation units compile in parallel; an object is rebuilt only when its source or a
header is newer.
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OBJ = PKG / "_build"
LIBDIR = PKG / "_lib"
ORACLE = ROOT / "oracle"
REFERENCE_SRC = Path("/root/reference")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")

CU_SOURCES = ["bp_exact.cu", "bp_fast.cu", "phasor.cu", "geometry.cu", "diag.cu", "octree.cu", "cnn.cu", "cnn_tc.cu", "rows.cu", "eval64.cu"]
CPP_SOURCES = ["capi.cpp", "capture.cpp", "shim.cpp", "synth.cpp", "tune.cpp", "npy.cpp",
               "octree_host.cpp"]

LIB_PATH = LIBDIR / "libbpgb300.so"
ORACLE_LIB = ORACLE / "_build" / "liboracle.so"
REF_CUBIN = ORACLE / "_ref" / "backproject_cuda_ref.cubin"
REF_LIB = ORACLE / "_ref" / "libbpref.so"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h*"))


def _compile_cu(src: Path, obj: Path) -> None:
    _run([NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)])


def _compile_cpp(src: Path, obj: Path) -> None:
    _run(["g++", "-std=c++17", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}", "-c", str(src), "-o", str(obj)])


def _pybind_include() -> str | None:
    spec = importlib.util.find_spec("pybind11")
    if spec and spec.origin:
        inc = Path(spec.origin).parent / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    spec = importlib.util.find_spec("torch")
    if spec and spec.origin:
        inc = Path(spec.origin).parent / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    return None


def build_library(verbose: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for name in CU_SOURCES + CPP_SOURCES:
        src = CSRC / name
        obj = OBJ / (name + ".o")
        objs.append(obj)
        if _stale(obj, [src, *hdrs]):
            jobs.append((src, obj))
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        futs = [ex.submit(_compile_cu if s.suffix == ".cu" else _compile_cpp, s, o) for s, o in jobs]
        for f in futs:
            f.result()
    if _stale(LIB_PATH, objs):
        _run([NVCC, "-shared", *ARCH, "-cudart", "static", "-o", str(LIB_PATH), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


def build_python_module(verbose: bool = False) -> Path | None:
    inc = _pybind_include()
    if inc is None:
        return None
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = PKG / f"nlosbpy{suffix}"
    src = CSRC / "nlosbpy.cpp"
    if _stale(out, [src, LIB_PATH, *_headers()]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{inc}",
              f"-I{sysconfig.get_paths()['include']}", f"-I{INCLUDE}", str(src), "-o", str(out),
              f"-L{LIBDIR}", "-lbpgb300", "-Wl,-rpath,$ORIGIN/_lib"])
    if verbose:
        print(f"built {out}")
    return out


def build_oracle(verbose: bool = False) -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    src = ORACLE / "oracle.c"
    if _stale(ORACLE_LIB, [src]):
        _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              str(src), "-o", str(ORACLE_LIB), "-lm"])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_reference(verbose: bool = False) -> Path | None:
    """Reference kernel from its own sources (only where they are mounted) and its loader."""
    REF_CUBIN.parent.mkdir(parents=True, exist_ok=True)
    src = REFERENCE_SRC / "backproject_cuda.cu"
    if src.exists() and _stale(REF_CUBIN, [src]):
        _run([NVCC, "-std=c++17", "-O3", *ARCH, "-cubin", f"-I{REFERENCE_SRC}", str(src),
              "-o", str(REF_CUBIN)])
    if not REF_CUBIN.exists():
        return None
    harness = ORACLE / "ref_harness.cu"
    if harness.exists() and _stale(REF_LIB, [harness]):
        _run([NVCC, "-std=c++17", "-O2", *ARCH, "-shared", "-Xcompiler", "-fPIC", str(harness),
              "-o", str(REF_LIB), f"-L{CUDA_HOME / 'lib64' / 'stubs'}", "-lcuda"])
    if verbose:
        print(f"built {REF_LIB}")
    return REF_LIB


CLI_PATH = LIBDIR / "bpgb_backprojector"


def build_cli(verbose: bool = False) -> Path:
    """The command-line tool (csrc/cli.cpp) linked against the library."""
    src = CSRC / "cli.cpp"
    if _stale(CLI_PATH, [src, LIB_PATH, *_headers()]):
        _run(["g++", "-std=c++17", "-O2", f"-I{INCLUDE}", f"-I{CSRC}", str(src), "-o",
              str(CLI_PATH), f"-L{LIBDIR}", "-lbpgb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {CLI_PATH}")
    return CLI_PATH


def build_all(verbose: bool = False) -> None:
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    with ThreadPoolExecutor(max_workers=3) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle, verbose)
        f_ref = ex.submit(build_reference, verbose)
        f_lib.result()
        f_orc.result()
        f_ref.result()
    build_python_module(verbose)
    build_cli(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
