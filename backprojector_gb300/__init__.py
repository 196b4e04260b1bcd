"""GB300-native NLOS backprojection engine (drop-in for mjgalindo/backprojector's GPU path).

Layers:
  include/backprojector_gb300.h   C ABI (extern "C", plain pointers, int status codes)
  csrc/                           sm_103a kernels, plans, host orchestration, pybind module
  capi.py                         ctypes binding of the C ABI (plans on device buffers)
  nlosbpy                         pybind11 module with the reference binding's functions
  synthetic.py                    seeded synthetic captures of the benchmark configurations
"""
from . import capi  # noqa: F401

__all__ = ["capi", "load_nlosbpy"]


def load_nlosbpy():
    """The compiled `nlosbpy` module (backproject / phasor), built by build.py."""
    from . import nlosbpy  # type: ignore[attr-defined]

    return nlosbpy
