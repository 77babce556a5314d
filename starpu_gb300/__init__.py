"""starpu_gb300: GB300-native tiled Cholesky / SPD solve behind StarPU's C API.

The product is the native library ``lib/libstarpu_gb300.so`` (C runtime +
C-ABI + sm_103a CUDA kernels).  This package only locates, builds and binds
it for Python hosts (tests, bench); it contains no numerical fallback: if the
library is missing every call raises.
"""
from .native import lib, load, build, lib_path, DeviceBuffer, Stream  # noqa: F401

__all__ = ["lib", "load", "build", "lib_path", "DeviceBuffer", "Stream"]
