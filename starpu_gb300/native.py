"""ctypes binding of ``libstarpu_gb300.so``.

Argument types are declared from the public headers in ``include/`` so a
Python host calls exactly the C-ABI a C host links against.  There is no
fallback path: a missing library or symbol raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import threading

from . import build as _build

_lock = threading.Lock()
_lib: C.CDLL | None = None

c_int, c_size_t, c_void_p, c_float, c_double, c_char_p = C.c_int, C.c_size_t, C.c_void_p, C.c_float, C.c_double, C.c_char_p
c_int64, c_uint64 = C.c_int64, C.c_uint64

_CTYPES = {
    "void": None, "int": c_int, "unsigned": C.c_uint, "size_t": c_size_t, "float": c_float, "double": c_double,
    "long": C.c_long, "int64_t": c_int64, "uint64_t": c_uint64, "uint32_t": C.c_uint32, "int32_t": C.c_int32,
    "const char*": c_char_p, "char*": c_char_p,
}


def lib_path() -> str:
    return _build.lib_path()


def build(verbose: bool = False) -> str:
    return _build.build(verbose=verbose)


def header_prototypes(header: str) -> dict[str, tuple[str, list[str]]]:
    """Parse the ``starpu_gb300_*`` function prototypes of a public header."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", " ", txt)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(starpu_gb300_\w+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("#") or "typedef" in ret:
            continue
        ret = " ".join(ret.split())
        alist = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret, alist)
    return out


def _ctype(decl: str):
    d = " ".join(decl.replace("*", " * ").split())
    d = re.sub(r"\s+\*", "*", d)
    if "*" in d:
        base = d.replace("const ", "")
        if base.startswith("char*") and d.count("*") == 1:
            return c_char_p
        return c_void_p
    # strip parameter name
    toks = d.replace("const ", "").split()
    for n in (2, 1):
        key = " ".join(toks[:n])
        if key in _CTYPES:
            return _CTYPES[key]
    if toks and toks[0] in ("struct", "enum"):
        return c_int
    raise TypeError(f"unmapped C type in prototype: {decl!r}")


# Public headers whose starpu_gb300_* functions live in libstarpu_gb300.so
# (starpu_gb300_chol.h belongs to the codelet library libstarpu_gb300_chol.so).
MAIN_HEADERS = ("starpu_gb300_kernels.h", "starpu_gb300_solver.h")


def _bind(dll: C.CDLL) -> None:
    inc = os.path.join(_build.ROOT, "include")
    for h in MAIN_HEADERS:
        for name, (ret, args) in header_prototypes(os.path.join(inc, h)).items():
            fn = getattr(dll, name)  # raises AttributeError if the symbol is missing
            fn.restype = _ctype(ret) if ret != "void" else None
            fn.argtypes = [_ctype(a) for a in args]


def load(rebuild: bool = False) -> C.CDLL:
    """Load (building first if needed) and bind the native library."""
    global _lib
    with _lock:
        if _lib is not None and not rebuild:
            return _lib
        path = lib_path()
        if rebuild or not os.path.exists(path):
            build()
        dll = C.CDLL(path, mode=C.RTLD_GLOBAL)
        _bind(dll)
        _lib = dll
        return dll


class _LazyLib:
    def __getattr__(self, name):
        return getattr(load(), name)


lib = _LazyLib()


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = load().starpu_gb300_last_error()
        raise RuntimeError(f"{what} failed with {rc}: {msg.decode() if msg else ''}")


class IrInfo(C.Structure):
    """ctypes mirror of starpu_gb300_ir_info (include/starpu_gb300_solver.h)."""
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("factor_terms", C.c_int), ("potrf_info", C.c_int),
                ("backward_error", C.c_double), ("anorm", C.c_double), ("method", C.c_int), ("fallback", C.c_int)]


class Request(C.Structure):
    """ctypes mirror of starpu_gb300_request (include/starpu_gb300_solver.h)."""
    _fields_ = [("n", C.c_int), ("nrhs", C.c_int), ("A", C.c_void_p), ("B", C.c_void_p), ("X", C.c_void_p),
                ("matrix_id", C.c_uint64), ("tol", C.c_double), ("max_iter", C.c_int), ("status", C.c_int),
                ("iterations", C.c_int), ("cache_hit", C.c_int), ("batched", C.c_int),
                ("backward_error", C.c_double), ("submit_us", C.c_double), ("start_us", C.c_double),
                ("end_us", C.c_double), ("done", C.c_int), ("reserved", C.c_int)]


class Stream:
    """A non-blocking CUDA stream owned by the native library."""

    def __init__(self):
        self.handle = load().starpu_gb300_stream_create()
        if not self.handle:
            raise RuntimeError("stream creation failed: " + load().starpu_gb300_last_error().decode())

    def sync(self):
        check(load().starpu_gb300_stream_sync(self.handle), "stream sync")

    def close(self):
        if self.handle:
            load().starpu_gb300_stream_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceBuffer:
    """Device allocation made through the C-ABI (cudaMalloc) with numpy up/download."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        self.ptr = load().starpu_gb300_device_malloc(self.nbytes)
        if not self.ptr:
            raise MemoryError("device allocation failed: " + load().starpu_gb300_last_error().decode())

    @classmethod
    def from_array(cls, arr, stream: Stream | None = None):
        import numpy as np
        a = np.asfortranarray(arr)
        b = cls(a.nbytes)
        b.upload(a, stream)
        return b

    def upload(self, arr, stream: Stream | None = None):
        import numpy as np
        a = np.asfortranarray(arr)
        assert a.nbytes <= self.nbytes
        s = stream.handle if stream else None
        check(load().starpu_gb300_memcpy_h2d(s, self.ptr, a.ctypes.data, a.nbytes), "h2d")
        check(load().starpu_gb300_stream_sync(s), "sync")

    def download(self, shape, dtype, stream: Stream | None = None):
        import numpy as np
        out = np.empty(shape, dtype=dtype, order="F")
        s = stream.handle if stream else None
        check(load().starpu_gb300_memcpy_d2h(s, out.ctypes.data, self.ptr, out.nbytes), "d2h")
        check(load().starpu_gb300_stream_sync(s), "sync")
        return out

    def free(self):
        if self.ptr:
            load().starpu_gb300_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __int__(self):
        return int(self.ptr)
