"""Build of the native library ``starpu_gb300/lib/libstarpu_gb300.so``.

One shared object holds the C runtime (StarPU API subset), the C-ABI kernel
layer and every sm_103a CUDA kernel.  Sources are compiled in parallel with
nvcc (``-gencode arch=compute_103a,code=sm_103a``) and gcc, in-tree, with an
mtime check so repeated builds are cheap.  No cmake.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libstarpu_gb300.so"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _headers() -> list[str]:
    hs = glob.glob(os.path.join(INCLUDE, "*.h"))
    for ext in ("*.h", "*.cuh"):
        hs += glob.glob(os.path.join(CSRC, "**", ext), recursive=True)
    return hs


def _stale(obj: str, src: str, deps_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return m < os.path.getmtime(src) or m < deps_mtime


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip() and os.environ.get("GB300_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout)


CHOL_LIBNAME = "libstarpu_gb300_chol.so"
LU_LIBNAME = "libstarpu_gb300_lu.so"
EXAMPLES = {"chol_implicit_gb300": CHOL_LIBNAME, "lu_gb300": LU_LIBNAME}
# perfmodel tools (csrc/tools/<name>.c), linked against libstarpu_gb300.so only
TOOLS = ("starpu_perfmodel_display", "starpu_perfmodel_plot")


def chol_lib_path() -> str:
    return os.path.join(LIBDIR, CHOL_LIBNAME)


def example_path(name: str) -> str:
    return os.path.join(LIBDIR, name)


def sources() -> tuple[list[str], list[str]]:
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "kernels", "*.cu")))
    c = sorted(glob.glob(os.path.join(CSRC, "runtime", "*.c")))
    return cu, c


def _build_codelets_and_examples(main_changed: bool) -> None:
    """libstarpu_gb300_chol.so (the Cholesky codelets) and the example drivers,
    linked against libstarpu_gb300.so."""
    inc = ["-I" + INCLUDE, "-I" + os.path.join(CUDA_HOME, "include")]
    rpath = "-Wl,-rpath," + LIBDIR + ":" + os.path.join(CUDA_HOME, "lib64")
    deps = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(lib_path())])
    # codelet libraries: the Cholesky codelets (codelets/) and the LU codelets (codelets_lu/)
    for sub, name in (("codelets", CHOL_LIBNAME), ("codelets_lu", LU_LIBNAME)):
        csrcs = sorted(glob.glob(os.path.join(CSRC, sub, "*.c")))
        out = os.path.join(LIBDIR, name)
        if main_changed or not os.path.exists(out) or any(_stale(out, s, deps) for s in csrcs):
            _run(["gcc", "-O2", "-g", "-fPIC", "-std=gnu11", "-Wall", "-shared", "-o", out + ".tmp", *csrcs, *inc,
                  "-L" + LIBDIR, "-lstarpu_gb300", rpath])
            os.replace(out + ".tmp", out)
    for ex, codelet_lib in EXAMPLES.items():
        src = os.path.join(CSRC, "examples", ex + ".c")
        exe = example_path(ex)
        lib = os.path.join(LIBDIR, codelet_lib)
        if main_changed or _stale(exe, src, max(deps, os.path.getmtime(lib))):
            _run(["gcc", "-O2", "-g", "-std=gnu11", "-Wall", "-o", exe + ".tmp", src, *inc, "-L" + LIBDIR,
                  "-l" + codelet_lib[3:-3], "-lstarpu_gb300", rpath, "-lm", "-lpthread"])
            os.replace(exe + ".tmp", exe)
    for tool in TOOLS:
        src = os.path.join(CSRC, "tools", tool + ".c")
        exe = example_path(tool)
        if main_changed or _stale(exe, src, deps):
            _run(["gcc", "-O2", "-g", "-std=gnu11", "-Wall", "-o", exe + ".tmp", src, *inc, "-L" + LIBDIR,
                  "-lstarpu_gb300", rpath, "-lm", "-lpthread"])
            os.replace(exe + ".tmp", exe)


def build(verbose: bool = False, extra_nvcc: list[str] | None = None) -> str:
    """Compile every source that changed and relink the library; return its path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OBJDIR, exist_ok=True)
    deps = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    cu, c = sources()
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]
    jobs = []
    objs = []
    for src in cu:
        rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
        obj = os.path.join(OBJDIR, rel + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-c", src, "-o", obj, *inc, *(extra_nvcc or [])]
            if verbose or os.environ.get("GB300_PTXAS_VERBOSE"):
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in c:
        rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
        obj = os.path.join(OBJDIR, rel + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append(["gcc", "-O2", "-g", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-function", "-pthread",
                         "-DSTARPU_GB300_BUILDING_LIB", "-c", src, "-o", obj, *inc])
    if jobs:
        with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
            list(ex.map(_run, jobs))
    out = lib_path()
    main_changed = bool(jobs) or not os.path.exists(out)
    if main_changed:
        tmp = out + ".tmp"
        _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared",
              "-Xlinker", "-rpath=" + os.path.join(CUDA_HOME, "lib64"), "-lpthread", "-ldl", "-lm"])
        os.replace(tmp, out)
    _build_codelets_and_examples(main_changed)
    return out


def clean() -> None:
    if os.path.isdir(LIBDIR):
        shutil.rmtree(LIBDIR)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
