"""The C-ABI libraries load (no GPU needed) and export every function that
the public headers in include/ declare; argument checking happens before any
device work."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions(header):
    txt = open(os.path.join(INC, header)).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    txt = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", " ", txt)
    txt = re.sub(r"#[^\n]*", " ", txt)
    names = set()
    for m in re.finditer(r"\b(starpu_\w+)\s*\(([^;{}]*?)\)\s*(__attribute__\s*\(\(.*?\)\))?\s*;", txt, flags=re.S):
        # skip function-pointer members "(*name)(...)"
        pre = txt[max(0, m.start() - 2):m.start()]
        if "(*" in pre or "*" == pre.strip()[-1:]:
            continue
        names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def libs():
    import starpu_gb300
    from starpu_gb300 import build as _b  # noqa: F401
    starpu_gb300.build()
    main = starpu_gb300.load()
    chol = C.CDLL(os.path.join(ROOT, "starpu_gb300", "lib", "libstarpu_gb300_chol.so"))
    return main, chol


def test_every_declared_function_is_exported(libs):
    main, chol = libs
    headers = sorted(h for h in os.listdir(INC) if h.endswith(".h"))
    missing = []
    total = 0
    for h in headers:
        lib = chol if h == "starpu_gb300_chol.h" else main
        for name in sorted(declared_functions(h)):
            total += 1
            if not hasattr(lib, name):
                missing.append(f"{h}: {name}")
    assert total > 100
    assert not missing, missing


def test_codelet_library_defines_the_reference_symbols(libs):
    _, chol = libs
    for sym in ("cl_potrf", "cl_trsm", "cl_syrk", "cl_gemm", "chol_model_potrf", "chol_model_gemm", "scratch",
                "devInfo", "cholesky_kernel_init", "cholesky_kernel_fini"):
        assert hasattr(chol, sym), sym


def test_lu_codelet_library_defines_the_reference_symbols(libs):
    lu = C.CDLL(os.path.join(ROOT, "starpu_gb300", "lib", "libstarpu_gb300_lu.so"))
    for sym in ("cl_getrf", "cl_getrf_pivot", "cl_trsm_ll", "cl_trsm_ru", "cl_gemm", "cl_pivot", "scratch",
                "devInfo", "lu_kernel_init", "lu_kernel_fini"):
        assert hasattr(lu, sym), sym


def test_tests_keep_device_buffers_alive():
    """A DeviceBuffer frees its memory when its last reference goes, so the
    pointer read off a buffer made inside a call's arguments is already freed
    when the kernel runs.  No test may pass one."""
    bad = []
    here = os.path.dirname(os.path.abspath(__file__))
    for name in sorted(os.listdir(here)):
        if name.endswith(".py"):
            for no, line in enumerate(open(os.path.join(here, name)), 1):
                if re.search(r"\)\.ptr\b", line.split("#")[0]):
                    bad.append(f"{name}:{no}: {line.strip()}")
    assert not bad, bad


def test_invalid_arguments_are_rejected_without_a_gpu(libs):
    main, _ = libs
    EINVAL = -22
    assert main.starpu_gb300_sgemm_nt_tile(None, -1, 1, 1, 1.0, None, 1, None, 1, 0.0, None, 1) == EINVAL
    assert main.starpu_gb300_dpotrf(None, 10, None, 5, 0, None) == EINVAL
    assert main.starpu_gb300_spotrs_noalloc(None, 16385, 1, None, 16385, None, 16385, None) == EINVAL
    assert main.starpu_gb300_dsposv(None, 10, 1, None, 10, None, 10, None, 10, 0, 2, 1e-12, 10, None, 0, None) == EINVAL
    assert main.starpu_gb300_dsposv_workspace(32768, 16, 1024) > 4 * 32768 * 32768
    assert main.starpu_gb300_server_wait(None, None) == EINVAL
    assert main.starpu_gb300_server_drain(None) == EINVAL
    assert main.starpu_gb300_server_submit(None, None) == EINVAL
    assert main.starpu_gb300_launch_count() == 0


def test_kernel_attributes_are_set_once_per_device(libs):
    """The dynamic shared memory limit of a kernel is set per function and
    device: the bookkeeping sets it again on a second device, on a larger
    request and after a failed attempt, and never twice otherwise."""
    main, _ = libs
    assert main.starpu_gb300_selftest_attr_book() == 0


@pytest.mark.parametrize("ntiles,spt", [(1, 1), (2, 32), (32, 32), (17, 3), (512, 1), (64, 32)])
def test_sweep_ticket_order(libs, ntiles, spt):
    """The tile sweeps' persistent CTAs take tasks by ticket; each ticket
    decodes to one task and every task it waits for has a smaller ticket."""
    main, _ = libs
    assert main.starpu_gb300_selftest_sweep_tickets(ntiles, spt) == 0


def test_wait_budget_knob_without_a_gpu(libs):
    main, _ = libs
    default = main.starpu_gb300_set_wait_budget_ns(0)
    assert default == 2_000_000_000
    assert main.starpu_gb300_set_wait_budget_ns(123) == default
    assert main.starpu_gb300_set_wait_budget_ns(0) == 123
