"""The allocation-free POTRS entry point (starpu_gb300_spotrs_noalloc).

Callers such as a codelet body inside a runtime that owns all device memory,
or a serving loop that must not allocate on its request path, cannot pass a
workspace.  This test checks, through the C-ABI, that the allocation-free
entry point gives the same solution as the workspace entry point
(starpu_gb300_spotrs_sweep) on two calls in a row -- the static scratch keeps
the previous call's contents, so the second call also checks that everything
that must start at zero is cleared -- and that sizes beyond the stated limit
are rejected.  The file is named so that pytest collects it last.
"""
import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu

GB300_EINVAL = -22
MAX_N = 16384


def _factor(oracle, n):
    i = np.arange(n, dtype=np.float64)
    A = 1.0 / (1.0 + i[:, None] + i[None, :]) + n * np.eye(n)
    return np.tril(oracle.potrf_tiled(A.astype(np.float32), max(1, n // 512))[0])


@pytest.mark.parametrize("n,nrhs", [(1000, 16), (2049, 20)])
def test_noalloc_matches_workspace_entry_point(gpu, oracle, n, nrhs):
    L = _factor(oracle, n)
    dL = DeviceBuffer.from_array(L)
    lw = gpu.starpu_gb300_spotrs_sweep_workspace(n)
    W = DeviceBuffer(lw)
    err = DeviceBuffer.from_array(np.zeros(1, np.int32))
    for call in range(2):
        Bm = oracle.uniform_rhs(n, nrhs, 100 + call).astype(np.float32)
        d_ref, d_new = DeviceBuffer.from_array(Bm), DeviceBuffer.from_array(Bm)
        check(gpu.starpu_gb300_spotrs_sweep(None, n, nrhs, dL.ptr, n, d_ref.ptr, n, W.ptr, lw, err.ptr))
        check(gpu.starpu_gb300_spotrs_noalloc(None, n, nrhs, dL.ptr, n, d_new.ptr, n, None))
        check(gpu.starpu_gb300_stream_sync(None))
        X_ref = d_ref.download(Bm.shape, np.float32)
        X_new = d_new.download(Bm.shape, np.float32)
        scale = np.max(np.abs(X_ref))
        assert np.max(np.abs(X_new - X_ref)) <= 1e-4 * scale, f"call {call}"
        assert err.download((1,), np.int32)[0] == 0


def test_noalloc_rejects_sizes_beyond_its_limit(gpu):
    n = MAX_N + 1
    rc = gpu.starpu_gb300_spotrs_noalloc(None, n, 1, None, n, None, n, None)
    assert rc == GB300_EINVAL
    assert b"STARPU_GB300_NOALLOC_MAX_N" in gpu.starpu_gb300_last_error()
