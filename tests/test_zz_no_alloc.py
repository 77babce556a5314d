"""The allocation-free POTRS entry point (starpu_gb300_spotrs_noalloc).

Callers such as a codelet body inside a runtime that owns all device memory,
or a serving loop that must not allocate on its request path, cannot pass a
workspace.  This test checks, through the C-ABI, that the allocation-free
entry point gives the same solution as the workspace entry point
(starpu_gb300_spotrs_sweep) on two calls in a row -- the static scratch keeps
the previous call's contents, so the second call also checks that everything
that must start at zero is cleared.  Both run the same kernels in the same
order, so the solutions must be bit for bit the same.  It also checks that a
wait that runs out is reported without a caller status word, and that sizes
beyond the stated limit are rejected.  The file is named so that pytest
collects it last.
"""
import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu

GB300_EINVAL = -22
GB300_ETIMEDOUT = -110
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
        assert np.array_equal(X_new, X_ref), f"call {call}"
        assert err.download((1,), np.int32)[0] == 0


def test_noalloc_with_caller_status_word_keeps_it(gpu, oracle):
    """A caller's d_err is set on a timeout and never cleared by the call."""
    n, nrhs = 1000, 4
    dL = DeviceBuffer.from_array(_factor(oracle, n))
    Bm = oracle.uniform_rhs(n, nrhs, 7).astype(np.float32)
    dB = DeviceBuffer.from_array(Bm)
    err = DeviceBuffer.from_array(np.array([5], np.int32))
    check(gpu.starpu_gb300_spotrs_noalloc(None, n, nrhs, dL.ptr, n, dB.ptr, n, err.ptr))
    check(gpu.starpu_gb300_stream_sync(None))
    assert err.download((1,), np.int32)[0] == 5


def test_noalloc_without_status_word_reports_timeout(gpu, oracle):
    """With d_err NULL a wait that runs out (1 ns limit) is returned as
    GB300_ETIMEDOUT; with the default limit the next call succeeds."""
    n, nrhs = 8192, 16
    i = np.arange(n)
    L = np.asfortranarray((np.tril(np.cos(i[:, None] * 0.37 + i[None, :]), -1) * (0.5 / n) + 2.0 * np.eye(n))
                          .astype(np.float32))
    dL = DeviceBuffer.from_array(L)
    Bm = oracle.uniform_rhs(n, nrhs, 8).astype(np.float32)
    dB = DeviceBuffer.from_array(Bm)
    check(gpu.starpu_gb300_spotrs_noalloc(None, n, nrhs, dL.ptr, n, dB.ptr, n, None))
    X0 = dB.download((n, nrhs), np.float32)
    dB.upload(Bm)
    prev = gpu.starpu_gb300_set_wait_budget_ns(1)
    try:
        rc = gpu.starpu_gb300_spotrs_noalloc(None, n, nrhs, dL.ptr, n, dB.ptr, n, None)
    finally:
        gpu.starpu_gb300_set_wait_budget_ns(prev)
    assert rc == GB300_ETIMEDOUT
    assert b"timed out" in gpu.starpu_gb300_last_error()
    dB.upload(Bm)
    check(gpu.starpu_gb300_spotrs_noalloc(None, n, nrhs, dL.ptr, n, dB.ptr, n, None))
    X = dB.download((n, nrhs), np.float32)
    np.testing.assert_array_equal(X, X0)
    L64, X = L.astype(np.float64), X.astype(np.float64)
    assert np.max(np.abs(L64 @ (L64.T @ X) - Bm)) <= 1e-4 * np.max(np.abs(Bm))


def test_noalloc_rejects_sizes_beyond_its_limit(gpu):
    n = MAX_N + 1
    rc = gpu.starpu_gb300_spotrs_noalloc(None, n, 1, None, n, None, n, None)
    assert rc == GB300_EINVAL
    assert b"STARPU_GB300_NOALLOC_MAX_N" in gpu.starpu_gb300_last_error()
