"""Bounded waits that run out: the sweeps' flag waits report a timeout and the
device stays usable.

The sweeps wait on flags that other CTAs of the same launch publish.  With the
wait limit set to 1 ns (starpu_gb300_set_wait_budget_ns) any wait that is not
satisfied at once runs out: the CTA records the timeout in the call's error
word, stops waiting and the launch still ends.  No kernel is made to fault,
trap or hang; the results of the timed-out calls are discarded.  The limit is
restored before the next calls, which must then succeed and agree with the
untimed-out results.
"""
import ctypes as C

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import IrInfo, check

pytestmark = pytest.mark.gpu

GB300_ETIMEDOUT = -110


def _lower(n, seed):
    """Well-conditioned lower-triangular FP32 factor: 2 on the diagonal, small
    entries below (row sums of |L_ij| / L_ii stay below 1/2)."""
    rng = np.random.default_rng(seed)
    L = np.tril(rng.uniform(-1.0, 1.0, (n, n)), -1) * (0.5 / n) + 2.0 * np.eye(n)
    return np.asfortranarray(L.astype(np.float32))


@pytest.fixture
def short_budget(gpu):
    """Sets a 1 ns wait limit for the test body and restores the default."""
    prev = gpu.starpu_gb300_set_wait_budget_ns(1)
    try:
        yield
    finally:
        gpu.starpu_gb300_set_wait_budget_ns(prev)


def test_set_wait_budget_returns_previous_and_zero_restores_default(gpu):
    default = gpu.starpu_gb300_set_wait_budget_ns(0)
    assert default == 2_000_000_000
    assert gpu.starpu_gb300_set_wait_budget_ns(5) == default
    assert gpu.starpu_gb300_set_wait_budget_ns(0) == 5
    assert gpu.starpu_gb300_set_wait_budget_ns(0) == default


def test_sweep_wait_runs_out_then_next_call_succeeds(gpu):
    n, nrhs = 16384, 32
    L = _lower(n, 1)
    Bm = np.asfortranarray(np.random.default_rng(2).uniform(-1, 1, (n, nrhs)).astype(np.float32))
    dL = DeviceBuffer.from_array(L)
    lw = gpu.starpu_gb300_spotrs_sweep_workspace(n)
    W = DeviceBuffer(lw)

    def sweep():
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        dB = DeviceBuffer.from_array(Bm)
        check(gpu.starpu_gb300_spotrs_sweep(None, n, nrhs, dL.ptr, n, dB.ptr, n, W.ptr, lw, err.ptr))
        check(gpu.starpu_gb300_stream_sync(None))
        return int(err.download((1,), np.int32)[0]), dB.download((n, nrhs), np.float32)

    err0, X0 = sweep()  # the default limit: the reference result
    assert err0 == 0
    prev = gpu.starpu_gb300_set_wait_budget_ns(1)
    try:
        timed_out, _ = sweep()
    finally:
        gpu.starpu_gb300_set_wait_budget_ns(prev)
    assert timed_out != 0, "a 1 ns wait limit must run out in a 256-block sweep"

    # the default limit again: the same call succeeds, bit for bit as before,
    # and solves L L^T X = B to FP32 accuracy
    err2, X2 = sweep()
    assert err2 == 0
    np.testing.assert_array_equal(X2, X0)
    L64, X = L.astype(np.float64), X2.astype(np.float64)
    R = L64 @ (L64.T @ X) - Bm
    assert np.max(np.abs(R)) <= 1e-4 * np.max(np.abs(Bm))


def test_mixed_solve_reports_timeout_then_converges(gpu, oracle, short_budget):
    n, nb, nrhs = 4096, 1024, 16
    A = oracle.spd_gram(n, 3, oracle.alpha_for_kappa(1e3))
    Bm = oracle.uniform_rhs(n, nrhs, 4)
    dA, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(Bm)
    dX = DeviceBuffer(8 * n * nrhs)
    lw = gpu.starpu_gb300_dsposv_workspace(n, nrhs, nb)
    W = DeviceBuffer(lw)
    info = IrInfo()
    rc = gpu.starpu_gb300_dsposv(None, n, nrhs, dA.ptr, n, dB.ptr, n, dX.ptr, n, nb, 3, 1e-12, 30, W.ptr, lw,
                                 C.byref(info))
    assert rc == GB300_ETIMEDOUT and info.status == GB300_ETIMEDOUT

    gpu.starpu_gb300_set_wait_budget_ns(0)
    info = IrInfo()
    check(gpu.starpu_gb300_dsposv(None, n, nrhs, dA.ptr, n, dB.ptr, n, dX.ptr, n, nb, 3, 1e-12, 30, W.ptr, lw,
                                  C.byref(info)), "dsposv after the timeout")
    X = dX.download((n, nrhs), np.float64)
    be, _ = oracle.backward_error(A, X, Bm)
    assert info.status == 0 and be <= 1e-12, (info.status, be)
