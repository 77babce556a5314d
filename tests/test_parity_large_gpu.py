"""Parity at the timed shapes' scale: the mixed solve and the plain FP64
factor + solve at n = 8192 against the FP64 oracle.

* Mixed (tile 1024, 16 RHS, kappa 1e4, the bench's tile and RHS count): the
  normwise backward error measured by the oracle in FP64 is <= 1e-12, the
  solver's own figure agrees with it, and the solution agrees with the FP64
  oracle solution (the CPU-path port's tiled FP64 Cholesky + dpotrs) to within
  the conditioning: forward error <= 10 kappa sqrt(n) max(berr, 1e-16).
* Plain FP64 (tile 512, 64 RHS, A = B B^T / n + 2 I: the FP64 configuration's
  factor at a quarter of its order): ||A - L L^T||_F / ||A||_F <= 1e-14, the
  solve's backward error <= 1e-12 and the same forward-error bound.
The inputs are made on the host with the oracle's generator (the device
generator's PCG64 row streams) through the host BLAS.
"""
import ctypes as C
import os

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import IrInfo, check

pytestmark = pytest.mark.gpu

N = 8192


@pytest.fixture(scope="module")
def cores(oracle):
    if not oracle.cpu_init():
        pytest.fail("the FP64 oracle needs scipy's OpenBLAS")
    return len(os.sched_getaffinity(0))


def test_dsposv_n8192_against_fp64_oracle(gpu, oracle, cores):
    n, nb, nrhs, kappa = N, 1024, 16, 1e4
    A = oracle.spd_gram_host_blas(n, 71, oracle.alpha_for_kappa(kappa), cores)
    B = oracle.uniform_rhs(n, nrhs, 72)
    dA, dB, dX = DeviceBuffer.from_array(A), DeviceBuffer.from_array(B), DeviceBuffer(8 * n * nrhs)
    lw = gpu.starpu_gb300_dsposv_workspace(n, nrhs, nb)
    W = DeviceBuffer(lw)
    info = IrInfo()
    check(gpu.starpu_gb300_dsposv(None, n, nrhs, dA.ptr, n, dB.ptr, n, dX.ptr, n, nb, 3, 1e-12, 30, W.ptr, lw,
                                  C.byref(info)), "dsposv")
    X = dX.download((n, nrhs), np.float64)
    be, per_col = oracle.backward_error(A, X, B)
    assert info.status == 0 and be <= 1e-12, (info.status, info.iterations, be)
    assert abs(be - info.backward_error) <= 1e-13 + 0.01 * be
    assert info.iterations <= 6
    Xo = oracle.cpu_solve(A, B, 1024, cores)
    fwd = np.max(np.abs(X - Xo), axis=0) / np.max(np.abs(Xo), axis=0)
    assert fwd.max() <= 10 * kappa * np.sqrt(n) * max(be, 1e-16), (fwd.max(), be)


def test_dposv_fp64_n8192_factor_and_solve_against_oracle(gpu, oracle, cores):
    n, nb, nrhs = N, 512, 64
    A = oracle.spd_gram_host_blas(n, 73, 2.0, cores)
    B = oracle.uniform_rhs(n, nrhs, 74)
    dL, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(B)
    dinfo = DeviceBuffer.from_array(np.zeros(1, np.int32))
    check(gpu.starpu_gb300_dpotrf(None, n, dL.ptr, n, nb, dinfo.ptr), "dpotrf")
    check(gpu.starpu_gb300_dpotrs(None, n, nrhs, dL.ptr, n, dB.ptr, n), "dpotrs")
    check(gpu.starpu_gb300_stream_sync(None))
    assert int(dinfo.download((1,), np.int32)[0]) == 0
    L = dL.download((n, n), np.float64)
    X = dB.download((n, nrhs), np.float64)
    assert oracle.llt_residual_blas(A, L) <= 1e-14
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12, be
    Xo = oracle.cpu_solve(A, B, 512, cores)
    kappa = (4.0 + 2.0) / 2.0  # Marchenko-Pastur edges [0, 4] shifted by 2
    fwd = np.max(np.abs(X - Xo), axis=0) / np.max(np.abs(Xo), axis=0)
    assert fwd.max() <= 10 * kappa * np.sqrt(n) * max(be, 1e-16), (fwd.max(), be)
