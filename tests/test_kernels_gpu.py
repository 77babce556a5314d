"""GPU parity of the C-ABI tile kernels and whole-matrix drivers against the
oracle (CPU restatement of the reference codelets), through the C-ABI."""
import ctypes as C

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer, Stream
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu


def up(a):
    return DeviceBuffer.from_array(np.asfortranarray(a))


def down(buf, like):
    return buf.download(like.shape, like.dtype)


def info_buf():
    b = DeviceBuffer(4)
    b.upload(np.zeros(1, dtype=np.int32))
    return b


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 5, 32, 33, 64, 65, 200, 512])
def test_potrf_tile(gpu, oracle, dtype, n):
    A = oracle.spd_gram(n, 100 + n, 1.0).astype(dtype)
    lda = n + 3
    Apad = np.zeros((lda, n), dtype=dtype, order="F")
    Apad[:n] = A
    d = up(Apad)
    info = info_buf()
    f = gpu.starpu_gb300_spotrf_tile if dtype == np.float32 else gpu.starpu_gb300_dpotrf_tile
    check(f(None, n, d.ptr, lda, info.ptr))
    L = np.tril(down(d, Apad)[:n])
    assert info.download((1,), np.int32)[0] == 0
    Lo, _ = oracle.potrf_tiled(A, 1)
    tol = 1e-5 if dtype == np.float32 else 1e-13
    assert np.max(np.abs(L - np.tril(Lo))) <= tol * np.max(np.abs(Lo))
    assert oracle.llt_residual(A.astype(np.float64), L) <= (1e-6 if dtype == np.float32 else 1e-14)
    # the strict upper triangle is not touched
    assert np.array_equal(np.triu(down(d, Apad)[:n], 1), np.triu(Apad[:n], 1))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("m,n", [(1, 1), (300, 64), (129, 65), (1000, 256), (7, 100)])
def test_trsm_tile(gpu, oracle, dtype, m, n):
    A = oracle.spd_gram(n, 7, 1.0)
    L = np.tril(oracle.potrf_tiled(A, 1)[0]).astype(dtype)
    rng = np.random.default_rng(m * 1000 + n)
    Bm = rng.uniform(-1, 1, (m, n)).astype(dtype)
    dL, dB = up(L), up(Bm)
    f = gpu.starpu_gb300_strsm_rltn_tile if dtype == np.float32 else gpu.starpu_gb300_dtrsm_rltn_tile
    check(f(None, m, n, 1.0, dL.ptr, n, dB.ptr, m))
    X = down(dB, Bm)
    ref = Bm.astype(np.float64) @ np.linalg.inv(L.astype(np.float64)).T
    tol = 1e-5 if dtype == np.float32 else 1e-12
    assert np.max(np.abs(X - ref)) <= tol * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (64, 64, 64), (300, 129, 77), (512, 512, 512), (130, 17, 256)])
def test_gemm_nt_tile(gpu, dtype, m, n, k):
    rng = np.random.default_rng(m + 7 * n + 13 * k)
    A = rng.standard_normal((m, k)).astype(dtype)
    Bm = rng.standard_normal((n, k)).astype(dtype)
    Cm = rng.standard_normal((m, n)).astype(dtype)
    dA, dB, dC = up(A), up(Bm), up(Cm)
    f = gpu.starpu_gb300_sgemm_nt_tile if dtype == np.float32 else gpu.starpu_gb300_dgemm_nt_tile
    check(f(None, m, n, k, -1.0, dA.ptr, m, dB.ptr, n, 1.0, dC.ptr, m))
    out = down(dC, Cm)
    ref = Cm.astype(np.float64) - A.astype(np.float64) @ Bm.astype(np.float64).T
    tol = 1e-5 if dtype == np.float32 else 1e-13
    assert np.max(np.abs(out - ref)) <= tol * np.sqrt(k) * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n,k", [(1, 1), (64, 64), (200, 33), (512, 512)])
def test_syrk_ln_tile(gpu, dtype, n, k):
    rng = np.random.default_rng(n + k)
    A = rng.standard_normal((n, k)).astype(dtype)
    Cm = rng.standard_normal((n, n)).astype(dtype)
    dA, dC = up(A), up(Cm)
    f = gpu.starpu_gb300_ssyrk_ln_tile if dtype == np.float32 else gpu.starpu_gb300_dsyrk_ln_tile
    check(f(None, n, k, -1.0, dA.ptr, n, 1.0, dC.ptr, n))
    out = down(dC, Cm)
    ref = Cm.astype(np.float64) - A.astype(np.float64) @ A.astype(np.float64).T
    tol = 1e-5 if dtype == np.float32 else 1e-13
    lo = np.tril_indices(n)
    assert np.max(np.abs(out[lo] - ref[lo])) <= tol * np.sqrt(k) * max(1.0, np.max(np.abs(ref)))
    up_ = np.triu_indices(n, 1)
    assert np.array_equal(out[up_], Cm[up_])  # upper triangle untouched (SYRK uplo=L)


@pytest.mark.parametrize("n,nb", [(256, 32), (2048, 256), (1000, 128), (2048, 512)])
def test_spotrf_hilbert_reference_check(gpu, oracle, n, nb):
    """Config-1 input through the whole-matrix FP32 driver; the reference's
    own acceptance criterion (cholesky_implicit.c:574-580)."""
    A = oracle.hilbert_f32(n)
    d = up(A)
    info = info_buf()
    check(gpu.starpu_gb300_spotrf(None, n, d.ptr, n, nb, info.ptr))
    L = down(d, A)
    assert info.download((1,), np.int32)[0] == 0
    bad, worst = oracle.check_hilbert(L, 1e-4)
    assert bad == 0, worst
    Lo, _ = oracle.potrf_tiled(A, max(1, n // nb))
    assert np.max(np.abs(np.tril(L) - np.tril(Lo))) <= 1e-5 * np.max(np.abs(Lo))


@pytest.mark.parametrize("n,nb,nrhs", [(1, 1, 1), (97, 32, 3), (1024, 256, 16), (1500, 512, 64)])
def test_dpotrf_dpotrs_fp64(gpu, oracle, n, nb, nrhs):
    A = oracle.spd_gram(n, 21, 2.0)
    Bm = oracle.uniform_rhs(n, nrhs, 22)
    dA, dB = up(A), up(Bm)
    info = info_buf()
    check(gpu.starpu_gb300_dpotrf(None, n, dA.ptr, n, nb, info.ptr))
    check(gpu.starpu_gb300_dpotrs(None, n, nrhs, dA.ptr, n, dB.ptr, n))
    assert info.download((1,), np.int32)[0] == 0
    L = np.tril(down(dA, A))
    X = down(dB, Bm)
    assert oracle.llt_residual(A, L) <= 1e-14
    be, _ = oracle.backward_error(A, X, Bm)
    assert be <= 1e-14
    Xo = oracle.potrs(np.tril(oracle.potrf_tiled(A, max(1, n // nb))[0]), Bm)
    assert np.max(np.abs(X - Xo)) <= 1e-10 * np.max(np.abs(Xo))


def test_spotrs_fp32(gpu, oracle):
    n, nrhs = 700, 5
    A = oracle.spd_gram(n, 5, 2.0)
    Bm = oracle.uniform_rhs(n, nrhs, 6)
    dA, dB = up(A.astype(np.float32)), up(Bm.astype(np.float32))
    check(gpu.starpu_gb300_spotrf(None, n, dA.ptr, n, 128, None))
    check(gpu.starpu_gb300_spotrs(None, n, nrhs, dA.ptr, n, dB.ptr, n))
    X = down(dB, Bm.astype(np.float32))
    be, _ = oracle.backward_error(A, X.astype(np.float64), Bm)
    assert be <= 1e-6


@pytest.mark.parametrize("n,nrhs", [(1, 1), (63, 3), (64, 16), (65, 17), (1000, 40), (4097, 16)])
def test_spotrs_sweep_matches_blocked_and_oracle(gpu, oracle, n, nrhs):
    A = oracle.spd_gram(min(n, 1200), 8, 2.0) if n <= 1200 else None
    if A is None:  # diagonally dominant FP32 input for the large case (oracle Gram is O(n^3))
        i = np.arange(n, dtype=np.float64)
        A = 1.0 / (1.0 + i[:, None] + i[None, :]) + n * np.eye(n)
    L = np.tril(oracle.potrf_tiled(A.astype(np.float32), max(1, n // 512))[0])
    Bm = oracle.uniform_rhs(n, nrhs, 9).astype(np.float32)
    dL = up(L)
    d1, d2 = up(Bm), up(Bm)
    lw = gpu.starpu_gb300_spotrs_sweep_workspace(n)
    W = DeviceBuffer(lw)
    err = info_buf()
    check(gpu.starpu_gb300_spotrs_sweep(None, n, nrhs, dL.ptr, n, d1.ptr, n, W.ptr, lw, err.ptr))
    check(gpu.starpu_gb300_spotrs(None, n, nrhs, dL.ptr, n, d2.ptr, n))
    X1, X2 = down(d1, Bm), down(d2, Bm)
    assert err.download((1,), np.int32)[0] == 0
    Xo = oracle.potrs(L, Bm)
    scale = np.max(np.abs(Xo))
    assert np.max(np.abs(X1 - Xo)) <= 1e-4 * scale
    assert np.max(np.abs(X1 - X2)) <= 1e-4 * scale
    # deterministic: the fixed accumulation order gives bit-identical repeats
    d3 = up(Bm)
    check(gpu.starpu_gb300_spotrs_sweep(None, n, nrhs, dL.ptr, n, d3.ptr, n, W.ptr, lw, err.ptr))
    np.testing.assert_array_equal(down(d3, Bm), X1)


def test_not_spd_sets_info_without_fault(gpu):
    n = 200
    A = np.eye(n) * 4.0
    A[150, 150] = -1.0
    d = up(A)
    info = info_buf()
    check(gpu.starpu_gb300_dpotrf(None, n, d.ptr, n, 64, info.ptr))
    gpu.starpu_gb300_stream_sync(None)
    assert info.download((1,), np.int32)[0] == 151
    # the context is still usable
    d4 = up(np.eye(4))
    check(gpu.starpu_gb300_dpotrf_tile(None, 4, d4.ptr, 4, None))
    gpu.starpu_gb300_stream_sync(None)
    np.testing.assert_array_equal(d4.download((4, 4), np.float64), np.eye(4))


def test_device_generator_matches_oracle(gpu, oracle):
    n = 130
    dA, dW = DeviceBuffer(n * n * 8), DeviceBuffer(n * n * 8)
    check(gpu.starpu_gb300_gen_spd_gram(None, n, 15, 0.1, dA.ptr, n, dW.ptr))
    A = dA.download((n, n), np.float64)
    np.testing.assert_allclose(A, oracle.spd_gram(n, 15, 0.1), rtol=1e-12, atol=1e-14)
    dB = DeviceBuffer(n * 3 * 8)
    check(gpu.starpu_gb300_gen_uniform_rhs(None, n, 3, 9, dB.ptr, n))
    np.testing.assert_array_equal(dB.download((n, 3), np.float64), oracle.uniform_rhs(n, 3, 9))


@pytest.mark.parametrize("m,n,k,lower", [(512, 512, 512, 0), (700, 300, 1024, 0), (513, 513, 256, 1)])
def test_tile_update_on_tensor_cores(gpu, m, n, k, lower):
    """The codelets' FP32 tile update on the tensor cores (row-scaled FP16
    splits): C -= A B^T within 1e-5 of the FP64 product relative to |A||B|^T,
    the SYRK form writing only the lower triangle, B == A split once."""
    rng = np.random.default_rng(m + n + k)
    A = np.asfortranarray(rng.standard_normal((m, k)).astype(np.float32))
    # rows of very different scales: the row scaling keeps each one's precision
    A *= np.float32(2.0) ** rng.integers(-20, 20, m)[:, None].astype(np.float32)
    B = A if lower else np.asfortranarray(rng.standard_normal((n, k)).astype(np.float32))
    C0 = np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32))
    dA, dC = DeviceBuffer.from_array(A), DeviceBuffer.from_array(C0)
    dB = dA if lower else DeviceBuffer.from_array(B)
    lw = gpu.starpu_gb300_tile_tc_workspace(max(m, n, k))
    W = DeviceBuffer(lw)
    err = DeviceBuffer.from_array(np.zeros(1, np.int32))
    check(gpu.starpu_gb300_tile_tc_prepare())
    check(gpu.starpu_gb300_sgemm_nt_tile_tc(None, m, n, k, dA.ptr, m, dB.ptr, n, dC.ptr, m, lower, W.ptr, lw,
                                            err.ptr))
    C = dC.download((m, n), np.float32).astype(np.float64)
    A64, B64 = A.astype(np.float64), B.astype(np.float64)
    ref = C0.astype(np.float64) - A64 @ B64.T
    scale = np.abs(A64) @ np.abs(B64).T + np.abs(C0)
    keep = np.tril(np.ones((m, n), bool)) if lower else np.ones((m, n), bool)
    assert np.max(np.abs(C - ref)[keep] / scale[keep]) <= 1e-5
    if lower:
        np.testing.assert_array_equal(C[~keep], C0.astype(np.float64)[~keep])
    assert err.download((1,), np.int32)[0] == 0
