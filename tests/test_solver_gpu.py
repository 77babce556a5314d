"""GPU parity of the mixed-precision solve (tensor-core factor + FP64
iterative refinement) against the FP64 oracle: the normwise backward error
must reach 1e-12 and the solution must match the FP64 LAPACK-style solution
to within the conditioning."""
import ctypes as C

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import IrInfo, check

pytestmark = pytest.mark.gpu

GB300_EDOM = -33
GB300_ETIMEDOUT = -110


def solve(gpu, A, B, nb, nterms, tol=1e-12, max_iter=30):
    n, nrhs = B.shape
    dA, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(B)
    dX = DeviceBuffer(n * nrhs * 8)
    lw = gpu.starpu_gb300_dsposv_workspace(n, nrhs, nb)
    W = DeviceBuffer(lw)
    info = IrInfo()
    rc = gpu.starpu_gb300_dsposv(None, n, nrhs, dA.ptr, n, dB.ptr, n, dX.ptr, n, nb, nterms, tol, max_iter, W.ptr, lw,
                                 C.byref(info))
    X = dX.download((n, nrhs), np.float64)
    # inputs are read-only
    np.testing.assert_array_equal(dA.download(A.shape, np.float64), A)
    return rc, info, X


@pytest.mark.parametrize("n,nb", [(1000, 256), (2048, 512)])
def test_factor_mirrors_lt_into_upper_part(gpu, oracle, n, nb):
    """After the mixed solve the workspace's FP32 factor W (its first n x n
    floats) holds L below the diagonal and, outside the diagonal tiles, L^T
    above it: the backward sweeps read that copy."""
    A = oracle.spd_gram(n, 41, oracle.alpha_for_kappa(1e3))
    B = oracle.uniform_rhs(n, 2, 42)
    dA, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(B)
    dX = DeviceBuffer(n * 2 * 8)
    lw = gpu.starpu_gb300_dsposv_workspace(n, 2, nb)
    W = DeviceBuffer(lw)
    info = IrInfo()
    rc = gpu.starpu_gb300_dsposv(None, n, 2, dA.ptr, n, dB.ptr, n, dX.ptr, n, nb, 3, 1e-12, 30, W.ptr, lw,
                                 C.byref(info))
    assert rc == 0
    Wf = W.download((n * n,), np.float32).reshape((n, n), order="F")
    tile = np.arange(n) // nb
    below = tile[:, None] > tile[None, :]          # (r, c) strictly below the diagonal tiles
    np.testing.assert_array_equal(Wf.T[below], Wf[below])


# plain BF16 (nterms=1, u ~ 4e-3) only refines when kappa * u < 1: kappa = 1e2
@pytest.mark.parametrize("kappa,nterms", [(1e2, 3), (1e4, 3), (1e2, 1)])
def test_dsposv_reaches_fp64_backward_error(gpu, oracle, kappa, nterms):
    n, nb, nrhs = 1024, 256, 4
    A = oracle.spd_gram(n, 31, oracle.alpha_for_kappa(kappa))
    B = oracle.uniform_rhs(n, nrhs, 32)
    rc, info, X = solve(gpu, A, B, nb, nterms)
    assert rc == 0 and info.status == 0, (rc, info.status, info.iterations, info.backward_error)
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12
    assert abs(be - info.backward_error) <= 1e-13 + 0.01 * be  # device-side norm agrees with the oracle's
    L = np.tril(oracle.potrf_tiled(A, 4)[0])
    Xo = oracle.potrs(L, B)
    fwd = np.max(np.abs(X - Xo)) / np.max(np.abs(Xo))
    # normwise bound: forward error <= cond * backward error (norm-equivalence factor sqrt(n))
    assert fwd <= 10 * kappa * np.sqrt(n) * max(be, 1e-16)
    if nterms == 3:
        assert info.iterations <= 6


@pytest.mark.parametrize("scale", [1e-34, 1e36])
def test_dsposv_scaled_matrix_residual(gpu, oracle, scale):
    """The refinement residual is formed from FP32 hi/lo pairs after scaling A
    and each column of X by powers of two, and each FP32 correction solve runs
    on a power-of-two-scaled residual: with A ~ 1e-34 or 1e36, whose low
    parts and late corrections lie far below FP32's normal range, the system
    must refine like an unscaled one."""
    n, nb, nrhs = 640, 128, 3
    A = oracle.spd_gram(n, 43, oracle.alpha_for_kappa(1e3)) * scale
    B = oracle.uniform_rhs(n, nrhs, 44)
    rc, info, X = solve(gpu, A, B, nb, 3)
    assert rc == 0 and info.status == 0, (rc, info.iterations, info.backward_error)
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12
    assert abs(be - info.backward_error) <= 1e-13 + 0.01 * be


@pytest.mark.parametrize("n,nb", [(1000, 256), (640, 128)])
def test_dsposv_reads_only_the_lower_triangle(gpu, oracle, n, nb):
    """LAPACK uplo = 'L': the strict upper triangle of A is never read, so
    filling it with NaN leaves the solution bit-identical."""
    nrhs = 5
    A = oracle.spd_gram(n, 45, oracle.alpha_for_kappa(1e3))
    B = oracle.uniform_rhs(n, nrhs, 46)
    rc, info, X = solve(gpu, A, B, nb, 3)
    assert rc == 0
    An = np.array(A, order="F")
    An[np.triu_indices(n, 1)] = np.nan
    rc2, info2, X2 = solve(gpu, An, B, nb, 3)
    assert rc2 == 0 and info2.iterations == info.iterations
    np.testing.assert_array_equal(X2, X)


def test_dsposv_ill_conditioned_converges(gpu, oracle):
    n, nb, nrhs = 768, 256, 2
    A = oracle.spd_gram(n, 33, oracle.alpha_for_kappa(1e6))
    B = oracle.uniform_rhs(n, nrhs, 34)
    rc, info, X = solve(gpu, A, B, nb, 3, max_iter=40)
    assert rc == 0, (rc, info.iterations, info.backward_error, info.fallback)
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12


@pytest.fixture
def refinement(gpu):
    """Sets the refinement mode for the test body and restores it."""
    prev = gpu.starpu_gb300_dsposv_set_refinement(-1)
    yield lambda m: gpu.starpu_gb300_dsposv_set_refinement(m)
    gpu.starpu_gb300_dsposv_set_refinement(prev)


def test_conjugate_gradients_rung_at_kappa_1e6(gpu, oracle, refinement):
    """kappa = 1e6: classic refinement contracts the error by ~0.3 per
    correction with the mixed factor; the automatic policy switches to
    preconditioned conjugate gradients after the first slow correction and
    needs fewer corrections, to the same backward error, and the solution
    agrees with the FP64 oracle's within kappa * 1e-12 (forward error)."""
    n, nb, nrhs = 4096, 1024, 4
    A = oracle.spd_gram(n, 35, oracle.alpha_for_kappa(1e6))
    B = oracle.uniform_rhs(n, nrhs, 36)
    refinement(0)
    rc0, info0, X0 = solve(gpu, A, B, nb, 3, max_iter=60)
    refinement(2)
    rc, info, X = solve(gpu, A, B, nb, 3, max_iter=60)
    assert rc0 == 0 and rc == 0, (rc0, rc)
    assert info0.method == 0 and info.method == 1 and info.fallback == 0
    assert info.iterations < info0.iterations, (info.iterations, info0.iterations)
    for Xk in (X0, X):
        be, _ = oracle.backward_error(A, Xk, B)
        assert be <= 1e-12
    Xo = oracle.cpu_solve(A, B, nb, 8)
    fe = np.max(np.abs(X - Xo)) / np.max(np.abs(Xo))
    assert fe <= 1e6 * 1e-12 * 10, fe


def test_pcg_only_matches_classic_on_easy_systems(gpu, oracle, refinement):
    """Conjugate gradients from the first correction also converge on a
    well-conditioned system (kappa = 1e2), to the same backward error."""
    n, nb, nrhs = 1024, 256, 3
    A = oracle.spd_gram(n, 37, oracle.alpha_for_kappa(1e2))
    B = oracle.uniform_rhs(n, nrhs, 38)
    refinement(1)
    rc, info, X = solve(gpu, A, B, nb, 3)
    assert rc == 0 and info.method == 1
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12


@pytest.fixture
def fallback(gpu):
    prev = gpu.starpu_gb300_dsposv_set_fp64_fallback(-1)
    yield lambda on: gpu.starpu_gb300_dsposv_set_fp64_fallback(on)
    gpu.starpu_gb300_dsposv_set_fp64_fallback(prev)


def _fp32_singular(n, seed):
    """SPD in FP64 (eigenvalues 1e-9 and 1 + (n - 1)(1 - 1e-9): kappa ~ n 1e9)
    but singular once rounded to FP32: every off-diagonal entry is 1 - 1e-9,
    which FP32 rounds to 1."""
    rng = np.random.default_rng(seed)
    A = np.full((n, n), 1.0 - 1e-9)
    np.fill_diagonal(A, 1.0)
    return np.asfortranarray(A), np.asfortranarray(rng.uniform(-1, 1, (n, 2)))


def test_fp64_fallback_when_the_mixed_factor_fails(gpu, oracle, fallback):
    """LAPACK dsposv semantics: the FP32-storage factorisation breaks down
    (or its refinement cannot converge) on a matrix that is SPD only in FP64;
    the FP64 factorisation on the GPU then solves it to FP64 accuracy.  With
    the fallback off the mixed outcome is returned as it is."""
    n, nb = 512, 256
    A, B = _fp32_singular(n, 39)
    assert np.linalg.eigvalsh(A).min() > 0
    fallback(1)
    rc, info, X = solve(gpu, A, B, nb, 3)
    assert rc == 0 and info.status == 0 and info.fallback in (1, 2), (rc, info.fallback, info.potrf_info)
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-12 and abs(be - info.backward_error) <= 1e-13 + 0.05 * be, (be, info.backward_error)
    fallback(0)
    rc0, info0, _ = solve(gpu, A, B, nb, 3)
    assert rc0 in (GB300_EDOM, GB300_ETIMEDOUT) and info0.fallback == 0


def test_dsposv_not_spd(gpu):
    n = 300
    A = np.eye(n)
    A[100, 100] = -2.0
    B = np.ones((n, 1))
    rc, info, X = solve(gpu, A, B, 128, 3)
    # the mixed factor fails, and so does the FP64 fallback, at the same pivot
    assert rc == GB300_EDOM and info.potrf_info == 101 and info.fallback == 1


def test_solver_context_host_buffers_match_device_call(gpu, oracle):
    n, nrhs, nb = 700, 3, 256
    A = oracle.spd_gram(n, 41, 0.5)
    B = oracle.uniform_rhs(n, nrhs, 42)
    h = gpu.starpu_gb300_solver_create(n, nrhs, nb, 3)
    assert h
    try:
        X = np.zeros((n, nrhs), order="F")
        info = IrInfo()
        rc = gpu.starpu_gb300_solver_dsposv_host(h, n, nrhs, A.ctypes.data, n, B.ctypes.data, n, X.ctypes.data, n,
                                                  1e-12, 30, C.byref(info))
        assert rc == 0
        rc2, info2, X2 = solve(gpu, A, B, nb, 3)
        assert rc2 == 0
        np.testing.assert_array_equal(X, X2)  # same kernels, same order: bit-identical
        assert info.iterations == info2.iterations
    finally:
        gpu.starpu_gb300_solver_destroy(h)


@pytest.mark.parametrize("overlap", [0, 1])
@pytest.mark.parametrize("n,nb", [(900, 256), (777, 256), (2600, 128)])
def test_solver_context_pinned_host_buffers(gpu, oracle, n, nb, overlap):
    """Pinned host input: the context reads A's lower triangle with a gather
    kernel instead of copies, writing the factor phase's FP32 copy and max
    |A_ij| on the way (odd n: columns start off 16-byte boundaries).  With
    the overlap on, the gather runs superblock by superblock beside the
    factorisation, whose updates of the late columns replay the stored
    panels in step order.  Either way the solution is bit-identical to the
    device call."""
    nrhs = 4
    A = np.asfortranarray(oracle.spd_gram(n, 47, 0.5))
    B = np.asfortranarray(oracle.uniform_rhs(n, nrhs, 48))
    hA = gpu.starpu_gb300_host_malloc_pinned(8 * n * n)
    hB = gpu.starpu_gb300_host_malloc_pinned(8 * n * nrhs)
    hX = gpu.starpu_gb300_host_malloc_pinned(8 * n * nrhs)
    h = gpu.starpu_gb300_solver_create(n, nrhs, nb, 3)
    assert hA and hB and hX and h
    gpu.starpu_gb300_solver_host_overlap(h, overlap)
    try:
        C.memmove(hA, A.ctypes.data, 8 * n * n)
        C.memmove(hB, B.ctypes.data, 8 * n * nrhs)
        info = IrInfo()
        for _ in range(2):
            rc = gpu.starpu_gb300_solver_dsposv_host(h, n, nrhs, hA, n, hB, n, hX, n, 1e-12, 30, C.byref(info))
            assert rc == 0
            X = np.ctypeslib.as_array((C.c_double * (n * nrhs)).from_address(hX)).reshape((n, nrhs), order="F").copy()
            rc2, info2, X2 = solve(gpu, A, B, nb, 3)
            np.testing.assert_array_equal(X, X2)
    finally:
        gpu.starpu_gb300_solver_destroy(h)
        for p in (hA, hB, hX):
            gpu.starpu_gb300_host_free_pinned(p)


def test_dposv_plain_fp64(gpu, oracle):
    n, nrhs = 900, 5
    A = oracle.spd_gram(n, 51, 1.0)
    B = oracle.uniform_rhs(n, nrhs, 52)
    dA, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(B)
    info = DeviceBuffer.from_array(np.zeros(1, np.int32))
    check(gpu.starpu_gb300_dposv(None, n, nrhs, dA.ptr, n, dB.ptr, n, 256, info.ptr))
    X = dB.download((n, nrhs), np.float64)
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-14


def test_profiling_counts_kernel_classes(gpu, oracle):
    n, nb, nrhs = 1024, 256, 2
    A = oracle.spd_gram(n, 61, 1.0)
    B = oracle.uniform_rhs(n, nrhs, 62)
    c0 = gpu.starpu_gb300_launch_count()
    gpu.starpu_gb300_profiling_reset()
    gpu.starpu_gb300_profiling_enable(1)
    rc, info, X = solve(gpu, A, B, nb, 3)
    gpu.starpu_gb300_profiling_enable(0)
    assert rc == 0
    assert gpu.starpu_gb300_launch_count() > c0
    launches, ms, fl = C.c_ulonglong(), C.c_double(), C.c_double()
    gpu.starpu_gb300_profiling_get(0, C.byref(launches), C.byref(ms), C.byref(fl), None)
    # per step with rows below the diagonal tile: the next column block, then
    # (when rows remain beyond it) the trailing triangle
    steps = n // nb - 1
    assert launches.value == steps + (steps - 1) and ms.value > 0
    expected = sum(3 * nb * (n - (k + 1) * nb) * (n - (k + 1) * nb + 1.0) for k in range(steps))
    assert abs(fl.value - expected) <= 1e-9 * expected
    share = C.c_double()
    check(gpu.starpu_gb300_profiling_sm_share(0, C.byref(share)))
    assert 0.0 < share.value <= 1.0
    # the per-launch timeline: one span per profiled launch of every class
    total = 0
    for kind in range(6):
        la = C.c_ulonglong()
        gpu.starpu_gb300_profiling_get(kind, C.byref(la), None, None, None)
        total += la.value
    cnt = gpu.starpu_gb300_profiling_timeline(0, None, None, None)
    assert cnt == total
    K, S, E = (C.c_int * cnt)(), (C.c_double * cnt)(), (C.c_double * cnt)()
    assert gpu.starpu_gb300_profiling_timeline(cnt, K, S, E) == cnt
    assert sum(1 for k in K if k == 0) == launches.value
    assert all(e >= s for s, e in zip(S, E)) and min(S) > -0.01 and max(E) > 0


def inv_tile_band(L32, nb):
    """Inverses of the nb x nb diagonal tiles of L, tile T as an ldd x ldd
    column-major block at T * ldd * ldd (zero above the diagonal)."""
    n = L32.shape[0]
    ldd = (nb + 63) // 64 * 64
    ntiles = (n + nb - 1) // nb
    band = np.zeros(ntiles * ldd * ldd, np.float32)
    for T in range(ntiles):
        t0 = T * nb
        kb = min(nb, n - t0)
        blk = np.zeros((ldd, ldd), np.float32, order="F")
        blk[:kb, :kb] = np.tril(np.linalg.inv(L32[t0:t0 + kb, t0:t0 + kb].astype(np.float64)))
        band[T * ldd * ldd:(T + 1) * ldd * ldd] = blk.ravel(order="F")
    return band, ldd


@pytest.mark.parametrize("n,nb,nrhs", [(2048, 1024, 16), (1000, 256, 5), (777, 96, 20), (64, 32, 1), (130, 64, 3)])
def test_spotrs_inv_tiles_matches_fp64_triangular_solves(gpu, oracle, n, nb, nrhs):
    """POTRS by tile-row sweeps with the diagonal-tile inverses supplied:
    agrees with an FP64 solve by the same FP32 factor to FP32 accuracy, and
    repeats bit-identically."""
    A = oracle.spd_gram(n, 71, 1.0)
    L32 = np.asfortranarray(np.tril(np.linalg.cholesky(A)).astype(np.float32))
    band, ldd = inv_tile_band(L32, nb)
    B = oracle.uniform_rhs(n, nrhs, 72).astype(np.float32)
    dL, dD = DeviceBuffer.from_array(L32), DeviceBuffer.from_array(band)
    lw = gpu.starpu_gb300_spotrs_inv_tiles_workspace(n, nb)
    W, err = DeviceBuffer(lw), DeviceBuffer.from_array(np.zeros(1, np.int32))
    outs = []
    for _ in range(2):
        dB = DeviceBuffer.from_array(B)
        check(gpu.starpu_gb300_spotrs_inv_tiles(None, n, nrhs, nb, dL.ptr, n, dD.ptr, ldd, dB.ptr, n, W.ptr, lw,
                                                 err.ptr))
        outs.append(dB.download((n, nrhs), np.float32))
    assert err.download((1,), np.int32)[0] == 0
    np.testing.assert_array_equal(outs[0], outs[1])
    L64 = L32.astype(np.float64)
    ref = np.linalg.solve(L64.T, np.linalg.solve(L64, B.astype(np.float64)))
    assert np.max(np.abs(outs[0] - ref)) / np.max(np.abs(ref)) < 2e-5


def test_spotrs_inv_tiles_rejects_bad_tiles(gpu):
    assert gpu.starpu_gb300_spotrs_inv_tiles_workspace(100, 48) == 0  # nb not a multiple of 32
    assert gpu.starpu_gb300_spotrs_inv_tiles(None, 100, 1, 48, None, 100, None, 64, None, 100, None, 0, None) == -22
    assert gpu.starpu_gb300_spotrs_inv_tiles(None, 100, 1, 2048, None, 100, None, 2048, None, 100, None, 0, None) == -22


def exact_residual(A, X, B):
    """B - A X to ~1 ulp: every product split exactly into 26-bit halves
    (Veltkamp), all terms of a row summed with math.fsum."""
    import math

    def split(v):
        c = v * 134217729.0  # 2^27 + 1
        hi = c - (c - v)
        return hi, v - hi
    Ah, Al = split(np.asarray(A, np.float64))
    R = np.empty_like(B)
    for j in range(X.shape[1]):
        xh, xl = split(X[:, j])
        for i in range(A.shape[0]):
            terms = np.concatenate([Ah[i] * xh, Ah[i] * xl, Al[i] * xh, Al[i] * xl])
            R[i, j] = math.fsum(np.concatenate([[B[i, j]], -terms]))
    return R


def dsyresidual(gpu, A, X, B):
    n, nrhs = X.shape
    dA, dX, dB = DeviceBuffer.from_array(A), DeviceBuffer.from_array(X), DeviceBuffer.from_array(B)
    dR = DeviceBuffer(8 * n * nrhs)
    lw = gpu.starpu_gb300_dsyresidual_workspace(n, nrhs)
    W, err = DeviceBuffer(lw), DeviceBuffer.from_array(np.zeros(1, np.int32))
    check(gpu.starpu_gb300_dsyresidual(None, n, nrhs, dA.ptr, n, dX.ptr, n, dB.ptr, n, dR.ptr, n, W.ptr, lw, err.ptr))
    R = dR.download((n, nrhs), np.float64)
    assert err.download((1,), np.int32)[0] == 0
    return R


@pytest.mark.parametrize("n,nrhs", [(128, 1), (500, 5), (777, 20)])
def test_dsyresidual_tensor_core_slices_are_fp64_accurate(gpu, oracle, n, nrhs):
    """The refinement residual from exact products of 7-bit slices on the
    tensor cores: within 2^-45 of ||A||_inf ||x_j||_inf of the exact residual
    (columns of very different scale, a zero column, negative entries),
    bit-identical on repeat, and the strict upper triangle is never read."""
    rng = np.random.default_rng(n + nrhs)
    A = oracle.spd_gram(n, n, 0.3)
    A[:, :] = A - 0.2 * np.mean(A)  # negative entries too (the residual needs no definiteness)
    A = np.asfortranarray(np.tril(A) + np.tril(A, -1).T)
    X = np.asfortranarray(rng.standard_normal((n, nrhs)) * np.exp(rng.uniform(-30, 30, nrhs)))
    X[:, nrhs // 2] = 0.0
    B = np.asfortranarray(A @ X + 1e-9 * rng.standard_normal((n, nrhs)) * np.abs(X).max(0))
    R = dsyresidual(gpu, A, X, B)
    Rx = exact_residual(A, X, B)
    anorm = np.abs(A).sum(1).max()
    for j in range(nrhs):
        scale = anorm * np.abs(X[:, j]).max()
        if scale == 0:
            np.testing.assert_array_equal(R[:, j], B[:, j])
        else:
            assert np.max(np.abs(R[:, j] - Rx[:, j])) <= 2.0 ** -45 * scale, j
    np.testing.assert_array_equal(dsyresidual(gpu, A, X, B), R)
    An = np.array(A, order="F")
    An[np.triu_indices(n, 1)] = np.nan
    np.testing.assert_array_equal(dsyresidual(gpu, An, X, B), R)
