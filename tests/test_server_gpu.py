"""Serving loop: mixed sizes and right-hand-side counts submitted together
(continuous batching, executors overlapping on the device), repeat
right-hand sides on cached device factors, an HBM budget, and every result
identical whether the request ran alone or in the mix."""
import ctypes as C

import numpy as np
import pytest

from starpu_gb300.native import Request

pytestmark = pytest.mark.gpu
GB = 1 << 30


def make(oracle, n, seed, kappa):
    Bn = oracle.normal_matrix(n, n, seed)
    A = np.asfortranarray(Bn @ Bn.T / n)
    A[np.diag_indices(n)] += oracle.alpha_for_kappa(kappa)
    return A


def request(A, B, matrix_id=0):
    n, nrhs = B.shape
    X = np.zeros((n, nrhs), order="F")
    r = Request()
    r.n, r.nrhs = n, nrhs
    r.A = A.ctypes.data if A is not None else None
    r.B = B.ctypes.data
    r.X = X.ctypes.data
    r.matrix_id = matrix_id
    r.tol = 1e-12
    r.max_iter = 40
    return r, X


@pytest.fixture(scope="module")
def problems(oracle):
    rng = np.random.default_rng(11)
    out = []
    for i, n in enumerate([64, 100, 300, 700, 1024, 1500, 2048, 1200]):
        kappa = float(np.exp(rng.uniform(np.log(1e2), np.log(1e5))))
        A = make(oracle, n, 40 + i, kappa)
        nrhs = int(rng.integers(1, 17))
        out.append((A, oracle.uniform_rhs(n, nrhs, 90 + i), i + 1))
    return out


def serve(gpu, reqs, executors=3, budget=24 * GB, mode=0):
    sv = gpu.starpu_gb300_server_create(budget, executors, 2048, 16, mode)
    assert sv, gpu.starpu_gb300_last_error()
    try:
        for r in reqs:
            assert gpu.starpu_gb300_server_submit(sv, C.byref(r)) == 0
        gpu.starpu_gb300_server_drain(sv)
        st = [C.c_ulonglong() for _ in range(4)]
        gpu.starpu_gb300_server_stats(sv, *[C.byref(x) for x in st], None)
        return [x.value for x in st]
    finally:
        gpu.starpu_gb300_server_destroy(sv)


def test_mixed_requests_all_reach_fp64_accuracy_and_match_alone(gpu, oracle, problems):
    mix = [request(A, B, mid) for A, B, mid in problems]
    served, batches, hits, _ = serve(gpu, [r for r, _ in mix])
    assert served == len(problems) and batches >= 1
    for (A, B, _), (r, X) in zip(problems, mix):
        assert r.done == 1 and r.status == 0, (A.shape, r.status)
        be, _ = oracle.backward_error(A, X, B)
        assert be <= 1e-12, (A.shape, be)
        assert r.batched == (1 if (A.shape[0] <= 1024 and B.shape[1] <= 8) else 0)
    # every request alone on a fresh server gives bit-identical results
    for k in (0, 3, 5, 6):
        A, B, mid = problems[k]
        r, X = request(A, B, mid)
        serve(gpu, [r], executors=1)
        np.testing.assert_array_equal(X, mix[k][1])


def test_repeat_rhs_reuses_the_device_factor(gpu, oracle, problems):
    A, B, _ = problems[6]  # n = 2048, large path
    B2 = oracle.uniform_rhs(A.shape[0], 5, 1234)
    r1, X1 = request(A, B, 777)
    r2, X2 = request(None, B2, 777)  # matrix not resent: the cached factor is used
    sv = gpu.starpu_gb300_server_create(24 * GB, 2, 2048, 16, 0)
    assert sv, gpu.starpu_gb300_last_error()
    try:
        assert gpu.starpu_gb300_server_submit(sv, C.byref(r1)) == 0
        assert gpu.starpu_gb300_server_wait(sv, C.byref(r1)) == 0
        assert gpu.starpu_gb300_server_submit(sv, C.byref(r2)) == 0
        assert gpu.starpu_gb300_server_wait(sv, C.byref(r2)) == 0
    finally:
        gpu.starpu_gb300_server_destroy(sv)
    assert r1.cache_hit == 0 and r2.cache_hit == 1
    be, _ = oracle.backward_error(A, X2, B2)
    assert be <= 1e-12
    # same result as solving the second right-hand side from scratch
    r3, X3 = request(A, B2, 0)
    serve(gpu, [r3], executors=1)
    np.testing.assert_array_equal(X2, X3)


def test_budget_too_small_for_the_cache_still_serves(gpu, oracle, problems):
    A, B, _ = problems[5]
    # the executor buffers alone, then a budget 1 MiB above them: no factor fits
    probe = gpu.starpu_gb300_server_create(64 * GB, 1, 2048, 16, 0)
    used = C.c_size_t()
    gpu.starpu_gb300_server_stats(probe, None, None, None, None, C.byref(used))
    gpu.starpu_gb300_server_destroy(probe)
    assert not gpu.starpu_gb300_server_create(used.value - 1, 1, 2048, 16, 0)  # below the executors' needs
    sv = gpu.starpu_gb300_server_create(used.value + (1 << 20), 1, 2048, 16, 0)
    assert sv
    try:
        reqs = [request(A, B, 55) for _ in range(3)]
        for r, _ in reqs:
            gpu.starpu_gb300_server_submit(sv, C.byref(r))
        gpu.starpu_gb300_server_drain(sv)
        for r, X in reqs:
            assert r.status == 0 and r.cache_hit == 0
            np.testing.assert_array_equal(X, reqs[0][1])
    finally:
        gpu.starpu_gb300_server_destroy(sv)


def test_plain_mode_baseline(gpu, oracle, problems):
    sub = [problems[1], problems[5]]
    reqs = [request(A, B) for A, B, _ in sub]
    serve(gpu, [r for r, _ in reqs], executors=1, mode=1)
    for (A, B, _), (r, X) in zip(sub, reqs):
        assert r.status == 0
        be, _ = oracle.backward_error(A, X, B)
        assert be <= 1e-14


def test_invalid_requests_are_rejected(gpu):
    sv = gpu.starpu_gb300_server_create(8 * GB, 1, 512, 4, 0)
    try:
        X = np.zeros((600, 1))
        r, _ = request(np.eye(600), X)
        assert gpu.starpu_gb300_server_submit(sv, C.byref(r)) == -22  # n > max_n
    finally:
        gpu.starpu_gb300_server_destroy(sv)
