"""GPU parity of the LU tile kernels (examples/lu codelet bodies) through the
C-ABI: against the golden outputs of the reference's own CPU codelets
(tests/golden/lu_golden.npz) and against the oracle (oracle/lu_oracle.c) at
the driver's tile sizes; pivoting follows the reference CUDA branch's choice
(the largest entry of the pivot row)."""
import os

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lu_golden.npz")
TOL = {"s": 5e-5, "d": 1e-12}
DT = {"s": np.float32, "d": np.float64}


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def up(a):
    return DeviceBuffer.from_array(np.asfortranarray(a))


def down(buf, like):
    return buf.download(like.shape, like.dtype)


def rel(a, b):
    return np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))


def status():
    return DeviceBuffer.from_array(np.zeros(1, np.int32))


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_tile_matches_reference(gpu, gold, p):
    A = gold[f"{p}_getrf_in"]
    n = A.shape[0]
    d, info = up(A), status()
    check(getattr(gpu, f"starpu_gb300_{p}getrf_tile")(None, n, d.ptr, n, info.ptr))
    assert info.download((1,), np.int32)[0] == 0
    assert rel(down(d, A), gold[f"{p}_getrf_out"]) <= TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
@pytest.mark.parametrize("n", [960, 333])
def test_getrf_tile_driver_sizes_vs_oracle(gpu, oracle, p, n):
    rng = np.random.default_rng(n)
    A = np.asfortranarray(rng.random((n, n)) + n * np.eye(n)).astype(DT[p])
    d, info = up(A), status()
    check(getattr(gpu, f"starpu_gb300_{p}getrf_tile")(None, n, d.ptr, n, info.ptr))
    out = down(d, A)
    ref = A.copy(order="F")
    assert oracle.lu_getrf(ref)[0] == 0
    assert info.download((1,), np.int32)[0] == 0
    assert rel(out, ref) <= TOL[p]
    L = np.tril(out).astype(np.float64)
    U = (np.triu(out, 1) + np.eye(n)).astype(np.float64)
    assert np.max(np.abs(L @ U - A)) / np.max(np.abs(A)) <= (1e-5 if p == "s" else 1e-13)


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_zero_pivot_reports_info_without_fault(gpu, p):
    n = 200
    A = np.eye(n, dtype=DT[p]) * 4
    A[70, 70] = 0
    d, info = up(A), status()
    check(getattr(gpu, f"starpu_gb300_{p}getrf_tile")(None, n, d.ptr, n, info.ptr))
    assert info.download((1,), np.int32)[0] == 71


@pytest.mark.parametrize("p", ["s", "d"])
def test_triangular_solves_and_gemm_match_reference(gpu, gold, p):
    L = gold[f"{p}_trsm_ll_l"]
    n = L.shape[0]
    dl = up(L)
    b = up(gold[f"{p}_trsm_ll_in"])
    check(getattr(gpu, f"starpu_gb300_{p}trsm_llnn_tile")(None, n, n, dl.ptr, n, b.ptr, n))
    assert rel(down(b, L), gold[f"{p}_trsm_ll_out"]) <= TOL[p]
    b2 = up(gold[f"{p}_trsm_ru_in"])
    check(getattr(gpu, f"starpu_gb300_{p}trsm_runu_tile")(None, n, n, dl.ptr, n, b2.ptr, n))
    assert rel(down(b2, L), gold[f"{p}_trsm_ru_out"]) <= TOL[p]
    a, bb, c = up(gold[f"{p}_gemm_a"]), up(gold[f"{p}_gemm_b"]), up(gold[f"{p}_gemm_in"])
    check(getattr(gpu, f"starpu_gb300_{p}gemm_nn_tile")(None, n, n, n, DT[p](-1), a.ptr, n, bb.ptr, n, DT[p](1), c.ptr, n))
    assert rel(down(c, L), gold[f"{p}_gemm_out"]) <= 10 * TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
@pytest.mark.parametrize("m,n", [(960, 960), (500, 300), (64, 1)])
def test_triangular_solves_ragged_vs_oracle(gpu, oracle, p, m, n):
    rng = np.random.default_rng(m + n)
    dt = DT[p]
    T = np.asfortranarray(rng.random((max(m, n), max(m, n))) + max(m, n) * np.eye(max(m, n))).astype(dt)
    oracle.lu_getrf(T)
    Lm = np.asfortranarray(T[:m, :m])
    Un = np.asfortranarray(T[:n, :n])
    B = np.asfortranarray(rng.standard_normal((m, n))).astype(dt)
    r1, r2 = B.copy(order="F"), B.copy(order="F")
    oracle.lu_trsm_ll(Lm, r1)
    oracle.lu_trsm_ru(Un, r2)
    b1, b2 = up(B), up(B)
    dl, du = up(Lm), up(Un)  # held until the kernels have run: a dropped buffer is freed at once
    check(getattr(gpu, f"starpu_gb300_{p}trsm_llnn_tile")(None, m, n, dl.ptr, m, b1.ptr, m))
    check(getattr(gpu, f"starpu_gb300_{p}trsm_runu_tile")(None, m, n, du.ptr, n, b2.ptr, m))
    assert rel(down(b1, B), r1) <= 10 * TOL[p]
    assert rel(down(b2, B), r2) <= 10 * TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_pivot_tile_pivots_like_the_cuda_branch(gpu, oracle, gold, p):
    A = gold[f"{p}_getrf_pivot_in"]
    n = A.shape[0]
    ref = A.copy(order="F")
    _, ipiv_ref = oracle.lu_getrf(ref, 1e-4)
    lw = getattr(gpu, f"starpu_gb300_{p}getrf_pivot_tile_workspace")(n)
    W, ip, info = DeviceBuffer(lw), DeviceBuffer(4 * n), status()
    d = up(A)
    check(getattr(gpu, f"starpu_gb300_{p}getrf_pivot_tile")(None, n, d.ptr, n, DT[p](1e-4), ip.ptr, W.ptr, lw,
                                                            info.ptr))
    np.testing.assert_array_equal(ip.download((n,), np.int32), ipiv_ref)
    assert (ipiv_ref >= 0).any()
    assert rel(down(d, A), ref) <= 50 * TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_pivot_tile_without_small_pivots_is_the_blocked_factor(gpu, gold, p):
    A = gold[f"{p}_getrf_in"]
    n = A.shape[0]
    lw = getattr(gpu, f"starpu_gb300_{p}getrf_pivot_tile_workspace")(n)
    W, ip, info = DeviceBuffer(lw), DeviceBuffer(4 * n), status()
    d1, d2 = up(A), up(A)
    check(getattr(gpu, f"starpu_gb300_{p}getrf_pivot_tile")(None, n, d1.ptr, n, DT[p](1e-4), ip.ptr, W.ptr, lw,
                                                            info.ptr))
    check(getattr(gpu, f"starpu_gb300_{p}getrf_tile")(None, n, d2.ptr, n, None))
    assert (ip.download((n,), np.int32) == -1).all()
    np.testing.assert_array_equal(down(d1, A), down(d2, A))


@pytest.mark.parametrize("p", ["s", "d"])
def test_swap_columns_matches_reference_pivot_codelet(gpu, gold, p):
    T = gold[f"{p}_pivot_in"]
    n = T.shape[0]
    ipiv = gold[f"{p}_getrf_pivot_ipiv"]
    pairs = np.array([[r, ipiv[r]] for r in range(n) if ipiv[r] != r], dtype=np.int32).ravel()
    d = up(T)
    check(getattr(gpu, f"starpu_gb300_{p}swap_columns_tile")(None, n, n, d.ptr, n, pairs.ctypes.data, len(pairs) // 2))
    np.testing.assert_array_equal(down(d, T), gold[f"{p}_pivot_out"])
    bad = np.array([0, n], dtype=np.int32)
    assert getattr(gpu, f"starpu_gb300_{p}swap_columns_tile")(None, n, n, d.ptr, n, bad.ctypes.data, 1) == -22
