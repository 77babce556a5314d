"""CPU tests of the LU oracle (oracle/lu_oracle.c) against the golden vectors
the reference's own LU codelets produced (tests/golden/make_lu_golden.py):
same factor form, same pivot choices, same column swaps."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lu_golden.npz")
TOL = {"s": 2e-5, "d": 1e-13}


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def rel(a, b):
    return np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_matches_reference(oracle, gold, p):
    A = np.array(gold[f"{p}_getrf_in"], order="F")
    info, ipiv = oracle.lu_getrf(A)
    assert info == 0 and (ipiv == -1).all()
    assert rel(A, gold[f"{p}_getrf_out"]) <= TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_pivot_matches_reference(oracle, gold, p):
    A = np.array(gold[f"{p}_getrf_pivot_in"], order="F")
    # the golden vectors come from the reference's CPU branch linked with a
    # Fortran-interface BLAS, whose 1-based ISAMAX it reads as 0-based
    info, ipiv = oracle.lu_getrf(A, 1e-4, iamax_shift=1)
    n = A.shape[0]
    # the reference writes ipiv[z] only when step z pivots (identity otherwise)
    ref = gold[f"{p}_getrf_pivot_ipiv"]
    np.testing.assert_array_equal(np.where(ipiv < 0, np.arange(n), ipiv), ref)
    assert (ipiv >= 0).any(), "the case must exercise pivoting"
    assert rel(A, gold[f"{p}_getrf_pivot_out"]) <= 50 * TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
def test_getrf_pivot_intended_choice_is_the_row_maximum(oracle, gold, p):
    """The CUDA branch's choice (1-based index corrected): the swapped-in
    column holds the largest magnitude of the pivot row."""
    A0 = np.array(gold[f"{p}_getrf_pivot_in"], order="F")
    A = A0.copy(order="F")
    info, ipiv = oracle.lu_getrf(A, 1e-4)
    assert ipiv[0] == int(np.argmax(np.abs(A0[0, :])))


@pytest.mark.parametrize("p", ["s", "d"])
def test_triangular_solves_and_gemm_match_reference(oracle, gold, p):
    L = np.array(gold[f"{p}_trsm_ll_l"], order="F")
    B = np.array(gold[f"{p}_trsm_ll_in"], order="F")
    oracle.lu_trsm_ll(L, B)
    assert rel(B, gold[f"{p}_trsm_ll_out"]) <= TOL[p]
    B2 = np.array(gold[f"{p}_trsm_ru_in"], order="F")
    oracle.lu_trsm_ru(L, B2)
    assert rel(B2, gold[f"{p}_trsm_ru_out"]) <= TOL[p]
    Cm = np.array(gold[f"{p}_gemm_in"], order="F")
    oracle.lu_gemm(gold[f"{p}_gemm_a"], gold[f"{p}_gemm_b"], Cm)
    assert rel(Cm, gold[f"{p}_gemm_out"]) <= 10 * TOL[p]


@pytest.mark.parametrize("p", ["s", "d"])
def test_pivot_swaps_match_reference(oracle, gold, p):
    T = np.array(gold[f"{p}_pivot_in"], order="F")
    oracle.lu_pivot(T, gold[f"{p}_getrf_pivot_ipiv"])
    np.testing.assert_array_equal(T, gold[f"{p}_pivot_out"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_lu_factor_reconstructs_input(oracle, dtype):
    rng = np.random.default_rng(3)
    n = 80
    A0 = np.asfortranarray(rng.random((n, n)) + n * np.eye(n)).astype(dtype)
    A = A0.copy(order="F")
    info, _ = oracle.lu_getrf(A)
    L = np.tril(A)
    U = np.triu(A, 1) + np.eye(n, dtype=dtype)
    assert info == 0
    assert np.max(np.abs(L @ U - A0)) / np.max(np.abs(A0)) <= (1e-5 if dtype == np.float32 else 1e-13)


def small_pivot_matrix(n, dtype, seed):
    """The GPU LU driver's -small-pivots input: a_ij uniform [0, 1), a_ii + n
    scaling of the diagonal, and row i zeroed up to its diagonal for
    i mod 97 = 5, so that step i's eliminated pivot is exactly zero."""
    rng = np.random.default_rng(seed)
    n_ = np.arange(n)
    A = rng.random((n, n))
    A[n_, n_] = (A[n_, n_] + 1.0) * n
    for i in range(5, n, 97):
        A[i, :i + 1] = 0.0
    return np.asfortranarray(A.astype(dtype))


def tiled_pivot_lu(oracle, A, nb, thr):
    """The tile DAG of the pivoting LU (examples/lu/xlu_implicit_pivot.c:
    165-210) in one topological order, on the oracle's codelets: GETRF_PIVOT
    of the diagonal tile, PIVOT of the other tiles of its block column, the
    two TRSMs, the GEMM updates.  Returns the global pivot record (ipiv[z] =
    z when step z did not swap)."""
    n = A.shape[0]
    nbk = n // nb
    T = lambda i, j: np.asfortranarray(A[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb])
    ipiv = np.arange(n)
    for k in range(nbk):
        Akk0 = T(k, k)
        info, loc = oracle.lu_getrf(Akk0, thr)
        assert info == 0
        A[k * nb:(k + 1) * nb, k * nb:(k + 1) * nb] = Akk0
        rec = np.where(loc < 0, np.arange(nb), loc)
        ipiv[k * nb:(k + 1) * nb] = rec + k * nb
        for i in range(nbk):
            if i != k:
                t = T(i, k)
                oracle.lu_pivot(t, rec)
                A[i * nb:(i + 1) * nb, k * nb:(k + 1) * nb] = t
        for i in range(k + 1, nbk):
            t = T(k, i)
            oracle.lu_trsm_ll(Akk0, t)
            A[k * nb:(k + 1) * nb, i * nb:(i + 1) * nb] = t
            t = T(i, k)
            oracle.lu_trsm_ru(Akk0, t)
            A[i * nb:(i + 1) * nb, k * nb:(k + 1) * nb] = t
        for i in range(k + 1, nbk):
            for j in range(k + 1, nbk):
                c = T(i, j)
                oracle.lu_gemm(T(i, k), T(k, j), c)
                A[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = c
    return ipiv


@pytest.mark.parametrize("dtype,thr", [(np.float32, 10e-5), (np.float64, 10e-10)])
def test_tiled_pivoting_lu_on_the_small_pivot_input(oracle, dtype, thr):
    """The algorithm the GPU LU driver runs with -piv -small-pivots: the zero
    pivots force column swaps, and A P = L U holds to the reference's bound
    ||A P - L U|| / (||A|| n) <= 1e-4 with P the recorded swaps in order."""
    n, nb = 1024, 256
    A0 = small_pivot_matrix(n, dtype, 3)
    A = A0.copy(order="F")
    ipiv = tiled_pivot_lu(oracle, A, nb, thr)
    assert (ipiv != np.arange(n)).sum() > 0
    perm = np.arange(n)
    for k in range(n):
        if ipiv[k] != k:
            perm[[k, ipiv[k]]] = perm[[ipiv[k], k]]
    L = np.tril(A).astype(np.float64)
    U = (np.triu(A, 1) + np.eye(n)).astype(np.float64)
    err = np.max(np.abs(A0.astype(np.float64)[:, perm] - L @ U)) / (np.max(np.abs(A0)) * n)
    assert err <= 1e-4, err
