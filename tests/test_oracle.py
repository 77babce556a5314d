"""CPU tests of the oracle: pinned against the reference's CLAPACK golden
vectors and against the reference driver's own -check criterion."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "chol_golden.npz")


def _cases():
    z = np.load(GOLD)
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    return [(k, z) for k in keys]


@pytest.mark.parametrize("key", [k for k, _ in _cases()])
def test_generator_matches_golden(oracle, key):
    z = np.load(GOLD)
    n, seed, alpha, _ = z[key + "_meta"]
    A = oracle.spd_gram(int(n), int(seed), float(alpha))
    # libm log/cos/sin may differ in the last ulp across machines
    np.testing.assert_allclose(A, z[key + "_A"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("key", [k for k, _ in _cases()])
@pytest.mark.parametrize("nblocks", [1, 3, 4])
def test_tiled_factor_matches_reference_clapack(oracle, key, nblocks):
    z = np.load(GOLD)
    A, Lref = z[key + "_A"], z[key + "_L"]
    n = A.shape[0]
    nb = min(nblocks, n)
    L, info = oracle.potrf_tiled(A, nb)
    assert info == 0
    L = np.tril(L)
    assert np.max(np.abs(L - Lref)) <= 1e-12 * max(1.0, np.max(np.abs(Lref)))
    assert oracle.llt_residual(A, L) <= 1e-14


@pytest.mark.parametrize("key", [k for k, _ in _cases()])
def test_potrs_matches_reference_clapack(oracle, key):
    z = np.load(GOLD)
    A, L, B, Xref = z[key + "_A"], z[key + "_L"], z[key + "_B"], z[key + "_X"]
    X = oracle.potrs(L, B)
    scale = np.max(np.abs(Xref))
    assert np.max(np.abs(X - Xref)) <= 1e-10 * scale
    be, _ = oracle.backward_error(A, X, B)
    assert be <= 1e-14


def test_reference_clapack_agrees_when_built(oracle):
    """Re-run the reference CLAPACK here (only where the reference tree was built)."""
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built on this machine")
    z = np.load(GOLD)
    A = z["n100_s15_A"]
    L, info = oracle.ref_dpotrf(A)
    assert info == 0
    np.testing.assert_allclose(np.tril(L), z["n100_s15_L"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("n,nblocks", [(256, 8), (300, 7), (2048, 8)])
def test_hilbert_passes_reference_check(oracle, n, nblocks):
    """Config 1 input and the reference's own acceptance test (relative error
    of L L^T vs the known input <= 1e-4, cholesky_implicit.c:574-580)."""
    if n >= 2048 and os.environ.get("GB300_QUICK"):
        pytest.skip("quick mode")
    A = oracle.hilbert_f32(n)
    L, info = oracle.potrf_tiled(A, nblocks)
    assert info == 0
    bad, worst = oracle.check_hilbert(L, 1e-4)
    assert bad == 0, worst


def test_chunking_matches_starpu_filters(oracle):
    # starpu_filter_nparts_compute_chunk_size_and_offset: remainder to the first chunks
    for n, p in [(10, 3), (2048, 8), (17, 17), (100, 7)]:
        sizes = [oracle.chunk(n, p, i) for i in range(p)]
        assert sum(s for s, _ in sizes) == n
        off = 0
        for i, (s, o) in enumerate(sizes):
            assert o == off
            assert s == n // p + (1 if i < n % p else 0)
            off += s


def test_not_spd_reports_info(oracle):
    A = np.eye(8)
    A[5, 5] = -1.0
    L, info = oracle.potrf_tiled(A, 2)
    assert info == 6


def test_ir_restatement_converges(oracle):
    n = 96
    A = oracle.spd_gram(n, 3, oracle.alpha_for_kappa(1e4))
    B = oracle.uniform_rhs(n, 3, 4)
    X, it, be = oracle.dsposv_ir(A, B, 4, tol=1e-12)
    assert it >= 0 and be <= 1e-12


def test_cpu_baseline_port_matches_oracle(oracle):
    if not oracle.cpu_init():
        pytest.skip("scipy OpenBLAS not found")
    A = oracle.hilbert_f32(512)
    L_or, _ = oracle.potrf_tiled(A, 4)
    A2 = np.array(A, order="F")
    assert oracle.cpu_potrf_tiled(A2, 4, 4) == 0
    assert np.max(np.abs(np.tril(A2) - np.tril(L_or))) <= 1e-4
    G = oracle.spd_gram(256, 5, 1.0)
    G2 = np.array(G, order="F")
    assert oracle.cpu_potrf_tiled(G2, 4, 3) == 0
    assert oracle.llt_residual(G, np.tril(G2)) <= 1e-14
