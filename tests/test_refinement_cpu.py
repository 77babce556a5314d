"""CPU checks of the mixed solve's refinement policy (starpu_gb300_dsposv):
the two facts its automatic rung choice rests on, restated in NumPy.

* The ratio of the largest to the smallest Cholesky pivot, max L_ii^2 /
  min L_ii^2, never exceeds kappa_2(A) (every pivot lies between the extreme
  eigenvalues), so a large ratio proves an ill-conditioned system; on the
  Gram test matrices it is about 0.6 sqrt(kappa).
* With a preconditioner as inexact as the tensor-core factor (relative
  factor error ~1e-6), flexible preconditioned conjugate gradients (Polak-
  Ribiere beta, recurrence residual checked against a true one) reach the
  1e-12 backward error in fewer corrections than classic refinement once
  kappa * error approaches 1, and in as few on a well-conditioned system.
"""
import numpy as np
import pytest
import scipy.linalg as sla

from oracle import oracle as O


def _backward_error(A, x, b):
    r = b - A @ x
    return np.max(np.abs(r)) / (np.max(np.sum(np.abs(A), axis=1)) * np.max(np.abs(x)) + np.max(np.abs(b)))


def _inexact_factor(A, eps, seed):
    """FP32 Cholesky factor of A + E with a random symmetric E of relative
    size eps (the tensor-core factor's backward error), as a solve."""
    n = A.shape[0]
    rng = np.random.default_rng(seed)
    E = rng.standard_normal((n, n))
    E = (E + E.T) / 2.0
    E *= eps * np.linalg.norm(A) / np.linalg.norm(E)
    L = np.linalg.cholesky(A + E).astype(np.float32)

    def solve(r):
        scale = np.max(np.abs(r)) or 1.0  # the device scales each FP32 solve by a power of two
        y = sla.solve_triangular(L, (r / scale).astype(np.float32), lower=True)
        return sla.solve_triangular(L.T, y, lower=False).astype(np.float64) * scale
    return solve


def _classic(A, b, M, tol=1e-12, max_iter=60):
    x = M(b)
    for it in range(max_iter + 1):
        if _backward_error(A, x, b) <= tol:
            return x, it
        x = x + M(b - A @ x)
    return x, None


def _flexible_pcg(A, b, M, tol=1e-12, max_iter=60):
    x = M(b)
    r = b - A @ x
    it, restart = 0, True
    while it <= max_iter:
        if _backward_error(A, x, b) <= tol:
            return x, it
        z = M(r)
        it += 1
        rz = r @ z
        if restart:
            p = z.copy()
        else:
            p = z + ((rz - r @ zp) / rho) * p
        zp, rho, restart = z, rz, False
        q = A @ p
        alpha = rz / (p @ q)
        x = x + alpha * p
        r = r - alpha * q
        if np.max(np.abs(r)) / (np.max(np.sum(np.abs(A), axis=1)) * np.max(np.abs(x)) + np.max(np.abs(b))) <= tol:
            r = b - A @ x  # accepted only once a true residual agrees
            restart = True
    return x, None


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6])
def test_pivot_ratio_bounds_kappa(kappa):
    n = 384
    A = O.spd_gram(n, 7, O.alpha_for_kappa(kappa))
    piv = np.diag(np.linalg.cholesky(A)) ** 2
    ev = np.linalg.eigvalsh(A)
    ratio, k2 = piv.max() / piv.min(), ev[-1] / ev[0]
    assert ratio <= k2 * (1 + 1e-10)
    # the device's switch point (300) is only passed for kappa well above 1e4
    assert (ratio > 300) == (kappa >= 1e6)


def test_conjugate_gradients_need_fewer_corrections_when_ill_conditioned():
    """A random perturbation is milder than the tensor-core factor's error
    (whose components along the small eigenvectors set the contraction), so
    at this small order the factor error is taken a few times larger (5e-6)
    for classic refinement to need several corrections at kappa = 1e6."""
    n = 512
    b = O.uniform_rhs(n, 1, 3)[:, 0]
    results = {}
    for kappa in (1e2, 1e6):
        A = O.spd_gram(n, 5, O.alpha_for_kappa(kappa))
        M = _inexact_factor(A, 5e-6, 11)
        x_ir, it_ir = _classic(A, b, M)
        x_cg, it_cg = _flexible_pcg(A, b, M)
        assert it_ir is not None and it_cg is not None, (kappa, it_ir, it_cg)
        assert _backward_error(A, x_cg, b) <= 1e-12
        results[kappa] = (it_ir, it_cg)
    assert results[1e2][1] <= results[1e2][0] + 1  # as few on an easy system (one more residual at most)
    assert results[1e6][1] < results[1e6][0], results
