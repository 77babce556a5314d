"""ORACLE -- test infrastructure only (tests/, smoke(), bench.py cpu_baseline).

ctypes binding of ``oracle/lib/liboracle.so`` (the C restatement of the
reference's tiled Cholesky plus the StarPU-CPU-path port) and, where it was
built from the reference tree, of ``oracle/_ref/libref_lapack.so`` (CLAPACK
dpotrf/dpotrs from min-dgels).  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libref_lapack.so")


def _reference_tree() -> str:
    """The reference checkout the build recipes compile from:
    STARPU_REFERENCE_TREE, else the REF_DEFAULT location of oracle/Makefile (the
    one recipe that names it).  An absent tree only skips the reference pins."""
    env = os.environ.get("STARPU_REFERENCE_TREE")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF_DEFAULT :="):
                return line.split("=", 1)[1].strip()
    return ""


REF_TREE = _reference_tree()

_o = None
_r = None
_blas_ready = False

vp, ci, cd, cu64 = C.c_void_p, C.c_int, C.c_double, C.c_uint64


# the reference driver sources staged for machines without the tree (git-ignored)
STAGED_TREE = os.path.join(HERE, "_ref", "src")


def build(with_ref: bool = True) -> None:
    """Compile the restatement; also the reference CLAPACK when the tree is
    present, and stage the unchanged drivers' sources for the GPU machine."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref and os.path.isdir(os.path.join(REF_TREE, "min-dgels")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "ref-stage", f"REF={REF_TREE}"], check=True)


def driver_tree() -> str | None:
    """Where the unchanged reference drivers compile from: the reference tree,
    else the staged copy of their sources, else None."""
    for t in (REF_TREE, STAGED_TREE):
        if t and os.path.isfile(os.path.join(t, "examples", "cholesky", "cholesky_implicit.c")):
            return t
    return None


def lib() -> C.CDLL:
    global _o
    if _o is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
                os.path.getmtime(os.path.join(HERE, f)) for f in ("chol_oracle.c", "cpu_chol.c", "lu_oracle.c")):
            build(with_ref=False)
        o = C.CDLL(LIB)
        o.oracle_hilbert_f32.argtypes = [ci, vp, ci]
        o.oracle_normal_matrix.argtypes = [ci, ci, cu64, vp, ci]
        o.oracle_normal_rows.argtypes = [ci, ci, ci, cu64, vp, ci]
        o.oracle_uniform_rhs.argtypes = [ci, ci, cu64, vp, ci]
        o.oracle_spd_gram.argtypes = [ci, cu64, cd, vp, ci]
        o.oracle_chunk.argtypes = [ci, ci, ci, vp, vp]
        o.oracle_potrf_tiled_f32.argtypes = [ci, vp, ci, ci]
        o.oracle_potrf_tiled_f64.argtypes = [ci, vp, ci, ci]
        o.oracle_potrs_f32.argtypes = [ci, ci, vp, ci, vp, ci]
        o.oracle_potrs_f64.argtypes = [ci, ci, vp, ci, vp, ci]
        o.oracle_check_hilbert_f32.argtypes = [ci, vp, ci, C.c_float, vp]
        o.oracle_llt_residual.argtypes = [ci, vp, ci, vp, ci, ci]
        o.oracle_llt_residual.restype = cd
        o.oracle_backward_error.argtypes = [ci, ci, vp, ci, vp, ci, vp, ci, vp]
        o.oracle_backward_error.restype = cd
        o.oracle_flops_potrf.argtypes = [cd]
        o.oracle_flops_potrf.restype = cd
        o.oracle_dsposv_ir.argtypes = [ci, ci, vp, ci, vp, ci, vp, ci, ci, cd, ci, vp]
        o.cpu_chol_init.argtypes = [C.c_char_p]
        o.cpu_chol_potrf_tiled_f32.argtypes = [ci, vp, ci, ci, ci]
        o.cpu_chol_potrf_tiled_f64.argtypes = [ci, vp, ci, ci, ci]
        o.cpu_chol_potrs_f64.argtypes = [ci, ci, vp, ci, vp, ci, ci]
        o.cpu_chol_set_blas_threads.argtypes = [ci]
        for p, t in (("s", C.c_float), ("d", C.c_double)):
            getattr(o, f"oracle_{p}lu_getrf").argtypes = [ci, vp, ci, t, vp, ci]
            getattr(o, f"oracle_{p}lu_trsm_ll").argtypes = [ci, ci, vp, ci, vp, ci]
            getattr(o, f"oracle_{p}lu_trsm_ru").argtypes = [ci, ci, vp, ci, vp, ci]
            getattr(o, f"oracle_{p}lu_gemm").argtypes = [ci, ci, ci, vp, ci, vp, ci, vp, ci]
            getattr(o, f"oracle_{p}lu_pivot").argtypes = [ci, vp, ci, vp]
        _o = o
    return _o


def ref_lib() -> C.CDLL | None:
    """CLAPACK from the reference tree (only where it was built)."""
    global _r
    if _r is None and os.path.exists(REFLIB):
        _r = C.CDLL(REFLIB)
    return _r


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- inputs
def hilbert_f32(n: int) -> np.ndarray:
    A = np.empty((n, n), dtype=np.float32, order="F")
    lib().oracle_hilbert_f32(n, _p(A), n)
    return A


def normal_matrix(rows: int, cols: int, seed: int) -> np.ndarray:
    B = np.empty((rows, cols), dtype=np.float64, order="F")
    lib().oracle_normal_matrix(rows, cols, seed, _p(B), rows)
    return B


def normal_matrix_threaded(rows: int, cols: int, seed: int, threads: int) -> np.ndarray:
    """normal_matrix, its row streams filled by `threads` host threads."""
    from concurrent.futures import ThreadPoolExecutor
    B = np.empty((rows, cols), dtype=np.float64, order="F")
    o = lib()
    step = max(1, (rows + threads - 1) // max(1, threads))
    base = B.ctypes.data

    def fill(r0):
        o.oracle_normal_rows(r0, min(step, rows - r0), cols, seed, C.c_void_p(base + 8 * r0), rows)
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        list(ex.map(fill, range(0, rows, step)))
    return B


def spd_gram_host_blas(n: int, seed: int, alpha: float, threads: int) -> np.ndarray:
    """spd_gram for large n: B from the same row streams, A = B B^T / n + alpha I
    through the host BLAS (scipy's dsyrk, lower), mirrored to the full matrix."""
    from scipy.linalg import blas
    assert cpu_init()
    lib().cpu_chol_set_blas_threads(threads)
    B = normal_matrix_threaded(n, n, seed, threads)
    A = blas.dsyrk(1.0 / n, B, lower=1, trans=0)
    del B
    A = np.asfortranarray(A)
    bs = 2048
    for j0 in range(0, n, bs):
        j1 = min(n, j0 + bs)
        D = A[j0:j1, j0:j1]
        A[j0:j1, j0:j1] = np.tril(D) + np.tril(D, -1).T
        if j1 < n:
            A[j0:j1, j1:] = A[j1:, j0:j1].T
    A[np.diag_indices(n)] += alpha
    lib().cpu_chol_set_blas_threads(1)
    return A


def uniform_rhs(n: int, nrhs: int, seed: int) -> np.ndarray:
    B = np.empty((n, nrhs), dtype=np.float64, order="F")
    lib().oracle_uniform_rhs(n, nrhs, seed, _p(B), n)
    return B


def spd_gram(n: int, seed: int, alpha: float) -> np.ndarray:
    A = np.empty((n, n), dtype=np.float64, order="F")
    lib().oracle_spd_gram(n, seed, alpha, _p(A), n)
    return A


def alpha_for_kappa(kappa: float) -> float:
    """Shift alpha so that (4 + alpha) / alpha = kappa for B B^T / n with B
    square iid N(0,1): its spectrum fills the Marchenko-Pastur range [0, 4]."""
    return 4.0 / (kappa - 1.0)


def chunk(n: int, parts: int, i: int) -> tuple[int, int]:
    s, o = C.c_int(), C.c_int()
    lib().oracle_chunk(n, parts, i, C.byref(s), C.byref(o))
    return s.value, o.value


# ------------------------------------------------------------ algorithms
def potrf_tiled(A: np.ndarray, nblocks: int) -> tuple[np.ndarray, int]:
    L = np.array(A, order="F", copy=True)
    n = L.shape[0]
    f = lib().oracle_potrf_tiled_f32 if L.dtype == np.float32 else lib().oracle_potrf_tiled_f64
    info = f(n, _p(L), n, nblocks)
    return L, info


def potrs(L: np.ndarray, B: np.ndarray) -> np.ndarray:
    L = np.asfortranarray(L)
    X = np.array(B, order="F", copy=True, dtype=L.dtype)
    n, nrhs = X.shape
    f = lib().oracle_potrs_f32 if L.dtype == np.float32 else lib().oracle_potrs_f64
    f(n, nrhs, _p(L), L.shape[0], _p(X), n)
    return X


def check_hilbert(L: np.ndarray, tol: float = 1e-4) -> tuple[int, float]:
    e = C.c_double()
    bad = lib().oracle_check_hilbert_f32(L.shape[0], _p(np.asfortranarray(L)), L.shape[0], tol, C.byref(e))
    return bad, e.value


def llt_residual(A: np.ndarray, L: np.ndarray) -> float:
    A = np.asfortranarray(A, dtype=np.float64)
    L = np.asfortranarray(L)
    return lib().oracle_llt_residual(A.shape[0], _p(A), A.shape[0], _p(L), L.shape[0], int(L.dtype == np.float32))


def backward_error(A: np.ndarray, X: np.ndarray, B: np.ndarray) -> tuple[float, np.ndarray]:
    A = np.asfortranarray(A, dtype=np.float64)
    X = np.asfortranarray(X, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    be = np.empty(X.shape[1])
    w = lib().oracle_backward_error(A.shape[0], X.shape[1], _p(A), A.shape[0], _p(X), X.shape[0], _p(B),
                                    B.shape[0], _p(be))
    return w, be


def llt_residual_blas(A: np.ndarray, L: np.ndarray) -> float:
    """llt_residual (||A - L L^T||_F / ||A||_F over the symmetric A) through
    numpy's BLAS, for orders where the plain-C loop is too slow."""
    Lt = np.tril(np.asarray(L, dtype=np.float64))
    R = np.asarray(A, dtype=np.float64) - Lt @ Lt.T
    return float(np.linalg.norm(R) / np.linalg.norm(A))


def cpu_solve(A: np.ndarray, B: np.ndarray, nb: int, nthreads: int) -> np.ndarray:
    """FP64 solution of A X = B by the StarPU CPU path port (tiled FP64
    Cholesky over OpenBLAS, pinned to CLAPACK dpotrf/dpotrs by the golden
    vectors) and LAPACK dpotrs: the FP64 oracle for large orders."""
    n = A.shape[0]
    L = np.array(A, dtype=np.float64, order="F", copy=True)
    X = np.array(B, dtype=np.float64, order="F", copy=True)
    info = cpu_potrf_tiled(L, max(1, min(512, round(n / nb))), nthreads)
    assert info == 0, info
    assert cpu_potrs(L, X, nthreads) == 0
    return X


def flops_potrf(n: float) -> float:
    return lib().oracle_flops_potrf(float(n))


def dsposv_ir(A, B, nblocks, tol=1e-12, max_iter=30):
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    X = np.zeros_like(B, order="F")
    be = C.c_double()
    it = lib().oracle_dsposv_ir(A.shape[0], B.shape[1], _p(A), A.shape[0], _p(B), B.shape[0], _p(X), X.shape[0],
                                nblocks, tol, max_iter, C.byref(be))
    return X, it, be.value


# ------------------------------------------------------ reference CLAPACK
def ref_dpotrf(A: np.ndarray) -> tuple[np.ndarray, int]:
    r = ref_lib()
    if r is None:
        raise FileNotFoundError("oracle/_ref/libref_lapack.so not built")
    L = np.array(A, dtype=np.float64, order="F", copy=True)
    n = C.c_long(L.shape[0])
    info = C.c_long(0)
    r._starpu_dpotrf_(b"L", C.byref(n), _p(L), C.byref(n), C.byref(info))
    return L, info.value


def ref_dpotrs(L: np.ndarray, B: np.ndarray) -> np.ndarray:
    r = ref_lib()
    X = np.array(B, dtype=np.float64, order="F", copy=True)
    n, nrhs = C.c_long(L.shape[0]), C.c_long(X.shape[1])
    info = C.c_long(0)
    r._starpu_dpotrs_(b"L", C.byref(n), C.byref(nrhs), _p(np.asfortranarray(L)), C.byref(n), _p(X), C.byref(n),
                      C.byref(info))
    assert info.value == 0
    return X


# -------------------------------------------------- StarPU CPU path port
def openblas_path() -> str | None:
    try:
        import scipy
    except ImportError:
        return None
    d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so*")))
    return c[0] if c else None


def cpu_init() -> bool:
    global _blas_ready
    if not _blas_ready:
        p = openblas_path()
        if p is None:
            return False
        _blas_ready = lib().cpu_chol_init(p.encode()) == 0
    return _blas_ready


def cpu_potrf_tiled(A: np.ndarray, nblocks: int, nthreads: int) -> int:
    assert cpu_init(), "scipy OpenBLAS not available"
    f = lib().cpu_chol_potrf_tiled_f32 if A.dtype == np.float32 else lib().cpu_chol_potrf_tiled_f64
    return f(A.shape[0], _p(A), A.shape[0], nblocks, nthreads)


def cpu_potrs(L: np.ndarray, B: np.ndarray, nthreads: int) -> int:
    assert cpu_init()
    return lib().cpu_chol_potrs_f64(L.shape[0], B.shape[1], _p(L), L.shape[0], _p(B), B.shape[0], nthreads)


# ------------------------------------------------------------------ LU (examples/lu)
def _lu_prefix(a: np.ndarray) -> str:
    return "s" if a.dtype == np.float32 else "d"


def lu_getrf(A: np.ndarray, thr: float = 0.0, iamax_shift: int = 0):
    """In-place LU of a Fortran-ordered tile (L non-unit, U unit); returns
    (info, ipiv) with ipiv[z] = the column swapped in at step z, -1 if none.
    iamax_shift = 1 reproduces the reference CPU branch built against a
    Fortran-interface BLAS (1-based ISAMAX used as 0-based)."""
    assert A.flags.f_contiguous and A.shape[0] == A.shape[1]
    n = A.shape[0]
    ipiv = np.full(n, -1, dtype=np.int32)
    info = getattr(lib(), f"oracle_{_lu_prefix(A)}lu_getrf")(n, _p(A), n, thr, _p(ipiv), iamax_shift)
    return info, ipiv


def lu_trsm_ll(L: np.ndarray, B: np.ndarray) -> None:
    getattr(lib(), f"oracle_{_lu_prefix(B)}lu_trsm_ll")(B.shape[0], B.shape[1], _p(L), L.shape[0], _p(B), B.shape[0])


def lu_trsm_ru(U: np.ndarray, B: np.ndarray) -> None:
    getattr(lib(), f"oracle_{_lu_prefix(B)}lu_trsm_ru")(B.shape[0], B.shape[1], _p(U), U.shape[0], _p(B), B.shape[0])


def lu_gemm(A: np.ndarray, B: np.ndarray, Cm: np.ndarray) -> None:
    getattr(lib(), f"oracle_{_lu_prefix(Cm)}lu_gemm")(Cm.shape[0], Cm.shape[1], A.shape[1], _p(A), A.shape[0], _p(B),
                                                       B.shape[0], _p(Cm), Cm.shape[0])


def lu_pivot(T: np.ndarray, ipiv_tile: np.ndarray) -> None:
    """Column swaps of the PIVOT codelet; ipiv_tile[r] = tile-local column (r = no swap)."""
    p = np.ascontiguousarray(ipiv_tile, dtype=np.int32)
    getattr(lib(), f"oracle_{_lu_prefix(T)}lu_pivot")(T.shape[0], _p(T), T.shape[0], _p(p))
