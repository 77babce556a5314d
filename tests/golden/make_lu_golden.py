"""Golden vectors of the reference's LU codelets (examples/lu/xlu_kernels.c,
CPU branches), computed by the reference's own code compiled from its tree:

    make -C oracle ref-lu && python tests/golden/make_lu_golden.py

writes tests/golden/lu_golden.npz: for FP32 and FP64, seeded inputs and the
outputs of GETRF, GETRF_PIVOT (a tile that needs pivots), TRSM_LL, TRSM_RU,
GEMM and PIVOT, each called like the runtime calls a codelet (an array of
matrix interfaces and the codelet argument).  Only the committed .npz is used
by the tests; this script needs the reference tree and runs only here.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref")


class MatrixInterface(C.Structure):
    # struct starpu_matrix_interface (include/starpu.h)
    _fields_ = [("id", C.c_int), ("ptr", C.c_void_p), ("dev_handle", C.c_void_p), ("offset", C.c_size_t),
                ("nx", C.c_size_t), ("ny", C.c_size_t), ("ld", C.c_size_t), ("elemsize", C.c_size_t),
                ("allocsize", C.c_size_t)]


class PivS(C.Structure):
    # struct piv_s of examples/lu/xlu.h
    _fields_ = [("piv", C.POINTER(C.c_uint)), ("first", C.c_uint), ("last", C.c_uint)]


def iface(a):
    assert a.flags.f_contiguous
    m = MatrixInterface()
    m.ptr = a.ctypes.data
    m.nx, m.ny, m.ld = a.shape[0], a.shape[1], a.shape[0]
    m.elemsize = a.itemsize
    return m


def call(fn, arrays, arg=None):
    ifs = [iface(a) for a in arrays]
    descr = (C.c_void_p * len(ifs))(*[C.addressof(i) for i in ifs])
    fn(descr, arg)


def cases(lib, prefix, dtype, n, rng):
    out = {}
    f = lambda name: getattr(lib, f"starpu_{prefix}lu_cpu_{name}")  # noqa: E731
    # GETRF: diagonally dominant like the reference driver's input (lu_example.c:221-233)
    A = np.asfortranarray(rng.random((n, n)) + np.eye(n) * n).astype(dtype)
    out["getrf_in"] = A.copy(order="F")
    call(f("getrf"), [A])
    out["getrf_out"] = A
    # GETRF_PIVOT: small and zero pivots force column swaps
    P = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    P[0, 0] = 0
    P[5, 5] = 1e-6
    P[n // 2, n // 2] = 0
    out["getrf_pivot_in"] = P.copy(order="F")
    ipiv = (C.c_uint * n)(*range(n))
    call(f("getrf_pivot"), [P], C.byref(PivS(C.cast(ipiv, C.POINTER(C.c_uint)), 0, n)))
    out["getrf_pivot_out"] = P
    out["getrf_pivot_ipiv"] = np.array(list(ipiv), dtype=np.int32)
    # TRSM_LL: B <- L^-1 B with the L of the GETRF output
    Lt = out["getrf_out"].copy(order="F")
    B = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    out["trsm_ll_l"], out["trsm_ll_in"] = Lt, B.copy(order="F")
    call(f("trsmll"), [Lt, B])
    out["trsm_ll_out"] = B
    # TRSM_RU: B <- B U^-1 with the unit U of the GETRF output
    B2 = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    out["trsm_ru_in"] = B2.copy(order="F")
    call(f("trsmru"), [Lt, B2])
    out["trsm_ru_out"] = B2
    # GEMM: C <- C - A B
    Ag = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    Bg = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    Cg = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    out["gemm_a"], out["gemm_b"], out["gemm_in"] = Ag, Bg, Cg.copy(order="F")
    call(f("gemm"), [Ag, Bg, Cg])
    out["gemm_out"] = Cg
    # PIVOT: the swaps recorded by GETRF_PIVOT applied to another tile
    T = np.asfortranarray(rng.standard_normal((n, n))).astype(dtype)
    out["pivot_in"] = T.copy(order="F")
    call(f("pivot"), [T], C.byref(PivS(C.cast(ipiv, C.POINTER(C.c_uint)), 0, n)))
    out["pivot_out"] = T
    return out


def main():
    rng = np.random.default_rng(20240)
    res = {}
    for prefix, dtype in (("s", np.float32), ("d", np.float64)):
        lib = C.CDLL(os.path.join(REF, f"libref_{prefix}lu.so"))
        for k, v in cases(lib, prefix, dtype, 64, rng).items():
            res[f"{prefix}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "lu_golden.npz"), **res)
    print("wrote", os.path.join(HERE, "lu_golden.npz"), len(res), "arrays")


if __name__ == "__main__":
    main()
