"""Generate the committed golden vectors under tests/golden/.

Run in a checkout where the reference tree is available (it builds
oracle/_ref/libref_lapack.so from the reference's min-dgels CLAPACK sources):

    python tests/golden/make_golden.py

Outputs
  chol_golden.npz : for each case (n, seed, alpha, nrhs): the SPD input A
                    (oracle generator), the lower factor computed by the
                    reference's CLAPACK dpotrf, right-hand sides B and the
                    solution computed by the reference's CLAPACK dpotrs.
  hilbert_ref.npz : FP32 tiled factor of the reference driver's input
                    (A_mn = 1/(1+m+n) + n delta_mn) computed by the reference's
                    own CPU codelets through the unchanged cholesky_implicit
                    driver, when that build is available (else omitted).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CASES = [  # n, seed, alpha, nrhs
    (1, 11, 1.0, 1),
    (2, 12, 1.0, 2),
    (17, 13, 0.5, 3),
    (64, 14, 1.0, 4),
    (100, 15, 0.1, 4),
    (130, 16, 2.0, 5),
    (96, 17, 4.0 / (1e4 - 1), 2),
]


def main():
    O.build(with_ref=True)
    assert O.ref_lib() is not None, "reference CLAPACK not built (is the reference tree present?)"
    out = {}
    for (n, seed, alpha, nrhs) in CASES:
        A = O.spd_gram(n, seed, alpha)
        L, info = O.ref_dpotrf(A)
        assert info == 0
        L = np.tril(L)
        B = O.uniform_rhs(n, nrhs, seed + 1000)
        X = O.ref_dpotrs(L, B)
        key = f"n{n}_s{seed}"
        out[key + "_A"] = A
        out[key + "_L"] = L
        out[key + "_B"] = B
        out[key + "_X"] = X
        out[key + "_meta"] = np.array([n, seed, alpha, nrhs], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "chol_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "chol_golden.npz"), len(CASES), "cases")


if __name__ == "__main__":
    main()
