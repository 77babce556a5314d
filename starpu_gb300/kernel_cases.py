"""Single-kernel cases for profiling (ncu) and quick timing, through the C-ABI.

    python -m starpu_gb300.kernel_cases tc_update --m 8192 --k 1024 --nterms 3 --reps 3
    python -m starpu_gb300.kernel_cases residual  --n 16384 --nrhs 16 --reps 3
    python -m starpu_gb300.kernel_cases potrs     --n 16384 --nrhs 16 --reps 3
    python -m starpu_gb300.kernel_cases sweep     --n 16384 --nrhs 16 --reps 3
    python -m starpu_gb300.kernel_cases dsposv    --n 8192  --nb 1024 --nrhs 16 --reps 2
    python -m starpu_gb300.kernel_cases spotrf_tc --n 8192  --nb 1024 --nterms 3 --reps 2
    python -m starpu_gb300.kernel_cases dpotrf    --n 8192  --nb 512 --reps 2
    python -m starpu_gb300.kernel_cases tile_ops  --n 1024 --reps 200
    python -m starpu_gb300.kernel_cases diag      --n 1024 --reps 50
    python -m starpu_gb300.kernel_cases tile_sweep --n 32768 --nb 1024 --nrhs 16 --reps 5
    python -m starpu_gb300.kernel_cases syresidual --n 32768 --nrhs 16 --reps 3

Each case allocates its operands once, runs `--reps` launches of the same
shape and prints the mean time per launch measured with CUDA events.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np

from . import load
from .native import DeviceBuffer, check


def _timed(L, fn, reps):
    fn()
    check(L.starpu_gb300_stream_sync(None))
    e0, e1 = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
    check(L.starpu_gb300_event_record(e0, None))
    for _ in range(reps):
        fn()
    check(L.starpu_gb300_event_record(e1, None))
    ms = L.starpu_gb300_event_elapsed_ms(e0, e1) / reps
    L.starpu_gb300_event_destroy(e0)
    L.starpu_gb300_event_destroy(e1)
    return ms


def oracle_free_spd(n):
    """FP32 SPD test matrix: 1 / (1 + i + j) plus n on the diagonal."""
    i = np.arange(n, dtype=np.float32)
    A = 1.0 / (1.0 + i[:, None] + i[None, :])
    A[np.diag_indices(n)] += n
    return A.astype(np.float32)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["tc_update", "residual", "potrs", "sweep", "spotrf_tc", "dpotrf", "dsposv",
                                     "tile_ops", "diag", "tile_sweep", "syresidual"])
    ap.add_argument("--kappa", type=float, default=1e4)
    ap.add_argument("--m", type=int, default=8192)
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--k", type=int, default=1024)
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--nterms", type=int, default=3)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    L = load()
    out = {"case": a.case}
    if a.case == "tc_update":
        m, k = a.m, a.k
        ldk = (k + 63) // 64 * 64
        P = DeviceBuffer(4 * m * k)
        hi, lo = DeviceBuffer(2 * m * ldk), DeviceBuffer(2 * m * ldk)
        Cb = DeviceBuffer(4 * m * m)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        check(L.starpu_gb300_memset(None, P.ptr, 0, 4 * m * k))
        check(L.starpu_gb300_memset(None, Cb.ptr, 0, 4 * m * m))
        check(L.starpu_gb300_split_bf16(None, m, k, P.ptr, m, hi.ptr, lo.ptr, ldk))
        ms = _timed(L, lambda: check(L.starpu_gb300_tc_update(None, m, m, k, hi.ptr, lo.ptr, ldk, hi.ptr, lo.ptr, ldk,
                                                               a.nterms, 1, Cb.ptr, m, err.ptr)), a.reps)
        fl = a.nterms * k * m * (m + 1.0)
        out.update(ms=ms, tflops=fl / ms / 1e9, algorithmic_bytes=8.0 * m * (m + 1) / 2 + 2.0 * m * ldk * 2)
    elif a.case in ("residual", "potrs", "sweep"):
        n, nrhs = a.n, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        Bd, Xd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 5, Xd.ptr, n))
        if a.case == "residual":
            lw = L.starpu_gb300_backward_error_workspace(n, nrhs)
            BW = DeviceBuffer(lw)
            be = np.zeros(nrhs)
            ms = _timed(L, lambda: check(L.starpu_gb300_backward_error(None, n, nrhs, A.ptr, n, Xd.ptr, n, Bd.ptr, n,
                                                                        BW.ptr, lw, be.ctypes.data)), a.reps)
            out.update(ms=ms, tflops=2.0 * n * n * nrhs / ms / 1e9, algorithmic_bytes=8.0 * n * n)
        else:
            # FP32 sweeps (the refinement's correction solve) with the lower part of a
            # diagonally dominant matrix as the factor
            i = np.arange(n, dtype=np.float32)
            Lh = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, :]), dtype=np.float32)
            Lh[np.diag_indices(n)] += n
            F = DeviceBuffer.from_array(Lh)
            Y = DeviceBuffer.from_array(np.ones((n, nrhs), np.float32))
            if a.case == "potrs":
                ms = _timed(L, lambda: check(L.starpu_gb300_spotrs(None, n, nrhs, F.ptr, n, Y.ptr, n)), a.reps)
            else:
                lw = L.starpu_gb300_spotrs_sweep_workspace(n)
                SW = DeviceBuffer(lw)
                err = DeviceBuffer.from_array(np.zeros(1, np.int32))
                ms = _timed(L, lambda: check(L.starpu_gb300_spotrs_sweep(None, n, nrhs, F.ptr, n, Y.ptr, n, SW.ptr, lw,
                                                                          err.ptr)), a.reps)
            # both sweeps read the lower triangle of L once: 2 * 4 * n^2 / 2 bytes
            out.update(ms=ms, gbs=4.0 * n * n / ms / 1e6)
    elif a.case == "spotrf_tc":
        n, nb = a.n, a.nb
        from_host = np.empty((n, n), np.float32, order="F")
        i = np.arange(n, dtype=np.float32)
        from_host[:] = 1.0 / (1.0 + i[:, None] + i[None, :])
        from_host[np.diag_indices(n)] += n
        F = DeviceBuffer.from_array(from_host)
        ws = L.starpu_gb300_spotrf_tc_workspace(n, nb)
        Wk = DeviceBuffer(ws)
        info, err = DeviceBuffer(4), DeviceBuffer.from_array(np.zeros(1, np.int32))

        def run():
            F.upload(from_host)
            check(L.starpu_gb300_spotrf_tc(None, n, F.ptr, n, nb, a.nterms, Wk.ptr, ws, info.ptr, err.ptr))
        ms = _timed(L, run, a.reps)
        out.update(ms_including_upload=ms)
    elif a.case == "tile_ops":
        # the FP32 pieces of the mixed solve's diagonal-tile factorisation: the
        # 64 x 64 leaf, the whole n x n tile, and one step's panel TRSM and SYRK
        # at their largest shape (n - 64 rows, 64 columns)
        n = a.n
        i = np.arange(n, dtype=np.float32)
        Ah = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, :]), dtype=np.float32)
        Ah[np.diag_indices(n)] += n
        A0, Aw = DeviceBuffer.from_array(Ah), DeviceBuffer(4 * n * n)
        info = DeviceBuffer(4)
        nbytes = 4 * n * n

        def restore():
            check(L.starpu_gb300_memcpy_d2d(None, Aw.ptr, A0.ptr, nbytes))
        ms_copy = _timed(L, restore, a.reps)

        def potrf(k):
            def f():
                restore()
                check(L.starpu_gb300_spotrf_tile(None, k, Aw.ptr, n, info.ptr))
            return f
        m, w = n - 64, 64
        ms_leaf = _timed(L, potrf(64), a.reps) - ms_copy
        ms_tile = _timed(L, potrf(n), a.reps) - ms_copy
        restore()
        check(L.starpu_gb300_spotrf_tile(None, n, Aw.ptr, n, info.ptr))
        Lw = DeviceBuffer.from_array(np.zeros((n, n), np.float32))
        check(L.starpu_gb300_memcpy_d2d(None, Lw.ptr, Aw.ptr, nbytes))
        ms_trsm = _timed(L, lambda: check(L.starpu_gb300_strsm_rltn_tile(None, m, w, 1.0, Lw.ptr, n, Aw.ptr + 4 * 64,
                                                                          n)), a.reps)
        ms_syrk = _timed(L, lambda: check(L.starpu_gb300_ssyrk_ln_tile(None, m, w, -1.0, Lw.ptr + 4 * 64, n, 1.0,
                                                                        Aw.ptr + 4 * (64 + 64 * n), n)), a.reps)
        out.update(n=n, ms_leaf64=ms_leaf, ms_tile=ms_tile, ms_trsm=ms_trsm, ms_syrk=ms_syrk, ms_restore=ms_copy,
                   tile_gflops=n ** 3 / 3 / ms_tile / 1e6)
    elif a.case == "diag":
        # the tensor-core Cholesky's diagonal-tile step alone: spotrf_tc of an
        # n x n matrix with nb = n (factor only), and of n + 64 with nb = n
        # (factor + inverse of the n x n tile, then a 64-row panel and update)
        n = a.n
        out.update(n=n)
        for tag, N in (("factor", n), ("factor_inverse_plus_64", n + 64)):
            Ah = np.asfortranarray(oracle_free_spd(N))
            A0, Aw = DeviceBuffer.from_array(Ah), DeviceBuffer(4 * N * N)
            ws = L.starpu_gb300_spotrf_tc_workspace(N, n)
            Wk = DeviceBuffer(ws)
            info, err = DeviceBuffer(4), DeviceBuffer.from_array(np.zeros(1, np.int32))

            def restore():
                check(L.starpu_gb300_memcpy_d2d(None, Aw.ptr, A0.ptr, 4 * N * N))

            def run():
                restore()
                check(L.starpu_gb300_spotrf_tc(None, N, Aw.ptr, N, n, 3, Wk.ptr, ws, info.ptr, err.ptr))
            ms_copy = _timed(L, restore, a.reps)
            out["ms_" + tag] = _timed(L, run, a.reps) - ms_copy
            out["err_" + tag] = int(DeviceBuffer.download(err, (1,), np.int32)[0])
    elif a.case == "tile_sweep":
        # both tile-row sweeps of one FP32 correction solve (identity
        # diagonal-tile inverses: the timing does not depend on the values)
        n, nb, nrhs = a.n, a.nb, a.nrhs
        i = np.arange(n, dtype=np.float32)
        F = DeviceBuffer(4 * n * n)
        for c0 in range(0, n, 2048):  # the factor column panel by column panel (host memory stays small)
            w = min(2048, n - c0)
            Lp = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, c0:c0 + w]), dtype=np.float32)
            Lp[np.arange(c0, c0 + w), np.arange(w)] += n
            check(L.starpu_gb300_memcpy_h2d(None, F.ptr + 4 * n * c0, Lp.ctypes.data, Lp.nbytes))
        ldd = (nb + 63) // 64 * 64
        ntiles = (n + nb - 1) // nb
        eye = np.asfortranarray(np.eye(ldd, dtype=np.float32))
        D = DeviceBuffer(4 * ntiles * ldd * ldd)
        for T in range(ntiles):
            check(L.starpu_gb300_memcpy_h2d(None, D.ptr + 4 * T * ldd * ldd, eye.ctypes.data, eye.nbytes))
        Y = DeviceBuffer.from_array(np.ones((n, nrhs), np.float32))
        lw = L.starpu_gb300_spotrs_inv_tiles_workspace(n, nb)
        Wk = DeviceBuffer(lw)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        ms = _timed(L, lambda: check(L.starpu_gb300_spotrs_inv_tiles(None, n, nrhs, nb, F.ptr, n, D.ptr, ldd, Y.ptr, n,
                                                                      Wk.ptr, lw, err.ptr)), a.reps)
        out.update(ms_two_sweeps=ms, gbs=4.0 * n * n / ms / 1e6, err=int(err.download((1,), np.int32)[0]))
    elif a.case == "syresidual":
        # the refinement residual R = B - A X on the tensor cores (symmetric A, lower triangle read)
        n, nrhs = a.n, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        del W
        Bd, Xd, Rd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 5, Xd.ptr, n))
        lw = L.starpu_gb300_dsyresidual_workspace(n, nrhs)
        Wk = DeviceBuffer(lw)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        ms = _timed(L, lambda: check(L.starpu_gb300_dsyresidual(None, n, nrhs, A.ptr, n, Xd.ptr, n, Bd.ptr, n, Rd.ptr, n,
                                                                 Wk.ptr, lw, err.ptr)), a.reps)
        out.update(ms=ms, tflops_fp64_equiv=2.0 * n * n * nrhs / ms / 1e9, err=int(err.download((1,), np.int32)[0]))
    elif a.case == "dpotrf":
        n, nb = a.n, a.nb
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        info = DeviceBuffer(4)

        def run():
            check(L.starpu_gb300_memcpy_d2d(None, W.ptr, A.ptr, 8 * n * n))
            check(L.starpu_gb300_dpotrf(None, n, W.ptr, n, nb, info.ptr))
        ms = _timed(L, run, a.reps)
        out.update(ms=ms, gflops=n ** 3 / 3 / ms / 1e6)
    elif a.case == "dsposv":
        from .native import IrInfo
        n, nb, nrhs = a.n, a.nb, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        Bd, Xd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 4.0 / (a.kappa - 1.0), A.ptr, n, W.ptr))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        lw = L.starpu_gb300_dsposv_workspace(n, nrhs, nb)
        Wk = DeviceBuffer(lw)
        info = IrInfo()
        ms = _timed(L, lambda: check(L.starpu_gb300_dsposv(None, n, nrhs, A.ptr, n, Bd.ptr, n, Xd.ptr, n, nb, a.nterms,
                                                            1e-12, 30, Wk.ptr, lw, C.byref(info))), a.reps)
        out.update(ms=ms, gflops=(n ** 3 / 3 + 2.0 * n * n * nrhs) / ms / 1e6, iterations=info.iterations,
                   backward_error=info.backward_error)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
