"""Batched SPD solve (many systems of uneven sizes, one persistent launch):
every system reaches the FP64 backward-error target, gives the same result
alone and in the mix, and a failing system does not disturb the others."""
import ctypes as C
import os

import numpy as np
import pytest

from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import check

pytestmark = pytest.mark.gpu


def make_system(oracle, n, seed, nrhs=4, shift=1.0):
    Bn = oracle.normal_matrix(n, n, seed)
    A = np.asfortranarray(Bn @ Bn.T / n)
    A[np.diag_indices(n)] += shift
    return A, oracle.uniform_rhs(n, nrhs, seed + 77)


def pack(systems, nrhs):
    ns = np.array([A.shape[0] for A, _ in systems], dtype=np.int32)
    a_off = np.zeros(len(ns), dtype=np.int64)
    b_off = np.zeros(len(ns), dtype=np.int64)
    a_off[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
    b_off[1:] = np.cumsum(ns.astype(np.int64) * nrhs)[:-1]
    Ap = np.concatenate([A.ravel(order="F") for A, _ in systems])
    Bp = np.concatenate([B.ravel(order="F") for _, B in systems])
    return ns, a_off, b_off, Ap, Bp


def run_batched(gpu, systems, nrhs=4, tol=1e-12, max_iter=20):
    ns, a_off, b_off, Ap, Bp = pack(systems, nrhs)
    dA, dB = DeviceBuffer.from_array(Ap), DeviceBuffer.from_array(Bp)
    dX = DeviceBuffer(Bp.nbytes)
    lw = gpu.starpu_gb300_dposv_batched_workspace(len(ns), ns.ctypes.data, nrhs)
    W = DeviceBuffer(lw)
    status = np.zeros(len(ns), dtype=np.int32)
    berr = np.zeros(len(ns))
    check(gpu.starpu_gb300_dposv_batched(None, len(ns), ns.ctypes.data, dA.ptr, a_off.ctypes.data, dB.ptr,
                                         b_off.ctypes.data, dX.ptr, nrhs, tol, max_iter, W.ptr, lw,
                                         status.ctypes.data, berr.ctypes.data))
    Xp = dX.download((Bp.size,), np.float64)
    Xs = [Xp[b_off[i]:b_off[i] + ns[i] * nrhs].reshape((ns[i], nrhs), order="F") for i in range(len(ns))]
    return status, berr, Xs


SIZES = [1, 5, 31, 32, 33, 64, 65, 100, 200, 257, 511, 513, 700, 1000, 1024]


def test_batched_uneven_sizes_reach_fp64_accuracy(gpu, oracle):
    systems = [make_system(oracle, n, 10 + i) for i, n in enumerate(SIZES)]
    status, berr, Xs = run_batched(gpu, systems)
    for (A, B), X, st, be in zip(systems, Xs, status, berr):
        assert st >= 0, (A.shape, st)
        ob, _ = oracle.backward_error(A, X, B)
        assert ob <= 1e-12, (A.shape, ob)
        assert abs(ob - be) <= 1e-13 + 0.05 * ob


def test_batched_same_result_alone_and_in_the_mix(gpu, oracle):
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(32), np.log(1024), 40)).astype(int)
    systems = [make_system(oracle, int(n), 200 + i) for i, n in enumerate(sizes)]
    _, _, X_mix = run_batched(gpu, systems)
    for i in (0, 7, 23, 39):
        _, _, X_alone = run_batched(gpu, [systems[i]])
        np.testing.assert_array_equal(X_alone[0], X_mix[i])


def test_batched_failing_system_is_isolated(gpu, oracle):
    good = [make_system(oracle, n, 300 + n) for n in (50, 300)]
    A_bad, B_bad = make_system(oracle, 128, 999)
    A_bad[40, 40] = -5.0
    status, berr, Xs = run_batched(gpu, [good[0], (A_bad, B_bad), good[1]])
    assert status[1] < 0
    assert status[0] >= 0 and status[2] >= 0
    for k in (0, 2):
        ob, _ = oracle.backward_error(good[k // 2][0], Xs[k], good[k // 2][1])
        assert ob <= 1e-12


def test_batched_autotuner_writes_table_next_to_perfmodels(gpu, tmp_path):
    os.environ["STARPU_PERF_MODEL_DIR"] = str(tmp_path)
    os.environ["STARPU_HOSTNAME"] = "tunehost"
    try:
        check(gpu.starpu_gb300_batched_autotune(64, 1))
        f = tmp_path / "codelets" / "45" / "gb300_chol_tuning.tunehost"
        assert f.exists()
        rows = [ln.split() for ln in f.read_text().splitlines() if ln and not ln.startswith("#")]
        assert len(rows) == 6 and all(int(r[2]) in (16, 32, 64) for r in rows)
        table = (C.c_byte * 6)()
        assert gpu.starpu_gb300_batched_get_tuning(table, 6) == 6
        assert [int(r[2]) for r in rows] == list(table)
    finally:
        del os.environ["STARPU_PERF_MODEL_DIR"]
        del os.environ["STARPU_HOSTNAME"]


_DENSE_TUNE = r"""
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import starpu_gb300
from starpu_gb300 import DeviceBuffer
from starpu_gb300.native import IrInfo, check
L = starpu_gb300.load()
check(L.starpu_gb300_dense_autotune(6144, 1024, 1), "dense autotune")
la, td, up, pr, st = C.c_int(), C.c_double(), C.c_double(), C.c_double(), C.c_double()
have = L.starpu_gb300_dense_get_tuning(1024, C.byref(la), C.byref(td), C.byref(up), C.byref(pr), C.byref(st))
# a solve with the stored schedule
n, nb, nrhs = 6144, 1024, 4
A, W0 = DeviceBuffer(8 * n * n), DeviceBuffer(8 * n * n)
check(L.starpu_gb300_gen_spd_gram(None, n, 3, 4.0 / (1e4 - 1), A.ptr, n, W0.ptr))
B, X = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, B.ptr, n))
lw = L.starpu_gb300_dsposv_workspace(n, nrhs, nb)
Wk = DeviceBuffer(lw)
info = IrInfo()
rc = L.starpu_gb300_dsposv(None, n, nrhs, A.ptr, n, B.ptr, n, X.ptr, n, nb, 3, 1e-12, 30, Wk.ptr, lw, C.byref(info))
print(json.dumps({"have": have, "la": la.value, "t_diag_us": td.value, "tflops": up.value, "panel_rate": pr.value,
                  "step_ms": st.value, "rc": rc, "berr": info.backward_error}))
"""


def test_dense_autotuner_stores_the_schedule_beside_the_perfmodels(gpu, tmp_path):
    """starpu_gb300_dense_autotune times the diagonal tile, the update and the
    panel solve, then whole factorisations under the model and fixed splits,
    and stores the fastest in gb300_chol_tuning.<host> beside the perfmodels,
    keeping the batched solver's lines; a solve afterwards uses it.  Run in a
    child process so that the stored schedule does not reach other tests."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    d = tmp_path / "codelets" / "45"
    d.mkdir(parents=True)
    f = d / "gb300_chol_tuning.tunehost"
    f.write_text("# an earlier batched tuning\n0 32 16 1.0\n1 64 32 1.0\n2 128 32 1.0\n3 256 64 1.0\n"
                 "4 512 64 1.0\n5 1024 64 1.0\n")
    env = dict(os.environ, STARPU_PERF_MODEL_DIR=str(tmp_path), STARPU_HOSTNAME="tunehost")
    env.pop("GB300_LOOKAHEAD_SMS", None)
    r = subprocess.run([sys.executable, "-c", _DENSE_TUNE, root], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["have"] == 1 and out["rc"] == 0 and out["berr"] <= 1e-12
    assert out["t_diag_us"] > 0 and out["tflops"] > 10 and out["panel_rate"] > 0 and out["step_ms"] > 0
    rows = [ln.split() for ln in f.read_text().splitlines() if ln and not ln.startswith("#")]
    dense = [r for r in rows if r[0] == "dense"]
    assert len(dense) == 1 and int(dense[0][1]) == 1024 and int(dense[0][2]) == out["la"]
    assert len([r for r in rows if r[0] != "dense"]) == 6  # the batched lines are kept
