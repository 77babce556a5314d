"""bench.py's reference arm on CPU: the StarPU CPU-path port timed on a small
sample prints one JSON line with the contract's keys (the GPU arm needs a
GB300), and the CPU-runnable configuration passes the reference's own check."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _openblas_or_skip():
    from oracle import oracle as O
    if not O.cpu_init():
        pytest.skip("scipy's OpenBLAS not found")


def test_reference_arm_json_line():
    _openblas_or_skip()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--cpu-n", "1024", "--cpu-nb", "256"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["backward_error"] < 1e-12


def test_cpu_config1_passes_reference_check():
    _openblas_or_skip()
    import bench
    r = bench.cpu_config1(reps=1)
    assert r["check_ok"] and r["max_rel_err"] <= 1e-4 and r["gflops"] > 0


def test_oracle_forward_error_helpers():
    """The bench's FP64 oracle solve (the CPU-path port) and its error
    measures on a small system, against numpy's own solve."""
    _openblas_or_skip()
    import numpy as np
    import bench
    from oracle import oracle as O
    n, nrhs, kappa = 700, 3, 1e3
    A = O.spd_gram(n, 5, O.alpha_for_kappa(kappa))
    B = O.uniform_rhs(n, nrhs, 6)
    Xo, t = bench.oracle_solve(A, B, 128, 2)
    Xn = np.linalg.solve(A, B)
    assert bench.forward_error(Xo, Xn) <= 1e-12 and t > 0
    assert bench.host_backward_error(A, Xo, B) <= 1e-15
    # a perturbed solution: the forward error sees it, relative to ||xo||_inf
    Xp = Xo.copy()
    Xp[0, 1] += 1e-6 * np.abs(Xo[:, 1]).max()
    assert abs(bench.forward_error(Xp, Xo) - 1e-6) <= 1e-9
    # the shifted system (A + s I) X = B, as the kappa sweep uses it
    s = 0.5
    Xs, _ = bench.oracle_solve(A, B, 128, 2, shift=s)
    r = bench.accuracy_of(A, B, Xs, np.linalg.solve(A + s * np.eye(n), B), kappa, shift=s)
    assert r["forward_error"] <= 1e-12 and r["backward_error_host"] <= 1e-15 and r["oracle_backward_error"] <= 1e-15


def test_reference_arm_names_the_gpu_arms_configuration():
    import argparse
    import bench
    args = argparse.Namespace(n=32768, nb=1024, nrhs=16, kappa=1e4)
    c = bench.bench_config(args, 1)
    assert (c["n"], c["nb"], c["nrhs"], c["kappa"]) == (32768, 1024, 16, 1e4)
    assert c == bench.bench_config(args, 1, n=32768, nb=1024)
