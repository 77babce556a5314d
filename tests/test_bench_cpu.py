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
