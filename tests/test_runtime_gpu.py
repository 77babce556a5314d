"""The StarPU-API runtime with the GB300 codelets on the GPU: a tiled Cholesky
submitted task by task (implicit dependencies) and run either as one CUDA
graph per DAG (every worker a CUDA worker) or task by task on the CUDA
worker's stream (CPU workers present, or STARPU_GB300_GRAPH=0).  The driver
checks L L^T against the input element-wise (relative 1e-4 FP32 / 1e-12 FP64)."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_driver(args, **env):
    import starpu_gb300
    starpu_gb300.build()
    exe = os.path.join(ROOT, "starpu_gb300", "lib", "chol_implicit_gb300")
    e = dict(os.environ)
    e.update({k: str(v) for k, v in env.items()})
    r = subprocess.run([exe, *args], env=e, capture_output=True, text=True, timeout=600)
    stats = dict(re.findall(r"(\w+)=([\d.]+)", r.stderr))
    return r, stats


@pytest.mark.parametrize("mode", ["graph", "per_task", "with_cpu_workers"])
@pytest.mark.parametrize("args", [["-size", "2048", "-nblocks", "8"], ["-size", "1000", "-nblocks", "7"],
                                  ["-size", "1536", "-nblocks", "6", "-double"], ["-size", "333", "-nblocks", "5", "-double"]])
def test_tiled_cholesky_through_the_runtime(mode, args):
    env = {"graph": dict(STARPU_NCPU=0), "per_task": dict(STARPU_NCPU=0, STARPU_GB300_GRAPH=0),
           "with_cpu_workers": dict(STARPU_NCPU=2)}[mode]
    r, st = run_driver(args + ["-check"], **env)
    assert r.returncode == 0, r.stdout + r.stderr
    nb = int(args[3])
    ntasks = nb + nb * (nb - 1) // 2 * 2 + nb * (nb - 1) * (nb - 2) // 6
    if mode == "graph":
        assert int(st["graph"]) == ntasks and int(st["graphs"]) >= 1
    else:
        assert int(st["cuda"]) == ntasks and int(st["graph"]) == 0
    assert re.search(r"^\d+\t\d+\t[\d.]+$", r.stdout, re.M)


@pytest.mark.parametrize("prec", [[], ["-double"]])
def test_indefinite_input_reported_by_status_word(prec):
    # pivot 300 lies in tile 2 of 4 (tile size 128); the tile's status is
    # relative to its diagonal block: 300 - 256 + 1 = 45
    r, _ = run_driver(["-size", "512", "-nblocks", "4", "-break", "300", *prec], STARPU_NCPU=0)
    assert r.returncode == 2, r.stdout + r.stderr
    assert "leading minor 45" in r.stderr
    # and the device is still usable: a normal run afterwards succeeds
    r2, _ = run_driver(["-size", "512", "-nblocks", "4", "-check", *prec], STARPU_NCPU=0)
    assert r2.returncode == 0, r2.stdout + r2.stderr


@pytest.mark.parametrize("mode", ["graph", "per_task"])
def test_tensor_core_tiles_through_the_runtime(mode):
    """The codelets' FP32 GEMM/SYRK tiles on the tensor cores (forced down to
    256-tiles): the driver's check holds and the factorisation is the same
    DAG."""
    env = {"graph": dict(STARPU_NCPU=0), "per_task": dict(STARPU_NCPU=0, STARPU_GB300_GRAPH=0)}[mode]
    r, st = run_driver(["-size", "2048", "-nblocks", "8", "-check"], STARPU_GB300_CHOL_TC_MIN=256, **env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert re.search(r"^\d+\t\d+\t[\d.]+$", r.stdout, re.M)
