"""The tiled LU through the StarPU-API runtime with the GB300 LU codelets on
the GPU (starpu_gb300/csrc/examples/lu_gb300.c, the DAG of the reference's
xlu_implicit.c / xlu_implicit_pivot.c): as one CUDA graph per DAG, task by
task, with CPU workers present, and with threshold pivoting (which runs task
by task: its GETRF_PIVOT fills a host pivot record).  The driver checks
||A P - L U|| / (||A|| n) <= 1e-4, the reference's bound."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_lu(args, **env):
    import starpu_gb300
    starpu_gb300.build()
    exe = os.path.join(ROOT, "starpu_gb300", "lib", "lu_gb300")
    e = dict(os.environ)
    e.update({k: str(v) for k, v in env.items()})
    r = subprocess.run([exe, *args], env=e, capture_output=True, text=True, timeout=600)
    stats = dict(re.findall(r"(\w+)=([\d.]+)", r.stderr))
    return r, stats


def ntasks(nb, piv):
    return nb + nb * (nb - 1) + sum((nb - k - 1) ** 2 for k in range(nb)) + (nb * (nb - 1) if piv else 0)


@pytest.mark.parametrize("prec", [[], ["-double"]])
@pytest.mark.parametrize("mode", ["graph", "per_task", "with_cpu_workers"])
def test_lu_through_the_runtime(prec, mode):
    env = {"graph": dict(STARPU_NCPU=0), "per_task": dict(STARPU_NCPU=0, STARPU_GB300_GRAPH=0),
           "with_cpu_workers": dict(STARPU_NCPU=2)}[mode]
    r, st = run_lu(["-size", "1920", "-nblocks", "4", "-check", *prec], **env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 pivoting steps" in r.stderr
    if mode == "graph":
        assert int(st["graph"]) == ntasks(4, False)
    else:
        assert int(st["cuda"]) == ntasks(4, False)
    assert re.search(r"^1920\t[\d.]+\t[\d.]+$", r.stdout, re.M)


@pytest.mark.parametrize("prec", [[], ["-double"]])
def test_lu_with_threshold_pivoting(prec):
    r, st = run_lu(["-size", "1024", "-nblocks", "4", "-check", "-piv", "-small-pivots", *prec], STARPU_NCPU=0)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"\((\d+) pivoting steps\)", r.stderr)
    assert m and int(m.group(1)) > 0, r.stderr
    assert int(st["cuda"]) == ntasks(4, True)


def test_lu_pivot_mode_without_small_pivots_matches_plain():
    r, _ = run_lu(["-size", "1024", "-nblocks", "8", "-check", "-piv"], STARPU_NCPU=0)
    assert r.returncode == 0 and "0 pivoting steps" in r.stderr, r.stdout + r.stderr
