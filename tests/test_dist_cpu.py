"""bench.py's multi-GPU path on CPU: two gloo ranks (one process each, as
torchrun starts them) share nothing but a barrier and the max over ranks of
the step time; the whole-job value is the ranks' total work over that max.
The reference arm runs on rank 0 only: the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys, time
sys.path.insert(0, os.environ["BENCH_ROOT"])
import bench
world, rank, local = bench.dist_setup()
d = bench.Dist(world, local)
d.barrier()
t0 = time.perf_counter()
time.sleep(0.05 * (rank + 1))          # rank 1 is the slower replica
d.barrier()
ms = d.max((time.perf_counter() - t0) * 1e3)
mine = d.max(float(rank + 10))
d.close()
print(json.dumps({"rank": rank, "world": world, "max_ms": ms, "max_rank_value": mine}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_barrier_and_max():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, CUDA_VISIBLE_DEVICES="", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), BENCH_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert [o["rank"] for o in outs] == [0, 1] and all(o["world"] == 2 for o in outs)
    # both ranks hold the same maximum, which is the slower replica's time
    assert outs[0]["max_ms"] == outs[1]["max_ms"] >= 100.0
    assert outs[0]["max_rank_value"] == outs[1]["max_rank_value"] == 11.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
