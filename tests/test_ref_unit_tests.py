"""StarPU's own unit tests of the task, tag and data API, unchanged, on this
runtime's CPU workers (tests/main and tests/datawizard of the reference:
insert_task, explicit task dependencies declared before or after the
predecessors' submission and from callbacks, tags, regenerated, restarted
and synchronous tasks, empty tasks as sync points, vector partitions,
readers/writers,
commuting writers (unordered among themselves, also against explicit
dependencies), void handles, pause/resume, tasks pinned to a worker, task
fault tolerance).  oracle/Makefile `ref-unit-tests` compiles each one
against include/ and links it with libstarpu_gb300.so; each must exit 0.

Not in the list: tests of what this runtime does not have (OpenCL/HIP
workers, NUMA nodes, memory reclaiming, hwloc, asynchronous partitioning,
reductions, more than STARPU_NMAXBUFS buffers per task), main/deadlock (a dependency cycle
that hangs by design), and main/tag_task_data_deps (passes, in about a
minute)."""
import os
import re
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.REF_TREE


def _tests():
    with open(os.path.join(ROOT, "oracle", "Makefile")) as f:
        text = f.read()
    m = re.search(r"^REF_UNIT_TESTS :=(.*?)^ref-unit-tests:", text, re.S | re.M)
    return m.group(1).replace("\\", " ").split()


TESTS = _tests()


@pytest.fixture(scope="module")
def built():
    if not os.path.isdir(os.path.join(REF, "tests", "main")):
        pytest.skip("reference tree not available on this machine")
    import starpu_gb300
    starpu_gb300.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "ref-unit-tests"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "tests")


def test_list_is_not_empty():
    assert len(TESTS) >= 30


@pytest.mark.parametrize("name", TESTS)
def test_reference_unit_test_passes(built, name, tmp_path):
    exe = os.path.join(built, name.replace("/", "_"))
    env = dict(os.environ, STARPU_NCUDA="0", STARPU_NCPU="4", STARPU_HOME=str(tmp_path),
               STARPU_PERF_MODEL_DIR=str(tmp_path / "models"))
    r = subprocess.run([exe], env=env, capture_output=True, text=True, timeout=120, cwd=tmp_path)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
