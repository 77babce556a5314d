"""The StarPU-API runtime of libstarpu_gb300.so on CPU workers.

* tests/c/test_runtime.c: implicit dependencies, filters, tags, values,
  callbacks, -ENODEV, history perfmodels, scheduling contexts, task fault
  tolerance (default retry policy), end dependencies, commuting writers and
  vector partitions (no GPU needed).
* The reference's own, unchanged examples/cholesky/cholesky_implicit.c
  compiled against include/ and linked with this runtime (oracle/Makefile
  `ref-driver`): with the reference's CPU codelets it must pass the
  reference's -check (config 1: N=2048, 8x8 tiles); with the GB300 codelet
  library and no GPU it must report "skipped" (exit 77) like the reference.
  Likewise cholesky_tag.c, cholesky_tile_tag.c, cholesky_grain_tag.c and
  cholesky_compil.c on the reference's CPU codelets.
"""
import os
import re
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.REF_TREE  # STARPU_REFERENCE_TREE, else the oracle recipe's location


def _lib():
    import starpu_gb300
    starpu_gb300.build()
    return os.path.join(ROOT, "starpu_gb300", "lib")


def _env(**kw):
    e = dict(os.environ)
    e.update({k: str(v) for k, v in kw.items()})
    return e


@pytest.fixture(scope="module")
def runtime_test_binary(tmp_path_factory):
    libdir = _lib()
    out = tmp_path_factory.mktemp("rt") / "test_runtime"
    subprocess.run(["gcc", "-std=gnu11", "-O1", "-g", "-o", str(out), os.path.join(ROOT, "tests", "c", "test_runtime.c"),
                    "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", "-L" + libdir,
                    "-lstarpu_gb300", "-Wl,-rpath," + libdir, "-lm", "-lpthread"], check=True)
    return str(out)


@pytest.mark.parametrize("ncpu", [1, 4])
def test_runtime_c_suite(runtime_test_binary, tmp_path, ncpu):
    # the tile task runs for about a microsecond: timer noise alone breaks the
    # 50 % outlier rule, so the rule is widened for the calibration check
    r = subprocess.run([runtime_test_binary], env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu, STARPU_PERF_MODEL_DIR=tmp_path,
                                                         STARPU_HOSTNAME="testhost", STARPU_HISTORY_MAX_ERROR=100000),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout + r.stderr
    assert (tmp_path / "codelets" / "45" / "gb300_test_tile_inc.testhost").exists()


def test_worker_stats_at_shutdown(runtime_test_binary, tmp_path):
    """STARPU_WORKER_STATS=1 prints, at shutdown, the tasks each worker ran
    (profiling_helpers.c:88-181 without per-task profiling)."""
    out = tmp_path / "stats.txt"
    r = subprocess.run([runtime_test_binary], env=_env(STARPU_NCUDA=0, STARPU_NCPU=2, STARPU_PERF_MODEL_DIR=tmp_path,
                                                         STARPU_HISTORY_MAX_ERROR=100000, STARPU_WORKER_STATS=1,
                                                         STARPU_WORKER_STATS_FILE=out),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    text = out.read_text()
    assert text.startswith("\n#---------------------\nWorker stats:\n") and text.endswith("#---------------------\n")
    counts = [int(c) for c in re.findall(r"^\t(\d+) task\(s\)$", text, re.M)]
    names = re.findall(r"^(CPU \d+) *$", text, re.M)
    assert names == ["CPU 0", "CPU 1"] and len(counts) == 2 and sum(counts) > 100, text


def _ref_driver(target):
    if not os.path.isdir(os.path.join(REF, "examples", "cholesky")):
        pytest.skip("reference tree not available on this machine")
    _lib()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", target], check=True)
    return os.path.join(ROOT, "oracle", target)


# Sizes divisible by nblocks: the reference's CPU TRSM codelet passes m = NY,
# n = NX to STRSM (examples/cholesky/cholesky_kernels.c:244-254), which is only
# right for square tiles, so ragged tilings fail its own -check.  (The GB300
# codelets pass the true dimensions; ragged tilings are covered on the GPU.)
@pytest.mark.parametrize("args", [["-size", "2048", "-nblocks", "8", "-check"],
                                  ["-size", "1008", "-nblocks", "7", "-check", "-no-prio"],
                                  ["-size", "960", "-nblocks", "6", "-check", "-niter", "3"],
                                  ["-size", "512", "-nblocks", "4", "-check", "-commute"],
                                  ["-size", "768", "-nblocks", "6", "-check", "-priority", "3"]])
def test_unchanged_reference_driver_on_cpu_workers(args):
    exe = _ref_driver("_ref/cholesky_implicit_cpu")
    r = subprocess.run([exe, *args], env=_env(STARPU_NCUDA=0, STARPU_NCPU=4), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"^(\d+)\t(\d+)\t([\d.]+)", r.stdout, re.M)
    assert m and int(m.group(1)) == int(args[1]) and float(m.group(3)) > 0, r.stdout


def test_unchanged_tile_tag_driver_explicit_tag_dependencies():
    """cholesky_tile_tag.c: tasks built with starpu_task_create, dependencies
    only through starpu_tag_declare_deps (default sequential consistency off)."""
    exe = _ref_driver("_ref/cholesky_tile_tag_cpu")
    for ncpu in (1, 4):
        r = subprocess.run([exe, "-size", "2048", "-nblocks", "8", "-check"], env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu),
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert re.search(r"^2048\t\d+\t[\d.]+", r.stdout, re.M)


def test_unchanged_tag_driver_entry_task_submitted_last():
    """cholesky_tag.c submits POTRF(0) last: every other task waits for its tag
    before that task exists.  Its own -check is not used: its GEMM task passes
    the operands as (A_nk, A_mk) (examples/cholesky/cholesky_tag.h:145-146),
    i.e. computes C_mn -= A_nk A_mk^T, and the reference's 1e-4 check fails on
    a few elements by a hair for every worker count; the run itself must
    complete and be identical for 1 and 4 workers."""
    exe = _ref_driver("_ref/cholesky_tag_cpu")
    outs = []
    for ncpu in (1, 4):
        r = subprocess.run([exe, "-size", "1024", "-nblocks", "8", "-check"], env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu),
                           capture_output=True, text=True, timeout=300)
        m = re.search(r"Error\[(\d+), (\d+)\] --> ([\d.]+)", r.stderr)
        outs.append(m.groups() if m else None)
    assert outs[0] is not None and outs[0] == outs[1], outs


@pytest.mark.parametrize("args", [["-size", "2048", "-nblocks", "8", "-check"],
                                  ["-size", "960", "-nblocks", "6", "-check", "-no-prio"]])
def test_unchanged_compil_driver_on_cpu_workers(args):
    """cholesky_compil.c: the tile DAG written as an externally generated loop
    nest (cholesky_compiled.c), submitted with starpu_task_insert; it must
    pass the reference's own -check."""
    exe = _ref_driver("_ref/cholesky_compil_cpu")
    for ncpu in (1, 4):
        r = subprocess.run([exe, *args], env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu), capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "comparing results" in r.stderr and "Error[" not in r.stderr
        assert re.search(rf"^{args[1]}\t\d+\t[\d.]+", r.stdout, re.M), r.stdout


@pytest.mark.parametrize("nbigblocks", [8, 4, 2])
def test_unchanged_grain_tag_driver_refines_the_trailing_matrix(nbigblocks):
    """cholesky_grain_tag.c: a tag DAG over 8 x 8 tiles for the first
    `nbigblocks` steps; the trailing matrix is then unpartitioned,
    unregistered, registered again in place (a sub-matrix of the same host
    array, ld = N) and factored with twice as many tiles per dimension.
    Its GEMM task has cholesky_tag.h's operand order (A_nk, A_mk), so the
    reference's 1e-4 check stops at its first element over the threshold by a
    hair, as for cholesky_tag.c; a wrong partition or a lost write-back would
    miss by orders of magnitude.  The run must otherwise complete, and its
    result must not depend on the worker count."""
    exe = _ref_driver("_ref/cholesky_grain_tag_cpu")
    outs = []
    for ncpu in (1, 4):
        r = subprocess.run([exe, "-size", "1024", "-nblocks", "8", "-nbigblocks", str(nbigblocks), "-check"],
                           env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu), capture_output=True, text=True, timeout=300)
        assert "comparing results" in r.stderr, r.stdout + r.stderr
        m = re.search(r"Error\[(\d+), (\d+)\] --> ([\d.]+) != ([\d.]+) \(err ([\d.]+)\)", r.stderr)
        if m:
            assert float(m.group(5)) < 2e-4, m.group(0)
        else:
            assert r.returncode == 0, r.stdout + r.stderr
        outs.append(m.groups() if m else None)
    assert outs[0] == outs[1], outs


@pytest.mark.parametrize("size", [1024, 2048])
def test_unchanged_grain_tag_driver_exact_check_through_the_refinement(size):
    """With 2 x 2 tiles and one coarse step every update is a SYRK (no GEMM
    between different tiles), so the operand order above never enters: the
    reference's own check must pass everywhere, including the trailing half
    that was unregistered, registered again as a sub-matrix and factored as
    2 x 2 finer tiles."""
    exe = _ref_driver("_ref/cholesky_grain_tag_cpu")
    for ncpu in (1, 4):
        r = subprocess.run([exe, "-size", str(size), "-nblocks", "2", "-nbigblocks", "1", "-check"],
                           env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu), capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "comparing results" in r.stderr and "Error[" not in r.stderr
        assert re.search(rf"^{size}\t\d+\t[\d.]+", r.stdout, re.M), r.stdout


@pytest.mark.parametrize("mode,nbench", [("-with_ctxs", 2), ("-with_noctxs", 2), ("-chole1", 1), ("-chole2", 1)])
def test_unchanged_driver_scheduling_contexts(mode, nbench):
    """cholesky_implicit.c's context modes (examples/sched_ctx_utils): two
    factorisations in two threads, each in its own context of two CPU
    workers (-with_ctxs; the first to finish hands its workers to the other,
    its inheritor), both in the initial context (-with_noctxs), or one of
    them alone (-chole1, -chole2).  Every factorisation must run (positive
    GFlop/s on the summary line)."""
    exe = _ref_driver("_ref/cholesky_implicit_cpu")
    sizes = ["-size1", "1024", "-nblocks1", "8", "-size2", "1024", "-nblocks2", "8"]
    r = subprocess.run([exe, mode, "-cpu1", "2", "-cpu2", "2", *sizes], env=_env(STARPU_NCUDA=0, STARPU_NCPU=4),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nums = [float(x) for x in r.stdout.strip().splitlines()[-1].split()]
    assert len(nums) == nbench + nbench + 1 and all(g > 0 for g in nums[:nbench]), r.stdout


def test_unchanged_driver_empty_contexts_submit_nothing():
    """Without -cpu1/-cpu2 the driver's two contexts hold no worker: every
    submission is refused with -ENODEV (workers.c _starpu_worker_exists), the
    driver skips the factorisations and reports 0 GFlop/s for both."""
    exe = _ref_driver("_ref/cholesky_implicit_cpu")
    r = subprocess.run([exe, "-with_ctxs", "-size1", "512", "-nblocks1", "4", "-size2", "512", "-nblocks2", "4"],
                       env=_env(STARPU_NCUDA=0, STARPU_NCPU=4), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nums = [float(x) for x in r.stdout.strip().splitlines()[-1].split()]
    assert nums[:2] == [0.0, 0.0], r.stdout


@pytest.mark.parametrize("ncpu", [1, 4])
def test_unchanged_fault_tolerance_retry_test(ncpu):
    """StarPU's own tests/fault-tolerance/retry.c, compiled unchanged (oracle
    recipe `ref-ft`): its task reports a failure ten times through
    starpu_task_ft_failed; starpu_task_ft_prologue and the test's check_ft
    callback resubmit it without dependencies until it succeeds, while the
    meta task holds the data.  x must stay 12 and y become 13."""
    if not os.path.isfile(os.path.join(REF, "tests", "fault-tolerance", "retry.c")):
        pytest.skip("reference tree not available on this machine")
    _lib()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "_ref/ft_retry_ref"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ft_retry_ref")
    r = subprocess.run([exe], env=_env(STARPU_NCUDA=0, STARPU_NCPU=ncpu), capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stderr.count("failing\n") == 10 and r.stderr.count("succeed\n") == 1, r.stderr
    assert "Value x = 12 (expected 12)" in r.stderr and "Value y = 13 (expected 13)" in r.stderr, r.stderr


def test_unchanged_reference_driver_links_gb300_codelets():
    exe = _ref_driver("_ref/cholesky_implicit_gb300")
    r = subprocess.run([exe, "-size", "256", "-nblocks", "2"], env=_env(STARPU_NCUDA=0, STARPU_NCPU=2),
                       capture_output=True, text=True, timeout=120)
    # CUDA-only codelets and no CUDA worker: starpu_task_insert returns -ENODEV,
    # _cholesky returns 77 and the reference's execute_cholesky ignores it
    # (cholesky_implicit.c:527), so the driver exits 0 without a timing line
    assert r.returncode == 0, r.stdout + r.stderr
    assert "GFlops" not in r.stdout


def test_gb300_driver_without_gpu_reports_skipped():
    libdir = _lib()
    r = subprocess.run([os.path.join(libdir, "chol_implicit_gb300"), "-size", "256", "-nblocks", "2"],
                       env=_env(STARPU_NCUDA=0, STARPU_NCPU=2), capture_output=True, text=True, timeout=120)
    assert r.returncode == 77, r.stdout + r.stderr


# The reference's unchanged LU drivers (examples/lu: lu_example.c with the
# implicit-dependency and the tag-based DAGs, xlu_implicit*.c / xlu*.c) and its
# CPU codelets on this runtime's CPU workers: each must pass its own check
# ||PA - LU|| / (||A|| N) <= PIVOT_THRESHHOLD (lu_example.c, check_result).
@pytest.mark.parametrize("prog", ["lu_implicit_float", "lu_tag_float", "lu_implicit_double", "lu_tag_double"])
@pytest.mark.parametrize("mode", [[], ["-piv"], ["-piv", "-no-stride"]])
def test_unchanged_reference_lu_drivers_on_cpu_workers(prog, mode):
    if not os.path.isdir(os.path.join(REF, "examples", "lu")):
        pytest.skip("reference tree not available on this machine")
    _lib()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "_ref/" + prog], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", prog)
    r = subprocess.run([exe, "-size", "768", "-nblocks", "4", "-check", *mode], env=_env(STARPU_NCUDA=0, STARPU_NCPU=4),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"\|\|P?A-LU\|\| / \(\|\|A\|\|\*N\) : ([0-9.e+-]+)", r.stderr)
    assert m and float(m.group(1)) <= 1e-6, r.stderr


@pytest.mark.parametrize("prog", ["lu_implicit_gb300_float", "lu_implicit_gb300_double"])
@pytest.mark.parametrize("mode", [[], ["-piv"]])
def test_unchanged_reference_lu_driver_links_gb300_lu_codelets(prog, mode):
    """The unchanged LU drivers link libstarpu_gb300_lu.so in place of
    xlu_kernels.c (every codelet, handle and init/fini symbol resolves).  Its
    codelets are CUDA-only, so without a CUDA worker every submit returns
    -ENODEV and the driver exits 77 (lu_example.c:537)."""
    if not os.path.isdir(os.path.join(REF, "examples", "lu")):
        pytest.skip("reference tree not available on this machine")
    _lib()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "_ref/" + prog], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", prog)
    r = subprocess.run([exe, "-size", "256", "-nblocks", "2", *mode], env=_env(STARPU_NCUDA=0, STARPU_NCPU=2),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 77, r.stdout + r.stderr
