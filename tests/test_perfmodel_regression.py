"""Regression-based and cost-function performance models on CPU.

* The runtime (rt_perfmodel.c, through tests/c/test_perfmodel_regression.c):
  linear and non-linear regression models record, predict, save and reload
  as the oracle's restatement of perfmodel_history.c and regression.c says;
  common, per-arch and per-worker models predict from their cost functions,
  and the scheduler places a task by its per-worker cost.
* The oracle's non-linear fit (perfmodel_oracle.nl_power_fit) is pinned to
  StarPU's own src/core/perfmodel/regression.c, compiled unchanged into
  oracle/_ref where the reference tree is present.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from oracle import perfmodel_oracle as PO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.REF_TREE

DIMS = [16, 24, 32, 48, 64, 96, 128]
SIZES = [4 * n * n for n in DIMS]                 # float n x n tiles
LIN_US = [26, 53, 89, 185, 310, 644, 1081]       # the C program's tables
NL_US = [14, 20, 29, 56, 96, 221, 407]


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    import importlib
    B = importlib.import_module("starpu_gb300.build")
    B.build()
    d = tmp_path_factory.mktemp("pmreg")
    exe = d / "test_perfmodel_regression"
    subprocess.run(["gcc", "-std=gnu11", "-O1", "-g", "-Wall", "-o", str(exe),
                    os.path.join(ROOT, "tests", "c", "test_perfmodel_regression.c"),
                    "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", "-L" + B.LIBDIR,
                    "-lstarpu_gb300", "-Wl,-rpath," + B.LIBDIR, "-lm", "-lpthread"], check=True)
    env = dict(os.environ)
    env.update(STARPU_PERF_MODEL_DIR=str(d / "models"), STARPU_HOME=str(d / "home"), STARPU_HOSTNAME="pmhost",
               STARPU_NCUDA="0", STARPU_NCPU="2")
    env.pop("STARPU_PERF_MODEL_PATH", None)
    r = subprocess.run([str(exe)], env=env, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("ALL OK"), r.stdout + r.stderr
    out = dict(l.split(" ", 1) for l in r.stdout.splitlines() if " " in l)
    out["_env"] = env
    out["_display"] = B.example_path("starpu_perfmodel_display")
    return out


def _model(path):
    with open(path) as f:
        text = f.read()
    m = PO.parse(text, PO.Registry())
    (pa,) = m.impls[m.combs[0]]
    return pa


def _e(x):
    return float(f"{x:e}")  # the file holds %e values


def test_linear_regression_records_and_predicts(run):
    o = PO.RegressionSums()
    for s, us in zip(SIZES, LIN_US):
        for _ in range(3):
            o.record(s, us)
    assert o.valid
    assert float(run["LIN_IN"]) == o.predict(4 * 64 * 64)
    assert math.isnan(float(run["LIN_OUT"])) and math.isnan(o.predict(4 * 256 * 256))
    pa = _model(run["LIN_PATH"])
    assert (pa.sumlnx, pa.sumlnx2, pa.sumlny, pa.sumlnxlny, pa.alpha, pa.beta) == \
        tuple(map(_e, (o.sumlnx, o.sumlnx2, o.sumlny, o.sumlnxlny, o.alpha, o.beta)))
    assert (pa.nsample, pa.minx, pa.maxx) == (21, 1024, 65536)
    assert math.isnan(pa.a) and math.isnan(pa.b) and math.isnan(pa.c)
    # the fit agrees with an ordinary least-squares line through the logs
    beta, lnalpha = np.polyfit(np.log(np.repeat(SIZES, 3)), np.log(np.repeat(LIN_US, 3)), 1)
    assert abs(beta - o.beta) < 1e-12 and abs(math.exp(lnalpha) - o.alpha) < 1e-12 * o.alpha
    # entries: a regression model keeps the first call of each size
    assert sorted((e.size, e.nsample, e.mean) for e in pa.entries) == [(s, 3, float(u)) for s, u in zip(SIZES, LIN_US)]
    # a runtime reload predicts from the file's fit
    assert float(run["LIN_RELOAD"]) == pa.alpha * math.pow(4 * 64 * 64, pa.beta)


def test_nonlinear_regression_fit_at_save(run):
    assert float(run["NL_BEFORE_FIT"]) == 96.0   # the entry's mean until a fit is loaded
    pa = _model(run["NL_PATH"])
    assert sorted((e.size, e.nsample, e.mean) for e in pa.entries) == [(s, 12, float(u)) for s, u in zip(SIZES, NL_US)]
    # the writer fits over its list, which is the file's entry order
    points = [(e.size, e.mean, e.nsample) for e in reversed(pa.entries)]
    a, b, c = PO.nl_power_fit(points)
    assert (pa.a, pa.b, pa.c) == (_e(a), _e(b), _e(c))
    assert abs(b - 1.1) < 0.01 and abs(c - 10) < 1.0   # the tables follow 2e-3 size^1.1 + 10
    o = PO.RegressionSums()
    for s, us in zip(SIZES, NL_US):
        for _ in range(12):
            o.record(s, us)
    assert (pa.sumlnx, pa.alpha, pa.beta, pa.nsample) == (_e(o.sumlnx), _e(o.alpha), _e(o.beta), 84)
    size = 4 * 64 * 64
    assert float(run["NL_RELOAD"]) == PO.nl_predict(pa.a, pa.b, pa.c, pa.minx, pa.maxx, size)
    assert math.isnan(float(run["NL_OUT"]))


@pytest.mark.parametrize("symbol,path_key", [("gb300_test_perfmodel_lreg", "LIN_PATH"),
                                             ("gb300_test_perfmodel_nlreg", "NL_PATH")])
@pytest.mark.parametrize("args,kw", [([], {}), (["-p", "alpha"], {"parameter": "alpha"}),
                                     (["-p", "beta"], {"parameter": "beta"}), (["-p", "a"], {"parameter": "a"}),
                                     (["-p", "c"], {"parameter": "c"})])
def test_display_tools_print_the_regression_models(run, symbol, path_key, args, kw):
    """The GB300 display tool, and StarPU's own tool compiled unchanged against
    this runtime where the reference tree is present, print the runtime's
    regression models as the oracle reads them."""
    with open(run[path_key]) as f:
        text = f.read()
    reg = PO.Registry()
    m = PO.parse(text, reg)
    want = PO.print_all(m, reg, **kw)
    t = subprocess.run([run["_display"], "-s", symbol, *args], env=run["_env"], capture_output=True, text=True,
                       timeout=60)
    assert t.returncode == 0, t.stderr
    assert t.stdout == want
    if os.path.isfile(os.path.join(REF, "tools", "starpu_perfmodel_display.c")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "ref-tools"], check=True)
        ref = os.path.join(ROOT, "oracle", "_ref", "starpu_perfmodel_display_ref")
        r = subprocess.run([ref, "-s", symbol, *args], env=run["_env"], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        assert r.stdout == want


def test_cost_function_models(run):
    speedup = PO.relative_speedup([("cpu", int(run["CPU_CORES"]))])
    assert float(run["SPEEDUP"]) == speedup
    assert float(run["COMMON"]) == 1000.0 / speedup
    assert float(run["PER_ARCH"]) == 4.0
    assert run["PER_WORKER_RAN_ON"] == "1"


# ------------------------------------------------- the oracle's fit, pinned


class _HEntry(C.Structure):
    _fields_ = [("mean", C.c_double), ("size", C.c_size_t), ("nsample", C.c_uint)]


class _HList(C.Structure):
    pass


_HList._fields_ = [("next", C.POINTER(_HList)), ("entry", C.POINTER(_HEntry))]


def _ref_fit(lib, points):
    keep = []
    head = None
    for size, mean, n in reversed(points):
        e = _HEntry(mean, size, n)
        node = _HList(head, C.pointer(e))
        keep += [e, node]
        head = C.pointer(node)
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    rc = lib._starpu_regression_non_linear_power(head, C.byref(a), C.byref(b), C.byref(c))
    return None if rc != 0 else (a.value, b.value, c.value)


def _same(x, y):
    return x == y or (math.isnan(x) and math.isnan(y))


def test_oracle_nl_fit_matches_the_reference_regression_c():
    src = os.path.join(REF, "src", "core", "perfmodel", "regression.c")
    if not os.path.isfile(src):
        pytest.skip("reference tree not available on this machine")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "ref-regression"], check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_regression.so"))
    lib._starpu_regression_non_linear_power.argtypes = [C.POINTER(_HList)] + [C.POINTER(C.c_double)] * 3
    lib._starpu_regression_non_linear_power.restype = C.c_int
    rng = np.random.default_rng(45)
    cases = [[(s, float(u), 12) for s, u in zip(SIZES, NL_US)],
             [(s, 3e-3 * s ** 0.8 + 40, 12) for s in SIZES],          # every weight vanishes: NaN fit
             [(1024, 5.0, 0), (4096, 9.0, 3)],                         # an entry without samples is skipped
             [(4096, 7.0, 0)],                                          # nothing to fit
             [(1024, 0.0, 5), (2048, 0.0, 5), (4096, 1.0, 5)],          # c stays 0: 0/0 weights
             [(1024, 2.0, 1), (1024, 3.0, 2), (1024, 4.0, 1)]]          # one size: no slope
    for _ in range(40):
        k = int(rng.integers(2, 12))
        sizes = np.sort(rng.choice(np.arange(256, 1 << 22), size=k, replace=False))
        a, b, c = 10 ** rng.uniform(-4, -1), rng.uniform(0.5, 1.6), rng.uniform(0, 50)
        noise = 1 + 0.05 * rng.standard_normal(k)
        cases.append([(int(s), float((a * s ** b + c) * z), int(rng.integers(0, 20))) for s, z in zip(sizes, noise)])
    for pts in cases:
        want = _ref_fit(lib, pts)
        got = PO.nl_power_fit(pts)
        if want is None:
            assert got is None, pts
            continue
        assert all(_same(x, y) for x, y in zip(got, want)), (pts, got, want)
