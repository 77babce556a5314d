"""Perfmodel files and tools on CPU: the runtime's version-45 reader/writer and
its starpu_perfmodel_display / starpu_perfmodel_plot tools, checked against
the Python restatement in oracle/perfmodel_oracle.py on a committed fixture,
on a model the runtime itself records, and (where the reference tree is
present) on every sample model StarPU ships and against StarPU's own display
tool compiled unchanged against this runtime."""
import os
import subprocess
import xml.etree.ElementTree as ET

import pytest

from oracle import oracle as O

from oracle import perfmodel_oracle as PO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE_DIR = os.path.join(ROOT, "tests", "golden", "perfmodel")
FIXTURE = "gb300_fixture_model.fixturehost"
REF = O.REF_TREE  # STARPU_REFERENCE_TREE, else the oracle recipe's location
REF_SAMPLES = os.path.join(REF, "tools", "perfmodels", "sampling")


@pytest.fixture(scope="module")
def tools():
    import importlib
    B = importlib.import_module("starpu_gb300.build")
    B.build()
    return {t: B.example_path(t) for t in B.TOOLS}


def _env(tmp_path, model_dir, **kw):
    e = dict(os.environ)
    e.update(STARPU_PERF_MODEL_DIR=str(model_dir), STARPU_HOME=str(tmp_path / "home"), STARPU_HOSTNAME="pmhost")
    e.pop("STARPU_PERF_MODEL_PATH", None)
    e.update({k: str(v) for k, v in kw.items()})
    return e


def _run(exe, args, env, cwd=None):
    r = subprocess.run([exe, *args], env=env, capture_output=True, text=True, timeout=60, cwd=cwd)
    return r


def _fixture_text():
    with open(os.path.join(FIXTURE_DIR, "codelets", "45", FIXTURE)) as f:
        return f.read()


VARIANTS = [([], {}), (["-a", "cpu"], {"arch": "cpu"}), (["-a", "cuda"], {"arch": "cuda"}),
            (["-a", "cuda0"], {"arch": "cuda0"}), (["-p", "mean"], {"parameter": "mean"}),
            (["-p", "stddev"], {"parameter": "stddev"}), (["-a", "cuda", "-p", "alpha"], {"arch": "cuda", "parameter": "alpha"}),
            (["-a", "cuda", "-p", "c"], {"arch": "cuda", "parameter": "c"}),
            (["-f", "0000beef"], {"footprint": 0xbeef})]


@pytest.mark.parametrize("args,kw", VARIANTS)
def test_display_fixture_matches_oracle(tools, tmp_path, args, kw):
    r = _run(tools["starpu_perfmodel_display"], ["-s", FIXTURE, *args], _env(tmp_path, FIXTURE_DIR))
    assert r.returncode == 0, r.stderr
    reg = PO.Registry()
    m = PO.parse(_fixture_text(), reg)
    assert r.stdout == PO.print_all(m, reg, **kw)


def test_display_fixture_xml(tools, tmp_path):
    r = _run(tools["starpu_perfmodel_display"], ["-x", "-s", FIXTURE], _env(tmp_path, FIXTURE_DIR))
    assert r.returncode == 0, r.stderr
    root = ET.fromstring(r.stdout.split("\n", 2)[2])  # past the XML declaration and doctype
    reg = PO.Registry()
    m = PO.parse(_fixture_text(), reg)
    combs = root.findall("combination")
    assert len(combs) == len(m.combs)
    for c, cid in zip(combs, m.combs):
        impls = c.findall("implementation")
        assert len(impls) == len(m.impls[cid])
        for im, pa in zip(impls, m.impls[cid]):
            got = [(int(e.get("footprint"), 16), int(e.get("size")), float(e.get("mean")), int(e.get("nsample")))
                   for e in im.findall("entry")]
            assert got == [(e.footprint, e.size, float(f"{e.mean:e}"), e.nsample) for e in pa.entries]


def test_display_dir_list_and_missing(tools, tmp_path):
    env = _env(tmp_path, FIXTURE_DIR)
    r = _run(tools["starpu_perfmodel_display"], ["-d"], env)
    assert r.stdout.splitlines() == [f"directory: <{FIXTURE_DIR}/codelets/45/>",
                                     f"directory: <{tmp_path}/home/.starpu/sampling/codelets/45/>"]
    r = _run(tools["starpu_perfmodel_display"], ["-l"], env)
    assert f"codelet directory: <{FIXTURE_DIR}/codelets/45/>" in r.stdout and f"file: <{FIXTURE}>" in r.stdout
    r = _run(tools["starpu_perfmodel_display"], ["-s", "no_such_symbol"], env)
    assert r.returncode == 1 and "could not be loaded" in r.stderr
    r = _run(tools["starpu_perfmodel_display"], [], env)
    assert r.returncode != 0 and "Incorrect usage" in r.stderr


def test_plot_fixture(tools, tmp_path):
    out = tmp_path / "plots"
    out.mkdir()
    r = _run(tools["starpu_perfmodel_plot"], ["-s", FIXTURE, "-o", str(out)], _env(tmp_path, FIXTURE_DIR))
    assert r.returncode == 0, r.stderr
    gp = (out / f"starpu_{FIXTURE}.gp").read_text()
    avg = out / f"starpu_{FIXTURE}_avg.data"
    assert gp.startswith("#!/usr/bin/gnuplot -persist\n")
    assert f'set output "starpu_{FIXTURE}.eps"' in gp and 'set ylabel "Time (ms)"' in gp
    assert 'title "Linear Regression cuda0_cores1_impl0 (Comb1)"' not in gp  # nl-valid: only the NL curve
    assert 'title "Non-Linear Regression cuda0_cores1_impl0 (Comb1)"' in gp
    assert gp.count("with errorlines") == 3 and os.access(out / f"starpu_{FIXTURE}.gp", os.X_OK)
    reg = PO.Registry()
    m = PO.parse(_fixture_text(), reg)
    assert avg.read_text() == PO.plot_averages(m)
    r = _run(tools["starpu_perfmodel_plot"], ["-s", FIXTURE, "-lc"], _env(tmp_path, FIXTURE_DIR))
    assert r.stdout.splitlines() == ["Model <%s>" % FIXTURE, "\tComb 0: 1 device",
                                     "\t\tDevice 0: type: cpu - devid: 0 - ncores: 1", "\tComb 1: 1 device",
                                     "\t\tDevice 0: type: cuda - devid: 0 - ncores: 1"]


@pytest.fixture(scope="module")
def perfmodel_binary(tmp_path_factory, tools):
    import importlib
    libdir = importlib.import_module("starpu_gb300.build").LIBDIR
    out = tmp_path_factory.mktemp("pm") / "test_perfmodel"
    subprocess.run(["gcc", "-std=gnu11", "-O1", "-g", "-o", str(out), os.path.join(ROOT, "tests", "c", "test_perfmodel.c"),
                    "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", "-L" + libdir,
                    "-lstarpu_gb300", "-Wl,-rpath," + libdir, "-lm", "-lpthread"], check=True)
    return str(out)


def test_runtime_written_model(perfmodel_binary, tools, tmp_path):
    models = tmp_path / "models"
    env = _env(tmp_path, models, STARPU_NCUDA=0, STARPU_NCPU=2)
    r = _run(perfmodel_binary, [], env)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout + r.stderr
    path = models / "codelets" / "45" / "gb300_test_perfmodel_io.pmhost"
    assert path.exists()
    text = path.read_text()
    reg = PO.Registry()
    m = PO.parse(text, reg)
    assert m.type == "history" and len(m.combs) == 1 and len(m.impls[m.combs[0]]) == 2
    impl0, impl1 = m.impls[m.combs[0]]
    # impl 0: 12 calls per size, the first opens the entry and is not kept,
    # the 10x outlier is an error -> 11 samples; impl 1: one batch of 4, kept
    assert sorted(e.nsample for e in impl0.entries) == [11, 11, 11]
    assert sorted(e.mean for e in impl0.entries) == [float(f"{100.0 * k + 6.0 / 11.0:e}") for k in (1, 2, 3)]
    assert sorted((e.nsample, e.mean) for e in impl1.entries) == [(4, 50.0), (4, 100.0), (4, 150.0)]
    assert sorted(e.flops for e in impl0.entries) == [2.0 * n ** 3 for n in (32, 64, 128)]
    # the same sequence replayed through the oracle's restatement of the rule
    for k, e in enumerate(sorted(impl0.entries, key=lambda e: e.mean)):
        o = PO.HistoryRecord()
        for i in range(12):
            o.record(100.0 * (k + 1) + (i & 1))
        o.record(1000.0 * (k + 1))
        as_written = lambda x: float(f"{x:e}")  # noqa: E731  (the file holds %e values)
        assert e.nsample == o.nsample
        assert (e.mean, e.sum, e.sum2, e.deviation) == tuple(map(as_written, (o.mean, o.sum, o.sum2, o.deviation)))
    est = next(l for l in r.stdout.splitlines() if l.startswith("ESTIMATIONS "))
    assert est.split()[1:] == ["1.005455e+02", "1.005455e+02"]  # STARPU_NCPU=2 workers
    # the in-process reload prints what the oracle reads from the file
    printed = r.stdout.split("BEGIN_PRINT\n")[1].split("END_PRINT\n")[0]
    assert printed == PO.print_all(m, reg)
    # and so does the display tool
    t = _run(tools["starpu_perfmodel_display"], ["-s", "gb300_test_perfmodel_io"], env)
    assert t.returncode == 0, t.stderr
    assert t.stdout == printed


def _ref_tool():
    if not os.path.isfile(os.path.join(REF, "tools", "starpu_perfmodel_display.c")):
        pytest.skip("reference tree not available on this machine")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF}", "ref-tools"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "starpu_perfmodel_display_ref")


@pytest.mark.parametrize("args", [["-s", FIXTURE], ["-x", "-s", FIXTURE], ["-s", FIXTURE, "-a", "cuda"],
                                  ["-s", FIXTURE, "-p", "mean"], ["-s", FIXTURE, "-f", "1a2b3c4d"], ["-d"], ["-l"]])
def test_reference_display_tool_unchanged(tools, tmp_path, args):
    """StarPU's own tools/starpu_perfmodel_display.c, compiled unchanged against
    this runtime, prints what the GB300 tool prints."""
    ref = _ref_tool()
    env = _env(tmp_path, FIXTURE_DIR)
    a = _run(ref, args, env)
    b = _run(tools["starpu_perfmodel_display"], args, env)
    assert a.returncode == b.returncode == 0, a.stderr + b.stderr
    assert a.stdout == b.stdout


def _sample_files():
    d = os.path.join(REF_SAMPLES, "codelets", "45")
    return sorted(os.listdir(d)) if os.path.isdir(d) else []


def test_reference_sample_models(tools, tmp_path):
    """Every model file StarPU ships (written by its own runtime on several
    machines) reads back as the oracle reads it, through both the GB300 tool
    and StarPU's unchanged display tool."""
    files = _sample_files()
    if not files:
        pytest.skip("reference tree not available on this machine")
    ref = _ref_tool()
    env = _env(tmp_path, REF_SAMPLES)
    malformed = []
    for name in files:
        with open(os.path.join(REF_SAMPLES, "codelets", "45", name)) as f:
            text = f.read()
        got = _run(tools["starpu_perfmodel_display"], ["-s", name], env)
        reg = PO.Registry()
        try:
            expect = PO.print_all(PO.parse(text, reg), reg)
        except (ValueError, IndexError, AssertionError):
            # a damaged file (StarPU's reader asserts on it): the load fails with 1
            malformed.append(name)
            assert got.returncode == 1 and "incorrect performance model file" in got.stderr, name
            continue
        assert got.returncode == 0, (name, got.stderr)
        assert got.stdout == expect, name
        assert _run(ref, ["-s", name], env).stdout == expect, name
    # the shipped idgraf double-LU GEMM models have their "a b c" line after the
    # coefficient count in one combination; every other file reads back
    assert malformed and all(n.startswith("starpu_dlu_lu_model_gemm") and n.endswith(".idgraf") for n in malformed)
    assert len(files) - len(malformed) >= 200


def test_model_directory_follows_environment(native, tmp_path):
    """A process may point successive calls at other model directories (the
    batched autotuner's table lives there too): the search list is rebuilt
    when STARPU_PERF_MODEL_DIR / STARPU_HOME / STARPU_PERF_MODEL_PATH change."""
    import ctypes
    f = native.starpu_perfmodel_get_model_path_default_location
    f.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
    f.restype = None
    saved = {k: os.environ.get(k) for k in ("STARPU_PERF_MODEL_DIR", "STARPU_HOSTNAME")}
    try:
        os.environ["STARPU_HOSTNAME"] = "envhost"
        for sub in ("a", "b"):
            os.environ["STARPU_PERF_MODEL_DIR"] = str(tmp_path / sub)
            buf = ctypes.create_string_buffer(4096)
            f(b"gb300_env_probe", buf, 4096)
            assert buf.value.decode() == f"{tmp_path / sub}/codelets/45/gb300_env_probe.envhost"
            assert (tmp_path / sub / "codelets" / "45").is_dir()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
