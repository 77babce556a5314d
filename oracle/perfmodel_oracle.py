"""ORACLE -- test infrastructure only (tests/).

A pure-Python restatement of StarPU's reader of version-45 performance model
files and of the text its perfmodel tools print for them, used to check the
runtime's C implementation (rt_perfmodel.c) and its perfmodel tools on the
same files.  The product never imports this module.

Followed:
  * src/core/perfmodel/perfmodel_history.c:763-812 parse_model_file,
    724-761 parse_comb, 682-722 parse_arch, 629-680 parse_per_arch_model_file,
    491-558 scan_reg_model, 577-628 scan_history_entry: '#' lines are
    comments; entries are put at the head of their list (655-657), so they
    come out in reverse file order; combinations get process-wide ids in the
    order they are first seen (187-230; the tools call no starpu_init, so
    device ids are never ignored when matching);
  * src/core/perfmodel/perfmodel_print.c:25-163 (starpu_perfmodel_print and
    the history lines), 166-285 (starpu_perfmodel_print_all);
  * src/core/perfmodel/perfmodel_history.c:1546-1560 (architecture names);
  * tools/starpu_perfmodel_plot.c:330-470 (the averages file);
  * src/core/perfmodel/perfmodel_history.c:1915-1990 (recording a measurement
    into a history entry: HistoryRecord).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


@dataclass
class Entry:
    footprint: int
    size: int
    flops: float
    mean: float
    deviation: float
    sum: float
    sum2: float
    nsample: int


@dataclass
class PerArch:
    sumlnx: float = 0.0
    sumlnx2: float = 0.0
    sumlny: float = 0.0
    sumlnxlny: float = 0.0
    alpha: float = math.nan
    beta: float = math.nan
    nsample: int = 0
    minx: int = 0
    maxx: int = 0
    a: float = math.nan
    b: float = math.nan
    c: float = math.nan
    coeff: list = field(default_factory=list)
    entries: list = field(default_factory=list)   # in list (reverse file) order


@dataclass
class Model:
    combs: list = field(default_factory=list)      # process-wide ids, file order
    impls: dict = field(default_factory=dict)      # comb id -> [PerArch]
    type: str = "invalid"


class Registry:
    """The process-wide table of architecture combinations."""

    def __init__(self):
        self.combs: list[tuple] = []   # each a tuple of (type, devid, ncores)

    def get(self, devices) -> int:
        for i, c in enumerate(self.combs):
            if len(c) != len(devices):
                continue
            matched = sum(1 for x in c for y in devices if x == y)
            if matched == len(devices):
                return i
        return -1

    def add(self, devices) -> int:
        i = self.get(devices)
        if i < 0:
            self.combs.append(tuple(devices))
            i = len(self.combs) - 1
        return i

    def name(self, comb: int, impl: int) -> str:
        typ = {0: "cpu", 1: "cuda"}
        devs = "_".join(f"{typ.get(t, '?')}{d}_cores{n}" for (t, d, n) in self.combs[comb])
        return f"{devs}_impl{impl} (Comb{comb})"


def _lines(text: str):
    for raw in text.split("\n"):
        s = raw.strip(" \t\r")
        if s and not s.startswith("#"):
            yield s


def _num(tok: str) -> float:
    return float(tok)  # Python reads "nan" like strtod


def parse(text: str, reg: Registry, calibrate_minimum: int = 10) -> Model:
    lines = list(_lines(text))
    pos = 0

    def line():
        nonlocal pos
        pos += 1
        return lines[pos - 1]

    m = Model()
    assert int(line().split()[0]) == 45, "not a version-45 model file"
    ncombs = int(line().split()[0])
    for _ in range(ncombs):
        ndev = int(line().split()[0])
        devs = []
        for _ in range(ndev):
            t = int(line().split()[0])
            d = int(line().split()[0])
            n = int(line().split()[0])
            devs.append((t, d, n))
        cid = reg.add(devs)
        if cid not in m.combs:
            m.combs.append(cid)
        nimpls = int(line().split()[0])
        m.impls[cid] = []
        for _ in range(nimpls):
            pa = PerArch()
            nentries = int(line().split()[0])
            t = line().split()
            (pa.sumlnx, pa.sumlnx2, pa.sumlny, pa.sumlnxlny, pa.alpha, pa.beta) = map(_num, t[:6])
            pa.nsample, pa.minx, pa.maxx = int(t[6]), int(t[7]), int(t[8])
            pa.a, pa.b, pa.c = map(_num, line().split()[:3])
            t = line().split()
            ncoeff = int(t[0])
            toks = t[1:]
            while len(toks) < ncoeff:
                toks += line().split()
            pa.coeff = [_num(x) for x in toks[:ncoeff]]
            for _ in range(nentries):
                t = line().split()
                if len(t) >= 8:
                    e = Entry(int(t[0], 16), int(t[1]), _num(t[2]), _num(t[3]), _num(t[4]), _num(t[5]),
                              _num(t[6]), int(t[7]))
                else:
                    e = Entry(int(t[0], 16), int(t[1]), 0.0, _num(t[2]), _num(t[3]), _num(t[4]), _num(t[5]),
                              int(t[6]))
                pa.entries.insert(0, e)
            if m.type == "invalid":
                if ncoeff:
                    m.type = "multiple"
                elif not any(math.isnan(v) for v in (pa.a, pa.b, pa.c)):
                    m.type = "nl"
                elif not any(math.isnan(v) for v in (pa.alpha, pa.beta)):
                    m.type = "linear"
                elif nentries:
                    m.type = "history"
            m.impls[cid].append(pa)
    return m


def _e(x: float) -> str:
    return "nan" if math.isnan(x) else f"{x:e}"


def _valid(pa: PerArch, calibrate_minimum: int) -> bool:
    return pa.minx < (9 * pa.maxx) // 10 and pa.nsample >= calibrate_minimum


def print_all(m: Model, reg: Registry, calibrate_minimum: int = 10, arch: str | None = None,
              parameter: str | None = None, footprint: int | None = None) -> str:
    """The text starpu_perfmodel_print_all writes (arch None, "cpu", "cuda", "cuda<d>")."""
    out = []

    def one(comb: int, impl: int):
        pa = m.impls[comb][impl]
        valid = not math.isnan(pa.alpha) and not math.isnan(pa.beta) and _valid(pa, calibrate_minimum)
        nl_valid = not any(math.isnan(v) for v in (pa.a, pa.b, pa.c)) and _valid(pa, calibrate_minimum)
        if pa.nsample or valid or nl_valid or pa.entries:
            out.append(f"# performance model for {reg.name(comb, impl)}\n")
        if parameter is None:
            if pa.nsample:
                out.append(f"\tRegression : #sample = {pa.nsample}\n")
            if valid:
                out.append(f"\tLinear: y = alpha size ^ beta\n\t\talpha = {_e(pa.alpha)}\n\t\tbeta = {_e(pa.beta)}\n")
            if nl_valid:
                out.append(f"\tNon-Linear: y = a size ^b + c\n\t\ta = {_e(pa.a)}\n\t\tb = {_e(pa.b)}\n"
                           f"\t\tc = {_e(pa.c)}\n")
            if pa.entries:
                out.append("# hash\t\tsize\t\tflops\t\tmean (us or J)\tstddev (us or J)\t\tn\n")
            for e in pa.entries:
                if footprint is None or e.footprint == footprint:
                    out.append(f"{e.footprint:08x}\t{e.size:<15d}\t{_e(e.flops):<15}\t{_e(e.mean):<15}\t"
                               f"{_e(e.deviation):<15}\t{e.nsample}\n")
        elif parameter in ("mean", "stddev"):
            for e in pa.entries:
                if footprint is None or e.footprint == footprint:
                    out.append(f"{_e(e.mean if parameter == 'mean' else e.deviation):<15}\n")
                    if parameter == "stddev":
                        break
        else:
            out.append(_e(getattr(pa, parameter)) + "\n")

    def combs_matching(pred):
        for cid in range(len(reg.combs)):
            if pred(reg.combs[cid]):
                for impl in range(len(m.impls.get(cid, []))):
                    one(cid, impl)

    if arch is None:
        combs_matching(lambda c: True)
    elif arch == "cpu":
        cid = reg.get([(0, 0, 1)])
        for impl in range(len(m.impls.get(cid, []))):
            one(cid, impl)
    elif arch == "cuda":
        for cid in range(len(reg.combs)):
            c = reg.combs[cid]
            if len(c) == 1 and c[0][0] == 1:
                for impl in range(len(m.impls.get(cid, []))):
                    one(cid, impl)
    elif arch.startswith("cuda"):
        d = int(arch[5:] if arch.startswith("cuda_") else arch[4:])
        cid = reg.get([(1, d, 1)])
        for impl in range(len(m.impls.get(cid, []))):
            one(cid, impl)
    return "".join(out)


def plot_averages(m: Model) -> str:
    """The averages file of starpu_perfmodel_plot (times in ms)."""
    lists = [pa for cid in m.combs for pa in m.impls[cid]]
    sizes = sorted({e.size for pa in lists for e in pa.entries if e.size > 0})
    rows = []
    for s in sizes:
        row = [f"{s:<15d} "]
        for pa in lists:
            hit = next((e for e in pa.entries if e.size == s), None)
            if hit is not None:
                row.append(f"\t{_e(0.001 * hit.mean):<15}\t{_e(0.001 * hit.deviation):<15}")
            elif pa.entries:
                row.append('\t""\t""')
        rows.append("".join(row) + "\n")
    return "".join(rows)


class HistoryRecord:
    """One history entry as StarPU's recording updates it
    (src/core/perfmodel/perfmodel_history.c:1915-1990), for one footprint.

    * A new entry of a history-based model does not keep a single first
      measurement (1926-1933); a batch (number != 1) or another model type
      keeps it.
    * Later, a measurement whose ratio to the mean exceeds
      1 + STARPU_HISTORY_MAX_ERROR/100 either way is an error, not a sample
      (1947-1949); once the errors reach the sample count the entry is
      flushed (1953-1964).
    * Otherwise sum, sum2 and nsample grow, the mean is sum / n and the
      deviation sqrt(|sum2 - sum^2 / n| / n) (1966-1973).
    """

    def __init__(self, history_based: bool = True, max_error: int = 50):
        self.history_based, self.max_error = history_based, max_error
        self.exists = False
        self.sum = self.sum2 = self.mean = self.deviation = 0.0
        self.nsample = self.nerror = 0

    def record(self, measured: float, number: int = 1) -> None:
        if not self.exists:
            self.exists = True
            if number != 1 or not self.history_based:
                self.sum, self.sum2 = measured * number, measured * measured * number
                self.nsample, self.mean = number, measured
            return
        ratio = measured / self.mean if self.mean else math.inf
        if self.nsample and (100 * ratio > 100 + self.max_error or 100 / ratio > 100 + self.max_error):
            self.nerror += number
            if self.nerror >= self.nsample:
                self.sum = self.sum2 = self.mean = self.deviation = 0.0
                self.nsample = self.nerror = 0
            return
        self.sum += measured * number
        self.sum2 += measured * measured * number
        self.nsample += number
        n = self.nsample
        self.mean = self.sum / n
        self.deviation = math.sqrt(abs(self.sum2 - self.sum * self.sum / n) / n)
