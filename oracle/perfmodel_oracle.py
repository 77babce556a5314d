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
    into a history entry: HistoryRecord);
  * src/core/perfmodel/perfmodel_history.c:1993-2023 and 66-67 (the log-log
    least-squares sums of a regression model: RegressionSums),
    src/core/perfmodel/regression.c:25-300 (the non-linear fit y = a x^b + c:
    nl_power_fit), perfmodel_history.c:1575-1680 (their predictions) and
    src/core/perfmodel/perfmodel.c:133-196 (cost-function models).
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


class RegressionSums:
    """The per-architecture regression of a (non-)linear regression model,
    perfmodel_history.c:1993-2023: every recorded call, whatever its batch
    size and whether or not its history entry kept it, adds ln(size) and
    ln(time) to the least-squares sums and widens [minx, maxx]; once
    VALID_REGRESSION holds (minx < 9 maxx / 10 in integer arithmetic, and
    at least STARPU_CALIBRATE_MINIMUM samples: 66-67) the fit time = alpha
    size^beta is recomputed."""

    def __init__(self, calibrate_minimum: int = 10):
        self.calibrate_minimum = calibrate_minimum
        self.sumlnx = self.sumlnx2 = self.sumlny = self.sumlnxlny = 0.0
        self.alpha = self.beta = 0.0
        self.nsample = self.minx = self.maxx = 0
        self.valid = False

    def record(self, size: int, measured: float) -> None:
        lx, ly = math.log(float(size)), math.log(measured)
        self.sumlnx += lx
        self.sumlnx2 += lx * lx
        self.sumlny += ly
        self.sumlnxlny += lx * ly
        if self.minx == 0 or size < self.minx:
            self.minx = size
        if self.maxx == 0 or size > self.maxx:
            self.maxx = size
        self.nsample += 1
        if self.minx < (9 * self.maxx) // 10 and self.nsample >= self.calibrate_minimum:
            n = float(self.nsample)
            self.beta = (n * self.sumlnxlny - self.sumlnx * self.sumlny) / (n * self.sumlnx2 - self.sumlnx * self.sumlnx)
            self.alpha = math.exp((self.sumlny - self.beta * self.sumlnx) / n)
            self.valid = True

    def predict(self, size: int) -> float:
        """perfmodel_history.c:1600-1601: only inside [0.9 minx, 1.1 maxx]."""
        if self.valid and self.minx * 0.9 <= size <= self.maxx * 1.1:
            return self.alpha * math.pow(float(size), self.beta)
        return math.nan


def _nl_level(t):
    # regression.c:25-35
    if t <= 0.0:
        return 0.0
    if t >= 1.0:
        return 1.0
    if t < 0.5:
        return -2 * t * t + 4 * t - 1
    return 2 * t * t


# IEEE double arithmetic where Python would raise (C gives inf / NaN there);
# exp, log and sqrt are the C library's, as in the compiled reference
def _div(a, b):
    if b != 0 or a != a or b != b:
        return a / b if b != 0 else math.nan
    return math.nan if a == 0 else math.copysign(math.inf, a) * math.copysign(1.0, b)


def _sqrt(x):
    return math.nan if x < 0 else math.sqrt(x)


def _log(x):
    return -math.inf if x == 0 else (math.nan if x < 0 else math.log(x))


def _exp(x):
    try:
        return math.exp(x)
    except OverflowError:
        return math.inf


def _nl_moments(c, x, y, pop):
    # regression.c:37-144: the weighted sums over the points whose weight
    # pop * level((y - c) / c - 1) is positive, in point order
    sxy = sx = sx2 = sy = sy2 = nn = 0.0
    for xi, yi, pi in zip(x, y, pop):
        w = pi * _nl_level(_div(yi - c, c) - 1.0)
        if w <= 0:  # a NaN weight is not skipped
            continue
        X, Y = _log(float(xi)), _log(yi - c)
        sxy += X * Y * w
        sx += X * w
        sx2 += X * X * w
        sy += Y * w
        sy2 += Y * Y * w
        nn += w
    return sxy, sx, sx2, sy, sy2, nn


def nl_power_fit(points):
    """regression.c:218-300 on `points` = [(size, mean, nsample), ...] in
    list order (entries without samples are skipped): (a, b, c) of
    time = a size^b + c, or None when no point holds samples.  IEEE double
    arithmetic throughout (a fit whose weights all vanish gives NaN, as in C)."""
    pts = [p for p in points if p[2]]
    if not pts:
        return None
    x = [p[0] for p in pts]
    y = [float(p[1]) for p in pts]
    pop = [p[2] for p in pts]
    cmin, cmax = 0.0, sorted(y)[len(y) // 3]
    err = 100000.0
    for _ in range(1000):
        c1 = cmin + 0.33 * (cmax - cmin)
        c2 = cmin + 0.67 * (cmax - cmin)
        r = []
        for c in (c1, c2):
            sxy, sx, sx2, sy, sy2, nn = _nl_moments(c, x, y, pop)
            r.append(_div(nn * sxy - sx * sy, _sqrt((nn * sx2 - sx * sx) * (nn * sy2 - sy * sy))))
        e1, e2 = abs(1.0 - r[0]), abs(1.0 - r[1])
        if e1 < e2:
            cmax = c2
        else:
            cmin = c1
        best = e1 if e1 < e2 else e2
        if abs(err - best) < 1.0e-10:
            break
        err = best
    c = (cmin + cmax) / 2
    sxy, sx, sx2, sy, sy2, nn = _nl_moments(c, x, y, pop)
    b = _div(nn * sxy - sx * sy, nn * sx2 - sx * sx)
    a = _exp(_div(sy - b * sx, nn))
    return a, b, c


def nl_predict(a, b, c, minx, maxx, size, entry_mean=math.nan):
    """perfmodel_history.c:1643-1663: the fit inside [0.9 minx, 1.1 maxx],
    else the calibrated mean of the task's history entry."""
    if minx * 0.9 <= size <= maxx * 1.1:
        return a * math.pow(float(size), b) + c
    return entry_mean


def relative_speedup(devices) -> float:
    """perfmodel.c:133-144 over [(archtype, ncores), ...]: CPU cores count
    0.5 each, CUDA devices 13.33 (the drivers' single-precision factors)."""
    import numpy as np
    coef = {"cpu": float(np.float32(0.5)), "cuda": float(np.float32(13.33))}
    return sum(coef[t] * n for t, n in devices)

