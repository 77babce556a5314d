#!/usr/bin/env python
"""Headline benchmark: SPD solve GFLOP/s at FP64-level backward error (<= 1e-12),
mixed precision vs plain FP64, on one GB300 per process.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one full solve through the C-ABI, inputs resident in HBM):
  mixed-precision SPD solve, N=32768, tile 1024, A = B B^T / N + alpha I
  (B iid N(0,1), alpha set for kappa = 1e4), 16 right-hand sides U[-1,1];
  tcgen05 factorisation on row-scaled FP16 split operands + FP64 iterative
  refinement to 1e-12.
  flops = N^3/3 + 2 N^2 nrhs (FP64-equivalent, LAPACK dsposv convention).
Beside it, in the same run: the plain FP64 GPU solve (dposv) of the same
system and of the FP64 config N=16384 / tile 512 / 64 RHS, a kappa sweep
{1e2, 1e4, 1e6}, the end-to-end host-buffer call, and StarPU's CPU path (the
port of its CPU codelets over OpenBLAS, FP64) on a bounded sample on the
host cores.  Multi-GPU: independent replicas, one per rank (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SPD solve GFLOP/s @1e-12 backward err, mixed vs FP64; solves/s + p99 latency"


# dram__bytes_read.sum + dram__bytes_write.sum of one tc_update_kernel launch,
# m = 8192, k = 1024, 3 scaled-FP16 split products (ncu, GB300)
TC_TRAFFIC_M8192 = 249.5e6

def solve_flops(n: int, nrhs: int) -> float:
    return n ** 3 / 3.0 + 2.0 * n * n * nrhs


def alpha_for_kappa(kappa: float) -> float:
    """Diagonal shift giving kappa for B B^T / n with B square iid N(0,1), whose
    spectrum fills the Marchenko-Pastur range [0, 4]: (4 + a) / a = kappa."""
    return 4.0 / (kappa - 1.0)


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs"), "bf16_tflops": d.get("bf16_tflops"),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    """Barrier + max-over-ranks through torch.distributed (plumbing only):
    NCCL on the rank's GPU, gloo on host tensors where no GPU is visible.
    The replicas exchange nothing else."""

    def __init__(self, world: int, local: int):
        self.world = world
        if world > 1:
            import torch
            import torch.distributed as dist
            self.device = "cpu"
            if torch.cuda.is_available():
                torch.cuda.set_device(local)
                self.device = f"cuda:{local}"
            dist.init_process_group("nccl" if self.device != "cpu" else "gloo")
            self.dist, self.torch = dist, torch

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ------------------------------------------------------------------ CPU path
def cpu_config1(reps: int = 3):
    """The reference's CPU-runnable configuration: plain FP32 tiled Cholesky,
    N=2048, 8x8 tiles of 256, A_ij = 1/(i+j+1) + N delta_ij (the input of
    examples/cholesky/cholesky_implicit.c:477-484), through the port of the CPU
    codelets on all host cores; GFLOP/s with FLOPS_SPOTRF (cholesky.h:95) and
    the reference's reconstruction check (max relative error <= 1e-4)."""
    from oracle import oracle as O
    if not O.cpu_init():
        return None
    n, nblocks = 2048, 8
    cores = len(os.sched_getaffinity(0))
    O.lib().cpu_chol_set_blas_threads(cores)
    A = O.hilbert_f32(n)
    times, ok, err = [], None, None
    for _ in range(reps):
        L = A.copy(order="F")
        t0 = time.perf_counter()
        info = O.cpu_potrf_tiled(L, nblocks, cores)
        times.append(time.perf_counter() - t0)
        assert info == 0
        ok, err = O.check_hilbert(L)
    t = min(times)
    return {"workload": "plain FP32 tiled Cholesky, N=2048, 8x8 tiles of 256, Hilbert + N*I", "cores": cores,
            "kind": "port", "gflops": O.flops_potrf(n) / t / 1e9, "ms": t * 1e3, "check_ok": bool(ok == 0),
            "max_rel_err": err, "best_of": reps}


# ------------------------------------------- FP64 oracle: forward errors
def host_backward_error(A, X, B):
    """Normwise backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf
    + ||b_j||_inf) in FP64 on the host BLAS (A symmetric, full)."""
    import numpy as np
    R = B - A @ X
    anorm = 0.0
    for j0 in range(0, A.shape[1], 2048):  # column sums = row sums (symmetric A)
        anorm = max(anorm, float(np.abs(A[:, j0:j0 + 2048]).sum(axis=0).max()))
    num = np.abs(R).max(axis=0)
    den = anorm * np.abs(X).max(axis=0) + np.abs(B).max(axis=0)
    return float((num / den).max())


def forward_error(X, Xo):
    """max_j ||x_j - xo_j||_inf / ||xo_j||_inf against the oracle solution Xo."""
    import numpy as np
    return float((np.abs(X - Xo).max(axis=0) / np.abs(Xo).max(axis=0)).max())


def oracle_solve(A, B, nb, cores, shift=0.0):
    """FP64 oracle solution of (A + shift I) X = B: the port of StarPU's CPU
    path (tiled FP64 Cholesky over OpenBLAS on all host cores, pinned to
    CLAPACK dpotrf/dpotrs by the golden vectors), then dpotrs.  Returns
    (X, seconds of the factor + solve)."""
    import numpy as np
    from oracle import oracle as O
    n = A.shape[0]
    L = np.array(A, order="F", copy=True)
    if shift:
        L[np.diag_indices(n)] += shift
    X = np.array(B, order="F", copy=True)
    t0 = time.perf_counter()
    info = O.cpu_potrf_tiled(L, max(1, min(512, round(n / nb))), cores)
    info2 = O.cpu_potrs(L, X, cores)
    t = time.perf_counter() - t0
    assert info == 0 and info2 == 0, (info, info2)
    return X, t


def accuracy_of(A, B, X, Xo, kappa, shift=0.0):
    """Accuracy of one GPU result against the FP64 oracle solution."""
    import numpy as np
    As = A
    if shift:
        As = np.array(A, order="F", copy=True)
        As[np.diag_indices(A.shape[0])] += shift
    return {"kappa": kappa, "forward_error": forward_error(X, Xo), "backward_error_host": host_backward_error(As, X, B),
            "oracle_backward_error": host_backward_error(As, Xo, B)}


def run_reference(args):
    """StarPU's CPU path (the port of its CPU codelets over OpenBLAS, FP64
    tiles, priority DAG on all host cores) on the bench configuration itself:
    N, tile, RHS and kappa of the GPU arm; one step = one factorisation +
    solve of the same A = B B^T / N + alpha I (same PCG64 row streams as the
    device generator), copied back from a pristine host copy before each step
    (not timed)."""
    import numpy as np
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle as O
    if not O.cpu_init():
        print(json.dumps({"impl": "reference", "unavailable": "scipy OpenBLAS not found on this host"}))
        return 0
    n, nb, nrhs = args.cpu_n or args.n, args.cpu_nb or args.nb, args.nrhs
    cores = len(os.sched_getaffinity(0))
    tg = time.perf_counter()
    A = O.spd_gram_host_blas(n, 1234, alpha_for_kappa(args.kappa), cores)
    rhs = O.uniform_rhs(n, nrhs, 99)
    gen_s = time.perf_counter() - tg
    L = np.empty_like(A, order="F")
    nblocks = max(1, min(512, round(n / nb)))
    times, X = [], None
    for i in range(args.warmup + args.steps):
        np.copyto(L, A)
        X = np.array(rhs, order="F", copy=True)
        t0 = time.perf_counter()
        info = O.cpu_potrf_tiled(L, nblocks, cores)
        info2 = O.cpu_potrs(L, X, cores)
        t = time.perf_counter() - t0
        assert info == 0 and info2 == 0
        if i >= args.warmup:
            times.append(t)
    t = sum(times) / len(times)
    val = solve_flops(n, nrhs) / t / 1e9
    berr = host_backward_error(A, X, rhs)
    sample = (f"FP64 tiled Cholesky (StarPU CPU codelets port, OpenBLAS, {cores} workers) + dpotrs, N={n}, "
              f"tile {n // nblocks}, {nrhs} RHS, kappa={args.kappa:g}: the full workload, every step")
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, world, n=n, nb=nb),
            "backward_error": berr, "generation_s": gen_s, "step_s": times,
            "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def bench_config(args, world, n=None, nb=None):
    """The workload both arms name: the mixed-precision solve's configuration."""
    n, nb = n or args.n, nb or args.nb
    return {"workload": f"SPD solve, N={n}, tile {nb}, A=B*B^T/N+alpha*I (kappa={args.kappa:g}), {args.nrhs} RHS "
                        f"U[-1,1], to backward error <= 1e-12 (GPU: scaled-FP16 split tcgen05 factor + FP64 iterative "
                        f"refinement)",
            "n": n, "nb": nb, "nrhs": args.nrhs, "kappa": args.kappa,
            "l2": "inputs larger than L2 (A is 8 GiB FP64 at N=32768; L2 129 MB)",
            "parallelism": f"replicas x{world}"}


# ------------------------------------------- config 4: batched uneven systems
def bench_batched(L, nsys=4096, nrhs=4, seed=2024):
    """4096 independent SPD systems, n log-uniform in [32, 1024],
    A = B B^T / n + I, 4 RHS: one persistent launch (FP32 factor + FP64
    refinement per system)."""
    import numpy as np
    from starpu_gb300 import DeviceBuffer
    from starpu_gb300.native import check
    rng = np.random.default_rng(seed)
    ns = np.clip(np.exp(rng.uniform(np.log(32), np.log(1024), nsys)).astype(np.int32), 32, 1024).astype(np.int32)
    a_off = np.zeros(nsys, np.int64)
    b_off = np.zeros(nsys, np.int64)
    a_off[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
    b_off[1:] = np.cumsum(ns.astype(np.int64) * nrhs)[:-1]
    atot, btot = int((ns.astype(np.int64) ** 2).sum()), int((ns.astype(np.int64) * nrhs).sum())
    dA, dB, dX = DeviceBuffer(8 * atot), DeviceBuffer(8 * btot), DeviceBuffer(8 * btot)
    wk = DeviceBuffer(8 * 1024 * 1024)
    for i in range(nsys):
        n = int(ns[i])
        check(L.starpu_gb300_gen_spd_gram(None, n, 7000 + i, 1.0, dA.ptr + 8 * int(a_off[i]), n, wk.ptr))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 9000 + i, dB.ptr + 8 * int(b_off[i]), n))
    check(L.starpu_gb300_stream_sync(None))
    lw = L.starpu_gb300_dposv_batched_workspace(nsys, ns.ctypes.data, nrhs)
    W = DeviceBuffer(lw)
    st, be = np.zeros(nsys, np.int32), np.zeros(nsys)
    flops = float((ns.astype(np.float64) ** 3 / 3 + 2 * ns.astype(np.float64) ** 2 * nrhs).sum())

    def call():
        check(L.starpu_gb300_dposv_batched(None, nsys, ns.ctypes.data, dA.ptr, a_off.ctypes.data, dB.ptr,
                                           b_off.ctypes.data, dX.ptr, nrhs, 1e-12, 20, W.ptr, lw, st.ctypes.data,
                                           be.ctypes.data))
    call()
    ts = []
    for _ in range(3):
        e0, e1 = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
        check(L.starpu_gb300_event_record(e0, None))
        call()
        check(L.starpu_gb300_event_record(e1, None))
        ts.append(L.starpu_gb300_event_elapsed_ms(e0, e1))
    ms = min(ts)
    tune = (C.c_byte * 6)()
    L.starpu_gb300_batched_get_tuning(tune, 6)
    # systems for the FP64 oracle: the 3 largest, the 2 smallest and 5 drawn at random
    order = np.argsort(ns)
    pick = sorted(set(order[-3:].tolist() + order[:2].tolist() +
                      np.random.default_rng(seed + 1).choice(nsys, 5, replace=False).tolist()))
    samples = []
    for i in pick:
        n = int(ns[i])
        Ai = np.empty((n, n), np.float64, order="F")
        Bi, Xi = np.empty((n, nrhs), np.float64, order="F"), np.empty((n, nrhs), np.float64, order="F")
        check(L.starpu_gb300_memcpy_d2h(None, Ai.ctypes.data, dA.ptr + 8 * int(a_off[i]), Ai.nbytes))
        check(L.starpu_gb300_memcpy_d2h(None, Bi.ctypes.data, dB.ptr + 8 * int(b_off[i]), Bi.nbytes))
        check(L.starpu_gb300_memcpy_d2h(None, Xi.ctypes.data, dX.ptr + 8 * int(b_off[i]), Xi.nbytes))
        check(L.starpu_gb300_stream_sync(None))
        samples.append({"system": int(i), "n": n, "kappa": None, "A": Ai, "B": Bi, "X": Xi})
    return {"workload": f"{nsys} SPD systems, n log-uniform [32,1024], A=B*B^T/n+I, {nrhs} RHS, one persistent launch",
            "ms": ms, "gflops": flops / (ms * 1e-3) / 1e9, "systems_per_s": nsys / (ms * 1e-3),
            "max_backward_error": float(be.max()), "all_converged": bool((st >= 0).all()),
            "corrections_max": int(st.max()), "tuning_nb_per_bucket": list(tune), "_samples": samples}


# --------------------------------------------------------- config 5: serving
def bench_serving(L, nreq=160, seed=5, repeat_frac=0.3, executors=4):
    """Poisson stream of solve requests: n log-uniform [64, 8192], 1-16 RHS,
    kappa log-uniform [1e2, 1e6], 30 % repeat right-hand sides on a cached
    device factor, 120 GB HBM budget.  Ours (continuous batching, executors
    overlapping, factor cache, mixed precision) against per-request plain
    launches (one at a time, FP64 dposv): throughput at saturation, then
    p50 / p99 latency under the same Poisson arrival rate."""
    import numpy as np
    from starpu_gb300 import DeviceBuffer
    from starpu_gb300.native import Request, check
    rng = np.random.default_rng(seed)
    ndistinct = int(nreq * (1 - repeat_frac)) + 1
    sizes = np.clip(np.exp(rng.uniform(np.log(64), np.log(8192), ndistinct)).astype(int), 64, 8192)
    kappas = np.exp(rng.uniform(np.log(1e2), np.log(1e6), ndistinct))
    mats = []
    wk = DeviceBuffer(8 * 8192 * 8192)
    for i, (n, k) in enumerate(zip(sizes, kappas)):
        d = DeviceBuffer(8 * int(n) * int(n))
        check(L.starpu_gb300_gen_spd_gram(None, int(n), 100 + i, 4.0 / (k - 1.0), d.ptr, int(n), wk.ptr))
        mats.append((int(n), d))
    del wk
    check(L.starpu_gb300_stream_sync(None))
    # request trace: first use of every matrix, then repeats of earlier ones (30 %)
    trace = []
    seen = []
    for q in range(nreq):
        if seen and rng.random() < repeat_frac:
            mi = int(rng.choice(seen))
        else:
            mi = len(seen) if len(seen) < ndistinct else int(rng.choice(seen))
            if mi not in seen:
                seen.append(mi)
        nrhs = int(rng.integers(1, 17))
        n = mats[mi][0]
        B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
        trace.append((mi, nrhs, B))
    flops_new = lambda n, r: n ** 3 / 3 + 2 * n * n * r  # noqa: E731

    kept = {}

    def run(mode, nexec, arrivals=None, keep_results=False):
        sv = L.starpu_gb300_server_create(120 * (1 << 30), nexec, 8192, 16, mode)
        assert sv, L.starpu_gb300_last_error()
        reqs, keep = [], []
        t0 = time.perf_counter()
        for q, (mi, nrhs, B) in enumerate(trace):
            n, d = mats[mi]
            X = np.zeros_like(B)
            r = Request()
            r.n, r.nrhs, r.A, r.B, r.X = n, nrhs, d.ptr, B.ctypes.data, X.ctypes.data
            r.matrix_id = (mi + 1) if mode == 0 else 0
            r.tol, r.max_iter = 1e-12, 40
            if arrivals is not None:
                delay = t0 + arrivals[q] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            check(L.starpu_gb300_server_submit(sv, C.byref(r)))
            reqs.append(r)
            keep.append(X)
        L.starpu_gb300_server_drain(sv)
        wall = time.perf_counter() - t0
        st = [C.c_ulonglong() for _ in range(4)]
        L.starpu_gb300_server_stats(sv, *[C.byref(x) for x in st], None)
        L.starpu_gb300_server_destroy(sv)
        lat = np.array([(r.end_us - r.submit_us) / 1e3 for r in reqs])
        ok = all(r.status == 0 for r in reqs)
        berr = max(r.backward_error for r in reqs) if mode != 1 else None
        if keep_results:
            kept["X"] = keep
        return {"solves_per_s": len(reqs) / wall, "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "all_ok": ok, "max_backward_error": berr,
                "batched_launches": st[1].value, "cache_hits": st[2].value}
    ours_sat = run(0, executors, keep_results=True)
    plain_sat = run(1, 1)
    mixed_sat = run(2, 1)  # the same mixed solves, one at a time: no batching, overlap or cache
    rate = 0.7 * plain_sat["solves_per_s"]  # a load the plain baseline can sustain
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    ours_lat = run(0, executors, arrivals)
    plain_lat = run(1, 1, arrivals)
    mixed_lat = run(2, 1, arrivals)
    # requests for the FP64 oracle: the largest new request, the largest repeat and 6 at random
    new_q = [q for q in range(nreq) if trace[q][0] not in [trace[p][0] for p in range(q)]]
    rep_q = [q for q in range(nreq) if q not in new_q]
    big = lambda qs: max(qs, key=lambda q: mats[trace[q][0]][0]) if qs else None  # noqa: E731
    pick = {big(new_q), big(rep_q)} | set(rng.choice(nreq, 6, replace=False).tolist())
    samples = []
    for q in sorted(p for p in pick if p is not None):
        mi, nrhs, B = trace[q]
        n, d = mats[mi]
        samples.append({"request": int(q), "n": n, "kappa": float(kappas[mi]), "repeat": q in rep_q,
                        "A": d.download((n, n), np.float64), "B": B, "X": kept["X"][q]})
    return {"workload": f"{nreq} requests, n log-uniform [64,8192], 1-16 RHS, kappa log-uniform [1e2,1e6], "
                        f"{int(repeat_frac * 100)}% repeat RHS, 120 GB budget, {executors} executors",
            "saturation": {"ours": ours_sat, "plain_per_request": plain_sat, "mixed_per_request": mixed_sat,
                           "speedup_solves_per_s": ours_sat["solves_per_s"] / plain_sat["solves_per_s"],
                           "speedup_vs_mixed_per_request": ours_sat["solves_per_s"] / mixed_sat["solves_per_s"],
                           "speedup_mixed_per_request_vs_plain": mixed_sat["solves_per_s"] / plain_sat["solves_per_s"]},
            "poisson_rate_per_s": rate,
            "at_rate": {"ours": ours_lat, "plain_per_request": plain_lat, "mixed_per_request": mixed_lat},
            "_samples": samples}


# ------------------------------------------------------------------ GPU path
def run_ours(args):
    import numpy as np
    import starpu_gb300
    from starpu_gb300 import DeviceBuffer
    from starpu_gb300.native import IrInfo, check

    world, rank, local = dist_setup()
    L = starpu_gb300.load()
    check(L.starpu_gb300_set_device(local), "set_device")
    dist = Dist(world, local)
    peaks = load_peaks()
    n, nb, nrhs = args.n, args.nb, args.nrhs
    stream = None  # legacy default stream; the library launches every kernel on it

    # ---- inputs resident in HBM: A (FP64, 8 GiB at N=32768) > L2 (129 MB)
    A = DeviceBuffer(8 * n * n)
    Bd = DeviceBuffer(8 * n * nrhs)
    Xd = DeviceBuffer(8 * n * nrhs)
    tg = time.perf_counter()
    with_work = DeviceBuffer(8 * n * n)
    alpha0 = 0.0
    check(L.starpu_gb300_gen_spd_gram(stream, n, 1234 + rank, alpha0, A.ptr, n, with_work.ptr), "gen")
    check(L.starpu_gb300_gen_uniform_rhs(stream, n, nrhs, 99 + rank, Bd.ptr, n), "rhs")
    check(L.starpu_gb300_stream_sync(stream))
    gen_s = time.perf_counter() - tg
    cur_alpha = 0.0

    def set_kappa(kappa):
        nonlocal cur_alpha
        a = alpha_for_kappa(kappa)
        check(L.starpu_gb300_shift_diagonal(stream, n, A.ptr, n, a - cur_alpha))
        cur_alpha = a

    # the schedule of the factorisation for this order and tile, tuned on this GPU and stored beside the
    # perfmodels (StarPU calibrates its perfmodels the same way before timing); not timed
    schedule = None
    if not args.no_autotune:
        ta = time.perf_counter()
        rc = L.starpu_gb300_dense_autotune(n, nb, 2)
        la, td, up, pr, st = C.c_int(), C.c_double(), C.c_double(), C.c_double(), C.c_double()
        if rc == 0 and L.starpu_gb300_dense_get_tuning(nb, C.byref(la), C.byref(td), C.byref(up), C.byref(pr),
                                                        C.byref(st)):
            schedule = {"lookahead_sms": la.value if la.value >= 0 else "per-step model",
                        "t_diag_us": td.value, "update_tflops": up.value, "panel_rate": pr.value,
                        "factor_ms": st.value, "tuning_s": time.perf_counter() - ta}
        else:
            schedule = {"autotune_rc": rc}
    lw = L.starpu_gb300_dsposv_workspace(n, nrhs, nb)
    W = DeviceBuffer(lw)
    info = IrInfo()

    def step(nterms=args.nterms):
        return L.starpu_gb300_dsposv(stream, n, nrhs, A.ptr, n, Bd.ptr, n, Xd.ptr, n, nb, nterms, 1e-12,
                                     args.max_iter, W.ptr, lw, C.byref(info))

    set_kappa(args.kappa)
    for _ in range(args.warmup):
        rc = step()
        assert rc == 0, f"dsposv failed rc={rc} status={info.status} it={info.iterations} be={info.backward_error}"
    e0, e1 = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
    clocks = ClockSampler(local)
    L.starpu_gb300_profiling_reset()
    dist.barrier()
    check(L.starpu_gb300_stream_sync(stream))
    clocks.start()
    L.starpu_gb300_profiling_enable(1)
    launches0 = L.starpu_gb300_launch_count()
    iters, berrs = [], []
    check(L.starpu_gb300_event_record(e0, stream))
    for _ in range(args.steps):
        rc = step()
        assert rc == 0, f"dsposv failed rc={rc}"
        iters.append(info.iterations)
        berrs.append(info.backward_error)
    check(L.starpu_gb300_event_record(e1, stream))
    check(L.starpu_gb300_stream_sync(stream))
    launches = L.starpu_gb300_launch_count() - launches0
    L.starpu_gb300_profiling_enable(0)
    clk = clocks.stop()
    want_oracle = rank == 0 and world == 1 and not args.no_cpu
    X_main = Xd.download((n, nrhs), np.float64) if want_oracle else None
    ms = L.starpu_gb300_event_elapsed_ms(e0, e1) / args.steps
    ms = dist.max(ms)
    flops = solve_flops(n, nrhs)
    value = world * flops / (ms * 1e-3) / 1e9
    # the refinement's stopping test uses the double-float residual; check the
    # last solution's backward error with the plain FP64 residual as well
    bw_ws = L.starpu_gb300_backward_error_workspace(n, nrhs)
    BWc = DeviceBuffer(bw_ws)
    hb = (C.c_double * nrhs)()
    check(L.starpu_gb300_backward_error(stream, n, nrhs, A.ptr, n, Xd.ptr, n, Bd.ptr, n, BWc.ptr, bw_ws, hb))
    berr_fp64_check = max(hb)
    del BWc

    # ---- roofline of the dominant kernel (tensor-core trailing update), live over the timed region
    prof = {}
    for kind, name in ((0, "tc_update"), (1, "panel"), (2, "residual_fp64"), (3, "trsv_fp32")):
        la, tms, fl, by = C.c_ulonglong(), C.c_double(), C.c_double(), C.c_double()
        L.starpu_gb300_profiling_get(kind, C.byref(la), C.byref(tms), C.byref(fl), C.byref(by))
        prof[name] = {"launches": la.value, "ms_per_step": tms.value / args.steps,
                      "share": None, "tflops": (fl.value / (tms.value * 1e-3) / 1e12) if tms.value else None,
                      "gbs": (by.value / (tms.value * 1e-3) / 1e9) if tms.value else None}
    for v in prof.values():
        v["share"] = v["ms_per_step"] / ms if ms else None
    # the trailing updates share the GPU with the next panel by design (the
    # panel and update classes overlap in time, so shares may sum above 1)
    sm_share = C.c_double(1.0)
    L.starpu_gb300_profiling_sm_share(0, C.byref(sm_share))
    prof["tc_update"]["sm_share"] = sm_share.value
    tc = prof["tc_update"]
    peak_tc = peaks["bf16_tflops_sustained"]
    traffic, traffic_src = args.tc_traffic, "given on the command line"
    if traffic is None:
        # DRAM bytes per launch: the ncu capture of one m = 8192, k = 1024
        # lower launch (dram__bytes_read.sum + dram__bytes_write.sum) scaled
        # to each update launch of the factorisation by its algorithmic bytes
        # (FP32 C read + written, two BF16 K-major panels), averaged over the
        # launches like `achieved`.  Per step (m = n - (k+1) nb rows below the
        # diagonal tile): the next column block (its kb1 x kb1 lower tile and
        # the m2 x kb1 rectangle below, m2 = m - kb1), then the trailing m2 x m2
        # lower triangle.
        ldk = (nb + 63) // 64 * 64

        def tc_bytes(m):
            return 8.0 * m * (m + 1) / 2 + 2.0 * m * ldk * 2

        launch_bytes = []
        for k in range((n + nb - 1) // nb - 1):
            m = n - (k + 1) * nb
            kb1 = min(nb, m)
            m2 = m - kb1
            launch_bytes.append(8.0 * (kb1 * (kb1 + 1) / 2 + m2 * kb1) + 2.0 * m * ldk * 2)
            if m2 > 0:
                launch_bytes.append(tc_bytes(m2))
        if launch_bytes:
            traffic = sum(TC_TRAFFIC_M8192 * b / tc_bytes(8192) for b in launch_bytes) / len(launch_bytes)
            traffic_src = (f"ncu capture of an m=8192 k=1024 launch ({TC_TRAFFIC_M8192 / 1e6:.1f} MB) scaled by "
                           f"algorithmic bytes to the {len(launch_bytes)} update launches of one factorisation "
                           "(next column block + trailing triangle per step), mean per launch")
    roofline = {"bound": "tensor", "achieved": tc["tflops"], "peak": peak_tc, "unit": "TFLOP/s",
                "frac": (tc["tflops"] / peak_tc) if tc["tflops"] else None,
                # the updates run on the SMs the concurrent panel leaves free:
                # their time-weighted mean share of the SMs, and the fraction
                # of the peak of that share they reach
                "sm_share": sm_share.value,
                "frac_of_sm_share": (tc["tflops"] / (peak_tc * sm_share.value)) if tc["tflops"] else None,
                "traffic": traffic, "traffic_source": traffic_src,
                "kernel": "tc_update_kernel (row-scaled FP16 split, tcgen05 trailing update)",
                "peak_source": f"{peaks['source']} bf16 sustained (kernel timed inside a long step)",
                "algorithmic": "flops = nterms * kb * 2 * (cells updated) per launch: per step the next column block "
                               "(kb1 lower tile + m2 x kb1 rectangle) and the m2 x m2 lower triangle beyond it; "
                               "summed over a step, nterms * kb * m*(m+1)"}

    # ---- kappa sweep (same Gram matrix, shifted diagonal)
    sweep = []
    if not args.no_sweep:
        # the default refinement policy at each kappa; at 1e6 also classic
        # corrections alone, the rung the policy switches away from
        for kap, modes in ((1e2, (2,)), (1e4, (2,)), (1e6, (2, 0))):
            set_kappa(kap)
            for mode in modes:
                prev_mode = L.starpu_gb300_dsposv_set_refinement(mode)
                t0e, t1e = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
                check(L.starpu_gb300_event_record(t0e, stream))
                rc = step(args.nterms)
                check(L.starpu_gb300_event_record(t1e, stream))
                tms = L.starpu_gb300_event_elapsed_ms(t0e, t1e)
                L.starpu_gb300_dsposv_set_refinement(prev_mode)
                sweep.append({"kappa": kap, "nterms": args.nterms, "status": rc, "iterations": info.iterations,
                              "refinement": ("classic", "pcg", "auto")[mode],
                              "method_at_end": ("classic", "pcg")[info.method], "fp64_fallback": info.fallback,
                              "factor_terms": info.factor_terms, "backward_error": info.backward_error,
                              "gflops": flops / (tms * 1e-3) / 1e9, "ms": tms,
                              "_X": Xd.download((n, nrhs), np.float64) if want_oracle and mode == 2 else None})
        set_kappa(args.kappa)

    # ---- plain FP64 GPU solve (the baseline of the ">= 3x" target)
    fp64 = []
    if not args.no_fp64:
        berr_ws = L.starpu_gb300_backward_error_workspace(n, nrhs)
        BW = DeviceBuffer(berr_ws)
        for (fn, fnb, frhs, same) in ((n, nb, nrhs, True), (args.fp64_n, 512, 64, False)):
            if fn <= 0 or (same and args.no_fp64_same_n):
                continue
            if same:
                Af, Bf = with_work, DeviceBuffer(8 * fn * frhs)
                src_A, src_B = A, Bd
            else:
                src_A, src_B = DeviceBuffer(8 * fn * fn), DeviceBuffer(8 * fn * frhs)
                tmp = DeviceBuffer(8 * fn * fn)
                check(L.starpu_gb300_gen_spd_gram(stream, fn, 4321, 2.0, src_A.ptr, fn, tmp.ptr))
                check(L.starpu_gb300_gen_uniform_rhs(stream, fn, frhs, 77, src_B.ptr, fn))
                Af, Bf = tmp, DeviceBuffer(8 * fn * frhs)
                BW = DeviceBuffer(L.starpu_gb300_backward_error_workspace(fn, frhs))
            dinfo = DeviceBuffer(4)
            ts = []
            for r in range(2 if same else 3):
                check(L.starpu_gb300_memcpy_d2d(stream, Af.ptr, src_A.ptr, 8 * fn * fn))
                check(L.starpu_gb300_memcpy_d2d(stream, Bf.ptr, src_B.ptr, 8 * fn * frhs))
                a0, a1 = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
                check(L.starpu_gb300_event_record(a0, stream))
                check(L.starpu_gb300_dposv(stream, fn, frhs, Af.ptr, fn, Bf.ptr, fn, fnb, dinfo.ptr))
                check(L.starpu_gb300_event_record(a1, stream))
                t_ms = L.starpu_gb300_event_elapsed_ms(a0, a1)
                if r > 0:
                    ts.append(t_ms)
            be = np.zeros(frhs)
            check(L.starpu_gb300_backward_error(stream, fn, frhs, src_A.ptr, fn, Bf.ptr, fn, src_B.ptr, fn, BW.ptr,
                                                L.starpu_gb300_backward_error_workspace(fn, frhs),
                                                be.ctypes.data))
            t_ms = min(ts)
            fp64.append({"n": fn, "nb": fnb, "nrhs": frhs, "ms": t_ms,
                         "gflops": solve_flops(fn, frhs) / (t_ms * 1e-3) / 1e9, "backward_error": float(be.max()),
                         "kappa": args.kappa if same else "B B^T/N + 2I",
                         "_X": Bf.download((fn, frhs), np.float64) if want_oracle else None,
                         "_A": src_A.download((fn, fn), np.float64) if want_oracle and not same else None,
                         "_B": src_B.download((fn, frhs), np.float64) if want_oracle and not same else None})
            if not same:
                del src_A, src_B, tmp
    del with_work

    # ---- end to end: host buffers through the C-ABI solver context (H2D + solve + D2H per step)
    e2e, X_e2e = None, None
    if not args.no_e2e:
        hA = L.starpu_gb300_host_malloc_pinned(8 * n * n)
        hB = L.starpu_gb300_host_malloc_pinned(8 * n * nrhs)
        hX = L.starpu_gb300_host_malloc_pinned(8 * n * nrhs)
        assert hA and hB and hX
        # the host inputs are written by the CPU, as a host program produces them:
        # pinned pages last written by a device-to-host copy read back at a
        # fraction of the link rate on this host, CPU-written ones at full rate
        tmp = L.starpu_gb300_host_malloc_pinned(8 * n * n)
        assert tmp
        for dst, src, nbytes in ((hA, A.ptr, 8 * n * n), (hB, Bd.ptr, 8 * n * nrhs)):
            check(L.starpu_gb300_memcpy_d2h(stream, tmp, src, nbytes))
            check(L.starpu_gb300_stream_sync(stream))
            C.memmove(dst, tmp, nbytes)
        L.starpu_gb300_host_free_pinned(tmp)
        del W  # the context owns its own workspace
        ctx = L.starpu_gb300_solver_create(n, nrhs, nb, args.nterms)
        assert ctx, L.starpu_gb300_last_error()
        einfo = IrInfo()

        def e2e_step():
            rc = L.starpu_gb300_solver_dsposv_host(ctx, n, nrhs, hA, n, hB, n, hX, n, 1e-12, args.max_iter,
                                                   C.byref(einfo))
            assert rc == 0, rc

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        dist.barrier()
        L.starpu_gb300_profiling_reset()
        L.starpu_gb300_profiling_enable(1)
        t0 = time.perf_counter()
        lat = []
        for _ in range(args.steps):
            s0 = time.perf_counter()
            e2e_step()
            lat.append(time.perf_counter() - s0)
        te = dist.max((time.perf_counter() - t0) / args.steps)
        L.starpu_gb300_profiling_enable(0)
        la, tms, by = C.c_ulonglong(), C.c_double(), C.c_double()
        L.starpu_gb300_profiling_get(5, C.byref(la), C.byref(tms), None, C.byref(by))
        xfer = {"ms_per_step": tms.value / args.steps, "bytes_per_step": by.value / args.steps,
                "gbs": (by.value / (tms.value * 1e-3) / 1e9) if tms.value else None}
        # the host path moves A's lower triangle as 512-column trapezoidal panels
        h2d = sum(8 * (n - j0) * min(512, n - j0) for j0 in range(0, n, 512)) + 8 * n * nrhs
        if want_oracle:
            X_e2e = np.empty((n, nrhs), np.float64, order="F")
            C.memmove(X_e2e.ctypes.data, hX, X_e2e.nbytes)
        e2e = {"value": world * flops / te / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": 8 * n * nrhs, "ms_per_step": te * 1e3,
               "solves_per_s": world / te, "p50_ms": 1e3 * statistics.median(lat),
               "p99_ms": 1e3 * sorted(lat)[min(len(lat) - 1, int(0.99 * len(lat)))],
               "backward_error": einfo.backward_error, "iterations": einfo.iterations, "transfers": xfer}
        L.starpu_gb300_solver_destroy(ctx)
        L.starpu_gb300_host_free_pinned(hA)
        L.starpu_gb300_host_free_pinned(hB)
        L.starpu_gb300_host_free_pinned(hX)

    # ---- configs 4 and 5
    batched = bench_batched(L) if not args.no_batched else None
    serving = bench_serving(L) if not args.no_serving else None

    # ---- CPU baseline (rank 0, N=1 only): StarPU CPU path port on the bench
    # system itself (one solve), whose FP64 solution is also the oracle for the
    # forward errors of every GPU result of this run
    cpu, accuracy = None, None
    if want_oracle:
        from oracle import oracle as O
        if O.cpu_init():
            cores = len(os.sched_getaffinity(0))
            Ah = A.download((n, n), np.float64)  # kappa = args.kappa (the sweep restored it)
            Bh = Bd.download((n, nrhs), np.float64)
            cnb = args.cpu_nb or nb
            Xo, t_cpu = oracle_solve(Ah, Bh, cnb, cores)
            cpu = {"value": flops / t_cpu / 1e9, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                   "sample": f"FP64 tiled Cholesky (StarPU CPU codelets port, OpenBLAS, {cores} workers) + dpotrs, "
                             f"the bench system itself: N={n}, tile {cnb}, {nrhs} RHS, kappa={args.kappa:g}; one solve",
                   "seconds_per_solve": t_cpu, "backward_error": host_backward_error(Ah, Xo, Bh)}
            cpu["config1"] = cpu_config1()
            oracle_note = ("FP64 oracle: the port of StarPU's CPU path (tiled FP64 Cholesky over OpenBLAS, pinned "
                           "to CLAPACK dpotrf/dpotrs) on the same inputs; forward error = max_j ||x_j - xo_j||_inf "
                           "/ ||xo_j||_inf; backward errors recomputed on the host in FP64")
            accuracy = {"oracle": oracle_note, "dsposv": accuracy_of(Ah, Bh, X_main, Xo, args.kappa)}
            if e2e is not None and X_e2e is not None:
                accuracy["e2e"] = accuracy_of(Ah, Bh, X_e2e, Xo, args.kappa)
            fp_same = next((f for f in fp64 if f["n"] == n), None)
            if fp_same is not None and fp_same["_X"] is not None:
                accuracy["fp64_plain_same_n"] = accuracy_of(Ah, Bh, fp_same["_X"], Xo, args.kappa)
            ks = []
            for sw in sweep:
                if sw["_X"] is None:
                    continue
                if sw["kappa"] == args.kappa:
                    ks.append(accuracy_of(Ah, Bh, sw["_X"], Xo, sw["kappa"]))
                    continue
                shift = alpha_for_kappa(sw["kappa"]) - alpha_for_kappa(args.kappa)
                Xk, _ = oracle_solve(Ah, Bh, cnb, cores, shift)
                ks.append(accuracy_of(Ah, Bh, sw["_X"], Xk, sw["kappa"], shift))
            accuracy["kappa_sweep"] = ks
            del Ah, Xo
            cfg2 = next((f for f in fp64 if f["n"] != n), None)
            if cfg2 is not None and cfg2["_A"] is not None:
                X2, _ = oracle_solve(cfg2["_A"], cfg2["_B"], cfg2["nb"], cores)
                accuracy["fp64_config2"] = accuracy_of(cfg2["_A"], cfg2["_B"], cfg2["_X"], X2, "B B^T/N + 2I")
            for key, res in (("batched", batched), ("serving", serving)):
                if res is None:
                    continue
                rows = []
                for smp in res["_samples"]:
                    Xs, _ = oracle_solve(smp["A"], smp["B"], 512, cores)
                    r = accuracy_of(smp["A"], smp["B"], smp["X"], Xs, smp["kappa"])
                    r.update({k: v for k, v in smp.items() if k not in ("A", "B", "X", "kappa")})
                    rows.append(r)
                accuracy[key] = {"samples": rows, "max_forward_error": max(r["forward_error"] for r in rows),
                                 "max_backward_error_host": max(r["backward_error_host"] for r in rows)}

    def public(x):
        """The result without the host copies kept for the oracle (keys starting with _)."""
        if isinstance(x, dict):
            return {k: public(v) for k, v in x.items() if not k.startswith("_")}
        if isinstance(x, list):
            return [public(v) for v in x]
        return x

    if rank == 0:
        fp64_same = next((f for f in fp64 if f["n"] == n), None)
        fp64, sweep, batched, serving = public(fp64), public(sweep), public(batched), public(serving)
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, world), "factor_terms": args.nterms, "generation_s": gen_s,
            "schedule": schedule,
            "backward_error": max(berrs), "backward_error_fp64_check": berr_fp64_check, "iterations": iters,
            "forward_error": accuracy["dsposv"]["forward_error"] if accuracy else None, "accuracy": accuracy,
            "vs_fp64_plain_same_n": (value / world / fp64_same["gflops"]) if fp64_same else None,
            "fp64_plain": fp64, "kappa_sweep": sweep, "batched": batched, "serving": serving,
            "roofline": roofline, "kernels": prof,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        }
        print(json.dumps(line))
    dist.close()
    return 0


# ------------------------------------------------------- single-kernel cases
KERNEL_CASES_DOC = """Single-kernel cases for profiling (ncu) and quick timing, through the C-ABI:

    python bench.py --case tc_update --m 8192 --k 1024 --nterms 3 --reps 3
    python bench.py --case residual  --n 16384 --nrhs 16 --reps 3
    python bench.py --case potrs     --n 16384 --nrhs 16 --reps 3
    python bench.py --case sweep     --n 16384 --nrhs 16 --reps 3
    python bench.py --case dsposv    --n 8192  --nb 1024 --nrhs 16 --reps 2
    python bench.py --case spotrf_tc --n 8192  --nb 1024 --nterms 3 --reps 2
    python bench.py --case dpotrf    --n 8192  --nb 512 --reps 2
    python bench.py --case tile_ops  --n 1024 --reps 200
    python bench.py --case diag      --n 1024 --reps 50
    python bench.py --case tile_sweep --n 32768 --nb 1024 --nrhs 16 --reps 5
    python bench.py --case syresidual --n 32768 --nrhs 16 --reps 3
    python bench.py --case batched --nsys 512 --reps 1
    python bench.py --case lu_tile --n 1024 --reps 3
    python bench.py --case dsposv_host --n 8192 --nb 1024 --nrhs 16 --reps 2
    python bench.py --case factor_error --n 8192 --nb 1024 --kappa 1e4
    python bench.py --case update_error --m 2048 --k 1024
    python bench.py --case tile_tc --m 8192 --k 1024 --reps 3

Each case allocates its operands once, runs `--reps` launches of the same
shape and prints the mean time per launch measured with CUDA events.
"""


def _timed(L, fn, reps):
    from starpu_gb300.native import check
    fn()
    check(L.starpu_gb300_stream_sync(None))
    e0, e1 = L.starpu_gb300_event_create(), L.starpu_gb300_event_create()
    check(L.starpu_gb300_event_record(e0, None))
    for _ in range(reps):
        fn()
    check(L.starpu_gb300_event_record(e1, None))
    ms = L.starpu_gb300_event_elapsed_ms(e0, e1) / reps
    L.starpu_gb300_event_destroy(e0)
    L.starpu_gb300_event_destroy(e1)
    return ms


def oracle_free_spd(n):
    import numpy as np
    """FP32 SPD test matrix: 1 / (1 + i + j) plus n on the diagonal."""
    i = np.arange(n, dtype=np.float32)
    A = 1.0 / (1.0 + i[:, None] + i[None, :])
    A[np.diag_indices(n)] += n
    return A.astype(np.float32)


def run_case(argv):
    """One single-kernel case (see KERNEL_CASES_DOC); prints one JSON line."""
    import numpy as np
    from starpu_gb300 import DeviceBuffer, load
    from starpu_gb300.native import check
    ap = argparse.ArgumentParser(prog="bench.py --case")
    ap.add_argument("case", choices=["tc_update", "residual", "potrs", "sweep", "spotrf_tc", "dpotrf", "dsposv",
                                     "tile_ops", "diag", "tile_sweep", "syresidual", "batched", "lu_tile",
                                     "dsposv_host", "factor_error", "update_error", "tile_tc"])
    ap.add_argument("--nsys", type=int, default=512)
    ap.add_argument("--kappa", type=float, default=1e4)
    ap.add_argument("--m", type=int, default=8192)
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--k", type=int, default=1024)
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--nterms", type=int, default=3)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    L = load()
    out = {"case": a.case}
    if a.case == "tc_update":
        m, k = a.m, a.k
        ldk = (k + 63) // 64 * 64
        P = DeviceBuffer(4 * m * k)
        hi, lo = DeviceBuffer(2 * m * ldk), DeviceBuffer(2 * m * ldk)
        Cb = DeviceBuffer(4 * m * m)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        check(L.starpu_gb300_memset(None, P.ptr, 0, 4 * m * k))
        check(L.starpu_gb300_memset(None, Cb.ptr, 0, 4 * m * m))
        check(L.starpu_gb300_split_bf16(None, m, k, P.ptr, m, hi.ptr, lo.ptr, ldk))
        ms = _timed(L, lambda: check(L.starpu_gb300_tc_update(None, m, m, k, hi.ptr, lo.ptr, ldk, hi.ptr, lo.ptr, ldk,
                                                               a.nterms, 1, Cb.ptr, m, err.ptr)), a.reps)
        fl = a.nterms * k * m * (m + 1.0)
        out.update(ms=ms, tflops=fl / ms / 1e9, algorithmic_bytes=8.0 * m * (m + 1) / 2 + 2.0 * m * ldk * 2)
    elif a.case in ("residual", "potrs", "sweep"):
        n, nrhs = a.n, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        Bd, Xd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 5, Xd.ptr, n))
        if a.case == "residual":
            lw = L.starpu_gb300_backward_error_workspace(n, nrhs)
            BW = DeviceBuffer(lw)
            be = np.zeros(nrhs)
            ms = _timed(L, lambda: check(L.starpu_gb300_backward_error(None, n, nrhs, A.ptr, n, Xd.ptr, n, Bd.ptr, n,
                                                                        BW.ptr, lw, be.ctypes.data)), a.reps)
            out.update(ms=ms, tflops=2.0 * n * n * nrhs / ms / 1e9, algorithmic_bytes=8.0 * n * n)
        else:
            # FP32 sweeps (the refinement's correction solve) with the lower part of a
            # diagonally dominant matrix as the factor
            i = np.arange(n, dtype=np.float32)
            Lh = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, :]), dtype=np.float32)
            Lh[np.diag_indices(n)] += n
            F = DeviceBuffer.from_array(Lh)
            Y = DeviceBuffer.from_array(np.ones((n, nrhs), np.float32))
            if a.case == "potrs":
                ms = _timed(L, lambda: check(L.starpu_gb300_spotrs(None, n, nrhs, F.ptr, n, Y.ptr, n)), a.reps)
            else:
                lw = L.starpu_gb300_spotrs_sweep_workspace(n)
                SW = DeviceBuffer(lw)
                err = DeviceBuffer.from_array(np.zeros(1, np.int32))
                ms = _timed(L, lambda: check(L.starpu_gb300_spotrs_sweep(None, n, nrhs, F.ptr, n, Y.ptr, n, SW.ptr, lw,
                                                                          err.ptr)), a.reps)
            # both sweeps read the lower triangle of L once: 2 * 4 * n^2 / 2 bytes
            out.update(ms=ms, gbs=4.0 * n * n / ms / 1e6)
    elif a.case == "spotrf_tc":
        n, nb = a.n, a.nb
        from_host = np.empty((n, n), np.float32, order="F")
        i = np.arange(n, dtype=np.float32)
        from_host[:] = 1.0 / (1.0 + i[:, None] + i[None, :])
        from_host[np.diag_indices(n)] += n
        F = DeviceBuffer.from_array(from_host)
        ws = L.starpu_gb300_spotrf_tc_workspace(n, nb)
        Wk = DeviceBuffer(ws)
        info, err = DeviceBuffer(4), DeviceBuffer.from_array(np.zeros(1, np.int32))

        def run():
            F.upload(from_host)
            check(L.starpu_gb300_spotrf_tc(None, n, F.ptr, n, nb, a.nterms, Wk.ptr, ws, info.ptr, err.ptr))
        ms = _timed(L, run, a.reps)
        out.update(ms_including_upload=ms)
    elif a.case == "tile_ops":
        # the FP32 pieces of the mixed solve's diagonal-tile factorisation: the
        # 64 x 64 leaf, the whole n x n tile, and one step's panel TRSM and SYRK
        # at their largest shape (n - 64 rows, 64 columns)
        n = a.n
        i = np.arange(n, dtype=np.float32)
        Ah = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, :]), dtype=np.float32)
        Ah[np.diag_indices(n)] += n
        A0, Aw = DeviceBuffer.from_array(Ah), DeviceBuffer(4 * n * n)
        info = DeviceBuffer(4)
        nbytes = 4 * n * n

        def restore():
            check(L.starpu_gb300_memcpy_d2d(None, Aw.ptr, A0.ptr, nbytes))
        ms_copy = _timed(L, restore, a.reps)

        def potrf(k):
            def f():
                restore()
                check(L.starpu_gb300_spotrf_tile(None, k, Aw.ptr, n, info.ptr))
            return f
        m, w = n - 64, 64
        ms_leaf = _timed(L, potrf(64), a.reps) - ms_copy
        ms_tile = _timed(L, potrf(n), a.reps) - ms_copy
        restore()
        check(L.starpu_gb300_spotrf_tile(None, n, Aw.ptr, n, info.ptr))
        Lw = DeviceBuffer.from_array(np.zeros((n, n), np.float32))
        check(L.starpu_gb300_memcpy_d2d(None, Lw.ptr, Aw.ptr, nbytes))
        ms_trsm = _timed(L, lambda: check(L.starpu_gb300_strsm_rltn_tile(None, m, w, 1.0, Lw.ptr, n, Aw.ptr + 4 * 64,
                                                                          n)), a.reps)
        ms_syrk = _timed(L, lambda: check(L.starpu_gb300_ssyrk_ln_tile(None, m, w, -1.0, Lw.ptr + 4 * 64, n, 1.0,
                                                                        Aw.ptr + 4 * (64 + 64 * n), n)), a.reps)
        out.update(n=n, ms_leaf64=ms_leaf, ms_tile=ms_tile, ms_trsm=ms_trsm, ms_syrk=ms_syrk, ms_restore=ms_copy,
                   tile_gflops=n ** 3 / 3 / ms_tile / 1e6)
    elif a.case == "diag":
        # the tensor-core Cholesky's diagonal-tile step alone: spotrf_tc of an
        # n x n matrix with nb = n (factor only), and of n + 64 with nb = n
        # (factor + inverse of the n x n tile, then a 64-row panel and update)
        n = a.n
        out.update(n=n)
        for tag, N in (("factor", n), ("factor_inverse_plus_64", n + 64)):
            Ah = np.asfortranarray(oracle_free_spd(N))
            A0, Aw = DeviceBuffer.from_array(Ah), DeviceBuffer(4 * N * N)
            ws = L.starpu_gb300_spotrf_tc_workspace(N, n)
            Wk = DeviceBuffer(ws)
            info, err = DeviceBuffer(4), DeviceBuffer.from_array(np.zeros(1, np.int32))

            def restore():
                check(L.starpu_gb300_memcpy_d2d(None, Aw.ptr, A0.ptr, 4 * N * N))

            def run():
                restore()
                check(L.starpu_gb300_spotrf_tc(None, N, Aw.ptr, N, n, 3, Wk.ptr, ws, info.ptr, err.ptr))
            ms_copy = _timed(L, restore, a.reps)
            out["ms_" + tag] = _timed(L, run, a.reps) - ms_copy
            out["err_" + tag] = int(DeviceBuffer.download(err, (1,), np.int32)[0])
    elif a.case == "tile_sweep":
        # both tile-row sweeps of one FP32 correction solve (identity
        # diagonal-tile inverses: the timing does not depend on the values)
        n, nb, nrhs = a.n, a.nb, a.nrhs
        i = np.arange(n, dtype=np.float32)
        F = DeviceBuffer(4 * n * n)
        for c0 in range(0, n, 2048):  # the factor column panel by column panel (host memory stays small)
            w = min(2048, n - c0)
            Lp = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, c0:c0 + w]), dtype=np.float32)
            Lp[np.arange(c0, c0 + w), np.arange(w)] += n
            check(L.starpu_gb300_memcpy_h2d(None, F.ptr + 4 * n * c0, Lp.ctypes.data, Lp.nbytes))
        ldd = (nb + 63) // 64 * 64
        ntiles = (n + nb - 1) // nb
        eye = np.asfortranarray(np.eye(ldd, dtype=np.float32))
        D = DeviceBuffer(4 * ntiles * ldd * ldd)
        for T in range(ntiles):
            check(L.starpu_gb300_memcpy_h2d(None, D.ptr + 4 * T * ldd * ldd, eye.ctypes.data, eye.nbytes))
        Y = DeviceBuffer.from_array(np.ones((n, nrhs), np.float32))
        lw = L.starpu_gb300_spotrs_inv_tiles_workspace(n, nb)
        Wk = DeviceBuffer(lw)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        ms = _timed(L, lambda: check(L.starpu_gb300_spotrs_inv_tiles(None, n, nrhs, nb, F.ptr, n, D.ptr, ldd, Y.ptr, n,
                                                                      Wk.ptr, lw, err.ptr)), a.reps)
        out.update(ms_two_sweeps=ms, gbs=4.0 * n * n / ms / 1e6, err=int(err.download((1,), np.int32)[0]))
    elif a.case == "syresidual":
        # the refinement residual R = B - A X on the tensor cores (symmetric A, lower triangle read)
        n, nrhs = a.n, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        del W
        Bd, Xd, Rd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 5, Xd.ptr, n))
        lw = L.starpu_gb300_dsyresidual_workspace(n, nrhs)
        Wk = DeviceBuffer(lw)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        ms = _timed(L, lambda: check(L.starpu_gb300_dsyresidual(None, n, nrhs, A.ptr, n, Xd.ptr, n, Bd.ptr, n, Rd.ptr, n,
                                                                 Wk.ptr, lw, err.ptr)), a.reps)
        out.update(ms=ms, tflops_fp64_equiv=2.0 * n * n * nrhs / ms / 1e9, err=int(err.download((1,), np.int32)[0]))
    elif a.case == "dpotrf":
        n, nb = a.n, a.nb
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 1.0, A.ptr, n, W.ptr))
        info = DeviceBuffer(4)

        def run():
            check(L.starpu_gb300_memcpy_d2d(None, W.ptr, A.ptr, 8 * n * n))
            check(L.starpu_gb300_dpotrf(None, n, W.ptr, n, nb, info.ptr))
        ms = _timed(L, run, a.reps)
        out.update(ms=ms, gflops=n ** 3 / 3 / ms / 1e6)
    elif a.case == "dsposv":
        from starpu_gb300.native import IrInfo
        n, nb, nrhs = a.n, a.nb, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        Bd, Xd = DeviceBuffer(8 * n * nrhs), DeviceBuffer(8 * n * nrhs)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 4.0 / (a.kappa - 1.0), A.ptr, n, W.ptr))
        check(L.starpu_gb300_gen_uniform_rhs(None, n, nrhs, 4, Bd.ptr, n))
        lw = L.starpu_gb300_dsposv_workspace(n, nrhs, nb)
        Wk = DeviceBuffer(lw)
        info = IrInfo()
        ms = _timed(L, lambda: check(L.starpu_gb300_dsposv(None, n, nrhs, A.ptr, n, Bd.ptr, n, Xd.ptr, n, nb, a.nterms,
                                                            1e-12, 30, Wk.ptr, lw, C.byref(info))), a.reps)
        out.update(ms=ms, gflops=(n ** 3 / 3 + 2.0 * n * n * nrhs) / ms / 1e6, iterations=info.iterations,
                   backward_error=info.backward_error)
    elif a.case == "batched":
        # the persistent batched solver on --nsys systems of the config's size distribution
        r = bench_batched(L, nsys=a.nsys)
        r.pop("_samples", None)
        out.update(r)
    elif a.case == "lu_tile":
        # the LU tile codelet body (no pivoting) on an n x n diagonally dominant FP32 tile
        n = a.n
        i = np.arange(n, dtype=np.float32)
        Ah = np.asfortranarray(1.0 / (1.0 + i[:, None] + i[None, :]), dtype=np.float32)
        Ah[np.diag_indices(n)] += n
        A0, Aw = DeviceBuffer.from_array(Ah), DeviceBuffer(4 * n * n)
        info = DeviceBuffer(4)

        def run():
            check(L.starpu_gb300_memcpy_d2d(None, Aw.ptr, A0.ptr, 4 * n * n))
            check(L.starpu_gb300_sgetrf_tile(None, n, Aw.ptr, n, info.ptr))
        ms = _timed(L, run, a.reps)
        out.update(n=n, ms_including_restore=ms, gflops=2.0 * n ** 3 / 3 / ms / 1e6)
    elif a.case == "dsposv_host":
        # the host-buffer solve of a solver context (gather over the host link with
        # the fused FP32 conversion, the solve, X back)
        from starpu_gb300.native import IrInfo
        n, nb, nrhs = a.n, a.nb, a.nrhs
        A = DeviceBuffer(8 * n * n)
        W = DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 3, 4.0 / (a.kappa - 1.0), A.ptr, n, W.ptr))
        del W
        # pinned host A: the context's gather kernel reads it over the host link.
        # Written by the CPU, as a host program produces it (pinned pages last
        # written by a device-to-host copy read back at a fraction of the link rate)
        hA = L.starpu_gb300_host_malloc_pinned(8 * n * n)
        tmp = L.starpu_gb300_host_malloc_pinned(8 * n * n)
        assert hA and tmp, L.starpu_gb300_last_error()
        check(L.starpu_gb300_memcpy_d2h(None, tmp, A.ptr, 8 * n * n))
        check(L.starpu_gb300_stream_sync(None))
        C.memmove(hA, tmp, 8 * n * n)
        L.starpu_gb300_host_free_pinned(tmp)
        hB = np.asfortranarray(np.random.default_rng(4).uniform(-1, 1, (n, nrhs)))
        hX = np.zeros((n, nrhs), order="F")
        ctx = L.starpu_gb300_solver_create(n, nrhs, nb, a.nterms)
        assert ctx, L.starpu_gb300_last_error()
        info = IrInfo()
        ms = _timed(L, lambda: check(L.starpu_gb300_solver_dsposv_host(ctx, n, nrhs, hA, n, hB.ctypes.data, n,
                                                                        hX.ctypes.data, n, 1e-12, 30, C.byref(info))),
                    a.reps)
        L.starpu_gb300_solver_destroy(ctx)
        L.starpu_gb300_host_free_pinned(hA)
        out.update(ms=ms, iterations=info.iterations, backward_error=info.backward_error)
    elif a.case == "factor_error":
        # ||A - L L^T||_F / ||A||_F of the FP32 factor of A = B B^T / n + alpha I (kappa), mixed (tensor-core)
        # factor with nterms 3 and 1, and the SIMT FP32 factor, FP64 on the host
        n, nb = a.n, a.nb
        dA, W0 = DeviceBuffer(8 * n * n), DeviceBuffer(8 * n * n)
        check(L.starpu_gb300_gen_spd_gram(None, n, 5, alpha_for_kappa(a.kappa), dA.ptr, n, W0.ptr))
        del W0
        A = dA.download((n, n), np.float64)
        del dA
        A32 = np.asfortranarray(A.astype(np.float32))
        for name, nt in (("mixed_nterms3", 3), ("mixed_nterms1", 1), ("simt_fp32", 0)):
            d = DeviceBuffer.from_array(A32)
            info, err = DeviceBuffer.from_array(np.zeros(1, np.int32)), DeviceBuffer.from_array(np.zeros(1, np.int32))
            if nt:
                ws = L.starpu_gb300_spotrf_tc_workspace(n, nb)
                Wk = DeviceBuffer(ws)
                check(L.starpu_gb300_spotrf_tc(None, n, d.ptr, n, nb, nt, Wk.ptr, ws, info.ptr, err.ptr))
            else:
                check(L.starpu_gb300_spotrf(None, n, d.ptr, n, nb, info.ptr))
            check(L.starpu_gb300_stream_sync(None))
            Lf = np.tril(d.download((n, n), np.float32).astype(np.float64))
            out[name] = float(np.linalg.norm(Lf @ Lf.T - A) / np.linalg.norm(A))
    elif a.case == "tile_tc":
        # the tensor-core tile update of the codelets on one m x m tile, K = k:
        # FP32 operand split to row-scaled FP16, lower update C -= A A^T
        m, k = a.m, a.k
        rng = np.random.default_rng(2)
        P = DeviceBuffer.from_array(np.asfortranarray(rng.standard_normal((m, k)).astype(np.float32)))
        Cb = DeviceBuffer.from_array(np.zeros((m, m), np.float32, order="F"))
        lw = L.starpu_gb300_tile_tc_workspace(max(m, k))
        Wk = DeviceBuffer(lw)
        err = DeviceBuffer.from_array(np.zeros(1, np.int32))
        check(L.starpu_gb300_tile_tc_prepare())
        ms = _timed(L, lambda: check(L.starpu_gb300_sgemm_nt_tile_tc(None, m, m, k, P.ptr, m, P.ptr, m, Cb.ptr, m, 1,
                                                                      Wk.ptr, lw, err.ptr)), a.reps)
        out.update(m=m, k=k, ms_including_split=ms, tflops=3.0 * k * m * (m + 1.0) / ms / 1e9)
    elif a.case == "update_error":
        # one BF16 split update C = -P P^T (m x K) against its FP64 product, rms relative error
        m, k = a.m, a.k
        rng = np.random.default_rng(1)
        P = np.asfortranarray(rng.standard_normal((m, k)).astype(np.float32) / 32)
        dP = DeviceBuffer.from_array(P)
        hi, lo = DeviceBuffer(2 * m * k), DeviceBuffer(2 * m * k)
        check(L.starpu_gb300_split_bf16(None, m, k, dP.ptr, m, hi.ptr, lo.ptr, k))
        ex = P.astype(np.float64) @ P.astype(np.float64).T
        for nt in (1, 3):
            dC = DeviceBuffer.from_array(np.zeros((m, m), np.float32))
            err = DeviceBuffer.from_array(np.zeros(1, np.int32))
            check(L.starpu_gb300_tc_update(None, m, m, k, hi.ptr, lo.ptr, k, hi.ptr, lo.ptr, k, nt, 0, dC.ptr, m,
                                           err.ptr))
            Cg = -dC.download((m, m), np.float32).astype(np.float64)
            out[f"bf16_nterms{nt}_rms"] = float(np.sqrt(((Cg - ex) ** 2).mean() / (ex ** 2).mean()))
    print(json.dumps(out))



def main():
    if "--case" in sys.argv[1:]:
        argv = sys.argv[1:]
        i = argv.index("--case")
        return run_case(argv[:i] + argv[i + 1:]) or 0
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=32768)
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--kappa", type=float, default=1e4)
    ap.add_argument("--nterms", type=int, default=3)
    ap.add_argument("--max-iter", type=int, default=30)
    ap.add_argument("--fp64-n", type=int, default=16384)
    ap.add_argument("--cpu-n", type=int, default=0, help="order of the reference arm's system (0: --n)")
    ap.add_argument("--cpu-nb", type=int, default=0, help="tile of the CPU path (0: --nb)")
    ap.add_argument("--tc-traffic", type=float, default=None,
                    help="DRAM bytes per trailing-update launch (default: the ncu capture of an m = 8192 launch "
                         "scaled to the factorisation's launches)")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the stored or default factorisation schedule")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-fp64-same-n", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # timing rule: at least 3 untimed warm-up steps
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
