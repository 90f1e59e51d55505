"""Benchmark of the SLQ log-determinant path (one JSON line on stdout).

Workload (default): the dense RBF kernel log-determinant of n = 16384 points
x ~ U[0, 1]^3, K = exp(-|x_i - x_j|^2 / (2 * 0.2^2)) + 1e-2 I, Lanczos depth
k = 64, p = 256 Rademacher probes, operator stored as a bf16 hi/lo split and
applied with the three-term split product on the tensor cores.  One step is
one complete log-determinant solve: build K from the points, draw the probes,
run the batched Arnoldi/CGS2 iteration, the tridiagonal eigensolves and the
quadrature, and average.  Inputs (operator 1.07 GB, Krylov basis 1.07 GB)
are larger than L2, so no flush is needed between steps.

--impl reference times the float64 NumPy restatement of matfree's algorithm
(the oracle; matfree itself is JAX and cannot run here) on the host cores on
a bounded probe sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (kind, n, k, p)
    "rbf16k": ("rbf", 16384, 64, 256),
    # small case of the same kernels for ncu captures (operator 268 MB and
    # basis 134 MB: both above L2)
    "rbf8k": ("rbf", 8192, 16, 256),
    # same, with the bench depth k = 64 (basis 537 MB) for captures of late steps
    "rbf8k64": ("rbf", 8192, 64, 256),
    # the bench's operator (n = 16384, 1.07 GB in bf16 hi + lo) at depth 4,
    # for captures of the full-size operator apply
    "rbf16k4": ("rbf", 16384, 4, 256),
    "dense1k": ("dense", 1000, 30, 100),
    # the sparse config's operator and panel at depth 4 (basis 1.07 GB), for
    # captures of the sparse product
    "laplace1m4": ("csr", 1024 * 1024, 4, 64),
    "laplace1m": ("csr", 1024 * 1024, 100, 64),
}
METRIC = "logdet solves/s"
UNIT = "solves/s"


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"hbm": float(d["hbm_gbs"]), "tensor_burst": float(d["bf16_tflops"]),
                "tensor_sustained": float(d["bf16_tflops_sustained"]), "source": "measured"}
    except Exception:
        return {"hbm": 6800.0, "tensor_burst": 1900.0, "tensor_sustained": 1700.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------


def _dist_init(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    return rank, world, local


def _barrier(world):
    from matfree_gb300 import replicas

    replicas.barrier(world)


def _max_over_ranks(x, world):
    from matfree_gb300 import replicas

    return replicas.max_over_ranks(x, world)


def build_problem(cfg, seed=0):
    """Host-side inputs of one solve (same seeds for both arms)."""
    kind, n, k, p = CONFIGS[cfg]
    if kind == "rbf":
        x = np.random.default_rng(seed).uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
        return {"kind": kind, "n": n, "k": k, "p": p, "x": x, "s2": 1.0, "ell": 0.2, "tau": 1e-2}
    if kind == "dense":
        B = np.random.default_rng(seed).standard_normal((n, n))
        return {"kind": kind, "n": n, "k": k, "p": p, "A": B @ B.T / n + np.eye(n)}
    m = int(round(math.sqrt(n)))
    import scipy.sparse as sp

    main = np.full(n, 4.0 + 0.1)
    side = -np.ones(n - 1)
    side[np.arange(1, n) % m == 0] = 0.0
    ud = -np.ones(n - m)
    A = sp.diags([main, side, side, ud, ud], [0, -1, 1, -m, m], format="csr")
    A.eliminate_zeros()
    A.sort_indices()
    return {"kind": kind, "n": n, "k": k, "p": p, "csr": A}


class _Slot:
    """One in-flight solve: its stream, workspace and result buffers."""

    def __init__(self, torch, dev):
        from matfree_gb300._panel import Workspace

        self.stream = torch.cuda.Stream(device=dev)
        self.ws = Workspace()
        self.mean_sem = torch.zeros(2, dtype=torch.float64, device=dev)
        self.host = torch.zeros(2, dtype=torch.float64).pin_memory()
        self.done = torch.cuda.Event()
        self.pending = None  # inputs of the solve in flight, until its status is read


def gpu_arm(args):
    import ctypes

    import torch

    import matfree_gb300 as mf
    from matfree_gb300 import _lib
    from matfree_gb300.funm import slq_retry_needed, slq_values

    rank, world, local = _dist_init(args.gpus)
    prob = build_problem(args.config)
    kind, n, k, p = prob["kind"], prob["n"], prob["k"], prob["p"]
    precision = args.precision
    tuned = None
    if precision in ("bf16", "bf16x3") and kind in ("rbf", "dense") and not args.no_autotune:
        # the tensor-core product's tile configuration for this GPU (timed once
        # per machine, outside the measured region, and cached)
        from matfree_gb300 import tuning

        rules = tuning.ensure(precision=precision)
        tuned = next((r for r in rules if r["n_lo"] <= n <= r["n_hi"] and r["p_lo"] <= min(p, 256) <= r["p_hi"]),
                     None)
    dev = torch.device("cuda", torch.cuda.current_device())
    key = mf.prng.prng_key(1 + rank)

    if kind == "rbf":
        x_host = torch.from_numpy(prob["x"]).pin_memory()
        x_dev = x_host.to(dev)
        static = None
    elif kind == "dense":
        static = mf.DenseOperator(torch.from_numpy(prob["A"]).to(dev), precision=precision)
        x_host = x_dev = None
    else:
        static = mf.CSROperator.from_scipy(prob["csr"], device=dev)
        x_host = x_dev = None
    sampler = mf.stochtrace.sampler_signs(torch.ones(n, device=dev), num=p)
    slots = [_Slot(torch, dev) for _ in range(max(1, args.inflight))]

    retries = [0]

    def solve(x, slot, h2d=False, two_sweep=None):
        """One complete solve enqueued on the slot's stream (its device status is
        read by finish() once the slot is reused)."""
        with torch.cuda.stream(slot.stream):
            if h2d:
                x = x_host.to(dev, non_blocking=True)
            if kind == "rbf":
                op = mf.RBFKernelOperator(x, s2=prob["s2"], ell=prob["ell"], tau=prob["tau"],
                                          precision=precision)
            else:
                op = static
            V = sampler(key)
            vals = slq_values(op, k, V, _lib.MFG_FUN_LOG, 0.0, mean_sem=slot.mean_sem,
                              workspace=slot.ws, two_sweep=two_sweep, check=False)
            if h2d:
                slot.host.copy_(slot.mean_sem, non_blocking=True)
            slot.done.record(slot.stream)
            slot.pending = (x, h2d)
        return vals

    def finish(slot):
        """Wait for the slot's solve; repeat it with the three-sweep form if the
        two-sweep step reported MFG_ERR_RETRY."""
        if slot.pending is None:
            return
        x, h2d = slot.pending
        slot.pending = None
        with torch.cuda.stream(slot.stream):
            if slq_retry_needed(slot.ws):
                retries[0] += 1
                solve(x, slot, h2d, two_sweep=False)
                slot.pending = None
                slot.done.synchronize()

    def join_all():
        cur = torch.cuda.current_stream()
        for s in slots:
            cur.wait_stream(s.stream)

    def fork_all():
        for s in slots:
            s.stream.wait_stream(torch.cuda.current_stream())

    for i in range(args.warmup):
        finish(slots[i % len(slots)])
        solve(x_dev, slots[i % len(slots)])
    for s_ in slots:
        finish(s_)
    join_all()
    torch.cuda.synchronize()
    lib = _lib.lib()

    # (1) throughput: solves round-robin over the in-flight slots, device-resident inputs
    lib.mfg_profile_enable(0)  # launch counting only
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    _barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        fork_all()
        for i in range(args.steps):
            slot = slots[i % len(slots)]
            finish(slot)  # the solve this slot ran before: done, status read
            starts[i].record(slot.stream)
            values = solve(x_dev, slot)
            ends[i].record(slot.stream)
        for s_ in slots:
            finish(s_)
        join_all()
        t1.record()
        torch.cuda.synchronize()
        _barrier(world)
    clocks = clk.summary()
    total_ms = _max_over_ranks(t0.elapsed_time(t1), world)
    step_ms = sorted(s.elapsed_time(e) for s, e in zip(starts, ends))
    nc = len(_lib.PROF_CLASSES)
    ln = (ctypes.c_int64 * nc)()
    _lib.check(lib.mfg_profile_read(nc, None, None, None, ln), "mfg_profile_read")
    launches = int(sum(ln))
    est = float(slots[(args.steps - 1) % len(slots)].mean_sem[0].item())

    # (2) roofline: the same steps on one stream, every launch bracketed by events
    lib.mfg_profile_enable(1)
    torch.cuda.synchronize()
    for i in range(args.steps):
        finish(slots[0])
        solve(x_dev, slots[0])
    finish(slots[0])
    torch.cuda.synchronize()
    ms = (ctypes.c_double * nc)()
    by = (ctypes.c_double * nc)()
    fl = (ctypes.c_double * nc)()
    ln1 = (ctypes.c_int64 * nc)()
    _lib.check(lib.mfg_profile_read(nc, ms, by, fl, ln1), "mfg_profile_read")
    lib.mfg_profile_enable(0)
    prof = {c: {"ms": ms[i], "bytes": by[i], "flops": fl[i], "launches": int(ln1[i])}
            for i, c in enumerate(_lib.PROF_CLASSES)}

    # (3) end to end through the public API: pinned host points in, (mean, sem) out
    e2e = None
    if kind == "rbf":
        torch.cuda.synchronize()
        _barrier(world)
        t_start = time.perf_counter()
        for i in range(args.steps):
            slot = slots[i % len(slots)]
            if i >= len(slots):
                slot.done.synchronize()
                finish(slot)
                _ = float(slot.host[0])  # the result of the solve this slot ran before
            solve(None, slot, h2d=True)
        for i in range(max(0, args.steps - len(slots)), args.steps):
            slots[i % len(slots)].done.synchronize()
            finish(slots[i % len(slots)])
            _ = float(slots[i % len(slots)].host[0])
        e2e_s = _max_over_ranks(time.perf_counter() - t_start, world)
        e2e = {"value": world * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(x_host.numel() * 4), "d2h_bytes_per_step": 16}

    # (4) the plain per-request FP32 drop-in on the same problem: fp32 operator
    # on the CUDA cores, one solve at a time (the comparison the metric names)
    plain = None
    if kind == "rbf" and precision != "fp32" and rank == 0 and not args.no_plain_fp32:
        def plain_simt():
            op = mf.RBFKernelOperator(x_dev, s2=prob["s2"], ell=prob["ell"], tau=prob["tau"],
                                      precision="fp32")
            return slq_values(op, k, sampler(key), _lib.MFG_FUN_LOG, 0.0, workspace=slots[0].ws)

        def plain_cublas():
            # the operator product as a library SGEMM (cuBLAS through torch, TF32
            # off) called back once per Krylov step; K symmetric, so V K = (K V^T)^T
            op = mf.RBFKernelOperator(x_dev, s2=prob["s2"], ell=prob["ell"], tau=prob["tau"],
                                      precision="fp32")
            K = op.a[:, :n]
            tau = prob["tau"]
            cb = mf.CallbackOperator(lambda X: torch.addmm(X, X, K, beta=tau), n, batched=True)
            return slq_values(cb, k, sampler(key), _lib.MFG_FUN_LOG, 0.0, workspace=slots[0].ws)

        tf32 = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        plain = {}
        for name, fn in (("simt", plain_simt), ("cublas", plain_cublas)):
            fn()
            torch.cuda.synchronize()
            t_p = time.perf_counter()
            for _ in range(2):
                pv = fn()
            torch.cuda.synchronize()
            plain[name] = {"solves_per_s": 2.0 / (time.perf_counter() - t_p), "values": pv}
        torch.backends.cuda.matmul.allow_tf32 = tf32

    result = {"rank": rank, "world": world, "total_ms": total_ms, "step_ms": step_ms, "prof": prof, "tuned": tuned,
              "clocks": clocks, "estimate": est, "e2e": e2e, "values": values, "key": key,
              "launches": launches, "plain": plain, "two_sweep_retries": retries[0]}
    return result, prob


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
# capture of that exact launch: --set full on `--config rbf16k4` (the same operator and
# panel as rbf16k), kernel dense_tcgen05_pair_kernel<1>: 1.107385 GB read + 3.65 MB written.
TRAFFIC = {("rbf16k", "bf16x3", "operator apply"): 1.107385e9 + 3.649536e6}


# FMA-pipe peaks of one GB300 (no measured figure exists for these pipes):
# fp32 = 152 SMs x 128 lanes x 2 flop x 2.07 GHz; fp64 = NVIDIA's published rate
SIMT_PEAKS = {"fp32": ("fp32 fma", 152 * 128 * 2 * 2.07e9 / 1e12, "nominal: 152 SMs x 128 FMA/clk x 2.07 GHz"),
              "fp64": ("fp64 fma", 1.25, "nominal: published GB300 FP64 rate")}


def _two_sweep(args, prob):
    """Whether the solves ran the two-sweep step (float bases, 2 <= k <= 129)."""
    return args.precision != "fp64" and 2 <= prob["k"] <= 129


def roofline(prof, peaks, steps, config=None, precision=None):
    """The class with the largest time share; HBM- or tensor-bound by its class."""
    total = sum(v["ms"] for v in prof.values()) or 1.0
    shares = {c: v["ms"] / total for c, v in prof.items()}
    cls = ("proj", "subproj", "sub")
    reortho_ms = sum(prof[c]["ms"] for c in cls)
    reortho_b = sum(prof[c]["bytes"] for c in cls)
    apply_ms = prof["apply"]["ms"]
    launches_reortho = sum(prof[c]["launches"] for c in cls)
    if reortho_ms >= apply_ms:
        per_launch_b = reortho_b / max(launches_reortho, 1)
        per_launch_s = reortho_ms / 1e3 / max(launches_reortho, 1)
        achieved = per_launch_b / per_launch_s / 1e9
        return {"kernel": "cgs2 reortho sweeps (proj, subproj, sub)", "bound": "hbm",
                "achieved": achieved, "peak": peaks["hbm"], "unit": "GB/s",
                "frac": achieved / peaks["hbm"], "traffic": None, "time_share": reortho_ms / total,
                "launches": launches_reortho, "shares": shares,
                "per_class_gbs": {c: (prof[c]["bytes"] / (prof[c]["ms"] / 1e3) / 1e9 if prof[c]["ms"] else None) for c in cls}}
    fl = prof["apply"]["flops"]
    launches = max(prof["apply"]["launches"], 1)
    if fl > 0:
        achieved = (fl / launches) / (apply_ms / 1e3 / launches) / 1e12
        if precision in SIMT_PEAKS:
            # fp32 / fp64 products run on the FMA pipes, not the tensor cores
            bound, peak, src = SIMT_PEAKS[precision]
            return {"kernel": "operator apply", "bound": bound, "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None, "peak_override": src,
                    "time_share": apply_ms / total, "launches": launches, "shares": shares}
        peak = peaks["tensor_burst"]
        return {"kernel": "operator apply", "bound": "tensor", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": TRAFFIC.get((config, precision, "operator apply")),
                "traffic_unit": "bytes per launch",
                "time_share": apply_ms / total, "launches": launches, "shares": shares}
    b = prof["apply"]["bytes"]
    achieved = (b / launches) / (apply_ms / 1e3 / launches) / 1e9
    return {"kernel": "operator apply", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm"],
            "unit": "GB/s", "frac": achieved / peaks["hbm"], "traffic": None,
            "time_share": apply_ms / total, "launches": launches, "shares": shares}


# --------------------------------------------------------------------------
# CPU arm (oracle restatement of matfree's algorithm, float64)
# --------------------------------------------------------------------------


def cpu_sample(prob, probes):
    """float64 SLQ of the given probe rows; returns (values, seconds, build seconds)."""
    from oracle import problems, slq

    t0 = time.perf_counter()
    if prob["kind"] == "rbf":
        K = problems.rbf_kernel(prob["x"].astype(np.float64), prob["s2"], prob["ell"], 0.0)
        K[np.diag_indices_from(K)] += prob["tau"]

        def matmat(X):
            return X @ K

    elif prob["kind"] == "dense":
        A = prob["A"].astype(np.float64)

        def matmat(X):
            return X @ A.T

    else:
        A = prob["csr"].astype(np.float64)

        def matmat(X):
            return (A @ X.T).T

    t1 = time.perf_counter()
    vals = slq.slq_batched(matmat, prob["k"], probes)
    t2 = time.perf_counter()
    return vals, t2 - t0, t1 - t0


CPU_BASIS_BYTES = 8e9  # host memory the float64 restatement may hold for its Krylov bases


def cpu_probe_count(prob):
    """All probes when their float64 Krylov bases fit in CPU_BASIS_BYTES,
    otherwise the largest probe count that does (the bases of laplace1m's 64
    probes alone would take 54 GB)."""
    per_probe = 8.0 * (prob["k"] + 1) * prob["n"]
    return int(max(1, min(prob["p"], CPU_BASIS_BYTES // per_probe)))


def rel_err_summary(got, want):
    """Relative error of the estimate (mean over all probes) against the float64
    oracle on identical probes, with the per-probe spread."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    per = np.abs(got - want) / np.abs(want)
    return {"value": float(abs(got.mean() - want.mean()) / abs(want.mean())),
            "on": f"mean over all {len(want)} probes, identical probe vectors",
            "per_probe_median": float(np.median(per)), "per_probe_max": float(per.max())}


def cpu_probe_sample(prob, key, num):
    from oracle import philox

    return philox.rademacher(key, num, prob["n"])[:num]


def reference_arm(args):
    import torch  # noqa: F401  (only for rank discovery parity)

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import matfree_gb300.prng as prng_host

    prob = build_problem(args.config)
    key = prng_host.prng_key(1)
    num = cpu_probe_count(prob)
    probes = cpu_probe_sample(prob, key, num)
    warm = probes[: min(8, num)]
    # warm-up steps page in the operator build and the BLAS thread pool on a
    # few probes; every timed step is one complete solve (all probes, full n, k)
    for _ in range(args.warmup):
        cpu_sample(prob, warm)
    # Complete solves take ~20 s on 16 cores: the timed steps stop once they
    # have used the time budget (at least one step), so that the run stays
    # within a few minutes; the line reports the steps actually timed.
    secs = []
    for _ in range(args.steps):
        _, s_, _ = cpu_sample(prob, probes)
        secs.append(s_)
        if sum(secs) >= args.reference_budget_s:
            break
    steps = len(secs)
    total = sum(secs)
    value = steps / total
    sample = (f"every timed step one complete solve: operator build and all {prob['p']} probes at "
              f"full n and k, no extrapolation (warm-up steps on {len(warm)} probes); {steps} of "
              f"{args.steps} requested steps timed within a {args.reference_budget_s:.0f} s budget")
    if num < prob["p"]:
        # bases of all probes exceed host memory: time the probe subset and scale
        value = value * num / prob["p"]
        sample = (f"every timed step {num} of {prob['p']} probes at full n and k (their float64 bases "
                  f"fill {CPU_BASIS_BYTES / 1e9:.0f} GB of host memory), rate scaled by {num}/{prob['p']}")
    cores = len(os.sched_getaffinity(0))
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": steps, "steps_requested": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample + "; float64 NumPy/OpenBLAS restatement of matfree's "
                                                "algorithm"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _config(args):
    kind, n, k, p = CONFIGS[args.config]
    desc = {"rbf": "dense RBF kernel log-det (x~U[0,1]^3, ell=0.2, tau=1e-2)",
            "dense": "dense SPD B B^T/n + I log-det", "csr": "5-point Laplacian + 0.1 I log-det (CSR)"}[kind]
    opdesc = "CSR fp32 (int32 indices)" if kind == "csr" else args.precision
    return {"workload": f"{desc}, n={n}, k={k}, p={p} Rademacher probes, operator {opdesc}",
            "n": n, "k": k, "p": p, "precision": args.precision, "parallelism": "replicas",
            "l2": "inputs larger than L2 (operator and Krylov basis > 129 MB); no flush"}


def _profiled(fn, steps):
    """Run fn() `steps` times with every library launch bracketed by CUDA
    events; returns the per-class profile (ms, bytes, flops, launches)."""
    import ctypes

    import torch

    from matfree_gb300 import _lib

    lib = _lib.lib()
    nc = len(_lib.PROF_CLASSES)
    lib.mfg_profile_enable(1)
    torch.cuda.synchronize()
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    ms, by, fl = (ctypes.c_double * nc)(), (ctypes.c_double * nc)(), (ctypes.c_double * nc)()
    ln = (ctypes.c_int64 * nc)()
    _lib.check(lib.mfg_profile_read(nc, ms, by, fl, ln), "mfg_profile_read")
    lib.mfg_profile_enable(0)
    return {c: {"ms": ms[i], "bytes": by[i], "flops": fl[i], "launches": int(ln[i])}
            for i, c in enumerate(_lib.PROF_CLASSES)}


def _launch_count(fn, steps):
    """Library kernel launches of `steps` calls of fn()."""
    import ctypes

    from matfree_gb300 import _lib

    lib = _lib.lib()
    nc = len(_lib.PROF_CLASSES)
    lib.mfg_profile_enable(0)
    for _ in range(steps):
        fn()
    ln = (ctypes.c_int64 * nc)()
    _lib.check(lib.mfg_profile_read(nc, None, None, None, ln), "mfg_profile_read")
    return int(sum(ln))


def grad_arm(args):
    """log det K(theta) and d/dtheta (RBF n=8192, k=48, p=128) per step."""
    import torch

    import matfree_gb300 as mf
    from matfree_gb300 import autodiff

    torch.cuda.set_device(0)
    n, k, p = 8192, 48, 128
    x = np.random.default_rng(0).uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    theta0 = np.array([0.0, math.log(0.2), math.log(1e-2)])
    key = mf.prng.prng_key(1)
    V = mf.stochtrace.sampler_signs(torch.ones(n, device="cuda"), num=p)(key)

    def step():
        th = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
        val = autodiff.rbf_logdet(xd, th, V, k, precision=args.precision)
        val.backward()
        return val.detach(), th.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            val, grad = step()
        torch.cuda.synchronize()
        secs = (time.perf_counter() - t0) / args.steps
    clocks = clk.summary()
    launches = _launch_count(step, 1) * args.steps
    prof = _profiled(step, args.steps)
    rl = roofline(prof, _peaks(), args.steps)
    rl["peak_source"] = rl.pop("peak_override", f"of {_peaks()['source']}")
    # float64 oracle gradient on every probe (same probe vectors)
    from oracle import adjoint as oadj
    from oracle import philox

    Vs = philox.rademacher(np.asarray(key, np.uint32), p, n)
    t1 = time.perf_counter()
    matmat, vjp_matmat = oadj.rbf_vjp_factory(x.astype(np.float64), theta0)
    v_ref, g_ref = oadj.slq_grad_batched(matmat, vjp_matmat, 3, k, Vs)
    cpu_s = time.perf_counter() - t1
    g_gpu = grad.numpy()
    rel = np.abs(g_gpu - g_ref) / np.abs(g_ref)
    line = {"metric": "logdet+grad solves/s", "value": 1.0 / secs, "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": f"f32 basis / {args.precision} operator / f64 reductions",
            "data": "synthetic (seeded)",
            "config": {"workload": f"GP log-det + d/dtheta, RBF n={n}, k={k}, p={p}, theta=(0, log 0.2, log 1e-2)"},
            "estimate": float(val), "grad": grad.tolist(),
            "rel_err_vs_fp64": {"value": abs(float(val) - v_ref) / abs(v_ref), "on": f"all {p} probes"},
            "grad_rel_err_vs_fp64_oracle": {"value": rel.tolist(), "on": f"all {p} probes, identical probes"},
            "roofline": rl, "clocks": clocks, "gpu_launches": launches,
            "kernel_ms_per_step": {c: v["ms"] / args.steps for c, v in prof.items()},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "solves/s",
                             "cores": len(os.sched_getaffinity(0)), "kind": "port",
                             "sample": f"one complete solve: value and gradient on all {p} probes "
                                       "(float64 forward + adjoint restatement)"}}
    print(json.dumps(line), flush=True)


def gp_arm(args):
    """GP log-pdf (SLQ log-det + CG solve) and d/dtheta, RBF n=8192, k=48, p=128, per step."""
    import torch

    import matfree_gb300 as mf

    torch.cuda.set_device(0)
    n, k, p, tol = 8192, 48, 128, 1e-5
    rng = np.random.default_rng(0)
    x = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    theta0 = np.array([0.0, math.log(0.2), math.log(1e-2)])
    key = mf.prng.prng_key(1)
    V = mf.stochtrace.sampler_signs(torch.ones(n, device="cuda"), num=p)(key)

    def step():
        th = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
        val = mf.gp.rbf_logpdf(xd, th, yd, V, k, precision=args.precision, cg_tol=tol)
        val.backward()
        return val.detach(), th.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        val, grad = step()
    torch.cuda.synchronize()
    secs = (time.perf_counter() - t0) / args.steps
    op = mf.RBFKernelOperator.from_theta(xd, theta0, precision=args.precision)
    _, its = mf.linalg.cg_batched(op, yd[None, :], tol=tol)
    its = int(its[0])
    # float64 oracle: log-det gradient on the first probes, CG for a bounded
    # number of iterations, both extrapolated (probes; CG iterations)
    from oracle import adjoint as oadj
    from oracle import gp as ogp
    from oracle import philox

    num = args.cpu_probes
    Vs = philox.rademacher(np.asarray(key, np.uint32), num, n)
    t1 = time.perf_counter()
    matmat, vjp_matmat = oadj.rbf_vjp_factory(x.astype(np.float64), theta0)
    _, g_ref = oadj.slq_grad_batched(matmat, vjp_matmat, 3, k, Vs)
    ld_s = time.perf_counter() - t1
    K, _, _ = oadj.rbf_matrices(x.astype(np.float64), theta0)
    cg_cap = min(its, 100)
    t2 = time.perf_counter()
    ogp.cg(lambda v: K @ v, y.astype(np.float64), tol=0.0, maxiter=cg_cap)
    cg_s = (time.perf_counter() - t2) * its / max(cg_cap, 1)
    cpu_s = ld_s * p / num + 2 * cg_s  # forward solve + the gradient's contractions reuse alpha
    line = {"metric": "GP logpdf+grad solves/s", "value": 1.0 / secs, "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": f"f32 basis / {args.precision} operator / f64 reductions",
            "data": "synthetic (seeded)",
            "config": {"workload": f"GP log-pdf (SLQ log-det + CG, tol {tol}) + d/dtheta, RBF n={n}, k={k}, "
                                   f"p={p}, theta=(0, log 0.2, log 1e-2)", "cg_iterations": its},
            "estimate": float(val), "grad": grad.tolist(),
            "logdet_grad_vs_fp64_oracle": {"oracle": g_ref.tolist(), "on": f"first {num} probes"},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "solves/s", "cores": len(os.sched_getaffinity(0)),
                             "kind": "port",
                             "sample": f"log-det gradient on {num} of {p} probes and {cg_cap} of {its} CG "
                                       "iterations (float64 restatement), extrapolated linearly"}}
    print(json.dumps(line), flush=True)


def product_arm(args):
    """Product log-determinant log det(A^T A) by Golub-Kahan SLQ, dense A n=8192, k=32, p=128."""
    import torch

    import matfree_gb300 as mf

    torch.cuda.set_device(0)
    n, k, p = 8192, 32, 128
    rng = np.random.default_rng(0)
    # singular values in about [1.5, 2.5]: well conditioned, and log det(A^T A)
    # far from zero, so that relative errors are meaningful
    A = (0.5 * rng.standard_normal((n, n)) / math.sqrt(n) + 2.0 * np.eye(n)).astype(np.float32)
    op = mf.DenseOperator(torch.from_numpy(A).cuda(), precision=args.precision)
    op.transpose()  # the transposed copy is built once, outside the timed steps
    key = mf.prng.prng_key(1)
    sampler = mf.stochtrace.sampler_signs(torch.ones(n, device="cuda"), num=p)
    integrand = mf.funm.monte_carlo_funm_product_logdet(mf.decomp.bidiag(k))
    estimate = mf.stochtrace.estimator_monte_carlo(integrand, sampler)
    for _ in range(args.warmup):
        estimate(op, key)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        val = estimate(op, key)
    torch.cuda.synchronize()
    secs = (time.perf_counter() - t0) / args.steps
    # float64 oracle on the first probes (same probe vectors), extrapolated in probes
    from oracle import bidiag as obidiag
    from oracle import philox

    num = args.cpu_probes
    Vs = philox.rademacher(np.asarray(key, np.uint32), num, n)
    Ad = A.astype(np.float64)
    t1 = time.perf_counter()
    ref = np.mean([obidiag.product_quadform(Ad, v, k) for v in Vs])
    cpu_s = (time.perf_counter() - t1) * p / num
    gpu_first = float(integrand.batched(op, sampler.panel(key)[:num]).mean())
    line = {"metric": "product log-det solves/s", "value": 1.0 / secs, "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": f"f32 basis / {args.precision} operator / f64 reductions",
            "data": "synthetic (seeded)",
            "config": {"workload": f"log det(A^T A), A = 2 I + 0.5 N(0,1)/sqrt(n), n={n}, k={k}, p={p} Rademacher probes, "
                                   f"operator {args.precision}"},
            "estimate": float(val),
            "rel_err_vs_fp64_oracle": {"value": abs(gpu_first - ref) / abs(ref), "on": f"first {num} probes"},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "solves/s", "cores": len(os.sched_getaffinity(0)),
                             "kind": "port", "sample": f"{num} of {p} probes (float64 restatement), "
                                                       "extrapolated linearly in probes"}}
    print(json.dumps(line), flush=True)


def _plain_fp32_request(req, dev="cuda"):
    """One request the plain way: fp32 RBF operator, the operator product as a
    cuBLAS SGEMM (TF32 off) called back once per Krylov step, one request at a
    time (the per-request FP32 drop-in of the serving comparison)."""
    import torch

    import matfree_gb300 as mf
    from matfree_gb300 import serve
    from matfree_gb300.funm import slq_values

    n = req.x.shape[0]
    xd = torch.from_numpy(np.ascontiguousarray(req.x, dtype=np.float32)).to(dev)
    op = mf.RBFKernelOperator(xd, s2=req.s2, ell=req.ell, tau=req.tau, precision="fp32")
    K = op.a[:, :n]
    cb = mf.CallbackOperator(lambda X: torch.addmm(X, X, K, beta=req.tau), n, batched=True)
    V = mf.stochtrace.sampler_signs(torch.ones(n, device=dev), num=req.p)(np.asarray(req.key, np.uint32))
    fun, param = serve._fun_code(req.fun)
    return slq_values(cb, req.k, V, fun, param).mean()


def serve_arm(args):
    """The serving stream through the continuous-batching server, with the plain
    per-request FP32 path timed on a prefix of the same stream and the served
    values checked against the float64 oracle on a seeded subset of requests."""
    import torch

    from matfree_gb300 import serve
    from oracle import philox, problems, slq

    torch.cuda.set_device(0)
    reqs = serve.synthetic_stream(args.requests, rate=args.rate, seed=0)
    warm = serve.synthetic_stream(8, rate=1e6, seed=99)
    srv = serve.SLQServer(slots=args.slots, budget_bytes=150e9, precision="bf16x3", autotune=True)
    def stalled(exc):
        print(json.dumps({"metric": METRIC, "value": None, "unit": UNIT, "n_gpus": 1,
                          "error": f"serving stalled: {exc}"}), flush=True)
        # leave without the interpreter's exit handlers, which would wait for
        # the solves that did not finish
        os._exit(3)

    try:
        srv.run(warm, realtime=False, stall_s=args.stall_s)
    except RuntimeError as exc:
        stalled(exc)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        try:
            res, stats = srv.run(reqs, realtime=True, stall_s=args.stall_s)
        except RuntimeError as exc:
            clk.__exit__(None, None, None)  # stop the clock sampler's nvidia-smi first
            stalled(exc)
    clocks = clk.summary()
    by_id = {r.rid: r for r in res}
    # plain per-request FP32 (cuBLAS SGEMM, TF32 off) on a prefix of the stream
    tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    base_reqs = reqs[: args.baseline_requests] if args.baseline_requests > 0 else reqs
    _plain_fp32_request(warm[0])
    torch.cuda.synchronize()
    t_p = time.perf_counter()
    for r in base_reqs:
        float(_plain_fp32_request(r))
    plain_s = time.perf_counter() - t_p
    torch.backends.cuda.matmul.allow_tf32 = tf32
    # the served value against the float64 oracle: the three largest requests
    # whose float64 solve stays under 6e12 flop, and the smallest request
    cost = {r.rid: 2.0 * r.x.shape[0] ** 2 * r.p * r.k for r in reqs}
    big = sorted((r for r in reqs if cost[r.rid] <= 6e12), key=lambda r: -r.x.shape[0])[:3]
    chosen = big + [min(reqs, key=lambda r: r.x.shape[0])]
    errs = []
    for r in chosen:
        K = problems.rbf_kernel(r.x.astype(np.float64), r.s2, r.ell, r.tau)
        V = philox.rademacher(np.asarray(r.key, np.uint32), r.p, r.x.shape[0])
        f = np.log if r.fun == "log" else (lambda t, a=float(r.fun.split(":")[1]): np.exp(a * t))
        want = slq.slq_batched(lambda X: X @ K, r.k, V, matfun=f).mean()
        del K
        errs.append({"rid": r.rid, "n": r.x.shape[0], "k": r.k, "p": r.p, "fun": r.fun,
                     "rel_err": abs(by_id[r.rid].mean - want) / abs(want)})
    work = sum(6.0 * r.x.shape[0] ** 2 * r.p * r.k for r in reqs)  # bf16x3: three products per step
    peaks = _peaks()
    tflops = work / stats["wall_s"] / 1e12
    plain_rate = len(base_reqs) / plain_s
    line = {"metric": METRIC, "value": stats["solves_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": len(reqs), "warmup": len(warm), "ms_per_step": 1e3 * stats["wall_s"] / len(reqs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 basis / bf16x3 operator / f64 reductions", "data": "synthetic (seeded)",
            "config": {"workload": f"serving stream: {len(reqs)} RBF log-det / trace-exp requests, Poisson "
                                   f"arrivals at {args.rate}/s, n log-uniform [512, 32768], k in "
                                   "{16,32,64,96}, p in {32,64,128,256}, bf16x3 operators built per request",
                       "slots": args.slots, "budget_gb": 150, "parallelism": "streams"},
            "latency_ms": {"p50": stats["p50_ms"], "p99": stats["p99_ms"], "mean": stats["mean_ms"]},
            "rel_err_vs_fp64": {"value": max(e["rel_err"] for e in errs), "on": errs},
            "plain_fp32_per_request": {"solves_per_s": plain_rate, "requests": len(base_reqs),
                                       "note": "the first requests of the same stream one at a time: fp32 "
                                               "operator, cuBLAS SGEMM (TF32 off) per Krylov step"},
            "speedup_vs_plain_fp32": stats["solves_per_s"] / plain_rate,
            "roofline": {"kernel": "operator products of all requests (bf16x3 tensor-core GEMMs)",
                         "bound": "tensor", "achieved": tflops, "peak": peaks["tensor_burst"],
                         "unit": "TFLOP/s", "frac": tflops / peaks["tensor_burst"], "traffic": None,
                         "peak_source": f"of {peaks['source']}",
                         "note": "algorithmic operator flops of the whole stream over its wall time"},
            "clocks": clocks, "packed_solves": stats["packed_solves"],
            "packed_requests": stats["packed_requests"],
            "gemm_tuning_rules": sum(1 for r in (srv.tuning or []) if r["bn"] or r["split_k"])}
    print(json.dumps(line), flush=True)


# The other benchmark configurations, run after the headline measurement of a
# default invocation (each in its own process, so that a failure in one cannot
# take the headline line with it) and reported under "other_configs".
OTHER_CONFIGS = [
    ("dense1k_fp64", ["--config", "dense1k", "--precision", "fp64", "--steps", "20"]),
    ("laplace1m", ["--config", "laplace1m", "--steps", "3"]),
    ("grad8k", ["--config", "grad8k", "--steps", "5"]),
    ("product8k", ["--config", "product8k", "--steps", "5"]),
    ("gp8k", ["--config", "gp8k", "--steps", "2"]),
    ("serve", ["--config", "serve"]),
]


def run_other_configs(timeout_s=900):
    out = {}
    for name, argv in OTHER_CONFIGS:
        cmd = [sys.executable, os.path.abspath(__file__), *argv, "--warmup", "3", "--no-other-configs"]
        t0 = time.perf_counter()
        try:
            proc = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout_s)
            lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
            if proc.returncode == 0 and lines:
                out[name] = json.loads(lines[-1])
            elif lines:  # a failure the arm reported itself (e.g. a serving stall)
                out[name] = json.loads(lines[-1])
                out[name]["rc"] = proc.returncode
            else:
                out[name] = {"error": f"rc {proc.returncode}", "stderr_tail": proc.stderr[-2000:]}
        except subprocess.TimeoutExpired:
            out[name] = {"error": f"timed out after {timeout_s} s"}
        out[name]["run_s"] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="rbf16k", choices=sorted(CONFIGS) + ["serve", "grad8k", "gp8k", "product8k"])
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--baseline-requests", type=int, default=200,
                    help="requests of the plain fp32 comparison (0: all of them)")
    ap.add_argument("--rate", type=float, default=150.0,
                    help="Poisson arrival rate of the serving stream (above the server's capacity, so "
                         "that solves/s measures the capacity and latencies include queueing)")
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--inflight", type=int, default=3,
                    help="independent solves in flight (round-robin over CUDA streams)")
    ap.add_argument("--precision", default="bf16x3", choices=["fp32", "bf16", "bf16x3", "fp64"])
    ap.add_argument("--cpu-probes", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-budget-s", type=float, default=180.0,
                    help="--impl reference: stop timing complete solves after this many seconds")
    ap.add_argument("--stall-s", type=float, default=60.0,
                    help="serve config: give up when no solve completes for this many seconds")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in tensor-core tile configuration")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="report the headline configuration only")
    ap.add_argument("--no-plain-fp32", action="store_true",
                    help="skip the plain per-request fp32 comparison solves")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.config == "serve" and args.impl == "ours":
        serve_arm(args)
        return
    if args.config == "grad8k" and args.impl == "ours":
        grad_arm(args)
        return
    if args.config == "gp8k" and args.impl == "ours":
        gp_arm(args)
        return
    if args.config == "product8k" and args.impl == "ours":
        product_arm(args)
        return
    if args.impl == "reference":
        line = reference_arm(args)
        if line is not None:
            print(json.dumps(line), flush=True)
        return

    res, prob = gpu_arm(args)
    if res["rank"] != 0:
        return
    world = res["world"]
    peaks = _peaks()
    value = world * args.steps / (res["total_ms"] / 1e3)
    rl = roofline(res["prof"], peaks, args.steps, args.config, args.precision)
    rl["peak_source"] = rl.pop("peak_override", f"of {peaks['source']}")
    launches = res["launches"]
    step_ms = res["step_ms"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 basis / bf16x3 operator / f64 reductions"
        if args.precision == "bf16x3" else args.precision, "data": "synthetic (seeded)",
        "config": _config(args),
        "latency_ms": {"p50": step_ms[len(step_ms) // 2], "p99": step_ms[min(len(step_ms) - 1, int(0.99 * len(step_ms)))]},
        "estimate": res["estimate"], "roofline": rl, "gpu_launches": launches,
        "clocks": res["clocks"], "e2e": res["e2e"],
        "kernel_ms_per_step": {c: v["ms"] / args.steps for c, v in res["prof"].items()},
        "gemm_tile": res["tuned"],
        "reortho": {"form": "two reads of the basis per step" if _two_sweep(args, prob)
                    else "three reads of the basis per step",
                    "retries": res["two_sweep_retries"]},
    }
    if prob["kind"] == "csr":
        # the sparse product (K2) beside the dominant class: algorithmic bytes
        # 8 nnz + 4 (n + 1) + 8 n p per launch over its event-timed duration
        ap = res["prof"]["apply"]
        if ap["ms"] > 0:
            gbs = ap["bytes"] / (ap["ms"] / 1e3) / 1e9
            line["spmm_roofline"] = {"kernel": "csr_spmm_window_kernel", "bound": "hbm", "achieved": gbs,
                                     "peak": peaks["hbm"], "unit": "GB/s", "frac": gbs / peaks["hbm"],
                                     "launches": ap["launches"],
                                     "ms_per_launch": ap["ms"] / max(ap["launches"], 1),
                                     "peak_source": f"of {peaks['source']}"}
    if not args.no_cpu_baseline:
        # one complete float64 solve on the host cores: every probe, full n and k
        # (a probe subset only where the bases would not fit in host memory)
        num = cpu_probe_count(prob)
        probes = cpu_probe_sample(prob, res["key"], num)
        vals, secs, build = cpu_sample(prob, probes)
        gpu_vals = res["values"][:num].cpu().numpy()
        if num == prob["p"]:
            rate = 1.0 / secs
            sample = (f"one complete solve: all {prob['p']} probes at full n and k (float64 NumPy/OpenBLAS "
                      f"restatement of matfree's algorithm; {secs:.1f} s incl. {build:.1f} s operator build)")
        else:
            rate = 1.0 / (build + (secs - build) * prob["p"] / num)
            sample = (f"{num} of {prob['p']} probes at full n and k (their float64 bases fill "
                      f"{CPU_BASIS_BYTES / 1e9:.0f} GB of host memory), extrapolated linearly in probes; "
                      f"{secs:.1f} s incl. {build:.1f} s operator build")
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": len(os.sched_getaffinity(0)),
                                "kind": "port", "sample": sample}
        line["rel_err_vs_fp64"] = rel_err_summary(gpu_vals, vals)
    if res["plain"] is not None:
        pl = res["plain"]
        best = max(pl.values(), key=lambda d: d["solves_per_s"])
        line["plain_fp32_per_request"] = {
            "solves_per_s": best["solves_per_s"], "speedup": value / best["solves_per_s"],
            "note": "same problem, fp32 operator, one solve at a time; the faster of the two fp32 "
                    "products: the library's CUDA-core kernel and cuBLAS SGEMM (TF32 off) through "
                    "CallbackOperator",
            "simt_solves_per_s": pl["simt"]["solves_per_s"],
            "cublas_solves_per_s": pl["cublas"]["solves_per_s"]}
        if not args.no_cpu_baseline:
            for name in ("simt", "cublas"):
                line["plain_fp32_per_request"][f"{name}_rel_err_vs_fp64"] = rel_err_summary(
                    pl[name]["values"].cpu().numpy(), vals)["value"]
    if args.config == "rbf16k" and world == 1 and not args.no_other_configs:
        del res
        import torch

        torch.cuda.empty_cache()
        line["other_configs"] = run_other_configs()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
