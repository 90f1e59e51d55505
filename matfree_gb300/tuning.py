"""Autotuner of the tensor-core operator product's tile configuration.

The CTA-pair GEMM covers an n x n operator with ceil(n / 256) row tiles per
probe tile.  With 76 CTA pairs on the GPU, some sizes fill the SMs in whole
waves and others leave up to half of them idle in a last partial wave
(n = 20000: 79 tiles, 1.04 waves).  Narrower probe tiles (more tiles, the
operator re-read once per tile), a K split over two CTAs (partial products
added into W) or the persistent form (one pair per two SMs; the last wave's
tiles split once along K, their tails packed onto the spare pairs) change
the wave count.  Which of these is fastest depends on n,
p and the precision, so ``autotune`` times every candidate on the device for a
grid of operator sizes and probe counts and installs the winners as rules in
the library (``mfg_gemm_tuning_add``); ``save`` / ``load`` keep them in a
JSON file keyed by the GPU name.  The defaults stand wherever no rule matches.
"""

from __future__ import annotations

import ctypes
import json
import math
import os

import torch

from . import _lib
from ._panel import Workspace, padded_ld, stream_ptr

# (probe tile, form): 0 built-in; form 1 one tile per CTA pair, 2 K halves,
# 3 persistent pairs with the last wave split along K
CANDIDATES = ((0, 0), (0, 1), (0, 2), (0, 3), (128, 1), (128, 2), (128, 3), (64, 1))
DEFAULT_NS = tuple(int(round(1024 * 2 ** (i / 2))) // 8 * 8 for i in range(11))  # 1024 .. 32768
DEFAULT_PS = (32, 64, 128, 256)
MARGIN = 0.03  # a candidate replaces the built-in choice only when this much faster


def cache_path() -> str:
    return os.path.join(os.path.dirname(_lib.library_path()), "gemm_tuning.json")


def _time_apply(op_struct, panel, out, p, ld, ws, reps):
    lib = _lib.lib()
    args = (ctypes.byref(op_struct), ctypes.c_void_p(panel.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            p, ld, ctypes.c_void_p(ws.data_ptr()), ws.numel(), stream_ptr())
    _lib.check(lib.mfg_operator_apply(*args), "mfg_operator_apply")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = math.inf
    for _ in range(reps):
        e0.record()
        _lib.check(lib.mfg_operator_apply(*args), "mfg_operator_apply")
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def pick(timings, margin: float = None):
    """(default_ms, (ms, bn, split)) from [(ms, bn, split), ...] that holds
    the built-in choice (0, 0): the fastest candidate, unless it is within
    `margin` of the built-in one, which then stays (it keeps the launch chain
    free of extra operations such as the zeroing before a K split)."""
    margin = MARGIN if margin is None else margin
    default_ms = next(t for t, b, sp in timings if b == 0 and sp == 0)
    best = min(timings)
    if best[0] > default_ms * (1.0 - margin):
        best = (default_ms, 0, 0)
    return default_ms, best


def _bounds(values, i):
    """Half-open log-midpoint range around values[i] (the rule's n or p range)."""
    lo = 0 if i == 0 else int(math.sqrt(values[i - 1] * values[i])) + 1
    hi = (1 << 40) if i == len(values) - 1 else int(math.sqrt(values[i] * values[i + 1]))
    return lo, hi


def autotune(ns=DEFAULT_NS, ps=DEFAULT_PS, precision: str = "bf16x3", reps: int = 3,
             candidates=CANDIDATES, device="cuda") -> list:
    """Time every candidate for each (n, p) of the grid and install the fastest
    as rules; returns them as dicts (n_lo, n_hi, p_lo, p_hi, bn, split_k, ms)."""
    from .operators import DenseOperator

    lib = _lib.lib()
    lib.mfg_gemm_tuning_clear()
    rules = []
    ns = sorted(int(n) for n in ns if n >= 1024)
    ps = sorted(int(p) for p in ps if p > 8)
    for i, n in enumerate(ns):
        ld = padded_ld(n)
        A = torch.randn((n, n), device=device) / math.sqrt(n)
        op = DenseOperator(A, precision=precision)
        del A
        s = op.c_struct()
        for j, p in enumerate(ps):
            panel = torch.zeros((p, ld), dtype=torch.float32, device=device)
            panel[:, :n].normal_()
            out = torch.zeros_like(panel)
            ws = Workspace()
            nbytes = lib.mfg_slq_workspace_bytes(ctypes.byref(s), 0, p, ld)
            wsb, _ = ws.get(nbytes, device)
            timings = []
            for bn, split in candidates:
                if bn and bn >= p:
                    continue  # not narrower than the default tile
                lib.mfg_gemm_tuning_clear()
                _lib.check(lib.mfg_gemm_tuning_add(n, n, p, p, bn, split), "mfg_gemm_tuning_add")
                timings.append((_time_apply(s, panel, out, p, ld, ws.buf, reps), bn, split))
            default_ms, (ms, bn, split) = pick(timings)
            n_lo, n_hi = _bounds(ns, i)
            p_lo, p_hi = _bounds(ps, j)
            rules.append({"n_lo": n_lo, "n_hi": n_hi, "p_lo": p_lo, "p_hi": p_hi, "bn": bn,
                          "split_k": split, "ms": ms, "n": n, "p": p, "default_ms": default_ms})
        del op
    install(rules)
    return rules


def install(rules) -> None:
    lib = _lib.lib()
    lib.mfg_gemm_tuning_clear()
    for r in rules:
        if r["bn"] or r["split_k"]:
            _lib.check(lib.mfg_gemm_tuning_add(r["n_lo"], r["n_hi"], r["p_lo"], r["p_hi"], r["bn"],
                                               r["split_k"]), "mfg_gemm_tuning_add")


def save(rules, path=None, precision="bf16x3") -> str:
    path = path or cache_path()
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[f"{torch.cuda.get_device_name()}|{precision}"] = rules
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    return path


def load(path=None, precision="bf16x3"):
    """Install the rules saved for this GPU and precision; None if there are none."""
    path = path or cache_path()
    if not os.path.exists(path):
        return None
    with open(path) as f:
        data = json.load(f)
    rules = data.get(f"{torch.cuda.get_device_name()}|{precision}")
    if rules is not None:
        install(rules)
    return rules


def ensure(precision="bf16x3", **kwargs):
    """Load this GPU's rules, or run the autotuner once and save them."""
    rules = load(precision=precision)
    if rules is None:
        rules = autotune(precision=precision, **kwargs)
        save(rules, precision=precision)
    return rules


def time_form(n: int, p: int, bn: int = 0, form: int = 0, precision: str = "bf16x3", reps: int = 10,
              seed: int = 0, device="cuda") -> dict:
    """Median device time of one operator product (n x n, p probes) under the
    tile rule (bn, form); L2 flushed before each timed launch."""
    from .operators import DenseOperator

    lib = _lib.lib()
    ld = padded_ld(n)
    g = torch.Generator(device=device).manual_seed(seed)
    A = torch.randn((n, n), device=device, generator=g) / math.sqrt(n)
    op = DenseOperator(A, precision=precision, shift=0.01)
    del A
    s = op.c_struct()
    panel = torch.zeros((p, ld), dtype=torch.float32, device=device)
    panel[:, :n].normal_(generator=g)
    out = torch.zeros_like(panel)
    ws = Workspace()
    ws.get(lib.mfg_slq_workspace_bytes(ctypes.byref(s), 0, p, ld), device)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=device)  # 256 MB > L2
    lib.mfg_gemm_tuning_clear()
    try:
        if bn or form:
            _lib.check(lib.mfg_gemm_tuning_add(n, n, p, p, bn, form), "mfg_gemm_tuning_add")
        args = (ctypes.byref(s), ctypes.c_void_p(panel.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                p, ld, ctypes.c_void_p(ws.buf.data_ptr()), ws.buf.numel(), stream_ptr())
        for _ in range(2):
            _lib.check(lib.mfg_operator_apply(*args), "mfg_operator_apply")
        times = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(lib.mfg_operator_apply(*args), "mfg_operator_apply")
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    finally:
        lib.mfg_gemm_tuning_clear()
    times.sort()
    ms = times[len(times) // 2]
    flop = (3 if precision == "bf16x3" else 1) * 2.0 * n * n * p
    return {"n": n, "p": p, "bn": bn, "form": form, "precision": precision, "median_ms": ms,
            "tflops": flop / (ms * 1e-3) / 1e12}


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="time one tensor-core operator product under a tile rule")
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--p", type=int, default=256)
    ap.add_argument("--bn", type=int, default=0)
    ap.add_argument("--form", type=int, default=0, help="0 built-in, 1 one tile per pair, 2 K halves, 3 persistent")
    ap.add_argument("--precision", default="bf16x3")
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args()
    print(json.dumps(time_form(a.n, a.p, a.bn, a.form, a.precision, a.reps)))
