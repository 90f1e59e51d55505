"""Continuous-batching SLQ log-det / trace-of-f(A) server on one GPU.

Requests (points x, depth k, probe count p, matrix function f) arrive over
time.  The loop admits a request as soon as a slot (a CUDA stream) is free
and its HBM footprint fits the budget, then enqueues the whole solve on that
slot's stream: host-to-device copy of the points, device build of the RBF
operator (bf16 hi/lo split by default), Philox probes, the batched Arnoldi /
CGS2 iteration, the tridiagonal eigensolves and the quadrature, and a
device-to-host copy of (mean, standard error).  Solves on different slots
overlap on the device; completions are detected with CUDA events, which
frees the slot and the budget for the next waiting request.

Every kernel of a solve is deterministic (fixed-order reductions, no
atomics in any sum), so a request returns bit-identical results whether it
runs alone or in a mix; ``tests/test_gpu_serve.py`` checks that.

Footprint per request (bytes): operator n * lda * (4 for bf16x3, 2 bf16,
4 fp32, 8 fp64) + mfg_slq workspace (Krylov basis p k ld, Hessenberg
p k^2, panels and reduction scratch) + the probe panel.
"""

from __future__ import annotations

import ctypes
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._panel import Workspace, padded_ld
from .operators import RBFKernelOperator


@dataclass
class Request:
    rid: int
    x: np.ndarray  # (n, 3) float32 points
    k: int
    p: int
    fun: str = "log"  # "log" or "exp:<scale>"
    arrival: float = 0.0  # seconds after the start of the stream
    key: tuple = (1, 0)
    s2: float = 1.0
    ell: float = 0.2
    tau: float = 1e-2


@dataclass
class Result:
    rid: int
    mean: float
    sem: float
    latency_ms: float
    start_ms: float
    end_ms: float
    n: int
    k: int
    p: int


def _fun_code(fun: str):
    if fun == "log":
        return _lib.MFG_FUN_LOG, 0.0
    if fun.startswith("exp:"):
        return _lib.MFG_FUN_EXP, float(fun.split(":", 1)[1])
    raise ValueError(f"unknown matrix function {fun!r}")


def footprint_bytes(n: int, k: int, p: int, precision: str) -> int:
    ld = padded_ld(n)
    op_bytes = {"bf16x3": 4, "bf16": 2, "fp32": 4, "fp64": 8}[precision] * n * ld
    s = _lib.MfgOperator()
    s.kind = _lib.MFG_OP_DENSE
    s.precision = _lib.PRECISIONS[precision]
    s.n, s.lda, s.a = n, ld, 4096
    s.a_lo = 4096 if precision == "bf16x3" else None
    ws = _lib.lib().mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, ld, _flags(k, precision))
    es = 8 if precision == "fp64" else 4
    return int(op_bytes + ws + p * ld * es + n * 3 * 4 + 4096)


def _flags(k: int, precision: str) -> int:
    """Two reads of the Krylov basis per step where that form applies."""
    return _lib.MFG_SLQ_TWO_SWEEP if precision != "fp64" and 2 <= k <= 129 else 0


@dataclass
class _Slot:
    stream: torch.cuda.Stream
    workspace: Workspace = field(default_factory=Workspace)
    busy: bool = False


class SLQServer:
    """Admission-controlled, stream-overlapped SLQ solves (see module docstring)."""

    def __init__(self, *, budget_bytes: float = 150e9, slots: int = 8, precision: str = "bf16x3",
                 device="cuda"):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.device = torch.device(device)
        self.slots = [_Slot(torch.cuda.Stream(device=self.device)) for _ in range(slots)]
        self.used = 0.0

    def _launch(self, slot: _Slot, req: Request, flags=None):
        lib = _lib.lib()
        n = req.x.shape[0]
        ld = padded_ld(n)
        fun, param = _fun_code(req.fun)
        with torch.cuda.stream(slot.stream):
            xh = torch.from_numpy(np.ascontiguousarray(req.x, dtype=np.float32)).pin_memory()
            xd = xh.to(self.device, non_blocking=True)
            op = RBFKernelOperator(xd, s2=req.s2, ell=req.ell, tau=req.tau, precision=self.precision)
            probes = torch.zeros((req.p, ld), dtype=op.basis_dtype, device=self.device)
            key = np.ascontiguousarray(np.asarray(req.key, dtype=np.uint32).reshape(2))
            st = lib.mfg_sampler_signs(key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), req.p, n, ld,
                                       _lib.MFG_F64 if op.basis_dtype == torch.float64 else _lib.MFG_F32,
                                       ctypes.c_void_p(probes.data_ptr()),
                                       ctypes.c_void_p(slot.stream.cuda_stream))
            _lib.check(st, "mfg_sampler_signs")
            values = torch.empty((req.p,), dtype=torch.float64, device=self.device)
            ms = torch.empty((2,), dtype=torch.float64, device=self.device)
            s = op.c_struct()
            if flags is None:
                flags = _flags(req.k, self.precision)
            nbytes = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), req.k, req.p, ld, flags)
            ws, wsb = slot.workspace.get(nbytes, self.device)
            st = lib.mfg_slq_ex(ctypes.byref(s), req.k, req.p, ctypes.c_void_p(probes.data_ptr()), ld, fun,
                                param, ctypes.c_void_p(values.data_ptr()), ctypes.c_void_p(ms.data_ptr()),
                                None, None, flags, ws, wsb, ctypes.c_void_p(slot.stream.cuda_stream))
            _lib.check(st, "mfg_slq_ex")
            out = torch.empty((2,), dtype=torch.float64, pin_memory=True)
            out.copy_(ms, non_blocking=True)
            done = torch.cuda.Event()
            done.record(slot.stream)
        # keep every buffer of the solve alive until its completion event fires
        return {"done": done, "out": out, "keep": (xh, xd, op, probes, values, ms), "flags": flags,
                "ws": ws}

    def run(self, requests, *, realtime: bool = True):
        """Serve the requests in arrival order; returns (results, stats)."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        inflight = {}
        results = []
        t0 = time.perf_counter()
        while pending or inflight:
            now = time.perf_counter() - t0
            for idx, (slot, req, st, fp, t_start) in list(inflight.items()):
                if st["done"].query() and st["flags"] and _lib.lib().mfg_workspace_status(
                        st["ws"], ctypes.c_void_p(slot.stream.cuda_stream)) == _lib.MFG_ERR_RETRY:
                    # the two-sweep step asked for the three-read form: run it again
                    inflight[idx] = (slot, req, self._launch(slot, req, flags=0), fp, t_start)
                    continue
                if st["done"].query():
                    t_end = time.perf_counter() - t0
                    mean, sem = (float(v) for v in st["out"])
                    arrival = req.arrival if realtime else 0.0
                    results.append(Result(req.rid, mean, sem, 1e3 * (t_end - arrival), 1e3 * t_start,
                                          1e3 * t_end, req.x.shape[0], req.k, req.p))
                    slot.busy = False
                    self.used -= fp
                    del inflight[idx]
            admitted = False
            while pending and (not realtime or pending[0].arrival <= now):
                req = pending[0]
                fp = footprint_bytes(req.x.shape[0], req.k, req.p, self.precision)
                if fp > self.budget:
                    raise ValueError(f"request {req.rid} needs {fp / 1e9:.1f} GB > budget")
                free = [s for s in self.slots if not s.busy]
                if not free or self.used + fp > self.budget:
                    break
                slot = free[0]
                slot.busy = True
                self.used += fp
                pending.popleft()
                t_start = time.perf_counter() - t0
                inflight[req.rid] = (slot, req, self._launch(slot, req), fp, t_start)
                admitted = True
            if not admitted:
                time.sleep(20e-6)
        wall = time.perf_counter() - t0
        lat = np.array([r.latency_ms for r in results])
        stats = {"solves": len(results), "wall_s": wall, "solves_per_s": len(results) / wall,
                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                 "mean_ms": float(lat.mean())}
        return sorted(results, key=lambda r: r.rid), stats


def synthetic_stream(num: int, *, rate: float, seed: int = 0, n_range=(512, 32768),
                     ks=(16, 32, 64, 96), ps=(32, 64, 128, 256), funs=("log", "exp:-0.1")):
    """Poisson arrivals of RBF log-det / trace-of-exp requests with fresh points.

    n log-uniform in n_range, k and p uniform over the given sets, f uniform.
    """
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(num):
        t += rng.exponential(1.0 / rate)
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        x = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
        out.append(Request(rid=i, x=x, k=int(rng.choice(ks)), p=int(rng.choice(ps)),
                           fun=str(rng.choice(funs)), arrival=t, key=(1 + i, 0)))
    return out
