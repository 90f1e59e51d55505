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

Small requests (n at most ``group_max_n``) that are waiting together and
share the depth k and the function f are packed into one solve: their probe
vectors form one panel of sum(p) rows zero-padded to a common length, the
operator is block-diagonal (member r's RBF matrix, zero-padded, applied to
its own rows by the tensor-core product), and every other kernel of the
Krylov step -- the streamed reorthogonalisation sweeps, the coefficient and
normalisation kernels, the tridiagonal eigensolves and the quadrature --
runs once for the whole group.  Zero padding leaves every member's Krylov
vectors in its own coordinates, so each member's value is its unpadded SLQ
value up to the order of floating-point sums.

Every kernel of a solve is deterministic (fixed-order reductions, no
atomics in any sum), so a request that runs alone returns bit-identical
results whether other requests run beside it or not; a request packed into
a group returns its alone value up to rounding (``tests/test_gpu_serve.py``).

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
from .operators import DenseOperator, RBFKernelOperator


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
    opbuf: Workspace = field(default_factory=Workspace)  # operator storage, reused by the slot
    busy: bool = False


def _operator_views(slot: _Slot, members_n: int, n: int, ld: int, precision: str, device):
    """Storage for `members_n` operators of n x ld entries in the slot's own
    grow-only buffer: requests of every size reuse the same device memory, so
    a long stream of mixed sizes does not fragment the allocator's cache (a
    fragmented cache ends in allocation retries that synchronise the device)."""
    es = {"bf16x3": 2, "bf16": 2, "fp32": 4, "fp64": 8}[precision]
    arrays = 2 if precision == "bf16x3" else 1
    one = n * ld * es
    slot.opbuf.get(members_n * arrays * one, device)
    buf = slot.opbuf.buf
    dt = {"bf16x3": torch.bfloat16, "bf16": torch.bfloat16, "fp32": torch.float32, "fp64": torch.float64}[precision]
    out = []
    for m in range(members_n):
        base = m * arrays * one
        a = buf[base:base + one].view(dt).view(n, ld)
        a_lo = buf[base + one:base + 2 * one].view(dt).view(n, ld) if arrays == 2 else None
        out.append((a, a_lo))
    return out


class _GroupOperator:
    """Block-diagonal operator over a packed probe panel: rows [start_r,
    start_r + p_r) are multiplied by member r's operator (every member n x n,
    zero-padded), one tensor-core product per member inside the library's
    callback, all on the solve's stream."""

    def __init__(self, ops, starts, counts, n, ld, device):
        self.ops = ops
        self.structs = [op.c_struct() for op in ops]
        self.starts, self.counts = list(starts), list(counts)
        self.n = int(n)
        self.precision = "fp32"
        self.error = None
        lib = _lib.lib()
        nbytes = max(lib.mfg_slq_workspace_bytes(ctypes.byref(st), 0, int(c), ld)
                     for st, c in zip(self.structs, self.counts))
        self.ws = torch.empty(int(nbytes), dtype=torch.uint8, device=device)

        def _apply(ctx, V, W, n_, p_, ld_, stream):
            try:
                for st, b0, pr in zip(self.structs, self.starts, self.counts):
                    off = int(b0) * int(ld_) * 4
                    rc = lib.mfg_operator_apply(ctypes.byref(st), ctypes.c_void_p(V + off),
                                                ctypes.c_void_p(W + off), int(pr), int(ld_),
                                                ctypes.c_void_p(self.ws.data_ptr()), self.ws.numel(),
                                                ctypes.c_void_p(stream))
                    if rc != _lib.MFG_OK:
                        return rc
                return 0
            except Exception as exc:  # reported by the caller through the status
                self.error = exc
                return 1

        self._cfn = _lib.APPLY_FN(_apply)

    def c_struct(self):
        st = _lib.MfgOperator()
        st.kind = _lib.MFG_OP_CALLBACK
        st.precision = _lib.MFG_PREC_FP32
        st.n = self.n
        st.apply = self._cfn
        st.ctx = None
        return st


def group_footprint_bytes(members, precision: str) -> int:
    """HBM of one packed solve: the members' zero-padded operators, the panel
    of all their probes and the solve's workspace at the padded length."""
    n = max(r.x.shape[0] for r in members)
    ld = padded_ld(n)
    P = sum(r.p for r in members)
    k = members[0].k
    op_bytes = {"bf16x3": 4, "bf16": 2, "fp32": 4, "fp64": 8}[precision] * n * ld * len(members)
    s = _lib.MfgOperator()
    s.kind = _lib.MFG_OP_CALLBACK
    s.precision = _lib.MFG_PREC_FP32
    s.n = n
    ws = _lib.lib().mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, P, ld, _flags(k, precision))
    return int(op_bytes + ws + 2 * P * ld * 4 + 4096 * len(members))


class SLQServer:
    """Admission-controlled, stream-overlapped SLQ solves (see module docstring).

    ``group_max_n``: requests up to this n may be packed into one solve with
    others of the same k and f (0 disables packing); a group holds at most
    ``group_probes`` probe vectors and ``group_members`` requests, whose n lie
    within a factor of two of each other.  ``autotune``: install the tensor-core
    tile configurations timed for this GPU (``matfree_gb300.tuning``)."""

    def __init__(self, *, budget_bytes: float = 150e9, slots: int = 8, precision: str = "bf16x3",
                 device="cuda", group_max_n: int = 4096, group_probes: int = 1024,
                 group_members: int = 16, autotune: bool = False):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.device = torch.device(device)
        self.slots = [_Slot(torch.cuda.Stream(device=self.device)) for _ in range(slots)]
        self.used = 0.0
        self.group_max_n = int(group_max_n)
        self.group_probes = int(group_probes)
        self.group_members = int(group_members)
        self.tuning = None
        if autotune and precision in ("bf16", "bf16x3"):
            # tile configurations of the tensor-core product for this GPU
            # (timed once, then loaded from the library's tuning file)
            from . import tuning

            self.tuning = tuning.ensure(precision=precision)

    def _launch(self, slot: _Slot, req: Request, flags=None):
        lib = _lib.lib()
        n = req.x.shape[0]
        ld = padded_ld(n)
        fun, param = _fun_code(req.fun)
        with torch.cuda.stream(slot.stream):
            xh = torch.from_numpy(np.ascontiguousarray(req.x, dtype=np.float32)).pin_memory()
            xd = xh.to(self.device, non_blocking=True)
            ((a, a_lo),) = _operator_views(slot, 1, n, ld, self.precision, self.device)
            st = lib.mfg_rbf_build(ctypes.c_void_p(xd.data_ptr()), n, 3, req.s2, req.ell,
                                   _lib.PRECISIONS[self.precision], ctypes.c_void_p(a.data_ptr()),
                                   ctypes.c_void_p(a_lo.data_ptr() if a_lo is not None else 0), ld,
                                   ctypes.c_void_p(slot.stream.cuda_stream))
            _lib.check(st, "mfg_rbf_build")
            op = DenseOperator._from_storage(n, self.precision, a, a_lo, req.tau)
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

    def _launch_group(self, slot: _Slot, members, flags=None):
        """One packed solve of several small requests on the slot's stream."""
        lib = _lib.lib()
        n = max(r.x.shape[0] for r in members)
        ld = padded_ld(n)
        counts = [r.p for r in members]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
        P = int(sum(counts))
        k = members[0].k
        fun, param = _fun_code(members[0].fun)
        keep = []
        with torch.cuda.stream(slot.stream):
            ops = []
            panel = torch.zeros((P, ld), dtype=torch.float32, device=self.device)
            views = _operator_views(slot, len(members), n, ld, self.precision, self.device)
            for r, b0, (a, a_lo) in zip(members, starts, views):
                nr = r.x.shape[0]
                xh = torch.from_numpy(np.ascontiguousarray(r.x, dtype=np.float32)).pin_memory()
                xd = xh.to(self.device, non_blocking=True)
                # rows nr..n-1 of the padded operator are zero (the builder writes rows < nr)
                a[nr:].zero_()
                if a_lo is not None:
                    a_lo[nr:].zero_()
                st = lib.mfg_rbf_build(ctypes.c_void_p(xd.data_ptr()), nr, 3, r.s2, r.ell,
                                       _lib.PRECISIONS[self.precision], ctypes.c_void_p(a.data_ptr()),
                                       ctypes.c_void_p(a_lo.data_ptr() if a_lo is not None else 0), ld,
                                       ctypes.c_void_p(slot.stream.cuda_stream))
                _lib.check(st, "mfg_rbf_build")
                ops.append(DenseOperator._from_storage(n, self.precision, a, a_lo, r.tau))
                key = np.ascontiguousarray(np.asarray(r.key, dtype=np.uint32).reshape(2))
                st = lib.mfg_sampler_signs(key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), r.p, nr, ld,
                                           _lib.MFG_F32, ctypes.c_void_p(panel[int(b0)].data_ptr()),
                                           ctypes.c_void_p(slot.stream.cuda_stream))
                _lib.check(st, "mfg_sampler_signs")
                keep += [xh, xd, a, a_lo]
            gop = _GroupOperator(ops, starts, counts, n, ld, self.device)
            values = torch.empty((P,), dtype=torch.float64, device=self.device)
            s = gop.c_struct()
            if flags is None:
                flags = _flags(k, self.precision)
            nbytes = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, P, ld, flags)
            ws, wsb = slot.workspace.get(nbytes, self.device)
            st = lib.mfg_slq_ex(ctypes.byref(s), k, P, ctypes.c_void_p(panel.data_ptr()), ld, fun, param,
                                ctypes.c_void_p(values.data_ptr()), None, None, None, flags, ws, wsb,
                                ctypes.c_void_p(slot.stream.cuda_stream))
            if gop.error is not None:
                raise gop.error
            _lib.check(st, "mfg_slq_ex")
            # per member: mean and standard error of its probes' values
            ms = torch.stack([torch.stack([values[b0:b0 + c].mean(),
                                           values[b0:b0 + c].std(unbiased=False) / math.sqrt(c)])
                              for b0, c in zip(starts.tolist(), counts)])
            out = torch.empty(ms.shape, dtype=torch.float64, pin_memory=True)
            out.copy_(ms, non_blocking=True)
            done = torch.cuda.Event()
            done.record(slot.stream)
        return {"done": done, "out": out, "keep": (keep, ops, gop, panel, values, ms), "flags": flags,
                "ws": ws, "group": members}

    def _take_group(self, pending, head, now, realtime):
        """The head request and the waiting requests packed with it."""
        n0 = head.x.shape[0]
        group, probes = [head], head.p
        rest = deque()
        while pending:
            r = pending.popleft()
            if realtime and r.arrival > now:
                rest.append(r)
                rest.extend(pending)
                pending.clear()
                break
            n = r.x.shape[0]
            if (len(group) < self.group_members and r.k == head.k and r.fun == head.fun
                    and n <= self.group_max_n and max(n, n0) <= 2 * min(n, n0)
                    and probes + r.p <= self.group_probes):
                group.append(r)
                probes += r.p
            else:
                rest.append(r)
        pending.extend(rest)
        return group

    def run(self, requests, *, realtime: bool = True, stall_s: float | None = None):
        """Serve the requests in arrival order; returns (results, stats).

        stall_s: if solves are in flight and none completes for this many
        seconds, raise RuntimeError describing the solves in flight (a solve
        that does not finish would otherwise keep the loop polling forever).
        """
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        packs = [0, 0]  # packed solves, requests in them
        inflight = {}
        results = []
        t0 = time.perf_counter()
        last_progress = t0
        while pending or inflight:
            now = time.perf_counter() - t0
            if stall_s is not None and inflight and time.perf_counter() - last_progress > stall_s:
                desc = []
                for idx, (slot, req, st, fp, t_start) in inflight.items():
                    members = st.get("group", [req])
                    desc.append({"rid": req.rid, "members": [(r.rid, r.x.shape[0], r.k, r.p) for r in members],
                                 "flags": st["flags"], "slot": self.slots.index(slot),
                                 "age_s": round(now - t_start, 3)})
                raise RuntimeError(f"no solve completed for {stall_s} s; in flight: {desc}; "
                                   f"{len(results)} done, {len(pending)} pending")
            for idx, (slot, req, st, fp, t_start) in list(inflight.items()):
                if st["done"].query() and st["flags"] and _lib.lib().mfg_workspace_status(
                        st["ws"], ctypes.c_void_p(slot.stream.cuda_stream)) == _lib.MFG_ERR_RETRY:
                    # the two-sweep step asked for the three-read form: run it again
                    again = (self._launch_group(slot, st["group"], flags=0) if "group" in st
                             else self._launch(slot, req, flags=0))
                    inflight[idx] = (slot, req, again, fp, t_start)
                    continue
                if st["done"].query():
                    t_end = time.perf_counter() - t0
                    members = st.get("group", [req])
                    out = st["out"].reshape(len(members), 2)
                    for r, (mean, sem) in zip(members, out.tolist()):
                        arrival = r.arrival if realtime else 0.0
                        results.append(Result(r.rid, mean, sem, 1e3 * (t_end - arrival), 1e3 * t_start,
                                              1e3 * t_end, r.x.shape[0], r.k, r.p))
                    slot.busy = False
                    self.used -= fp
                    del inflight[idx]
                    last_progress = time.perf_counter()
            admitted = False
            while pending and (not realtime or pending[0].arrival <= now):
                req = pending[0]
                small = req.x.shape[0] <= self.group_max_n
                fp = footprint_bytes(req.x.shape[0], req.k, req.p, self.precision)
                if fp > self.budget:
                    raise ValueError(f"request {req.rid} needs {fp / 1e9:.1f} GB > budget")
                free = [s for s in self.slots if not s.busy]
                if not free or self.used + fp > self.budget:
                    break
                pending.popleft()
                slot = free[0]
                if small:
                    group = self._take_group(pending, req, now, realtime)
                    if len(group) > 1:
                        gfp = group_footprint_bytes(group, self.precision)
                        if self.used + gfp > self.budget:
                            # the group does not fit: the head runs alone, the rest wait
                            for r in reversed(group[1:]):
                                pending.appendleft(r)
                            group = [req]
                        else:
                            fp = gfp
                slot.busy = True
                self.used += fp
                t_start = time.perf_counter() - t0
                if small and len(group) > 1:
                    launched = self._launch_group(slot, group)
                    packs[0] += 1
                    packs[1] += len(group)
                else:
                    launched = self._launch(slot, req)
                inflight[req.rid] = (slot, req, launched, fp, t_start)
                admitted = True
            if not admitted:
                time.sleep(20e-6)
        wall = time.perf_counter() - t0
        lat = np.array([r.latency_ms for r in results])
        stats = {"solves": len(results), "wall_s": wall, "solves_per_s": len(results) / wall,
                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                 "mean_ms": float(lat.mean()), "packed_solves": packs[0], "packed_requests": packs[1]}
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
