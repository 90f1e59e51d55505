"""Operator descriptors: the ``matvec`` argument of the SLQ path.

matfree accepts any callable ``matvec(v, *params)`` (matfree/funm.py:231-235,
decomp.py:380-386) and evaluates it under ``vmap`` over the probes
(stochtrace.py:49).  Here the operator is applied to the whole probe panel at
once by a CUDA kernel, so the operator must be described to the library:

* ``DenseOperator``    dense matrix, fp32 / fp64 CUDA-core product or bf16 /
                        bf16x3-split tcgen05 tensor-core product;
* ``RBFKernelOperator`` dense RBF kernel matrix built on the device;
* ``CSROperator``      CSR sparse matrix (int32 indices, fp32 values);
* ``CallbackOperator`` any torch function of a (p, n) CUDA panel (the
                        library calls back into it once per Krylov step).

Every descriptor is itself a callable ``op(v, *params)``, so it still
satisfies matfree's matvec protocol.  A plain Python callable passed where an
operator is expected is wrapped in a ``CallbackOperator`` (vectorised with
``torch.vmap``).
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._panel import Workspace, padded_ld, require_cuda, stream_ptr, wrap_device


class Operator:
    n: int
    precision: str = "fp32"
    shift: float = 0.0

    @property
    def basis_dtype(self):
        return torch.float64 if self.precision == "fp64" else torch.float32

    def c_struct(self) -> _lib.MfgOperator:
        raise NotImplementedError

    def matmat(self, V: torch.Tensor) -> torch.Tensor:
        """Apply to the rows of V (p, n); returns (p, n)."""
        from ._panel import as_panel

        V = require_cuda(V, "V")
        p = V.shape[0]
        panel, ld = as_panel(V, self.n, self.basis_dtype)
        out = torch.zeros((p, ld), dtype=self.basis_dtype, device=V.device)
        op = self.c_struct()
        nbytes = _lib.lib().mfg_slq_workspace_bytes(ctypes.byref(op), 0, p, ld)
        ws, wsb = self._ws.get(nbytes, V.device)
        st = _lib.lib().mfg_operator_apply(ctypes.byref(op), ctypes.c_void_p(panel.data_ptr()),
                                           ctypes.c_void_p(out.data_ptr()), p, ld, ws, wsb, stream_ptr())
        _lib.check(st, "mfg_operator_apply")
        return out[:, : self.n]

    def __call__(self, v, *params):
        if v.dim() == 1:
            return self.matmat(v[None, :])[0]
        return self.matmat(v)

    @property
    def _ws(self):
        if not hasattr(self, "_workspace"):
            self._workspace = Workspace()
        return self._workspace


class DenseOperator(Operator):
    """A + shift I for a dense (n, n) CUDA matrix A.

    precision: "fp32" (CUDA cores), "fp64" (CUDA cores, float64 basis),
    "bf16" (tcgen05, A rounded to bf16) or "bf16x3" (tcgen05, A and the
    panel split into bf16 hi + lo, three products hi*hi + hi*lo + lo*hi).
    """

    def __init__(self, A: torch.Tensor, *, precision: str = "fp32", shift: float = 0.0):
        A = require_cuda(A, "A")
        if A.dim() != 2 or A.shape[0] != A.shape[1]:
            raise ValueError("A must be square")
        if precision not in _lib.PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_lib.PRECISIONS)}")
        self.n = int(A.shape[0])
        self.precision = precision
        self.shift = float(shift)
        self.lda = padded_ld(self.n)
        n, lda = self.n, self.lda
        self.a_lo = None
        if precision in ("fp32", "fp64"):
            dt = torch.float32 if precision == "fp32" else torch.float64
            self.a = torch.zeros((n, lda), dtype=dt, device=A.device)
            self.a[:, :n].copy_(A)
        else:
            src = torch.zeros((n, lda), dtype=torch.float32, device=A.device)
            src[:, :n].copy_(A)
            self.a = torch.zeros((n, lda), dtype=torch.bfloat16, device=A.device)
            lo = torch.zeros((n, lda), dtype=torch.bfloat16, device=A.device) if precision == "bf16x3" else None
            st = _lib.lib().mfg_split_bf16(
                ctypes.c_void_p(src.data_ptr()), n, lda, lda, ctypes.c_void_p(self.a.data_ptr()),
                ctypes.c_void_p(lo.data_ptr() if lo is not None else 0), lda, stream_ptr())
            _lib.check(st, "mfg_split_bf16")
            self.a_lo = lo

    @classmethod
    def _from_storage(cls, n, precision, a, a_lo, shift):
        obj = cls.__new__(cls)
        obj.n, obj.precision, obj.a, obj.a_lo, obj.shift = int(n), precision, a, a_lo, float(shift)
        obj.lda = a.shape[1]
        return obj

    def c_struct(self):
        s = _lib.MfgOperator()
        s.kind = _lib.MFG_OP_DENSE
        s.precision = _lib.PRECISIONS[self.precision]
        s.n = self.n
        s.a = self.a.data_ptr()
        s.a_lo = self.a_lo.data_ptr() if self.a_lo is not None else None
        s.lda = self.lda
        s.shift = self.shift
        return s

    def transpose(self) -> "DenseOperator":
        """A^T + shift I in the same storage (an explicit transposed copy, cached)."""
        cached = getattr(self, "_transpose", None)
        if cached is not None:
            return cached
        n = self.n

        def tr(a):
            if a is None:
                return None
            t = torch.zeros_like(a)
            t[:, :n] = a[:, :n].t()
            return t

        out = DenseOperator._from_storage(n, self.precision, tr(self.a), tr(self.a_lo), self.shift)
        out._transpose = self
        self._transpose = out
        return out

    def dense(self) -> torch.Tensor:
        """The operator as a float64 (n, n) matrix (for checks)."""
        a = self.a[:, : self.n].double()
        if self.a_lo is not None:
            a = a + self.a_lo[:, : self.n].double()
        return a + self.shift * torch.eye(self.n, dtype=torch.float64, device=a.device)


class RBFKernelOperator(DenseOperator):
    """K = s2 exp(-|x_i - x_j|^2 / (2 ell^2)) + tau I from points x (n, dim).

    The exponential part is built on the device in the requested storage;
    the nugget tau is the operator shift (applied exactly in fp32).  The
    hyper-parameters are theta = (log s2, log ell, log tau).
    """

    def __init__(self, x: torch.Tensor, *, s2: float = 1.0, ell: float = 0.2, tau: float = 1e-2,
                 precision: str = "bf16x3"):
        x = require_cuda(x, "x")
        if precision not in _lib.PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(_lib.PRECISIONS)}")
        x = x.to(torch.float32).contiguous()
        self.x = x
        self.n = int(x.shape[0])
        self.dim = int(x.shape[1])
        self.s2, self.ell, self.tau = float(s2), float(ell), float(tau)
        self.precision = precision
        self.shift = self.tau
        self.lda = padded_ld(self.n)
        dt = {"fp32": torch.float32, "fp64": torch.float64, "bf16": torch.bfloat16, "bf16x3": torch.bfloat16}[precision]
        self.a = torch.empty((self.n, self.lda), dtype=dt, device=x.device)
        self.a_lo = torch.empty((self.n, self.lda), dtype=dt, device=x.device) if precision == "bf16x3" else None
        st = _lib.lib().mfg_rbf_build(
            ctypes.c_void_p(x.data_ptr()), self.n, self.dim, self.s2, self.ell,
            _lib.PRECISIONS[precision], ctypes.c_void_p(self.a.data_ptr()),
            ctypes.c_void_p(self.a_lo.data_ptr() if self.a_lo is not None else 0), self.lda, stream_ptr())
        _lib.check(st, "mfg_rbf_build")

    @property
    def theta(self):
        return (math.log(self.s2), math.log(self.ell), math.log(self.tau))

    @classmethod
    def from_theta(cls, x, theta, precision="bf16x3"):
        s2, ell, tau = (float(math.exp(t)) for t in theta)
        return cls(x, s2=s2, ell=ell, tau=tau, precision=precision)


class CSROperator(Operator):
    """A + shift I for a CSR matrix (int32 row_ptr / col_idx, float32 values)."""

    def __init__(self, row_ptr, col_idx, values, n: int, *, shift: float = 0.0):
        row_ptr = require_cuda(row_ptr, "row_ptr")
        col_idx = require_cuda(col_idx, "col_idx")
        values = require_cuda(values, "values")
        self.row_ptr = row_ptr.to(torch.int32).contiguous()
        self.col_idx = col_idx.to(torch.int32).contiguous()
        self.values = values.to(torch.float32).contiguous()
        self.n = int(n)
        self.nnz = int(self.values.numel())
        self.shift = float(shift)
        self.precision = "fp32"
        if self.row_ptr.numel() != self.n + 1:
            raise ValueError("row_ptr must have n + 1 entries")

    @classmethod
    def from_scipy(cls, A, *, shift: float = 0.0, device="cuda"):
        A = A.tocsr()
        return cls(torch.from_numpy(np.asarray(A.indptr, dtype=np.int32)).to(device),
                   torch.from_numpy(np.asarray(A.indices, dtype=np.int32)).to(device),
                   torch.from_numpy(np.asarray(A.data, dtype=np.float32)).to(device),
                   A.shape[0], shift=shift)

    def c_struct(self):
        s = _lib.MfgOperator()
        s.kind = _lib.MFG_OP_CSR
        s.precision = _lib.MFG_PREC_FP32
        s.n = self.n
        s.row_ptr = self.row_ptr.data_ptr()
        s.col_idx = self.col_idx.data_ptr()
        s.values = self.values.data_ptr()
        s.nnz = self.nnz
        s.shift = self.shift
        return s


class CallbackOperator(Operator):
    """Any torch function of a CUDA panel.

    ``fn(V)`` maps a (p, n) tensor to (p, n) when ``batched`` is True;
    otherwise ``fn(v, *params)`` maps (n,) to (n,) and is vectorised with
    ``torch.vmap`` (falling back to a loop over the rows on the GPU).
    """

    def __init__(self, fn, n: int, *, dtype=torch.float32, batched: bool = False, params=()):
        self.fn = fn
        self.n = int(n)
        self.precision = "fp64" if dtype == torch.float64 else "fp32"
        self.batched = batched
        self.params = tuple(params)
        self.error = None
        dtype_ = dtype

        def _apply(ctx, V, W, n, p, ld, stream):
            try:
                Vt = wrap_device(V, (p, n), (ld, 1), dtype_)
                Wt = wrap_device(W, (p, n), (ld, 1), dtype_)
                Wt.copy_(self._apply_rows(Vt))
                return 0
            except Exception as exc:  # reported by the caller through the status
                self.error = exc
                return 1

        self._cfn = _lib.APPLY_FN(_apply)

    def _apply_rows(self, V):
        if self.batched:
            return self.fn(V, *self.params)
        try:
            return torch.vmap(lambda v: self.fn(v, *self.params))(V)
        except Exception:
            return torch.stack([self.fn(v, *self.params) for v in V])

    def with_params(self, params):
        self.params = tuple(params)
        return self

    def c_struct(self):
        s = _lib.MfgOperator()
        s.kind = _lib.MFG_OP_CALLBACK
        s.precision = _lib.PRECISIONS[self.precision]
        s.n = self.n
        s.apply = self._cfn
        s.ctx = None
        return s


def as_operator(matvec, n: int, dtype=torch.float32, params=()) -> Operator:
    """Return ``matvec`` as an operator descriptor (wrapping callables)."""
    if isinstance(matvec, CallbackOperator):
        return matvec.with_params(params) if params else matvec
    if isinstance(matvec, Operator):
        if matvec.n != n:
            raise ValueError(f"operator dimension {matvec.n} does not match vector length {n}")
        return matvec
    if callable(matvec):
        return CallbackOperator(matvec, n, dtype=dtype, params=params)
    raise TypeError("matvec must be an operator descriptor or a callable")
