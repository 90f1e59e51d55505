"""Linear solves on the GPU: conjugate gradients.

matfree's Gaussian log-density (tutorials/8_gaussian_logpdf.py:44-50) solves
K alpha = y with ``jax.scipy.sparse.linalg.cg``.  ``cg`` below keeps that
call's signature and stopping rule (||r||^2 <= max(tol^2 ||b||^2, atol^2),
at most ``maxiter`` = 10 n iterations, x0 = 0, no preconditioner) and runs in
``libmatfree_gb300`` (``mfg_cg``): the operator application is the same
tensor-core / CUDA-core / sparse kernel as in the Lanczos iteration, and the
vector updates carry the float64 residual norm.  ``cg_batched`` solves one
system per row of a (p, n) panel, as ``vmap(cg)`` does: rows that have
converged stay fixed while the others iterate.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._panel import Workspace, as_panel, require_cuda, stream_ptr
from .operators import as_operator

_WS = Workspace()


def cg_batched(op, B: torch.Tensor, *, tol: float = 1e-5, atol: float = 0.0, maxiter=None,
               workspace=None):
    """Solve op X_b = B_b for every row b of B (p, n); returns (X (p, n), iterations (p,))."""
    B = require_cuda(B, "B")
    if B.dim() != 2:
        raise ValueError("B must be a (p, n) panel")
    p, n = B.shape
    op = as_operator(op, n, B.dtype, ())
    if op.n != n:
        raise ValueError(f"operator of size {op.n} applied to vectors of size {n}")
    panel, ld = as_panel(B, n, op.basis_dtype)
    X = torch.zeros((p, ld), dtype=op.basis_dtype, device=B.device)
    iters = torch.zeros((p,), dtype=torch.int32, device=B.device)
    s = op.c_struct()
    lib = _lib.lib()
    nbytes = lib.mfg_cg_workspace_bytes(ctypes.byref(s), p, ld)
    if nbytes == 0:
        raise ValueError("unsupported operator for conjugate gradients")
    ws, wsb = (workspace or _WS).get(nbytes, B.device)
    st = lib.mfg_cg(ctypes.byref(s), p, ctypes.c_void_p(panel.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                    ld, float(tol), float(atol), int(maxiter) if maxiter is not None else 0,
                    ctypes.c_void_p(iters.data_ptr()), ws, wsb, stream_ptr())
    err = getattr(op, "error", None)
    if err is not None:
        op.error = None
        raise err
    _lib.check(st, "mfg_cg")
    out_dt = B.dtype if B.dtype in (torch.float32, torch.float64) else torch.float32
    return X[:, :n].to(out_dt), iters


def cg(A, b: torch.Tensor, x0=None, *, tol: float = 1e-5, atol: float = 0.0, maxiter=None, M=None):
    """``jax.scipy.sparse.linalg.cg(A, b, x0, tol=, atol=, maxiter=, M=)`` for one vector.

    Returns ``(x, None)`` like JAX.  The start vector must be zero (or None) and
    no preconditioner is supported.
    """
    if M is not None:
        raise NotImplementedError("preconditioned CG is not supported")
    if x0 is not None and bool(torch.any(x0 != 0)):
        raise NotImplementedError("CG starts from x0 = 0")
    b = require_cuda(b, "b")
    X, _ = cg_batched(A, b.reshape(1, -1), tol=tol, atol=atol, maxiter=maxiter)
    return X[0].reshape(b.shape), None
