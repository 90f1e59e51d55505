"""Matrix functions and the SLQ integrands (GPU).

``monte_carlo_funm_sym(dense_funm, tridiag_sym)`` and
``monte_carlo_funm_sym_logdet(tridiag_sym)`` build the integrand
``quadform(matvec, v, *params) = ||v||^2 e1^T f(T) e1`` of matfree/funm.py:186-243;
``dense_funm_sym_eigh(matfun)`` is matfree/funm.py:322-335.  Called on one
vector the integrand behaves exactly like matfree's.  The estimators in
``stochtrace`` call ``integrand.batched(matvec, samples)`` instead of vmap:
one ``mfg_slq`` call runs the Krylov iteration for all probes, then the
batched tridiagonal eigensolve + quadrature kernel.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._panel import Workspace, as_panel, require_cuda, stream_ptr
from .decomp import _flat_operator, _TridiagSymFull, full_reortho, run_hessenberg, two_sweep_applies
from .operators import CallbackOperator, Operator, as_operator
from .tree import ravel_pytree

_LOGS = {np.log, math.log, torch.log}
_EXPS = {np.exp, math.exp, torch.exp}


class DenseFunmSymEigh:
    """f(M) = V diag(f(lambda)) V^T for a dense symmetric matrix (funm.py:322-335).

    ``kind``/``param`` identify f for the fused device quadrature (log,
    exp(param x), x**param); any other callable runs as torch code on the
    eigenvalues produced by the device eigensolver.
    """

    def __init__(self, matfun, kind=None, param=0.0):
        self.matfun = matfun
        if kind is None:
            if matfun in _LOGS:
                kind, param = _lib.MFG_FUN_LOG, 0.0
            elif matfun in _EXPS:
                kind, param = _lib.MFG_FUN_EXP, 1.0
        self.kind = kind
        self.param = float(param)

    def __call__(self, dense_matrix: torch.Tensor) -> torch.Tensor:
        dense_matrix = require_cuda(dense_matrix, "dense_matrix")
        w, V = torch.linalg.eigh(dense_matrix)
        return V @ torch.diag_embed(self.apply_scalar(w)) @ V.transpose(-1, -2)

    def apply_scalar(self, x: torch.Tensor) -> torch.Tensor:
        if self.kind == _lib.MFG_FUN_LOG:
            return torch.log(x)
        if self.kind == _lib.MFG_FUN_EXP:
            return torch.exp(self.param * x)
        if self.kind == _lib.MFG_FUN_POW:
            return x ** self.param
        out = self.matfun(x)
        return out if isinstance(out, torch.Tensor) else torch.as_tensor(out, device=x.device)


def dense_funm_sym_eigh(matfun):
    """matfree/funm.py:322-335."""
    return DenseFunmSymEigh(matfun)


def funm_exp(scale: float = 1.0) -> DenseFunmSymEigh:
    """f(x) = exp(scale x) with the fused device quadrature."""
    return DenseFunmSymEigh(lambda x: torch.exp(scale * x), kind=_lib.MFG_FUN_EXP, param=scale)


def funm_pow(power: float) -> DenseFunmSymEigh:
    """f(x) = x ** power with the fused device quadrature."""
    return DenseFunmSymEigh(lambda x: x ** power, kind=_lib.MFG_FUN_POW, param=power)


_WS = Workspace()


class MonteCarloFunmSym:
    """The SLQ integrand (matfree/funm.py:205-243)."""

    def __init__(self, dense_funm, tridiag_sym):
        if not isinstance(dense_funm, DenseFunmSymEigh):
            dense_funm = DenseFunmSymEigh(dense_funm)
        if not isinstance(tridiag_sym, _TridiagSymFull):
            raise TypeError("tridiag_sym must come from matfree_gb300.decomp.tridiag_sym(k, reortho='full')")
        self.dense_funm = dense_funm
        self.tridiag_sym = tridiag_sym

    # single vector: the matfree call signature
    def __call__(self, matvec, v0, *parameters):
        flat, unravel = ravel_pytree(v0)
        flat = require_cuda(flat, "v0")
        op = _flat_operator(matvec, unravel, flat.numel(), flat.dtype, parameters)
        return self.batched(op, flat[None, :])[0]

    def batched(self, matvec, samples: torch.Tensor, *parameters) -> torch.Tensor:
        """Integrand values (p,) float64 for the rows of samples (p, n)."""
        samples = require_cuda(samples, "samples")
        p, n = samples.shape
        k = self.tridiag_sym.num_matvecs
        if isinstance(matvec, Operator):
            op = as_operator(matvec, n, samples.dtype, parameters)
        else:
            op = _flat_operator(matvec, lambda v: v, n, samples.dtype, parameters)
        if k < 0 or k > n:
            from .decomp import _error_num_matvecs

            raise ValueError(_error_num_matvecs(k, maxval=n, minval=0))
        if k > 0 and isinstance(op, CallbackOperator):
            from .autodiff import callback_quadform, params_require_grad

            if params_require_grad(op.params):
                # differentiable in the matvec's parameters (the custom VJP
                # of tridiag_sym, decomp.py:420-422)
                return callback_quadform(op.fn, n, k, samples, self.dense_funm, op.params,
                                         batched=op.batched)
        if self.dense_funm.kind is not None:
            return slq_values(op, k, samples, self.dense_funm.kind, self.dense_funm.param)
        # arbitrary f: device Krylov + device eigensolve, f evaluated by torch on the GPU
        _, H, _, c = run_hessenberg(op, k, samples, reortho=full_reortho(op, k))
        lam, fsq = tridiag_eigh_first(H)
        length_sq = 1.0 / (c * c)
        return length_sq * (self.dense_funm.apply_scalar(lam) * fsq).sum(-1)


def slq_values(op, k: int, samples: torch.Tensor, fun: int, param: float, mean_sem=None,
               workspace=None, two_sweep=None, check=True):
    """One ``mfg_slq_ex`` call: values (p,) float64 of ||v||^2 e1^T f(T) e1.

    ``two_sweep`` (default: where it applies) runs the full reorthogonalisation
    in two reads of the Krylov basis per step.  With ``check`` the call waits
    for the solve and, if the device reports ``MFG_ERR_RETRY`` (a step whose
    second projection was too large for the two-sweep form), repeats it with
    the three-sweep form; callers that keep several solves in flight pass
    ``check=False`` and call :func:`slq_retry_needed` once the solve is done.
    """
    p, n = samples.shape
    panel, ld = as_panel(samples, n, op.basis_dtype)
    values = torch.empty((p,), dtype=torch.float64, device=samples.device)
    if two_sweep is None:
        two_sweep = two_sweep_applies(op, k)
    flags = _lib.MFG_SLQ_TWO_SWEEP if two_sweep else 0
    s = op.c_struct()
    lib = _lib.lib()
    nbytes = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, ld, flags)
    ws, wsb = (workspace or _WS).get(nbytes, samples.device)
    ms = ctypes.c_void_p(mean_sem.data_ptr()) if mean_sem is not None else ctypes.c_void_p(0)
    st = lib.mfg_slq_ex(ctypes.byref(s), k, p, ctypes.c_void_p(panel.data_ptr()), ld, fun, param,
                        ctypes.c_void_p(values.data_ptr()), ms, None, None, flags, ws, wsb,
                        stream_ptr())
    err = getattr(op, "error", None)
    if err is not None:
        op.error = None
        raise err
    _lib.check(st, "mfg_slq_ex")
    if two_sweep and check and slq_retry_needed(workspace or _WS):
        return slq_values(op, k, samples, fun, param, mean_sem, workspace, two_sweep=False)
    return values


def slq_retry_needed(workspace) -> bool:
    """Wait for the last solve on ``workspace``; True if it must be repeated
    without the two-sweep form (device status ``MFG_ERR_RETRY``)."""
    buf = workspace.buf
    st = _lib.lib().mfg_workspace_status(ctypes.c_void_p(buf.data_ptr()), stream_ptr())
    if st == _lib.MFG_ERR_RETRY:
        return True
    _lib.check(st, "mfg_slq_ex (device status)")
    return False


def tridiag_eigh_first(H: torch.Tensor):
    """Eigenvalues (ascending) and squared first eigenvector components of the
    tridiagonal part of (H + H^T)/2 for a stack H (p, k, k) float64."""
    p, k, _ = H.shape
    H = H.contiguous()
    lam = torch.empty((p, k), dtype=torch.float64, device=H.device)
    fsq = torch.empty((p, k), dtype=torch.float64, device=H.device)
    st = _lib.lib().mfg_tridiag_quadrature(k, p, ctypes.c_void_p(H.data_ptr()), _lib.MFG_FUN_NONE, 0.0,
                                           None, None, ctypes.c_void_p(lam.data_ptr()),
                                           ctypes.c_void_p(fsq.data_ptr()), stream_ptr())
    _lib.check(st, "mfg_tridiag_quadrature")
    return lam, fsq


def tridiag_eigh(H: torch.Tensor):
    """Eigenvalues (ascending, (p, k)) and eigenvectors (columns of (p, k, k)) of
    the tridiagonal part of (H + H^T)/2 for a stack H (p, k, k) float64."""
    p, k, _ = H.shape
    H = H.contiguous()
    w = torch.empty((p, k), dtype=torch.float64, device=H.device)
    S = torch.empty((p, k, k), dtype=torch.float64, device=H.device)
    Z = torch.empty((p, k, k), dtype=torch.float64, device=H.device)
    st = _lib.lib().mfg_tridiag_eigh(k, p, ctypes.c_void_p(H.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                     ctypes.c_void_p(S.data_ptr()), ctypes.c_void_p(Z.data_ptr()),
                                     stream_ptr())
    _lib.check(st, "mfg_tridiag_eigh")
    return w, S


def monte_carlo_funm_sym(dense_funm, tridiag_sym, /):
    """matfree/funm.py:205-243."""
    return MonteCarloFunmSym(dense_funm, tridiag_sym)


def monte_carlo_funm_sym_logdet(tridiag_sym, /):
    """matfree/funm.py:186-202 (f = log)."""
    return MonteCarloFunmSym(dense_funm_sym_eigh(torch.log), tridiag_sym)


# The spec name of the same integrand.
integrand_funm_sym_logdet = monte_carlo_funm_sym_logdet


class FunmLanczosSym:
    """f(A) v by Lanczos: ||v|| Q^T f(T) e1 (matfree/funm.py:114-147).

    ``batched(matvec, V)`` evaluates every row of V (p, n) at once: one batched
    decomposition, the device eigensolver for f(T) e1 (mfg_tridiag_eigh, every
    eigenvector) and the device back-projection Q^T (f(T) e1)
    (mfg_basis_combine).  With the decomposition's custom VJP the result is
    differentiable in V and in a callable matvec's parameters.
    """

    def __init__(self, dense_funm, tridiag_sym):
        if not isinstance(dense_funm, DenseFunmSymEigh):
            dense_funm = DenseFunmSymEigh(dense_funm)
        self.dense_funm = dense_funm
        self.tridiag_sym = tridiag_sym

    def __call__(self, matvec, vec, *parameters):
        flat, unravel = ravel_pytree(vec)
        flat = require_cuda(flat, "vec")
        op = _flat_operator(matvec, unravel, flat.numel(), flat.dtype, parameters) \
            if not isinstance(matvec, Operator) else matvec
        return unravel(self.batched(op, flat[None, :])[0])

    def batched(self, matvec, V: torch.Tensor, *parameters) -> torch.Tensor:
        from .autodiff import basis_combine, funm_e1
        from .decomp import _todense_tridiag_sym

        V = require_cuda(V, "vectors")
        length = torch.linalg.vector_norm(V, dim=1)
        Q, T, *_ = self.tridiag_sym.batched(matvec, V / length[:, None], *parameters)
        if isinstance(T, tuple):
            T = _todense_tridiag_sym(*T)
        if T.shape[-1] == 0:
            return torch.zeros_like(V)
        coef = funm_e1(T, self.dense_funm) * length.to(torch.float64)[:, None]
        return basis_combine(Q, coef).to(V.dtype)


def funm_lanczos_sym(dense_funm, tridiag_sym, /):
    """f(A) v via Lanczos (matfree/funm.py:114-147): ||v|| Q^T f(T) e1."""
    return FunmLanczosSym(dense_funm, tridiag_sym)


# ---------------------------------------------------------------------------
# Matrix functions of products A^T A (matfree/funm.py:246-320)
# ---------------------------------------------------------------------------


class DenseFunmProductSvd(DenseFunmSymEigh):
    """f(B^T B) through the SVD of B (matfree/funm.py:306-320).

    ``kind``/``param`` name the fused device quadrature of f on the
    eigenvalues of B^T B (log, or x ** param for Schatten norms).
    """

    def __call__(self, matrix: torch.Tensor) -> torch.Tensor:
        matrix = require_cuda(matrix, "matrix")
        _, S, Vt = torch.linalg.svd(matrix)
        eigvecs = Vt.transpose(-1, -2)
        return eigvecs @ torch.diag_embed(self.apply_scalar(S * S)) @ eigvecs.transpose(-1, -2)


def dense_funm_product_svd(matfun):
    """matfree/funm.py:306-320."""
    return DenseFunmProductSvd(matfun)


class MonteCarloFunmProduct:
    """The integrand ||v||^2 e1^T f(B^T B) e1 of matfree/funm.py:276-303."""

    def __init__(self, dense_funm, bidiag):
        from .decomp import _Bidiag

        if not isinstance(dense_funm, DenseFunmProductSvd):
            dense_funm = DenseFunmProductSvd(dense_funm)
        if not isinstance(bidiag, _Bidiag):
            raise TypeError("bidiag must come from matfree_gb300.decomp.bidiag(k)")
        self.dense_funm = dense_funm
        self.bidiag = bidiag

    def __call__(self, matvec, v0, *parameters):
        flat, unravel = ravel_pytree(v0)
        flat = require_cuda(flat, "v0")
        if isinstance(matvec, Operator):
            return self.batched(matvec, flat[None, :], *parameters)[0]

        def flat_matvec(x, *p):
            return ravel_pytree(matvec(unravel(x), *p))[0]

        return self.batched(flat_matvec, flat[None, :], *parameters)[0]

    def batched(self, matvec, samples: torch.Tensor, *parameters) -> torch.Tensor:
        """Integrand values (p,) float64 for the rows of samples (p, n_cols)."""
        samples = require_cuda(samples, "samples")
        k = self.bidiag.num_matvecs
        if self.dense_funm.kind is not None:
            return _slq_product_values(self.bidiag, matvec, samples, k, self.dense_funm.kind,
                                       self.dense_funm.param, parameters)
        _, _, alphas, betas, _, c = self.bidiag.batched(matvec, samples, *parameters)
        lam, fsq = tridiag_eigh_first(_gram(alphas, betas))
        return (1.0 / (c * c)) * (self.dense_funm.apply_scalar(lam) * fsq).sum(-1)


def _gram(alphas: torch.Tensor, betas: torch.Tensor) -> torch.Tensor:
    """B^T B (p, k, k) for the upper bidiagonal B (alphas; betas[:, 1:] above)."""
    p, k = alphas.shape
    d = alphas * alphas
    d[:, 1:] += betas[:, 1:] * betas[:, 1:]
    o = alphas[:, :-1] * betas[:, 1:]
    return torch.diag_embed(d) + torch.diag_embed(o, 1) + torch.diag_embed(o, -1)


def _slq_product_values(bidiag, matvec, samples, k, kind, param, parameters):
    """One ``mfg_slq_product`` call for all rows of samples."""
    p, ncols = samples.shape
    A, At, nrows, _ = bidiag._operators(matvec, samples[0], parameters)
    if k < 1 or k > min(nrows, ncols):
        from .decomp import _error_num_matvecs

        raise ValueError(_error_num_matvecs(k, maxval=min(nrows, ncols), minval=0))
    N = A.n
    dt = A.basis_dtype
    V0p = torch.zeros((p, N), dtype=dt, device=samples.device)
    V0p[:, :ncols] = samples
    panel, ld = as_panel(V0p, N, dt)
    values = torch.empty((p,), dtype=torch.float64, device=samples.device)
    sA, sT = A.c_struct(), At.c_struct()
    lib = _lib.lib()
    nbytes = lib.mfg_bidiag_workspace_bytes(ctypes.byref(sA), ctypes.byref(sT), k, p, ld)
    if nbytes == 0:
        raise ValueError("unsupported operator pair for bidiagonalisation")
    ws, wsb = _WS.get(nbytes, samples.device)
    st = lib.mfg_slq_product(ctypes.byref(sA), ctypes.byref(sT), k, p, ctypes.c_void_p(panel.data_ptr()), ld,
                             kind, param, ctypes.c_void_p(values.data_ptr()), None, ws, wsb, stream_ptr())
    for op in (A, At):
        err = getattr(op, "error", None)
        if err is not None:
            op.error = None
            raise err
    _lib.check(st, "mfg_slq_product")
    return values


def monte_carlo_funm_product(dense_funm, bidiag, /):
    """matfree/funm.py:276-303."""
    return MonteCarloFunmProduct(dense_funm, bidiag)


def monte_carlo_funm_product_logdet(bidiag, /):
    """matfree/funm.py:246-256: log det(A^T A)."""
    return MonteCarloFunmProduct(DenseFunmProductSvd(torch.log, kind=_lib.MFG_FUN_LOG), bidiag)


def monte_carlo_funm_product_schatten_norm(power, bidiag, /):
    """matfree/funm.py:259-273: the power-th power of the Schatten-power norm."""
    fn = DenseFunmProductSvd(lambda x: x ** (power / 2), kind=_lib.MFG_FUN_POW, param=power / 2)
    return MonteCarloFunmProduct(fn, bidiag)
