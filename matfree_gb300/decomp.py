"""Krylov decompositions on the GPU: ``tridiag_sym`` and ``hessenberg``.

Same constructors, call signature, outputs and errors as matfree/decomp.py:
``tridiag_sym(num_matvecs, /, *, materialize=True, reortho="full",
custom_vjp=True)`` returns ``decompose(matvec, vec, *params) ->
_DecompResult(Q_tall, J_small, residual, init_length_inv)``
(matfree/decomp.py:30-152).  As in matfree, the full-reorthogonalisation
tridiagonalisation runs the Arnoldi iteration with classical Gram-Schmidt
applied twice and returns the tridiagonal part of T = (H + H^T)/2
(decomp.py:125-145).  The iteration itself runs in ``libmatfree_gb300``
(``mfg_hessenberg``), batched over any number of vectors via ``.batched``.
"""

from __future__ import annotations

import ctypes
from typing import NamedTuple, Union

import torch

from . import _lib
from ._panel import Workspace, as_panel, require_cuda, stream_ptr
from .operators import as_operator
from .tree import ravel_pytree


class _DecompResult(NamedTuple):
    # matfree/decomp.py:15-27
    Q_tall: Union[torch.Tensor, tuple]
    J_small: Union[torch.Tensor, tuple]
    residual: torch.Tensor
    init_length_inv: torch.Tensor


def _error_num_matvecs(num, maxval, minval):
    # matfree/decomp.py:753-756
    msg1 = f"Parameter 'num_matvecs'={num} exceeds the acceptable range. "
    msg2 = f"Expected: {minval} <= num_matvecs <= {maxval}."
    return msg1 + msg2


_WS = Workspace()


def two_sweep_applies(op, k: int) -> bool:
    """Whether the two-sweep step (``mfg_slq_ex`` flag MFG_SLQ_TWO_SWEEP,
    ``mfg_hessenberg`` reortho 3) runs for this operator and k: float bases,
    2 <= k <= 129."""
    return op.basis_dtype == torch.float32 and 2 <= k <= 129


def full_reortho(op, k: int) -> str:
    """The fastest full-reorthogonalisation form for this operator and k."""
    return "full-two-sweep" if two_sweep_applies(op, k) else "full"


def run_hessenberg(op, k: int, V: torch.Tensor, *, reortho: str = "full", workspace=None):
    """Batched Arnoldi over the rows of V (p, n) on the GPU.

    ``reortho``: "full" (Gram-Schmidt twice, three reads of the basis per
    step), "full-two-sweep" (the same in two reads, repeated as "full" when
    the device reports a step near an invariant subspace), "none", or
    "lanczos" (the three-term recurrence).
    Returns (Q (p, k, n), H (p, k, k) float64, residual (p, n), 1/||v|| (p,)).
    """
    V = require_cuda(V, "vectors")
    n = op.n
    p = V.shape[0]
    if k < 0 or k > n:
        raise ValueError(_error_num_matvecs(k, maxval=n, minval=0))
    dt = op.basis_dtype
    panel, ld = as_panel(V, n, dt)
    Q = torch.zeros((p, max(k, 0), ld), dtype=dt, device=V.device)
    H = torch.zeros((p, k, k), dtype=torch.float64, device=V.device)
    R = torch.zeros((p, ld), dtype=dt, device=V.device)
    c = torch.zeros((p,), dtype=torch.float64, device=V.device)
    s = op.c_struct()
    lib = _lib.lib()
    mode = {"none": 0, "full": 1, "lanczos": 2, "full-two-sweep": 3}[reortho]
    flags = _lib.MFG_SLQ_TWO_SWEEP if mode == 3 else 0
    nbytes = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, ld, flags)
    ws, wsb = (workspace or _WS).get(nbytes, V.device)
    st = lib.mfg_hessenberg(ctypes.byref(s), k, p, ctypes.c_void_p(panel.data_ptr()), ld, mode,
                            ctypes.c_void_p(Q.data_ptr() if k > 0 else 0),
                            ctypes.c_void_p(H.data_ptr() if k > 0 else 0),
                            ctypes.c_void_p(R.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                            ws, wsb, stream_ptr())
    err = getattr(op, "error", None)
    if err is not None:
        op.error = None
        raise err
    _lib.check(st, "mfg_hessenberg")
    if mode == 3:
        # the two-sweep step asks for the three-sweep form near an invariant subspace
        dst = lib.mfg_workspace_status(ws, stream_ptr())
        if dst == _lib.MFG_ERR_RETRY:
            return run_hessenberg(op, k, V, reortho="full", workspace=workspace)
        _lib.check(dst, "mfg_hessenberg (device status)")
    return Q[:, :, :n], H, R[:, :n], c


def _tridiag_from_hessenberg(H):
    # matfree/decomp.py:133-135
    T = 0.5 * (H + H.transpose(-1, -2))
    return torch.diagonal(T, 0, -2, -1), torch.diagonal(T, 1, -2, -1)


def _todense_tridiag_sym(diag, off_diag):
    # matfree/decomp.py:148-152
    return torch.diag_embed(diag) + torch.diag_embed(off_diag, -1) + torch.diag_embed(off_diag, 1)


class _Decomposition:
    reortho = "full"

    def __init__(self, num_matvecs: int, *, materialize: bool, custom_vjp: bool):
        self.num_matvecs = int(num_matvecs)
        self.materialize = materialize
        self.custom_vjp = custom_vjp

    def _prepare(self, matvec, vec, params):
        flat, unravel = ravel_pytree(vec)
        n = flat.numel()
        if self.num_matvecs < 0 or self.num_matvecs > n:
            raise ValueError(_error_num_matvecs(self.num_matvecs, maxval=n, minval=0))
        flat = require_cuda(flat, "vec")
        op = _flat_operator(matvec, unravel, n, flat.dtype, params)
        return flat, unravel, op

    def __call__(self, matvec, vec, *params):
        flat, unravel, op = self._prepare(matvec, vec, params)
        out = self.batched(op, flat[None, :])
        Q, J, r, c = out
        J = tuple(x[0] for x in J) if isinstance(J, tuple) else J[0]
        return _DecompResult(Q_tall=unravel(Q[0]), J_small=J, residual=unravel(r[0]),
                             init_length_inv=c[0])


def _differentiable_forward(dec, op, k, V):
    """run_hessenberg with full reorthogonalisation, behind the Hessenberg
    adjoint when V or the matvec's parameters require gradients (the custom
    VJP of matfree/decomp.py:393-422); plain otherwise."""
    from .autodiff import arnoldi_full, wants_grad

    if k > 0 and wants_grad(V, op):
        if not dec.custom_vjp:
            raise NotImplementedError(
                "gradients of the decomposition need custom_vjp=True: the Krylov loop runs as CUDA "
                "kernels, so it is differentiated by the Hessenberg adjoint, not traced")
        return arnoldi_full(op, k, V)
    return run_hessenberg(op, k, V, reortho=full_reortho(op, k))


class _TridiagSymFull(_Decomposition):
    def batched(self, matvec, V: torch.Tensor, *params) -> _DecompResult:
        """Decompose every row of V (p, n) at once; outputs carry a leading p axis.

        Differentiable in V and in the tensor leaves of a callable matvec's
        parameters (custom_vjp=True, the default)."""
        V = require_cuda(V, "vectors")
        op = as_operator(matvec, V.shape[1], V.dtype, params)
        k = self.num_matvecs
        Q, H, r, c = _differentiable_forward(self, op, k, V)
        d, e = _tridiag_from_hessenberg(H)
        out_dt = V.dtype if V.dtype in (torch.float32, torch.float64) else torch.float32
        d, e = d.to(out_dt), e.to(out_dt)
        J = _todense_tridiag_sym(d, e) if self.materialize else (d, e)
        return _DecompResult(Q_tall=Q, J_small=J, residual=r, init_length_inv=c.to(out_dt))


class _TridiagSymNone(_Decomposition):
    """Three-term Lanczos without reorthogonalisation (matfree/decomp.py:155-291)."""

    reortho = "none"

    def batched(self, matvec, V: torch.Tensor, *params) -> _DecompResult:
        op = as_operator(matvec, V.shape[1], V.dtype, params)
        k = self.num_matvecs
        # k = 0 still applies the operator once for the residual (decomp.py:230-237)
        Q, H, r, c = run_hessenberg(op, max(k, 1), V, reortho="lanczos")
        Q, H = Q[:, :k], H[:, :k, :k]
        out_dt = V.dtype if V.dtype in (torch.float32, torch.float64) else torch.float32
        d = torch.diagonal(H, 0, -2, -1).to(out_dt)
        e = torch.diagonal(H, -1, -2, -1).to(out_dt)
        J = _todense_tridiag_sym(d, e) if self.materialize else (d, e)
        return _DecompResult(Q_tall=Q, J_small=J, residual=r, init_length_inv=c.to(out_dt))


class _Hessenberg(_Decomposition):
    def __init__(self, num_matvecs, *, reortho, custom_vjp, reortho_vjp):
        super().__init__(num_matvecs, materialize=True, custom_vjp=custom_vjp)
        self.reortho = reortho
        self.reortho_vjp = reortho if reortho_vjp == "match" else reortho_vjp

    def batched(self, matvec, V: torch.Tensor, *params) -> _DecompResult:
        V = require_cuda(V, "vectors")
        op = as_operator(matvec, V.shape[1], V.dtype, params)
        k = self.num_matvecs
        if self.reortho == "full":
            Q, H, r, c = _differentiable_forward(self, op, k, V)
        else:
            from .autodiff import wants_grad

            if k > 0 and wants_grad(V, op):
                raise NotImplementedError("gradients are provided for reortho='full' only")
            Q, H, r, c = run_hessenberg(op, k, V, reortho=self.reortho)
        out_dt = V.dtype if V.dtype in (torch.float32, torch.float64) else torch.float32
        return _DecompResult(Q_tall=Q, J_small=H.to(out_dt), residual=r, init_length_inv=c.to(out_dt))


def _flat_operator(matvec, unravel, n, dtype, params):
    """The matvec over flat vectors (pytree in, pytree out, as decomp.py:383-384)."""
    from .operators import CallbackOperator, Operator

    if isinstance(matvec, Operator):
        return as_operator(matvec, n, dtype, params)

    def flat_fn(v, *p):
        return ravel_pytree(matvec(unravel(v), *p))[0]

    return CallbackOperator(flat_fn, n, dtype=dtype, params=params)


def tridiag_sym(num_matvecs: int, /, *, materialize: bool = True, reortho: str = "full",
                custom_vjp: bool = True):
    """Tridiagonalisation with full reorthogonalisation (matfree/decomp.py:30-122)."""
    if reortho == "full":
        return _TridiagSymFull(num_matvecs, materialize=materialize, custom_vjp=custom_vjp)
    if reortho == "none":
        return _TridiagSymNone(num_matvecs, materialize=materialize, custom_vjp=custom_vjp)
    msg = f"reortho={reortho} unsupported. Choose eiter {'full', 'none'}."
    raise ValueError(msg)


class _Bidiag:
    """Golub-Kahan bidiagonalisation with full reorthogonalisation (matfree/decomp.py:608-750).

    The iteration runs in ``libmatfree_gb300`` (``mfg_bidiag``) for all rows
    of a panel at once.  The vector-matrix product u -> A^T u comes from the
    operator's ``transpose()`` (dense descriptors) or, for a callable matvec,
    from ``torch.func.vjp`` of it, as matfree uses ``jax.vjp``
    (decomp.py:711-725).  Rectangular maps (n_rows != n_cols) are handled by
    zero-padding both spaces to the larger size: padded coordinates stay
    exactly zero, so the iteration is the unpadded one.
    """

    def __init__(self, num_matvecs: int, materialize: bool):
        self.num_matvecs = int(num_matvecs)
        self.materialize = materialize

    @staticmethod
    def _operators(Av, x_like: torch.Tensor, params):
        """(A, A^T) as square descriptors of size N, n_rows, n_cols."""
        from .operators import CallbackOperator, DenseOperator, Operator

        ncols = x_like.shape[-1]
        dt = x_like.dtype if x_like.dtype in (torch.float32, torch.float64) else torch.float32
        if isinstance(Av, DenseOperator):
            if Av.n != ncols:
                raise ValueError(f"operator dimension {Av.n} does not match vector length {ncols}")
            return Av, Av.transpose(), ncols, ncols
        if isinstance(Av, Operator):
            raise TypeError("bidiag needs a dense operator descriptor or a callable matvec")

        def av(x):
            return ravel_pytree(Av(x, *params))[0]

        nrows = av(torch.zeros(ncols, dtype=dt, device=x_like.device)).numel()
        N = max(nrows, ncols)

        def pad(X):
            out = torch.zeros((X.shape[0], N), dtype=dt, device=X.device)
            out[:, : X.shape[1]] = X
            return out

        def rows(fn, X):
            try:
                return torch.vmap(fn)(X)
            except Exception:
                return torch.stack([fn(x) for x in X])

        def A_rows(V):
            return pad(rows(av, V[:, :ncols]))

        def At_rows(U):
            _, vjp_fn = torch.func.vjp(av, torch.zeros(ncols, dtype=dt, device=U.device))
            return pad(rows(lambda u: vjp_fn(u)[0], U[:, :nrows]))

        A = CallbackOperator(A_rows, N, dtype=dt, batched=True)
        At = CallbackOperator(At_rows, N, dtype=dt, batched=True)
        return A, At, nrows, ncols

    def batched(self, Av, V0: torch.Tensor, *params):
        """Bidiagonalise from every row of V0 (p, n_cols).

        Returns (U (p, k, n_rows), V (p, k, n_cols), alphas (p, k), betas (p, k),
        residual (p, n_cols), 1/||v0|| (p,)); betas[:, 0] = 0 as in matfree.
        """
        V0 = require_cuda(V0, "V0")
        p, ncols = V0.shape
        A, At, nrows, _ = self._operators(Av, V0[0], params)
        k = self.num_matvecs
        if k < 0 or k > min(nrows, ncols):
            raise ValueError(_error_num_matvecs(k, maxval=min(nrows, ncols), minval=0))
        N = A.n
        dt = A.basis_dtype
        V0p = torch.zeros((p, N), dtype=dt, device=V0.device)
        V0p[:, :ncols] = V0
        panel, ld = as_panel(V0p, N, dt)
        kk = max(k, 1)
        U = torch.zeros((p, kk, ld), dtype=dt, device=V0.device)
        V = torch.zeros((p, kk, ld), dtype=dt, device=V0.device)
        alphas = torch.zeros((p, kk), dtype=torch.float64, device=V0.device)
        betas = torch.zeros((p, kk), dtype=torch.float64, device=V0.device)
        R = torch.zeros((p, ld), dtype=dt, device=V0.device)
        c = torch.zeros((p,), dtype=torch.float64, device=V0.device)
        sA, sT = A.c_struct(), At.c_struct()
        lib = _lib.lib()
        nbytes = lib.mfg_bidiag_workspace_bytes(ctypes.byref(sA), ctypes.byref(sT), k, p, ld)
        if nbytes == 0:
            raise ValueError("unsupported operator pair for bidiagonalisation")
        ws, wsb = _WS.get(nbytes, V0.device)
        st = lib.mfg_bidiag(ctypes.byref(sA), ctypes.byref(sT), k, p, ctypes.c_void_p(panel.data_ptr()), ld,
                            ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(V.data_ptr()),
                            ctypes.c_void_p(alphas.data_ptr()), ctypes.c_void_p(betas.data_ptr()),
                            ctypes.c_void_p(R.data_ptr()), ctypes.c_void_p(c.data_ptr()), ws, wsb, stream_ptr())
        for op in (A, At):
            err = getattr(op, "error", None)
            if err is not None:
                op.error = None
                raise err
        _lib.check(st, "mfg_bidiag")
        return (U[:, :k, :nrows], V[:, :k, :ncols], alphas[:, :k], betas[:, :k], R[:, :ncols], c)

    def __call__(self, Av, v0, *params) -> _DecompResult:
        from .operators import Operator

        flat, unravel = ravel_pytree(v0)
        flat = require_cuda(flat, "v0")
        if isinstance(Av, Operator):
            U, V, alphas, betas, R, c = self.batched(Av, flat[None, :], *params)
            out_like, u_unravel = flat, unravel
        else:
            def av_flat(x, *p):
                return Av(unravel(x), *p)

            U, V, alphas, betas, R, c = self.batched(av_flat, flat[None, :], *params)
            out_like = av_flat(flat, *params)
            _, u_unravel = ravel_pytree(out_like)
        out_dt = flat.dtype if flat.dtype in (torch.float32, torch.float64) else torch.float32
        d, e = alphas[0].to(out_dt), betas[0, 1:].to(out_dt)
        J = torch.diag_embed(d) + torch.diag_embed(e, 1) if self.materialize else (d, e)
        U0, V0 = U[0].to(out_dt), V[0].to(out_dt)
        return _DecompResult(Q_tall=(_stack_unravel(u_unravel, U0, out_like), _stack_unravel(unravel, V0, v0)),
                             J_small=J, residual=unravel(R[0].to(out_dt)), init_length_inv=c[0].to(out_dt))


def _stack_unravel(unravel, M: torch.Tensor, like):
    """k stacked flat vectors (k, n) -> a stack in the shape of ``like``."""
    if isinstance(like, torch.Tensor):
        return M.reshape(M.shape[0], *like.shape)
    return torch.vmap(unravel)(M)


def bidiag(num_matvecs: int, /, materialize: bool = True, reortho: str = "full"):
    """Golub-Kahan bidiagonalisation (matfree/decomp.py:641-750)."""
    if reortho != "full":
        raise NotImplementedError("bidiag is provided with full reorthogonalisation only")
    return _Bidiag(num_matvecs, materialize)


def hessenberg(num_matvecs, /, *, reortho: str, custom_vjp: bool = True, reortho_vjp: str = "match"):
    """Arnoldi / Hessenberg factorisation (matfree/decomp.py:353-423)."""
    reortho_expected = ["none", "full"]
    if reortho not in reortho_expected:
        msg = f"Unexpected input for {reortho}: either of {reortho_expected} expected."
        raise TypeError(msg)
    return _Hessenberg(num_matvecs, reortho=reortho, custom_vjp=custom_vjp, reortho_vjp=reortho_vjp)
