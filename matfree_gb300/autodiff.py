"""Gradients of SLQ estimates with respect to operator hyper-parameters.

The reverse pass mirrors what JAX differentiates in matfree:

1. the quadrature ``||v||^2 e1^T f(T) e1`` (funm.py:239-241) through the
   symmetric eigendecomposition of T (funm.py:330-333): the Daleckii-Krein
   formula gives d/dT = S (F o s1 s1^T) S^T with F the divided differences
   of f at the eigenvalues (f' on the diagonal);
2. T = tridiagonal part of (H + H^T)/2 (decomp.py:133-135, 148-152) -> dH;
3. the Hessenberg adjoint (decomp.py:480-600) on the GPU
   (``mfg_hessenberg_adjoint``), which returns the adjoint states Lambda;
4. the parameter part of each step's matvec VJP, summed over steps and
   probes: sum lambda_idx^T (dA/dtheta) q_idx = <Lambda, (dA/dtheta) Q>,
   evaluated for all steps at once by applying dA/dtheta to the stacked
   Krylov basis (one tensor-core operator application per parameter).

Step 1 runs as batched torch linear algebra on the GPU on p small k x k
matrices; everything of size n runs in the CUDA library.

``rbf_logdet`` does step 4 for the RBF kernel's three log-parameters;
``callback_quadform`` does it for any callable matvec(v, *params) with one
autograd VJP of the callable over the stacked basis.
"""

from __future__ import annotations

import ctypes
import math

import torch

from . import _lib
from ._panel import Workspace, as_panel, padded_ld, require_cuda, stream_ptr
from .decomp import run_hessenberg, two_sweep_applies
from .operators import CallbackOperator, DenseOperator, RBFKernelOperator
from .tree import _rebuild, tree_leaves

_WS = Workspace()


def quadform_dH(H: torch.Tensor, scale: torch.Tensor, f, fprime) -> tuple[torch.Tensor, torch.Tensor]:
    """Values scale_b e1^T f(T_b) e1 and their cotangent with respect to H.

    H: (p, k, k) float64; scale: (p,) float64.  Returns (values (p,), dH (p, k, k)).
    """
    from .funm import tridiag_eigh

    p, k = H.shape[0], H.shape[1]
    w, S = tridiag_eigh(H)  # the eigh of T = tridiagonal part of (H + H^T)/2
    fw = f(w)
    s1 = S[:, 0, :]
    values = scale * (fw * s1 * s1).sum(-1)
    diff = w[:, :, None] - w[:, None, :]
    same = diff.abs() <= 1e-13 * torch.clamp(w.abs()[:, :, None], min=1.0)
    F = (fw[:, :, None] - fw[:, None, :]) / torch.where(same, torch.ones_like(diff), diff)
    F = torch.where(same, fprime(0.5 * (w[:, :, None] + w[:, None, :])), F)
    G = S @ (F * s1[:, :, None] * s1[:, None, :]) @ S.transpose(-1, -2)
    G = G * scale[:, None, None]
    # T_dense = diag(d) + diag(e, 1) + diag(e, -1), d = diag(H), e = (H[i,i+1] + H[i+1,i])/2
    dH = torch.zeros_like(H)
    i = torch.arange(k, device=H.device)
    dH[:, i, i] = G[:, i, i]
    if k > 1:
        de = G[:, i[:-1], i[1:]] + G[:, i[1:], i[:-1]]
        dH[:, i[:-1], i[1:]] = 0.5 * de
        dH[:, i[1:], i[:-1]] = 0.5 * de
    return values, dH


def hessenberg_adjoint(op, Q, H, R, c, dH, dr=None, dc=None, dQ=None):
    """GPU reverse pass.  Q (p, k, ld) / R (p, ld) are the forward panels;
    dQ (p, k, ld) and dr (p, ld) are optional cotangents in the same layout.

    Returns (Lambda (p, k, ld), dv (p, ld)).
    """
    p, k, ld = Q.shape
    if k == 0:
        # matfree/decomp.py:483-486
        raise ValueError("Custom Hessenberg-adjoints are not implemented for num_matvecs = 0.")
    Lam = torch.zeros_like(Q)
    dv = torch.zeros_like(R)
    s = op.c_struct()
    lib = _lib.lib()
    nbytes = lib.mfg_adjoint_workspace_bytes(ctypes.byref(s), k, p, ld)
    ws, wsb = _WS.get(nbytes, Q.device)
    vp = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)  # noqa: E731
    st = lib.mfg_hessenberg_adjoint_ex(ctypes.byref(s), k, p, ld, vp(Q), vp(H.contiguous()), vp(R), vp(c),
                                       vp(dQ), vp(dH.contiguous()), vp(dr), vp(dc), vp(Lam), vp(dv), ws,
                                       wsb, stream_ptr())
    err = getattr(op, "error", None)
    if err is not None:  # a callback operator raised inside the reverse sweep
        op.error = None
        raise err
    _lib.check(st, "mfg_hessenberg_adjoint_ex")
    return Lam, dv


def _log(x):
    return torch.log(x)


def _dlog(x):
    return 1.0 / x


def backward_bytes_per_probe(n: int, k: int, dtype=torch.float32) -> int:
    """Device bytes one probe holds between the forward and the backward pass
    (Krylov basis Q, adjoint states Lambda and the residual, in the basis type)."""
    es = 8 if dtype == torch.float64 else 4
    return int((2 * k + 1) * padded_ld(n) * es)


def probe_chunks(p: int, n: int, k: int, dtype, budget_bytes) -> list:
    """Probe ranges [b0, b1) whose bases fit ``budget_bytes`` (all probes at once
    when no budget is given or they fit)."""
    if budget_bytes is None:
        return [(0, p)]
    per = backward_bytes_per_probe(n, k, dtype)
    pc = max(1, min(p, int(budget_bytes // per)))
    return [(b0, min(p, b0 + pc)) for b0 in range(0, p, pc)]


class _RBFLogdet(torch.autograd.Function):
    """mean_b ||v_b||^2 e1^T log(T_b) e1 for K(theta), differentiable in theta.

    When the bases of all probes (Q, Lambda, residual: (2k + 1) n elements per
    probe) exceed ``budget_bytes``, the probes are processed in chunks that
    fit: the forward pass keeps only each chunk's H and 1/||v||, and the
    backward pass recomputes the chunk's Krylov basis (the same deterministic
    kernels on the same probes) before running its adjoint.  Probes are
    independent, so the gradient is that of the unchunked computation."""

    @staticmethod
    def forward(ctx, theta, x, probes, k, precision, budget_bytes):
        s2, ell, tau = (float(math.exp(t)) for t in theta.detach().cpu().tolist())
        op = RBFKernelOperator(x, s2=s2, ell=ell, tau=tau, precision=precision)
        n = op.n
        panel, ld = as_panel(probes, n, op.basis_dtype)
        p = panel.shape[0]
        chunks = probe_chunks(p, n, k, op.basis_dtype, budget_bytes)
        vals, saved = [], []
        for b0, b1 in chunks:
            Q, H, R, c = _forward_panels(op, k, panel[b0:b1], ld)
            values, dH = quadform_dH(H, 1.0 / (c * c), _log, _dlog)
            vals.append(values)
            if len(chunks) == 1:
                saved.append((Q, H, R, c, dH))
            else:
                del Q, R  # recomputed in the backward pass
                saved.append((None, H, None, c, dH))
        ctx.save_for_backward(theta, x)
        ctx.saved = (op, panel, ld, chunks, saved, p, precision)
        return torch.cat(vals).mean()

    @staticmethod
    def backward(ctx, grad_out):
        theta, x = ctx.saved_tensors
        op, panel, ld, chunks, saved, p, precision = ctx.saved
        grad = None
        dl = _rbf_dlogell_operator(op, x)
        for (b0, b1), (Q, H, R, c, dH) in zip(chunks, saved):
            if Q is None:
                Q, H, R, c = _forward_panels(op, H.shape[-1], panel[b0:b1], ld)
            Lam, _dv = hessenberg_adjoint(op, Q, H, R, c, dH * (grad_out.double() / p))
            g = rbf_theta_contractions(op, x, Q, Lam, dl=dl)
            grad = g if grad is None else grad + g
            del Q, R, Lam
        return grad.to(device=theta.device, dtype=theta.dtype), None, None, None, None, None


def _forward_panels(op, k, panel, ld):
    """mfg_hessenberg keeping the padded (p, k, ld) / (p, ld) panels."""
    p = panel.shape[0]
    dt = op.basis_dtype
    Q = torch.zeros((p, k, ld), dtype=dt, device=panel.device)
    H = torch.zeros((p, k, k), dtype=torch.float64, device=panel.device)
    R = torch.zeros((p, ld), dtype=dt, device=panel.device)
    c = torch.zeros((p,), dtype=torch.float64, device=panel.device)
    s = op.c_struct()
    lib = _lib.lib()
    # full reorthogonalisation in two reads of the basis per step where it
    # applies, repeated in the three-read form if the device asks for it
    for mode in ((3, 1) if two_sweep_applies(op, k) else (1,)):
        flags = _lib.MFG_SLQ_TWO_SWEEP if mode == 3 else 0
        nbytes = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, ld, flags)
        ws, wsb = _WS.get(nbytes, panel.device)
        st = lib.mfg_hessenberg(ctypes.byref(s), k, p, ctypes.c_void_p(panel.data_ptr()), ld, mode,
                                ctypes.c_void_p(Q.data_ptr()), ctypes.c_void_p(H.data_ptr()),
                                ctypes.c_void_p(R.data_ptr()), ctypes.c_void_p(c.data_ptr()), ws,
                                wsb, stream_ptr())
        err = getattr(op, "error", None)
        if err is not None:  # a callback operator raised inside the Krylov loop
            op.error = None
            raise err
        _lib.check(st, "mfg_hessenberg")
        if mode == 1:
            break
        dst = lib.mfg_workspace_status(ws, stream_ptr())
        if dst != _lib.MFG_ERR_RETRY:
            _lib.check(dst, "mfg_hessenberg (device status)")
            break
    return Q, H, R, c


def rbf_theta_contractions(op: RBFKernelOperator, x, Q, Lam, dl=None) -> torch.Tensor:
    """d/dtheta of sum_idx lambda_idx^T K(theta) q_idx for theta = (log s2, log ell, log tau).

    dK/dlog s2 = K - tau I,  dK/dlog ell = s2 E o D / ell^2,  dK/dlog tau = tau I.
    """
    p, k, ld = Q.shape
    n = op.n
    rows = Q.reshape(p * k, ld)[:, :n]
    lam = Lam.reshape(p * k, ld)[:, :n].double()
    # the stored exponential part (without the nugget) is dK/dlog s2
    base = DenseOperator._from_storage(n, op.precision, op.a, op.a_lo, 0.0)
    g0 = (lam * base.matmat(rows).double()).sum()
    if dl is None:
        dl = _rbf_dlogell_operator(op, x)
    g1 = (lam * dl.matmat(rows).double()).sum()
    g2 = op.tau * (lam * rows.double()).sum()
    return torch.stack([g0, g1, g2])


def _rbf_dlogell_operator(op: RBFKernelOperator, x) -> DenseOperator:
    lda = padded_ld(op.n)
    dt = op.a.dtype
    a = torch.empty((op.n, lda), dtype=dt, device=x.device)
    a_lo = torch.empty((op.n, lda), dtype=dt, device=x.device) if op.precision == "bf16x3" else None
    st = _lib.lib().mfg_rbf_build_dlogell(
        ctypes.c_void_p(op.x.data_ptr()), op.n, op.dim, op.s2, op.ell, _lib.PRECISIONS[op.precision],
        ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(a_lo.data_ptr() if a_lo is not None else 0), lda,
        stream_ptr())
    _lib.check(st, "mfg_rbf_build_dlogell")
    return DenseOperator._from_storage(op.n, op.precision, a, a_lo, 0.0)


def rbf_logdet(x: torch.Tensor, theta: torch.Tensor, probes: torch.Tensor, num_matvecs: int,
               precision: str = "bf16x3", budget_bytes=None) -> torch.Tensor:
    """SLQ estimate of log det K(theta) on the given probes, differentiable in theta.

    theta = (log s2, log ell, log tau) as a CUDA or CPU tensor of 3 values;
    probes (p, n) CUDA tensor; returns a 0-d float64 tensor.  ``budget_bytes``
    caps the device memory the Krylov bases hold between the forward and the
    backward pass (probe chunks recomputed in the backward pass; see
    ``backward_bytes_per_probe``).
    """
    x = require_cuda(x, "x")
    probes = require_cuda(probes, "probes")
    if num_matvecs <= 0 or num_matvecs > x.shape[0]:
        from .decomp import _error_num_matvecs

        raise ValueError(_error_num_matvecs(num_matvecs, maxval=x.shape[0], minval=0))
    return _RBFLogdet.apply(theta, x.to(torch.float32).contiguous(), probes, int(num_matvecs), precision,
                            budget_bytes)


def _fun_pair(dense_funm):
    """(f, f') on float64 eigenvalue tensors for an integrand's matrix function.

    log, exp(a x) and x**a have closed-form derivatives; any other elementwise
    torch callable is differentiated with torch autograd.
    """
    kind, a = dense_funm.kind, dense_funm.param
    if kind == _lib.MFG_FUN_LOG:
        return torch.log, lambda x: 1.0 / x
    if kind == _lib.MFG_FUN_EXP:
        return (lambda x: torch.exp(a * x)), (lambda x: a * torch.exp(a * x))
    if kind == _lib.MFG_FUN_POW:
        return (lambda x: x ** a), (lambda x: a * x ** (a - 1.0))
    f = dense_funm.apply_scalar

    def fprime(x):
        with torch.enable_grad():
            xr = x.detach().requires_grad_(True)
            (g,) = torch.autograd.grad(f(xr).sum(), xr)
        return g

    return f, fprime


def params_require_grad(params) -> bool:
    """Whether autograd should see the matvec's parameters."""
    return torch.is_grad_enabled() and any(
        isinstance(t, torch.Tensor) and t.requires_grad for t in tree_leaves(params))


class _CallbackQuadform(torch.autograd.Function):
    """Values ||v_b||^2 e1^T f(T_b) e1 of a callable matvec(v, *params), with
    the gradient in the tensor leaves of params.

    This is the SLQ integrand (matfree/funm.py:226-241) behind the custom VJP
    of the decomposition (decomp.py:420-422, 480-600).  The forward pass keeps
    the Krylov panels; the backward pass forms dH from the eigenvectors of T
    (``quadform_dH``), runs the Hessenberg adjoint on the GPU for Lambda
    (``mfg_hessenberg_adjoint``) and contracts
    sum_{b,j} lambda_bj^T d(A(params) q_bj)/d params with one batched autograd
    VJP of the matvec over all p*k basis vectors (the reference takes the same
    VJP one step at a time, decomp.py:587-589).  dQ = dr = 0 (the integrand
    reads only T), and the probes get no gradient.
    """

    @staticmethod
    def forward(ctx, spec, samples, *leaves):
        fn, n, k, f, fprime, batched, params_tree = spec
        params = _rebuild(params_tree, iter(leaves))
        op = CallbackOperator(fn, n, dtype=samples.dtype, batched=batched, params=params)
        panel, ld = as_panel(samples, n, op.basis_dtype)
        Q, H, R, c = _forward_panels(op, k, panel, ld)
        values, dH = quadform_dH(H, 1.0 / (c * c), f, fprime)
        ctx.save_for_backward(Q, H, R, c, dH)
        ctx.spec = spec
        ctx.op = op
        ctx.leaves = leaves
        return values

    @staticmethod
    def backward(ctx, gvals):
        Q, H, R, c, dH = ctx.saved_tensors
        fn, n, k, _f, _fp, batched, params_tree = ctx.spec
        leaves = ctx.leaves
        want = [i for i in range(len(leaves)) if ctx.needs_input_grad[2 + i]]
        grads = [None] * len(leaves)
        if want:
            Lam, _dv = hessenberg_adjoint(ctx.op, Q, H, R, c, dH * gvals.to(dH.dtype)[:, None, None])
            p = Q.shape[0]
            Qf = Q[:, :, :n].reshape(p * k, n)
            Lf = Lam[:, :, :n].reshape(p * k, n)
            with torch.enable_grad():
                live = [t.detach().requires_grad_(True) if i in want else t for i, t in enumerate(leaves)]
                params = _rebuild(params_tree, iter(live))
                AQ = CallbackOperator(fn, n, dtype=Q.dtype, batched=batched, params=params)._apply_rows(Qf)
                total = (Lf.to(AQ.dtype) * AQ).sum()
                gs = torch.autograd.grad(total, [live[i] for i in want], allow_unused=True)
            for i, g in zip(want, gs):
                grads[i] = torch.zeros_like(leaves[i]) if g is None else g.to(leaves[i].dtype)
        return (None, None, *grads)


def _params_vjp(fn, batched, params_tree, leaves, want, Qf, Lf):
    """sum_j Lf_j^T d(A(params) Qf_j)/d params for the leaves listed in want
    (one autograd VJP of the matvec over all stacked basis vectors)."""
    grads = [None] * len(leaves)
    if not want:
        return grads
    n = Qf.shape[1]
    with torch.enable_grad():
        live = [t.detach().requires_grad_(True) if i in want else t for i, t in enumerate(leaves)]
        params = _rebuild(params_tree, iter(live))
        AQ = CallbackOperator(fn, n, dtype=Qf.dtype, batched=batched, params=params)._apply_rows(Qf)
        total = (Lf.to(AQ.dtype) * AQ).sum()
        gs = torch.autograd.grad(total, [live[i] for i in want], allow_unused=True)
    for i, g in zip(want, gs):
        grads[i] = torch.zeros_like(leaves[i]) if g is None else g.to(leaves[i].dtype)
    return grads


class _ArnoldiFull(torch.autograd.Function):
    """Batched Arnoldi with full reorthogonalisation whose backward pass is the
    Hessenberg adjoint: the custom VJP that matfree puts on the decomposition
    (matfree/decomp.py:393-422).

    Inputs: the starting vectors V (p, n) and the tensor leaves of the matvec's
    parameters.  Outputs: Q (p, k, n), H (p, k, k) float64, residual (p, n)
    and 1/||v|| (p,) float64, as ``run_hessenberg``.  The backward pass takes
    the cotangents of all four (dQ, dH, dr, dc; absent ones are zero), runs
    ``mfg_hessenberg_adjoint_ex`` on the GPU and returns dV = lambda c and the
    parameter gradient sum_{b,j} lambda_bj^T d(A q_bj)/d params.
    """

    @staticmethod
    def forward(ctx, spec, V, *leaves):
        op_fixed, fn, n, k, batched, params_tree = spec
        if op_fixed is not None:
            op = op_fixed
        else:
            params = _rebuild(params_tree, iter(leaves))
            op = CallbackOperator(fn, n, dtype=V.dtype, batched=batched, params=params)
        panel, ld = as_panel(V.detach(), n, op.basis_dtype)
        Q, H, R, c = _forward_panels(op, k, panel, ld)
        ctx.save_for_backward(Q, H, R, c)
        ctx.op, ctx.spec, ctx.leaves = op, spec, leaves
        return Q[:, :, :n], H, R[:, :n], c

    @staticmethod
    def backward(ctx, dQ, dH, dR, dc):
        Q, H, R, c = ctx.saved_tensors
        op_fixed, fn, n, k, batched, params_tree = ctx.spec
        p, _, ld = Q.shape
        leaves = ctx.leaves
        want = [i for i in range(len(leaves)) if ctx.needs_input_grad[2 + i]]
        if not ctx.needs_input_grad[1] and not want:
            return (None, None, *([None] * len(leaves)))
        dQp = None
        if dQ is not None:
            dQp = torch.zeros_like(Q)
            dQp[:, :, :n] = dQ.to(Q.dtype)
        dRp = None
        if dR is not None:
            dRp = torch.zeros_like(R)
            dRp[:, :n] = dR.to(R.dtype)
        dH = torch.zeros_like(H) if dH is None else dH.to(torch.float64).contiguous()
        dc = None if dc is None else dc.to(torch.float64).contiguous()
        Lam, dv = hessenberg_adjoint(ctx.op, Q, H, R, c, dH, dr=dRp, dc=dc, dQ=dQp)
        dV = dv[:, :n] if ctx.needs_input_grad[1] else None
        grads = [None] * len(leaves)
        if want and op_fixed is None:
            grads = _params_vjp(fn, batched, params_tree, leaves, want,
                                Q[:, :, :n].reshape(p * k, n), Lam[:, :, :n].reshape(p * k, n))
        return (None, dV, *grads)


def arnoldi_full(op, k: int, V: torch.Tensor):
    """Differentiable batched Arnoldi (full reorthogonalisation) of the rows of V.

    ``op`` is an operator descriptor (gradients flow to V only) or a
    ``CallbackOperator`` (gradients also flow to the tensor leaves of its
    parameters).  Returns (Q (p, k, n), H (p, k, k), residual (p, n), 1/||v|| (p,)).
    """
    if k <= 0:
        # decomp.py:483-486
        raise ValueError("Custom Hessenberg-adjoints are not implemented for num_matvecs = 0.")
    if isinstance(op, CallbackOperator):
        spec = (None, op.fn, int(op.n), int(k), op.batched, tuple(op.params))
        leaves = tree_leaves(tuple(op.params))
    else:
        spec = (op, None, int(op.n), int(k), False, ())
        leaves = []
    return _ArnoldiFull.apply(spec, V, *leaves)


def wants_grad(V, op) -> bool:
    """Whether the decomposition of V under op must be differentiable."""
    if not torch.is_grad_enabled():
        return False
    if isinstance(V, torch.Tensor) and V.requires_grad:
        return True
    return isinstance(op, CallbackOperator) and params_require_grad(op.params)


class _FunmE1(torch.autograd.Function):
    """f(T) e1 (p, k) for a stack of symmetric tridiagonal T (p, k, k) float64,
    through the device eigensolver (mfg_tridiag_eigh); the backward pass is the
    Daleckii-Krein formula dL/dT = S (F o (S^T dy)(S^T e1)^T) S^T, with F the
    divided differences of f at the eigenvalues (f' on the diagonal) -- what
    autodiff through eigh computes for matfree's dense_funm_sym_eigh
    (matfree/funm.py:322-335)."""

    @staticmethod
    def forward(ctx, T, f, fprime):
        from .funm import tridiag_eigh

        w, S = tridiag_eigh(T.detach().contiguous())
        fw = f(w)
        s1 = S[:, 0, :]
        y = torch.einsum("pij,pj->pi", S, fw * s1)
        ctx.save_for_backward(w, S)
        ctx.fun = (f, fprime)
        return y

    @staticmethod
    def backward(ctx, dy):
        w, S = ctx.saved_tensors
        f, fprime = ctx.fun
        fw = f(w)
        diff = w[:, :, None] - w[:, None, :]
        same = diff.abs() <= 1e-13 * torch.clamp(w.abs()[:, :, None], min=1.0)
        F = (fw[:, :, None] - fw[:, None, :]) / torch.where(same, torch.ones_like(diff), diff)
        F = torch.where(same, fprime(0.5 * (w[:, :, None] + w[:, None, :])), F)
        u = torch.einsum("pji,pj->pi", S, dy.to(torch.float64))
        v = S[:, 0, :]
        G = S @ (F * u[:, :, None] * v[:, None, :]) @ S.transpose(-1, -2)
        return G, None, None


def funm_e1(T: torch.Tensor, dense_funm) -> torch.Tensor:
    """Differentiable f(T) e1 for a stack of symmetric tridiagonal matrices."""
    f, fprime = _fun_pair(dense_funm)
    return _FunmE1.apply(T.to(torch.float64), f, fprime)


class _BasisCombine(torch.autograd.Function):
    """y_b = sum_i coef[b, i] q_{b,i} (the back-projection of funm.py:142-146) on
    the device (mfg_basis_combine); backward: dcoef = Q dy, dQ = coef dy^T."""

    @staticmethod
    def forward(ctx, Q, coef):
        p, k, n = Q.shape
        ld = Q.stride(1) if k > 1 else padded_ld(n)
        base = Q
        if Q.stride(2) != 1 or ld % 8 or ld < n or Q.data_ptr() % 16 or (p > 1 and Q.stride(0) != k * ld):
            base = torch.zeros((p, k, padded_ld(n)), dtype=Q.dtype, device=Q.device)
            base[:, :, :n] = Q
            ld = base.shape[2]
        out = torch.zeros((p, ld), dtype=Q.dtype, device=Q.device)
        cf = coef.to(torch.float64).contiguous()
        dt = _lib.MFG_F64 if Q.dtype == torch.float64 else _lib.MFG_F32
        st = _lib.lib().mfg_basis_combine(dt, k, p, n, ld, ctypes.c_void_p(base.data_ptr()),
                                          ctypes.c_void_p(cf.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                          stream_ptr())
        _lib.check(st, "mfg_basis_combine")
        ctx.save_for_backward(Q, coef)
        return out[:, :n]

    @staticmethod
    def backward(ctx, dy):
        Q, coef = ctx.saved_tensors
        dQ = dcoef = None
        if ctx.needs_input_grad[0]:
            dQ = coef.to(Q.dtype)[:, :, None] * dy.to(Q.dtype)[:, None, :]
        if ctx.needs_input_grad[1]:
            dcoef = torch.einsum("pkn,pn->pk", Q.double(), dy.double()).to(coef.dtype)
        return dQ, dcoef


def basis_combine(Q: torch.Tensor, coef: torch.Tensor) -> torch.Tensor:
    """Differentiable sum_i coef[b, i] Q[b, i, :] on the device."""
    return _BasisCombine.apply(Q, coef)


def callback_quadform(fn, n: int, k: int, samples: torch.Tensor, dense_funm, params=(),
                      batched: bool = False) -> torch.Tensor:
    """Differentiable integrand values (p,) float64 for a callable matvec
    ``fn(v, *params)`` (or ``fn(V, *params)`` on (p, n) panels if ``batched``)."""
    if k <= 0:
        # decomp.py:483-486
        raise ValueError("Custom Hessenberg-adjoints are not implemented for num_matvecs = 0.")
    f, fprime = _fun_pair(dense_funm)
    spec = (fn, int(n), int(k), f, fprime, batched, tuple(params))
    return _CallbackQuadform.apply(spec, samples, *tree_leaves(tuple(params)))


__all__ = ["quadform_dH", "hessenberg_adjoint", "rbf_logdet", "rbf_theta_contractions",
           "run_hessenberg", "callback_quadform", "params_require_grad", "arnoldi_full", "wants_grad",
           "funm_e1", "basis_combine", "backward_bytes_per_probe", "probe_chunks"]
