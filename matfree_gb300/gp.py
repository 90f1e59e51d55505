"""Gaussian-process log-density: SLQ log-determinant plus a CG solve.

Mirrors matfree's tutorial composition (tutorials/8_gaussian_logpdf.py:36-55):

    logpdf(y) = -1/2 (y^T K^{-1} y + log det K + n log(2 pi))

with log det K from the SLQ estimator (``tridiag_sym`` -> ``monte_carlo_funm_
sym_logdet`` -> ``estimator_monte_carlo`` with Rademacher probes) and K^{-1} y
from conjugate gradients (``linalg.cg``).  ``rbf_logpdf`` is the same
quantity for the RBF kernel K(theta) = s2 exp(-|x_i - x_j|^2 / (2 ell^2)) +
tau I, differentiable in theta = (log s2, log ell, log tau):

    d/dtheta (y^T K^{-1} y) = -alpha^T (dK/dtheta) alpha,   alpha = K^{-1} y,

evaluated with the same derivative operators as the log-determinant's
adjoint (``autodiff.rbf_theta_contractions``), and d/dtheta log det K from
the Hessenberg adjoint (``autodiff.rbf_logdet``).
"""

from __future__ import annotations

import math

import torch

from . import decomp, funm, linalg, stochtrace
from ._panel import padded_ld, require_cuda
from .autodiff import rbf_logdet, rbf_theta_contractions
from .operators import RBFKernelOperator


def create_logpdf(matvec, vec_like, *, num_matvecs: int = 6, num_samples: int = 500,
                  cg_tol: float = 1e-5):
    """``create_logpdf`` of tutorials/8_gaussian_logpdf.py:36-55 on the GPU."""
    tridiag = decomp.tridiag_sym(num_matvecs)
    integrand = funm.monte_carlo_funm_sym_logdet(tridiag)
    sampler = stochtrace.sampler_signs(vec_like, num=num_samples)
    estimator = stochtrace.estimator_monte_carlo(integrand, sampler=sampler)

    def logpdf(y, key, *params):
        dim = y.numel()
        logdet = estimator(matvec, key, *params)
        op = matvec if not params else (lambda v: matvec(v, *params))
        y_solve, _ = linalg.cg(op, y, tol=cg_tol)
        quad = torch.dot(y.double().reshape(-1), y_solve.double().reshape(-1))
        return -0.5 * (quad + torch.as_tensor(logdet, dtype=torch.float64, device=quad.device)
                       + dim * math.log(2 * math.pi))

    return logpdf


class _RBFQuad(torch.autograd.Function):
    """y^T K(theta)^{-1} y by CG, with d/dtheta = -alpha^T (dK/dtheta) alpha."""

    @staticmethod
    def forward(ctx, theta, x, y, precision, tol):
        op = RBFKernelOperator.from_theta(x, [float(t) for t in theta.detach().cpu()], precision=precision)
        y = y.to(op.basis_dtype)
        alpha, _ = linalg.cg(op, y, tol=tol)
        ctx.save_for_backward(theta)
        ctx.op, ctx.x, ctx.alpha = op, x, alpha
        return torch.dot(y.double(), alpha.double())

    @staticmethod
    def backward(ctx, grad_out):
        (theta,) = ctx.saved_tensors
        op, alpha = ctx.op, ctx.alpha
        n = op.n
        a = torch.zeros((1, 1, padded_ld(n)), dtype=op.basis_dtype, device=alpha.device)
        a[0, 0, :n] = alpha
        g = -rbf_theta_contractions(op, ctx.x, a, a)
        grad = (grad_out.double() * g).to(device=theta.device, dtype=theta.dtype)
        return grad, None, None, None, None


def rbf_logpdf(x: torch.Tensor, theta: torch.Tensor, y: torch.Tensor, probes: torch.Tensor,
               num_matvecs: int, precision: str = "bf16x3", cg_tol: float = 1e-6) -> torch.Tensor:
    """GP log-density of y under the RBF kernel K(theta), differentiable in theta.

    x (n, dim) CUDA points, theta = (log s2, log ell, log tau), y (n,) CUDA
    observations, probes (p, n) CUDA Rademacher probes of the log-determinant.
    Returns a 0-d float64 tensor.
    """
    x = require_cuda(x, "x")
    y = require_cuda(y, "y")
    n = x.shape[0]
    quad = _RBFQuad.apply(theta, x.to(torch.float32).contiguous(), y.reshape(-1), precision, cg_tol)
    logdet = rbf_logdet(x, theta, probes, num_matvecs, precision=precision)
    return -0.5 * (quad.to(torch.float64).to(logdet.device) + logdet.to(torch.float64)
                   + n * math.log(2 * math.pi))
