"""Oracle for the Gaussian log-density row (test infrastructure only).

CPU float64 restatement of matfree's GP log-density tutorial
(tutorials/8_gaussian_logpdf.py:36-55):

    logpdf(y) = -1/2 (y^T K^{-1} y + logdet_SLQ(K) + n log(2 pi))

The linear solve there is ``jax.scipy.sparse.linalg.cg`` (a jax dependency:
jax/jaxlib have no pinned version in the reference's pyproject.toml and are
not vendored).  ``cg`` below restates its published algorithm (Hestenes-
Stiefel conjugate gradients, x0 = 0, no preconditioner, stop once
r^T r <= max(tol^2 b^T b, atol^2), at most 10 n iterations by default).
Pinned against ``numpy.linalg.solve`` and ``scipy.stats.multivariate_normal``
in tests/test_oracle_gp.py.
"""

from __future__ import annotations

import numpy as np

from . import adjoint, slq


def cg(matvec, b, *, tol=1e-5, atol=0.0, maxiter=None):
    """Return (x, iterations)."""
    b = np.asarray(b, dtype=np.float64)
    n = b.shape[0]
    maxiter = 10 * n if maxiter is None else maxiter
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rs = r @ r
    thr = max(tol * tol * (b @ b), atol * atol)
    k = 0
    while rs > thr and k < maxiter:
        Ap = matvec(p)
        alpha = rs / (p @ Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        rs_new = r @ r
        p = r + (rs_new / rs) * p
        rs = rs_new
        k += 1
    return x, k


def logpdf_dense(K, y):
    """Exact zero-mean Gaussian log-density by Cholesky."""
    L = np.linalg.cholesky(K)
    z = np.linalg.solve(L, y)
    n = len(y)
    return -0.5 * (z @ z + 2.0 * np.sum(np.log(np.diag(L))) + n * np.log(2 * np.pi))


def rbf_logpdf_slq(x, theta, y, probes, num_matvecs):
    """Value and theta-gradient of the SLQ log-density on fixed probes.

    The quadratic term and its gradient -alpha^T (dK/dtheta) alpha use an
    exact solve; the log-determinant and its gradient the SLQ estimate and the
    Hessenberg adjoint (``adjoint.slq_grad_batched``).
    """
    K, E, D = adjoint.rbf_matrices(x, theta)
    s2, ell, tau = np.exp(theta)
    alpha = np.linalg.solve(K, y)
    quad = y @ alpha
    dK = [s2 * E, s2 * E * D / (ell * ell), tau * np.eye(len(y))]
    dquad = np.array([-(alpha @ (Ki @ alpha)) for Ki in dK])
    matmat, vjp = adjoint.rbf_vjp_factory(x, theta)
    logdet, dlogdet = adjoint.slq_grad_batched(matmat, vjp, 3, num_matvecs, probes)
    n = len(y)
    value = -0.5 * (quad + logdet + n * np.log(2 * np.pi))
    return value, -0.5 * (dquad + dlogdet)


def slq_logdet(K, probes, num_matvecs):
    """SLQ estimate of log det K on fixed probes (mean of the quadratic forms)."""
    return slq.slq_batched(lambda V: V @ K.T, num_matvecs, probes).mean()
