"""Oracle for Golub-Kahan bidiagonalisation and the product SLQ integrand.

Test infrastructure only: a CPU float64 restatement of
matfree/decomp.py:641-750 (``bidiag`` with full reorthogonalisation: each new
left / right vector is projected out of all vectors of its side twice) and of
the product integrand matfree/funm.py:246-320 (``||v||^2 e1^T f(B^T B) e1``
through the SVD of B).  Pinned by matfree's known-answer tests for these
functions (tests/test_decomp/test_bidiag.py,
tests/test_funm/test_monte_carlo_funm_product_logdet.py) in
tests/test_oracle_bidiag.py.
"""

from __future__ import annotations

import numpy as np


def bidiag(Av, vA, num_matvecs, v0, nrows):
    """Return (U (k, nrows), B (k, k), V (k, ncols), residual (ncols,), 1/||v0||)."""
    v0 = np.asarray(v0, dtype=np.float64)
    ncols = v0.shape[0]
    k = num_matvecs
    if k < 0 or k > min(nrows, ncols):
        raise ValueError("num_matvecs out of range")
    length = np.linalg.norm(v0)
    vk = v0 / length
    vk = vk / np.linalg.norm(vk)  # init() normalises again (decomp.py:697-698)
    Us = np.zeros((k, nrows))
    Vs = np.zeros((k, ncols))
    alphas = np.zeros(k)
    betas = np.zeros(k)
    beta = 0.0
    for i in range(k):
        Vs[i] = vk
        betas[i] = beta
        uk = Av(vk) - beta * (Us[i - 1] if i > 0 else 0.0)
        uk = uk - Us.T @ (Us @ uk)
        uk = uk - Us.T @ (Us @ uk)
        alpha = np.linalg.norm(uk)
        uk = uk / alpha
        Us[i] = uk
        alphas[i] = alpha
        vk = vA(uk) - alpha * vk
        vk = vk - Vs.T @ (Vs @ vk)
        vk = vk - Vs.T @ (Vs @ vk)
        beta = np.linalg.norm(vk)
        vk = vk / beta
    B = np.diag(alphas) + np.diag(betas[1:], 1)
    return Us, B, Vs, beta * vk, 1.0 / length


def product_quadform(A, v0, num_matvecs, matfun=np.log):
    """||v||^2 e1^T f(B^T B) e1 (matfree/funm.py:276-320) for a dense matrix A."""
    _, B, _, _, _ = bidiag(lambda v: A @ v, lambda u: A.T @ u, num_matvecs, v0, A.shape[0])
    _, S, Vt = np.linalg.svd(B)
    w = Vt.T[0, :]
    return (np.linalg.norm(v0) ** 2) * np.sum(matfun(S * S) * w * w)
