"""Float64 restatement of matfree's Hessenberg adjoint (oracle; test infrastructure).

``hessenberg_adjoint`` follows matfree/decomp.py:480-544 (set-up of gamma,
lambda_k, Pi_xi, Pi_gamma, the masks and the reverse scan) and
matfree/decomp.py:547-600 (one reverse step: masked re-projection of lambda,
one vector-Jacobian product of the matvec, Gamma and Lambda updates).  The
batched variant runs the same recurrences for p probes at once.

``slq_grad_batched`` chains the SLQ integrand (funm.py:226-241), the eigh-based
matrix function (funm.py:330-333; derivative by the Daleckii-Krein formula),
the symmetrisation T = (H + H^T)/2 (decomp.py:133-135) and the adjoint, giving
d/dtheta of mean_b ||v_b||^2 e1^T f(T_b) e1 for a parametrised operator.
"""

from __future__ import annotations

import numpy as np

from oracle import problems, slq


def _lower(m):
    m_tril = np.tril(m)
    return m_tril - 0.5 * np.diag(np.diag(m_tril))


def hessenberg_adjoint(vjp_matvec, params, *, Q, H, r, c, dQ, dH, dr, dc, reortho="full"):
    """Reverse pass of the Arnoldi iteration for one vector.

    vjp_matvec(q, lam) must return (A^T lam, tuple of d(lam^T A(params) q)/dparams).
    Q, dQ are (n, k) as in matfree's internal layout; H, dH are (k, k).
    Returns (dv, dparams).
    """
    n, k = Q.shape
    if k == 0:
        raise ValueError("Custom Hessenberg-adjoints are not implemented for num_matvecs = 0.")
    eye = np.eye(k)
    e_K = eye[-1]
    e_1 = eye[0]
    lower_mask = _lower(np.ones((k, k)))

    gamma = dH @ e_K - Q.T @ dr
    lambda_k = dr + Q @ gamma
    Lambda = np.zeros_like(Q)
    Gamma = np.zeros((k, k))
    dp = [np.zeros_like(np.asarray(p, dtype=np.float64)) for p in params]

    Pi_xi = dQ.T + np.outer(gamma, r)
    Pi_gamma = -dc * c * np.outer(e_1, e_1) + H @ dH.T - (dQ.T @ Q)
    reortho_mask = np.tril(np.ones((k, k)), 1)

    beta_minuses = np.concatenate([np.ones((1,)), np.diagonal(H, -1)])
    alphas = np.diagonal(H)
    beta_pluses = H - np.diag(np.diagonal(H)) - np.diag(np.diagonal(H, -1), -1)

    for idx in reversed(range(k)):
        if reortho == "full":
            mask = reortho_mask[idx]
            Qm = mask[None, :] * Q
            rhs = mask * dH[:, idx]
            lambda_k = lambda_k - Qm @ (Qm.T @ lambda_k) + Qm @ rhs
        vecmat_lambda, dp_inc = vjp_matvec(Q[:, idx], lambda_k)
        dp = [a + b for a, b in zip(dp, dp_inc)]
        Gamma[idx, :] = lower_mask[idx] * (Pi_gamma[idx] - vecmat_lambda @ Q)
        Lambda[:, idx] = lambda_k
        xi = Pi_xi[idx] + (Gamma + Gamma.T)[idx, :] @ Q.T
        lambda_k = xi - (alphas[idx] * lambda_k - vecmat_lambda) - beta_pluses[idx] @ Lambda.T
        lambda_k = lambda_k / beta_minuses[idx]
    return lambda_k * c, dp


def hessenberg_adjoint_batched(vjp_matmat, nparams, *, Q, H, r, dH, c):
    """The same reverse pass for p probes with dQ = 0, dr = 0, dc = 0.

    This is the case the SLQ integrand produces (it only reads T).  Q is
    (p, k, n) (probe-major basis), r is (p, n), H and dH are (p, k, k).  vjp_matmat(q_panel,
    lam_panel) returns (A^T lam (p, n), array (nparams,) of summed parameter
    cotangents).  Returns (dv (p, n), dparams (nparams,)).
    """
    p, k, n = Q.shape
    lower_mask = _lower(np.ones((k, k)))
    reortho_mask = np.tril(np.ones((k, k)), 1)
    gamma = dH[:, :, k - 1]  # dH @ e_K with dr = 0
    lam = slq.combine(Q, gamma)
    Lam = np.zeros((p, k, n))
    Gamma = np.zeros((p, k, k))
    dp = np.zeros(nparams)
    Pi_gamma = np.einsum("pij,pkj->pik", H, dH)  # H dH^T (dc = 0, dQ = 0)
    beta_minus = np.concatenate([np.ones((p, 1)), np.diagonal(H, -1, -2, -1)], axis=1)
    alphas = np.diagonal(H, 0, -2, -1)
    beta_plus = H.copy()
    idx_all = np.arange(k)
    beta_plus[:, idx_all, idx_all] = 0.0
    beta_plus[:, idx_all[1:], idx_all[:-1]] = 0.0
    for idx in reversed(range(k)):
        # the mask row tril(1, 1)[idx] keeps columns 0..idx+1 (decomp.py:558-566)
        m = int(reortho_mask[idx].sum())
        Qm = Q[:, :m, :]
        rhs = dH[:, :m, idx]
        proj = slq.project(Qm, lam)
        lam = lam - slq.combine(Qm, proj) + slq.combine(Qm, rhs)
        At_lam, dp_inc = vjp_matmat(Q[:, idx, :], lam)
        dp = dp + dp_inc
        Gamma[:, idx, :] = lower_mask[idx][None, :] * (Pi_gamma[:, idx, :] - slq.project(Q, At_lam))
        Lam[:, idx, :] = lam
        G = Gamma[:, idx, :] + Gamma[:, :, idx]
        # Pi_xi[idx] = dQ^T[idx] + gamma[idx] r = gamma[idx] r
        xi = gamma[:, idx, None] * r + slq.combine(Q, G)
        lam = xi - (alphas[:, idx, None] * lam - At_lam) - slq.combine(Lam, beta_plus[:, idx, :])
        lam = lam / beta_minus[:, idx, None]
    return lam * c[:, None], dp


def _loewner_first_row(w, S, f, fprime):
    """d(e1^T f(T) e1)/dT for symmetric T = S diag(w) S^T (Daleckii-Krein)."""
    diff = w[:, None] - w[None, :]
    fw = f(w)
    same = np.abs(diff) <= 1e-14 * np.maximum(1.0, np.abs(w[:, None]))
    with np.errstate(divide="ignore", invalid="ignore"):
        F = np.where(same, 0.0, (fw[:, None] - fw[None, :]) / np.where(same, 1.0, diff))
    avg = 0.5 * (w[:, None] + w[None, :])
    F = np.where(same, fprime(avg), F)
    s1 = S[0, :]
    return S @ (F * np.outer(s1, s1)) @ S.T


def dT_to_dH(G):
    """Pull a symmetric cotangent of the dense tridiagonal back to H.

    T_dense = diag(d) + diag(e, 1) + diag(e, -1) with d = diag(H) and
    e_i = (H[i, i+1] + H[i+1, i]) / 2 (decomp.py:133-135, 148-152).
    """
    k = G.shape[-1]
    dH = np.zeros_like(G)
    i = np.arange(k)
    dH[..., i, i] = G[..., i, i]
    if k > 1:
        de = G[..., i[:-1], i[1:]] + G[..., i[1:], i[:-1]]
        dH[..., i[:-1], i[1:]] = 0.5 * de
        dH[..., i[1:], i[:-1]] = 0.5 * de
    return dH


def slq_grad_batched(matmat, vjp_matmat, nparams, num_matvecs, V, f=np.log, fprime=None):
    """Value and theta-gradient of mean_b ||v_b||^2 e1^T f(T_b) e1 (fixed probes V)."""
    if fprime is None:
        fprime = lambda x: 1.0 / x  # noqa: E731  (derivative of log)
    V = np.asarray(V, dtype=np.float64)
    p = V.shape[0]
    length = np.linalg.norm(V, axis=1)
    Vn = V / length[:, None]
    Q, H, r, c = slq.hessenberg_forward_batched(matmat, num_matvecs, Vn)
    d, e = slq.tridiag_from_hessenberg(H)
    k = num_matvecs
    vals = np.zeros(p)
    G = np.zeros((p, k, k))
    idx = np.arange(k)
    for b in range(p):
        T = np.zeros((k, k))
        T[idx, idx] = d[b]
        if k > 1:
            T[idx[:-1], idx[1:]] = e[b]
            T[idx[1:], idx[:-1]] = e[b]
        w, S = np.linalg.eigh(T)
        vals[b] = length[b] ** 2 * np.sum(f(w) * S[0, :] ** 2)
        G[b] = length[b] ** 2 * _loewner_first_row(w, S, f, fprime) / p
    dH = dT_to_dH(G)
    _dv, dtheta = hessenberg_adjoint_batched(vjp_matmat, nparams, Q=Q, H=H, r=r, dH=dH, c=c)
    return vals.mean(), dtheta


# ---------------------------------------------------------------------------
# The RBF kernel operator K(theta) = s2 exp(-D / (2 l^2)) + tau I, theta = logs
# ---------------------------------------------------------------------------


def rbf_matrices(x, theta):
    """Return (K, E, D) in float64 for points x (n, d) and theta=(log s2, log l, log tau)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    s2, ell, tau = np.exp(theta)
    D = np.empty((n, n))
    E = np.empty((n, n))
    K = np.empty((n, n))

    def fill(lo, hi):
        D[lo:hi] = problems.sqdist_rows(x, lo, hi)
        E[lo:hi] = np.exp(-D[lo:hi] / (2.0 * ell * ell))
        K[lo:hi] = s2 * E[lo:hi]

    problems.row_blocks(n, fill)
    K[np.diag_indices(n)] += tau
    return K, E, D


def rbf_vjp_factory(x, theta):
    """matmat and vjp_matmat for the RBF operator (dense float64)."""
    K, E, D = rbf_matrices(x, theta)
    s2, ell, tau = np.exp(theta)
    dK0 = s2 * E  # dK/dlog s2
    dK1 = s2 * E * D / (ell * ell)  # dK/dlog l
    del E, D

    def matmat(Vp):
        return Vp @ K.T

    def vjp_matmat(Qp, Lp):
        At = Lp @ K  # A^T lam for each probe
        g0 = np.einsum("pn,pn->", Lp, Qp @ dK0.T)
        g1 = np.einsum("pn,pn->", Lp, Qp @ dK1.T)
        g2 = tau * np.einsum("pn,pn->", Lp, Qp)
        return At, np.array([g0, g1, g2])

    return matmat, vjp_matmat
