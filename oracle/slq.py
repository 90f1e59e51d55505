"""Float64 NumPy restatement of matfree's SLQ path (oracle; test infrastructure).

Every function cites the matfree file and lines it follows.  Single-vector
functions mirror the reference step by step (including its quirks); the
``*_batched`` functions run the same arithmetic over a (p, n) probe panel and
are used for larger parity cases and for the timed CPU baseline.
"""

from __future__ import annotations

import numpy as np


def error_num_matvecs(num, maxval, minval):
    """Message of matfree/decomp.py:753-756."""
    msg1 = f"Parameter 'num_matvecs'={num} exceeds the acceptable range. "
    msg2 = f"Expected: {minval} <= num_matvecs <= {maxval}."
    return msg1 + msg2


# ---------------------------------------------------------------------------
# Arnoldi / Hessenberg forward pass
# ---------------------------------------------------------------------------


def hessenberg_forward(matvec, num_matvecs, v, *, reortho="full"):
    """Arnoldi with classical Gram-Schmidt, applied twice when reortho='full'.

    Follows matfree/decomp.py:426-451 (initialisation, k=0 case, loop) and
    matfree/decomp.py:454-477 (one step: normalise, store, matvec, project
    against *all* k columns, re-project, norm, ``h[idx+1] = length`` which is
    dropped at the last step because the index is out of range).

    Returns (Q (n, k), H (k, k), residual (n,), 1/||v||).
    """
    if reortho not in ("none", "full"):
        raise TypeError(f"Unexpected input for {reortho}: either of ['none', 'full'] expected.")
    v = np.asarray(v)
    v = v.astype(np.result_type(v.dtype, np.float64))  # complex input: complex-step checks
    (n,) = v.shape
    k = num_matvecs
    if k < 0 or k > n:
        raise ValueError(error_num_matvecs(k, maxval=n, minval=0))
    Q = np.zeros((n, k), dtype=v.dtype)
    H = np.zeros((k, k), dtype=v.dtype)
    initlength = np.sqrt(v @ v)
    length = initlength
    for idx in range(k):
        v = v / length
        Q[:, idx] = v
        v = matvec(v)
        h = Q.T @ v
        v = v - Q @ h
        if reortho != "none":
            v = v - Q @ (Q.T @ v)
        length = np.sqrt(v @ v)
        if idx + 1 < k:  # JAX drops out-of-bounds .at[].set
            h[idx + 1] = length
        H[:, idx] = h
    return Q, H, v, 1.0 / initlength


def tridiag_sym_full(matvec, num_matvecs, v, *, materialize=True):
    """matfree/decomp.py:125-145: Arnoldi, then T = (H + H^T)/2 and its diagonals.

    Returns (Q_tall (k, n), T (k, k) or (diag, offdiag), residual, 1/||v||).
    """
    Q, H, r, c = hessenberg_forward(matvec, num_matvecs, v, reortho="full")
    T = 0.5 * (H + H.T)
    diags = np.diagonal(T, 0).copy()
    offdiags = np.diagonal(T, 1).copy()
    J = todense_tridiag_sym(diags, offdiags) if materialize else (diags, offdiags)
    return Q.T.copy(), J, r, c


def tridiag_sym_none(matvec, num_matvecs, vec, *, materialize=True):
    """matfree/decomp.py:155-212 and 215-291: three-term Lanczos, no reorthogonalisation.

    v0 = vec/||vec||; a = v.Av; r = Av - a v - b v_prev; b = ||r||; x = r/b.
    Returns (Q_tall (k, n), T or (diag, offdiag), residual = b x, 1/||vec||).
    """
    vec = np.asarray(vec, dtype=np.float64)
    n = vec.shape[0]
    k = num_matvecs
    if k < 0 or k > n:
        raise ValueError(error_num_matvecs(k, maxval=n, minval=0))
    vectors = np.zeros((k + 1, n))
    diags = np.zeros(k)
    offdiags = np.zeros(k)
    v0 = vec / np.linalg.norm(vec)
    vectors[0] = v0
    Av = matvec(v0)
    a = v0 @ Av
    r = Av - a * v0
    b = np.linalg.norm(r)
    x = r / b
    if k == 0:
        Q, d, e = vectors[:-1], diags, offdiags[:-1]
    else:
        vectors[1], offdiags[0], diags[0] = x, b, a
        v1, v_prev = x, v0
        for i in range(1, k):
            Av = matvec(v1)
            a = v1 @ Av
            r = Av - a * v1 - b * v_prev
            b = np.linalg.norm(r)
            x = r / b
            vectors[i + 1], offdiags[i], diags[i] = x, b, a
            v1, v_prev = x, v1
        Q, d, e = vectors[:-1], diags, offdiags[:-1]
    J = todense_tridiag_sym(d, e) if materialize else (d, e)
    return Q, J, b * x, 1.0 / np.linalg.norm(vec)


def todense_tridiag_sym(diag, off_diag):
    """matfree/decomp.py:148-152."""
    return np.diag(diag) + np.diag(off_diag, -1) + np.diag(off_diag, 1)


# ---------------------------------------------------------------------------
# Matrix functions and the SLQ integrand
# ---------------------------------------------------------------------------


def dense_funm_sym_eigh(matfun):
    """matfree/funm.py:322-335: f(T) = V diag(f(lambda)) V^T via eigh."""

    def fun(dense_matrix):
        w, V = np.linalg.eigh(dense_matrix)
        return V @ np.diag(matfun(w)) @ V.T

    return fun


def monte_carlo_funm_sym(dense_funm, num_matvecs):
    """matfree/funm.py:226-241: ||v||^2 e1^T f(T) e1 after normalising v."""

    def quadform(matvec, v0):
        v0 = np.asarray(v0, dtype=np.float64)
        length = np.linalg.norm(v0)
        v0 = v0 / length
        _, dense, *_ = tridiag_sym_full(matvec, num_matvecs, v0, materialize=True)
        fA = dense_funm(dense)
        return length**2 * fA[0, 0]

    return quadform


def monte_carlo_funm_sym_logdet(num_matvecs):
    """matfree/funm.py:186-202 (f = log)."""
    return monte_carlo_funm_sym(dense_funm_sym_eigh(np.log), num_matvecs)


def funm_lanczos_sym(dense_funm, num_matvecs):
    """matfree/funm.py:114-147: f(A) v = ||v|| Q^T f(T) e1 (Q_tall (k, n))."""

    def estimate(matvec, vec):
        vec = np.asarray(vec, dtype=np.float64)
        length = np.linalg.norm(vec)
        Q, dense, *_ = tridiag_sym_full(matvec, num_matvecs, vec / length, materialize=True)
        fA = dense_funm(dense)
        e1 = np.eye(len(dense))[0, :]
        return length * (Q.T @ (fA @ e1))

    return estimate


def estimator_monte_carlo(integrand, matvec, samples):
    """matfree/stochtrace.py:47-50: mean of the integrand over the samples."""
    vals = np.array([integrand(matvec, s) for s in samples])
    return vals.mean(axis=0)


def estimator_monte_carlo_mean_and_sem(integrand, matvec, samples):
    """matfree/stochtrace.py:82-87: (mean, std / sqrt(num))."""
    vals = np.array([integrand(matvec, s) for s in samples])
    return vals.mean(axis=0), vals.std(axis=0) / np.sqrt(vals.shape[0])


# ---------------------------------------------------------------------------
# Batched (probe-panel) restatement, same arithmetic as above per probe
# ---------------------------------------------------------------------------


def project(Qa, w):
    """Q_b^T w_b for every probe b: (p, j, n), (p, n) -> (p, j) (batched BLAS GEMV)."""
    return np.matmul(Qa, w[:, :, None])[:, :, 0]


def combine(Qa, h):
    """Q_b h_b for every probe b: (p, j, n), (p, j) -> (p, n) (batched BLAS GEMV)."""
    return np.matmul(h[:, None, :], Qa)[:, 0, :]


def hessenberg_forward_batched(matmat, num_matvecs, V, *, reortho="full"):
    """matfree/decomp.py:426-477 applied to every row of V (p, n) at once.

    ``matmat`` maps a (p, n) panel to (p, n) (the operator applied to each
    row).  The projection uses only the columns written so far: the columns
    matfree still holds at zero contribute exact zeros.

    Returns Q (p, k, n), H (p, k, k), residual (p, n), 1/||v|| (p,).
    """
    V = np.asarray(V, dtype=np.float64)
    p, n = V.shape
    k = num_matvecs
    if k < 0 or k > n:
        raise ValueError(error_num_matvecs(k, maxval=n, minval=0))
    Q = np.zeros((p, k, n))
    H = np.zeros((p, k, k))
    initlength = np.sqrt(np.einsum("pn,pn->p", V, V))
    length = initlength
    w = V
    for idx in range(k):
        v = w / length[:, None]
        Q[:, idx, :] = v
        w = matmat(v)
        Qa = Q[:, : idx + 1, :]
        h = project(Qa, w)
        w = w - combine(Qa, h)
        if reortho != "none":
            h2 = project(Qa, w)
            w = w - combine(Qa, h2)
        length = np.sqrt(np.einsum("pn,pn->p", w, w))
        H[:, : idx + 1, idx] = h
        if idx + 1 < k:
            H[:, idx + 1, idx] = length
    return Q, H, w, 1.0 / initlength


def tridiag_from_hessenberg(H):
    """decomp.py:133-135 for a stack (p, k, k): diag(T) and diag(T, 1) of T=(H+H^T)/2."""
    T = 0.5 * (H + np.swapaxes(H, -1, -2))
    return np.diagonal(T, 0, -2, -1).copy(), np.diagonal(T, 1, -2, -1).copy()


def quadrature_batched(diags, offdiags, matfun):
    """e1^T f(T) e1 for each tridiagonal in a stack (funm.py:239-241, 330-333)."""
    p, k = diags.shape
    T = np.zeros((p, k, k))
    idx = np.arange(k)
    T[:, idx, idx] = diags
    if k > 1:
        T[:, idx[:-1], idx[1:]] = offdiags
        T[:, idx[1:], idx[:-1]] = offdiags
    w, S = np.linalg.eigh(T)
    return np.einsum("pi,pi->p", matfun(w), S[:, 0, :] ** 2)


def slq_batched(matmat, num_matvecs, V, matfun=np.log):
    """Per-probe SLQ quadratic forms ||v||^2 e1^T f(T) e1 for a (p, n) panel.

    Same arithmetic as ``monte_carlo_funm_sym(...)`` applied to each row.
    """
    V = np.asarray(V, dtype=np.float64)
    length = np.linalg.norm(V, axis=1)
    V = V / length[:, None]
    _, H, _, _ = hessenberg_forward_batched(matmat, num_matvecs, V)
    d, e = tridiag_from_hessenberg(H)
    return length**2 * quadrature_batched(d, e, matfun)
