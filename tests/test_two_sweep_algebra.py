"""The two-sweep Arnoldi step, restated in float64 NumPy, against the oracle's
CGS2 step (matfree/decomp.py:454-477).  No GPU.

The device step (``mfg_hessenberg`` reortho 3, ``mfg_slq_ex`` with
MFG_SLQ_TWO_SWEEP) applies the operator to qt_j = u_j / nu_j, where u_j is
the previous step's first-projected vector, performs the delayed second
projection together with step j's first projection, and recovers A q_j from
the Arnoldi relation A Q_{j-1} = Q_j Hh (Hh: h + h2 and beta).  This module
restates that recurrence (the same quantities the two streamed passes, the
coefficient kernel and the finish kernel form) and checks that H, Q and the
residual equal the reference's, and that the device's retry criterion
(||Q^T qt||^2 > 0.01 ||qt||^2) fires where the recovered product loses
accuracy (a vector left inside the basis by one projection).
"""

import numpy as np
import pytest

from oracle import problems, slq


def two_sweep(A, v, k):
    """Returns (Q (n, k), H (k, k), residual, retry flag)."""
    n = len(v)
    Q = np.zeros((k, n))
    H = np.zeros((k, k))
    Hh = np.zeros((k + 1, k))  # full coefficients: h + h2 above, beta below
    Q[0] = v / np.linalg.norm(v)
    w = A @ Q[0]
    H[0, 0] = Q[0] @ w
    u = w - Q[0] * H[0, 0]
    nu = np.linalg.norm(u)
    qt = u / nu
    retry = False
    for j in range(1, k + 1):
        Qp = Q[:j]
        hq = Qp @ qt  # delayed second projection of u_j = nu qt
        b = qt - Qp.T @ hq  # = w''_{j-1} / nu
        nb = b @ b
        if j < k:  # the step that recovers A q_j checks; the final residual does not
            retry |= hq @ hq > 0.01 * (hq @ hq + nb)
        rho = np.sqrt(nb)
        beta = nu * rho
        Hh[:j, j - 1] = H[:j, j - 1] + nu * hq
        Hh[j, j - 1] = beta
        if j == k:
            return Q.T, H, nu * b, retry
        H[j, j - 1] = beta
        wt = A @ qt  # the operator on the not yet reorthogonalised vector
        g = Qp @ wt
        c = qt @ wt
        z = wt - Qp.T @ g
        qw = (c - hq @ g) / rho  # q_j . A qt
        m = Hh[: j + 1, :j] @ hq
        H[: j + 1, j] = nu * (np.concatenate([g, [qw]]) - m) / beta
        Q[j] = b / rho
        y = z - Q[j] * qw  # (I - Q_j Q_j^T) A qt
        s = np.linalg.norm(y)
        qt = y / s
        nu = s / rho
    raise AssertionError("unreachable")


def _cases():
    rng = np.random.default_rng(0)
    yield "spd", problems.dense_spd(300, seed=1), rng.standard_normal(300), 40
    n = 12
    hilbert = 1.0 / (np.arange(1, n + 1)[:, None] + np.arange(n)[None, :])
    yield "hilbert", hilbert, np.flip(np.arange(1.0, 1.0 + n)).copy(), n
    yield "full rank", problems.dense_spd(30, seed=2), rng.standard_normal(30), 30
    eig = np.arange(1.0, 2.0, 1.0 / 20)
    yield "graded", problems.hermitian_matrix_from_eigenvalues(eig, rng), rng.standard_normal(20), 15


@pytest.mark.parametrize("name,A,v,k", list(_cases()), ids=lambda c: c if isinstance(c, str) else "")
def test_two_sweep_equals_cgs2(name, A, v, k):
    Qo, Ho, ro, _ = slq.hessenberg_forward(lambda x: A @ x, k, v)
    Q, H, r, retry = two_sweep(A, v, k)
    scale = np.abs(Ho).max()
    np.testing.assert_allclose(H, Ho, atol=1e-12 * scale)
    assert not retry
    if name != "hilbert":  # after a Krylov breakdown the later columns are noise in both
        np.testing.assert_allclose(Q, Qo, atol=1e-10)
        np.testing.assert_allclose(r, ro, atol=1e-10 * max(np.abs(ro).max(), 1.0))


def test_retry_criterion_fires_near_an_invariant_subspace():
    # rank 10 plus 1e-8 I: the Krylov space is exhausted after ~10 steps
    rng = np.random.default_rng(0)
    U = rng.standard_normal((200, 10))
    A = U @ U.T + 1e-8 * np.eye(200)
    v = rng.standard_normal(200)
    _, H, _, retry = two_sweep(A, v, 30)
    assert retry
    # up to the exhaustion the recurrence still matches the reference
    _, Ho, _, _ = slq.hessenberg_forward(lambda x: A @ x, 10, v)
    _, H10, _, retry10 = two_sweep(A, v, 10)
    assert not retry10
    np.testing.assert_allclose(H10, Ho, atol=1e-9 * np.abs(Ho).max())
