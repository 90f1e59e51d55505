"""The GP log-density oracle against exact references (CPU)."""

import numpy as np
import pytest
from scipy import stats

from oracle import adjoint, gp


def _rbf_problem(n=80, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(size=(n, 2))
    theta = np.array([0.0, np.log(0.3), np.log(0.1)])
    K, _, _ = adjoint.rbf_matrices(x, theta)
    y = rng.standard_normal(n)
    return x, theta, K, y


def test_cg_matches_dense_solve():
    _, _, K, y = _rbf_problem()
    x, its = gp.cg(lambda v: K @ v, y, tol=1e-12)
    np.testing.assert_allclose(x, np.linalg.solve(K, y), rtol=1e-8, atol=1e-8)
    assert 0 < its <= 10 * len(y)


def test_cg_stops_at_the_tolerance_and_maxiter():
    _, _, K, y = _rbf_problem()
    x, its = gp.cg(lambda v: K @ v, y, tol=1e-3)
    r = y - K @ x
    assert r @ r <= 1e-6 * (y @ y)
    _, its2 = gp.cg(lambda v: K @ v, y, tol=1e-12, maxiter=3)
    assert its2 == 3
    x0, its0 = gp.cg(lambda v: K @ v, np.zeros(5))
    assert its0 == 0 and not x0.any()


def test_dense_logpdf_matches_scipy():
    _, _, K, y = _rbf_problem()
    want = stats.multivariate_normal(mean=np.zeros(len(y)), cov=K).logpdf(y)
    assert abs(gp.logpdf_dense(K, y) - want) < 1e-9 * abs(want)


def test_slq_logpdf_exact_for_full_depth_and_gradient_vs_differences():
    x, theta, K, y = _rbf_problem(n=24)
    n = len(y)
    probes = np.eye(n)  # e_i probes: sum_i e_i^T log(K) e_i = tr log K at full depth
    val, grad = gp.rbf_logpdf_slq(x, theta, y, probes, n - 1)
    # mean over n unit probes times n = log det
    exact = gp.logpdf_dense(K, y)
    logdet_slq = gp.slq_logdet(K, probes, n - 1) * n
    value_from_mean = -0.5 * (y @ np.linalg.solve(K, y) + logdet_slq + n * np.log(2 * np.pi))
    assert abs(value_from_mean - exact) < 1e-8 * abs(exact)
    # central differences of the same (fixed-probe) estimate
    h = 1e-5
    for i in range(3):
        e = np.zeros(3)
        e[i] = h
        fp, _ = gp.rbf_logpdf_slq(x, theta + e, y, probes, 6)
        fm, _ = gp.rbf_logpdf_slq(x, theta - e, y, probes, 6)
        _, g6 = gp.rbf_logpdf_slq(x, theta, y, probes, 6)
        assert abs((fp - fm) / (2 * h) - g6[i]) <= 1e-5 * max(1.0, abs(g6[i]))
