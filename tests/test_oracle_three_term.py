"""The oracle's three-term Lanczos (reortho="none") against matfree's known answers.

Ports tests/test_decomp/test_tridiag_sym.py:7-65 and test_consistency.py for
reortho="none", with matfree's tolerances for that setting.
"""

import numpy as np
import pytest

from oracle import problems, slq


def _matrix(n=12):
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    return problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))


def test_full_rank_reconstruction_without_reortho():
    n = 12
    A = _matrix(n)
    v = np.flip(np.arange(1.0, 1.0 + n))
    Q, T, _, _ = slq.tridiag_sym_none(lambda x: A @ x, n, v)
    assert np.allclose(Q.T @ T @ Q, A, atol=1e-1, rtol=1e-1)


@pytest.mark.parametrize("k", [1, 5, 11])
def test_mid_rank_relation_without_reortho(k):
    n = 12
    A = _matrix(n)
    v = np.flip(np.arange(1.0, 1.0 + n))
    Q, T, q, _ = slq.tridiag_sym_none(lambda x: A @ x, k, v)
    e_K = np.eye(k)[-1]
    assert np.allclose(A @ Q.T - Q.T @ T - np.outer(q, e_K), 0.0, atol=1e-6)


@pytest.mark.parametrize("k", [6, 13, 0])
def test_shapes_without_reortho(k):
    rng = np.random.default_rng(1)
    n = 13
    A = rng.standard_normal((n, n))
    Q, T, r, c = slq.tridiag_sym_none(lambda x: A @ x, k, rng.standard_normal(n))
    assert Q.shape == (k, n) and T.shape == (k, k) and r.shape == (n,) and np.shape(c) == ()


def test_three_term_matches_full_reortho_early_on():
    # before orthogonality is lost both recurrences give the same tridiagonal
    A = problems.dense_spd(60, seed=3)
    v = np.random.default_rng(2).standard_normal(60)
    _, T1, _, _ = slq.tridiag_sym_none(lambda x: A @ x, 5, v)
    _, T2, _, _ = slq.tridiag_sym_full(lambda x: A @ x, 5, v)
    np.testing.assert_allclose(T1, T2, atol=1e-10)
