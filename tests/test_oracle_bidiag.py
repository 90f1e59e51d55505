"""The bidiagonalisation oracle against matfree's known answers (CPU).

Restates tests/test_decomp/test_bidiag.py and
tests/test_funm/test_monte_carlo_funm_product_logdet.py with NumPy probes.
"""

import numpy as np
import pytest

from oracle import bidiag, problems


def _make_A(nrows, ncols, num_significant, base):
    n = min(nrows, ncols)
    d = np.arange(n) + base
    d[num_significant:] = 0.001
    return problems.asymmetric_matrix_from_singular_values(d, nrows=nrows, ncols=ncols)


def _check(A, U, B, V, res, ln, v0, k):
    np.testing.assert_allclose(U @ U.T, np.eye(k), atol=1e-8)
    np.testing.assert_allclose(V @ V.T, np.eye(k), atol=1e-8)
    em = np.eye(k)[:, -1]
    np.testing.assert_allclose(A @ V.T - U.T @ B, 0.0, atol=1e-6)
    np.testing.assert_allclose(A.T @ U.T - V.T @ B.T - np.outer(res, em), 0.0, atol=1e-6)
    np.testing.assert_allclose(1.0 / np.linalg.norm(v0), ln)


def test_bidiag_decomposition_is_satisfied():
    A = _make_A(50, 49, 4, 10.0)
    v0 = np.random.default_rng(1).standard_normal(49)
    U, B, V, res, ln = bidiag.bidiag(lambda v: A @ v, lambda u: A.T @ u, 6, v0, 50)
    _check(A, U, B, V, res, ln, v0, 6)


@pytest.mark.parametrize("nrows", [15, 13])
@pytest.mark.parametrize("ncols", [15, 13])
def test_bidiag_decomposition_is_satisfied_hilbert(nrows, ncols):
    a = np.arange(0, max(ncols, nrows))
    A = 1.0 / (1.0 + a[:, None] + a[None, :])[:nrows, :ncols]
    v0 = np.random.default_rng(1).standard_normal(ncols)
    U, B, V, res, ln = bidiag.bidiag(lambda v: A @ v, lambda u: A.T @ u, 12, v0, nrows)
    _check(A, U, B, V, res, ln, v0, 12)


def test_logdet_product():
    A = _make_A(50, 30, 30, 1.0)
    rng = np.random.default_rng(3)
    probes = rng.choice([-1.0, 1.0], size=(400, 30))
    est = np.mean([bidiag.product_quadform(A, v, 20) for v in probes])
    want = np.linalg.slogdet(A.T @ A)[1]
    assert np.allclose(est, want, atol=1e-2, rtol=1e-2)


def test_logdet_product_exact_for_full_num_matvecs():
    n = 50
    A = problems.asymmetric_matrix_from_singular_values(np.sqrt(np.arange(1.0, 1.0 + n)), n, n)
    x = np.random.default_rng(1).standard_normal(n) + 1
    received = bidiag.product_quadform(A, x, n - 1)
    w, S = np.linalg.eigh(A.T @ A)
    expected = x @ (S @ np.diag(np.log(w)) @ S.T) @ x
    assert np.allclose(received, expected, atol=1e-3, rtol=1e-3)


def test_bidiag_rejects_too_many_matvecs():
    A = np.eye(5)
    with pytest.raises(ValueError):
        bidiag.bidiag(lambda v: A @ v, lambda u: A.T @ u, 6, np.ones(5), 5)
