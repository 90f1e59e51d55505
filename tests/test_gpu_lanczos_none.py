"""tridiag_sym(reortho="none") on the GPU vs the oracle's three-term Lanczos."""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from oracle import problems, slq

pytestmark = pytest.mark.gpu


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


@pytest.mark.parametrize("k", [0, 1, 5, 20])
def test_three_term_fp64_matches_oracle(k):
    n = 200
    A = problems.dense_spd(n, seed=8)
    v = np.random.default_rng(9).standard_normal(n)
    Q, T, r, c = mf.decomp.tridiag_sym(k, reortho="none")(mf.DenseOperator(_t(A), precision="fp64"), _t(v))
    Qo, To, ro, co = slq.tridiag_sym_none(lambda x: A @ x, k, v)
    assert Q.shape == (k, n) and T.shape == (k, k)
    np.testing.assert_allclose(T.cpu().numpy(), To, atol=1e-9)
    np.testing.assert_allclose(Q.cpu().numpy(), Qo, atol=1e-9)
    np.testing.assert_allclose(r.cpu().numpy(), ro, atol=1e-8)
    np.testing.assert_allclose(float(c), co, rtol=1e-13)


@pytest.mark.parametrize("k", [1, 5, 11])
def test_three_term_relation(k):
    # tests/test_decomp/test_tridiag_sym.py:43-65 with reortho="none"
    n = 12
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    A = problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))
    v = _t(np.flip(np.arange(1.0, 1.0 + n)).copy())
    Q, T, q, _ = mf.decomp.tridiag_sym(k, reortho="none")(mf.DenseOperator(_t(A), precision="fp64"), v)
    Q, T, q = (x.cpu().numpy() for x in (Q, T, q))
    assert np.allclose(A @ Q.T - Q.T @ T - np.outer(q, np.eye(k)[-1]), 0.0, atol=1e-6)


def test_three_term_materialize_false():
    n, k = 50, 7
    A = problems.dense_spd(n, seed=1)
    v = _t(np.random.default_rng(2).standard_normal(n))
    _, (d, e), _, _ = mf.decomp.tridiag_sym(k, reortho="none", materialize=False)(
        mf.DenseOperator(_t(A), precision="fp64"), v)
    assert d.shape == (k,) and e.shape == (k - 1,)
