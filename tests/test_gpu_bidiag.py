"""Golub-Kahan bidiagonalisation and product log-determinants on the GPU vs the oracle."""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from oracle import bidiag as obidiag
from oracle import problems

pytestmark = pytest.mark.gpu


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


def _make_A(nrows, ncols, num_significant, base):
    n = min(nrows, ncols)
    d = np.arange(n) + base
    d[num_significant:] = 0.001
    return problems.asymmetric_matrix_from_singular_values(d, nrows=nrows, ncols=ncols)


@pytest.mark.parametrize("nrows,ncols,k", [(50, 49, 6), (15, 13, 12), (13, 15, 12), (40, 40, 10)])
def test_bidiag_pytree_callable_matches_oracle(nrows, ncols, k):
    # tests/test_decomp/test_bidiag.py:16-46: tuple in, list-of-tuple out
    A = _make_A(nrows, ncols, 4, 10.0)
    v0 = np.random.default_rng(1).standard_normal(ncols)
    At = _t(A)

    def Av(v):
        (x,) = v
        return [(At @ x,)]

    (U_tree, V_tree), B, res_tree, ln = mf.decomp.bidiag(k)(Av, (_t(v0),))
    [(U,)] = U_tree
    (V,) = V_tree
    (res,) = res_tree
    Uo, Bo, Vo, reso, lno = obidiag.bidiag(lambda v: A @ v, lambda u: A.T @ u, k, v0, nrows)
    assert U.shape == (k, nrows) and V.shape == (k, ncols) and B.shape == (k, k)
    np.testing.assert_allclose(B.cpu().numpy(), Bo, atol=1e-10)
    np.testing.assert_allclose(float(ln), lno, rtol=1e-14)
    # the relations matfree tests (near breakdown, past the significant
    # singular values, the vectors themselves are rounding-determined)
    U, V, B, res = (z.cpu().numpy() for z in (U, V, B, res))
    np.testing.assert_allclose(U @ U.T, np.eye(k), atol=1e-8)
    np.testing.assert_allclose(V @ V.T, np.eye(k), atol=1e-8)
    em = np.eye(k)[:, -1]
    np.testing.assert_allclose(A @ V.T - U.T @ B, 0.0, atol=1e-6)
    np.testing.assert_allclose(A.T @ U.T - V.T @ B.T - np.outer(res, em), 0.0, atol=1e-6)


def test_bidiag_dense_operator_batched_relations():
    n, k, p = 300, 20, 5
    rng = np.random.default_rng(2)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    V0 = rng.standard_normal((p, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    U, V, alphas, betas, R, c = mf.decomp.bidiag(k).batched(op, _t(V0))
    for b in range(p):
        Uo, Bo, Vo, reso, lno = obidiag.bidiag(lambda v: A @ v, lambda u: A.T @ u, k, V0[b], n)
        B = np.diag(alphas[b].cpu().numpy()) + np.diag(betas[b, 1:].cpu().numpy(), 1)
        np.testing.assert_allclose(B, Bo, atol=1e-10)
        np.testing.assert_allclose(U[b].cpu().numpy(), Uo, atol=1e-9)
        np.testing.assert_allclose(R[b].cpu().numpy(), reso, atol=1e-9)


def test_bidiag_tensor_core_operator_pair_form():
    # n >= 1024 and 64 probes: the CTA-pair GEMM applies both A and A^T
    n, k, p = 1100, 12, 64
    rng = np.random.default_rng(3)
    A = (rng.standard_normal((n, n)) / np.sqrt(n)).astype(np.float32)
    V0 = rng.standard_normal((p, n)).astype(np.float32)
    op = mf.DenseOperator(_t(A, torch.float32), precision="bf16x3")
    U, V, alphas, betas, R, c = mf.decomp.bidiag(k).batched(op, _t(V0, torch.float32))
    Ad = op.dense().cpu().numpy()
    for b in (0, 31, 63):
        _, Bo, _, _, _ = obidiag.bidiag(lambda v: Ad @ v, lambda u: Ad.T @ u, k, V0[b].astype(np.float64), n)
        np.testing.assert_allclose(alphas[b].cpu().numpy(), np.diag(Bo), rtol=2e-4)
        np.testing.assert_allclose(betas[b, 1:].cpu().numpy(), np.diag(Bo, 1), rtol=2e-4)
    Uc = U.double().cpu().numpy()
    G = Uc @ Uc.transpose(0, 2, 1)
    assert np.abs(G - np.eye(k)).max() < 5e-5


def test_product_logdet_estimator_matches_oracle_on_the_same_probes():
    # tests/test_funm/test_monte_carlo_funm_product_logdet.py:16-37 with a dict pytree
    A = _make_A(50, 30, 30, 1.0)
    At = _t(A)

    def matvec(x):
        return {"fx": At @ x["fx"]}

    x_like = {"fx": _t(np.ones(30))}
    sampler = mf.stochtrace.sampler_signs(x_like, num=400)
    integrand = mf.funm.monte_carlo_funm_product_logdet(mf.decomp.bidiag(20))
    estimate = mf.stochtrace.estimator_monte_carlo(integrand, sampler)
    key = mf.prng.prng_key(3)
    received = float(estimate(matvec, key))
    probes = sampler.panel(key).cpu().numpy()
    want = np.mean([obidiag.product_quadform(A, v, 20) for v in probes])
    assert abs(received - want) <= 1e-9 * abs(want)
    assert np.allclose(received, np.linalg.slogdet(A.T @ A)[1], atol=1e-2, rtol=1e-2)


def test_product_exact_for_full_num_matvecs():
    n = 50
    A = problems.asymmetric_matrix_from_singular_values(np.sqrt(np.arange(1.0, 1.0 + n)), n, n)
    x = np.random.default_rng(1).standard_normal(n) + 1
    integrand = mf.funm.monte_carlo_funm_product_logdet(mf.decomp.bidiag(n - 1))
    received = float(integrand(mf.DenseOperator(_t(A), precision="fp64"), _t(x)))
    w, S = np.linalg.eigh(A.T @ A)
    expected = x @ (S @ np.diag(np.log(w)) @ S.T) @ x
    assert np.allclose(received, expected, atol=1e-3, rtol=1e-3)


@pytest.mark.parametrize("power", [1, 2, 3])
def test_schatten_norm_and_general_function_agree_with_the_oracle(power):
    A = _make_A(40, 40, 40, 1.0)
    op = mf.DenseOperator(_t(A), precision="fp64")
    V = np.random.default_rng(power).choice([-1.0, 1.0], size=(8, 40))
    fused = mf.funm.monte_carlo_funm_product_schatten_norm(power, mf.decomp.bidiag(15))
    general = mf.funm.monte_carlo_funm_product(lambda x: x ** (power / 2), mf.decomp.bidiag(15))
    got = fused.batched(op, _t(V)).cpu().numpy()
    got2 = general.batched(op, _t(V)).cpu().numpy()
    want = np.array([obidiag.product_quadform(A, v, 15, lambda s: s ** (power / 2)) for v in V])
    np.testing.assert_allclose(got, want, rtol=1e-9)
    np.testing.assert_allclose(got2, want, rtol=1e-9)
