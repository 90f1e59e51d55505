"""GP log-density on the GPU: CG solves and the differentiable RBF log-pdf vs the oracle."""

import math

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from oracle import gp, problems

pytestmark = pytest.mark.gpu


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


def test_cg_fp64_matches_oracle_iterates():
    n = 300
    A = problems.dense_spd(n, seed=2)
    b = np.random.default_rng(3).standard_normal(n)
    op = mf.DenseOperator(_t(A), precision="fp64")
    X, its = mf.linalg.cg_batched(op, _t(b)[None, :], tol=1e-10)
    xo, ko = gp.cg(lambda v: A @ v, b, tol=1e-10)
    assert int(its[0]) == ko
    np.testing.assert_allclose(X[0].cpu().numpy(), xo, rtol=1e-10, atol=1e-12)
    x, info = mf.linalg.cg(op, _t(b), tol=1e-10)
    assert info is None and torch.equal(x, X[0])


def test_cg_batched_rows_run_independently():
    # one row converges in one step (an eigenvector), one never starts (zero),
    # the others need many: each row equals its own single-vector solve
    n = 200
    rng = np.random.default_rng(4)
    A = problems.dense_spd(n, seed=5)
    w, S = np.linalg.eigh(A)
    B = np.stack([S[:, 3], np.zeros(n), rng.standard_normal(n), rng.standard_normal(n)])
    op = mf.DenseOperator(_t(A), precision="fp64")
    X, its = mf.linalg.cg_batched(op, _t(B), tol=1e-9)
    for i in range(len(B)):
        xo, ko = gp.cg(lambda v: A @ v, B[i], tol=1e-9)
        assert int(its[i]) == ko
        np.testing.assert_allclose(X[i].cpu().numpy(), xo, rtol=1e-9, atol=1e-12)
    assert int(its[0]) == 1 and int(its[1]) == 0


def test_cg_maxiter_stops_every_row():
    n = 150
    A = problems.dense_spd(n, seed=6)
    B = np.random.default_rng(7).standard_normal((3, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    X, its = mf.linalg.cg_batched(op, _t(B), tol=1e-14, maxiter=4)
    assert (its.cpu().numpy() == 4).all()
    for i in range(3):
        xo, _ = gp.cg(lambda v: A @ v, B[i], tol=1e-14, maxiter=4)
        np.testing.assert_allclose(X[i].cpu().numpy(), xo, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("n", [500, 1500])
def test_cg_tensor_core_rbf_operator(n):
    # bf16x3 RBF operator: the fp32 CG solution against a float64 solve of
    # the stored operator
    x = torch.rand((n, 3), generator=torch.Generator().manual_seed(n)).cuda()
    op = mf.RBFKernelOperator(x, s2=1.0, ell=0.2, tau=0.5, precision="bf16x3")
    b = torch.randn(n, generator=torch.Generator().manual_seed(1)).cuda()
    sol, _ = mf.linalg.cg(op, b, tol=1e-6)
    K = op.dense().cpu().numpy()
    want = np.linalg.solve(K, b.double().cpu().numpy())
    assert np.abs(sol.double().cpu().numpy() - want).max() <= 1e-4 * np.abs(want).max()


def test_cg_long_vectors_multi_launch_iteration():
    # n above the one-CTA-per-probe step (8192): the iteration runs as a
    # projection, an update and a direction launch; a zero row never starts
    import scipy.sparse as sp

    n = 40000
    L = sp.diags([-np.ones(n - 1), 2.0 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1], format="csr")
    op = mf.CSROperator.from_scipy(L, shift=1.0)
    rng = np.random.default_rng(11)
    B = np.stack([rng.standard_normal(n), np.zeros(n), rng.standard_normal(n)])
    X, its = mf.linalg.cg_batched(op, _t(B, torch.float32), tol=1e-6)
    A = L + sp.identity(n)
    for i in (0, 2):
        xo, ko = gp.cg(lambda v: A @ v, B[i], tol=1e-6)
        assert abs(int(its[i]) - ko) <= 2
        np.testing.assert_allclose(X[i].double().cpu().numpy(), xo, atol=1e-5 * np.abs(xo).max())
    assert int(its[1]) == 0 and not X[1].any()


def test_rbf_logpdf_value_and_gradient_fp64_vs_oracle():
    n, k, p = 256, 20, 16
    rng = np.random.default_rng(10)
    xs = rng.uniform(size=(n, 3))
    theta0 = np.array([0.1, np.log(0.3), np.log(0.2)])
    y = rng.standard_normal(n)
    probes = rng.choice([-1.0, 1.0], size=(p, n))
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    val = mf.gp.rbf_logpdf(_t(xs, torch.float32), theta, _t(y), _t(probes), k, precision="fp64",
                           cg_tol=1e-13)
    # the points enter in float32 on the device: the oracle gets the same points
    xs32 = xs.astype(np.float32).astype(np.float64)
    want, gwant = gp.rbf_logpdf_slq(xs32, theta0, y, probes, k)
    assert abs(float(val.detach()) - want) <= 1e-8 * abs(want)
    val.backward()
    np.testing.assert_allclose(theta.grad.numpy(), gwant, rtol=1e-6, atol=1e-6)


def test_create_logpdf_follows_the_tutorial_composition():
    # tutorials/8_gaussian_logpdf.py:36-55 with a dense fp64 covariance
    n = 120
    xs = np.linspace(0.0, 1.0, n)
    K = np.exp(-((xs[:, None] - xs[None, :]) ** 2) / 2.0) + np.exp(-2.0) * np.eye(n)
    op = mf.DenseOperator(_t(K), precision="fp64")
    y = np.random.default_rng(1).standard_normal(n)
    vec_like = _t(np.zeros(n))
    logpdf = mf.gp.create_logpdf(op, vec_like, num_matvecs=6, num_samples=50, cg_tol=1e-12)
    key = mf.prng.prng_key(2)
    val = float(logpdf(_t(y), key))
    probes = mf.stochtrace.sampler_signs(vec_like, num=50).panel(key).cpu().numpy()
    logdet = gp.slq_logdet(K, probes, 6)
    want = -0.5 * (y @ np.linalg.solve(K, y) + logdet + n * math.log(2 * math.pi))
    assert abs(val - want) <= 1e-9 * abs(want)
