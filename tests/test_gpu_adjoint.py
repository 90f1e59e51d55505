"""GPU Hessenberg adjoint and SLQ hyper-parameter gradients vs the float64 oracle.

matfree checks its custom VJP against JAX autodiff
(tests/test_decomp/test_hessenberg_adjoint.py, test_tridiag_sym_adjoint.py).
Here the oracle's float64 restatement of the same adjoint (itself checked
against complex-step differentiation on the CPU) and central finite
differences of the GPU estimator stand in for autodiff.
"""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import autodiff
from oracle import adjoint as oadj
from oracle import philox, problems, slq

pytestmark = pytest.mark.gpu


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


@pytest.mark.parametrize("n,k,p", [(40, 6, 3), (300, 20, 5)])
def test_batched_adjoint_fp64_matches_oracle(n, k, p):
    rng = np.random.default_rng(n)
    A = problems.dense_spd(n, seed=2)
    V = rng.standard_normal((p, n))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    dH = rng.standard_normal((p, k, k))
    E = rng.standard_normal((n, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    panel, ld = mf._panel.as_panel(_t(V), n, torch.float64)
    Q, H, R, c = autodiff._forward_panels(op, k, panel, ld)
    Lam, dv = autodiff.hessenberg_adjoint(op, Q, H, R, c, _t(dH))

    Qo, Ho, ro, co = slq.hessenberg_forward_batched(lambda X: X @ A.T, k, V)

    def vjp_matmat(Qp, Lp):
        return Lp @ A, np.array([np.sum(Lp * (Qp @ E.T))])

    dvo, dpo = oadj.hessenberg_adjoint_batched(vjp_matmat, 1, Q=Qo, H=Ho, r=ro, dH=dH, c=co)
    np.testing.assert_allclose(dv[:, :n].cpu().numpy(), dvo, rtol=1e-7, atol=1e-8)
    # parameter direction E: sum_idx lambda_idx^T E q_idx
    Qn = Q[:, :, :n].cpu().numpy()
    Ln = Lam[:, :, :n].cpu().numpy()
    got = np.einsum("pkn,pkn->", Ln, Qn @ E.T)
    np.testing.assert_allclose(got, dpo[0], rtol=1e-7)


def test_adjoint_k_zero_raises():
    # tests/test_decomp/test_hessenberg_adjoint.py:43-61
    op = mf.DenseOperator(_t(np.eye(3)), precision="fp64")
    Q = torch.zeros((1, 0, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="= 0"):
        autodiff.hessenberg_adjoint(op, Q, torch.zeros((1, 0, 0), dtype=torch.float64, device="cuda"),
                                    torch.zeros((1, 8), dtype=torch.float64, device="cuda"),
                                    torch.ones(1, dtype=torch.float64, device="cuda"),
                                    torch.zeros((1, 0, 0), dtype=torch.float64, device="cuda"))


def _rbf_case(n, p, seed=3):
    x = problems.rbf_points(n, seed=seed).astype(np.float32)
    V = philox.rademacher(philox.prng_key(seed + 1), p, n)
    return x, V


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("bf16x3", 2e-3), ("fp32", 1e-3)])
def test_rbf_logdet_gradient_matches_oracle(precision, tol):
    n, k, p = 600, 20, 16
    x, V = _rbf_case(n, p)
    theta0 = np.array([0.0, np.log(0.2), np.log(1e-2)])
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    dt = torch.float64 if precision == "fp64" else torch.float32
    val = autodiff.rbf_logdet(_t(x, torch.float32), theta, _t(V, dt), k, precision=precision)
    val.backward()
    matmat, vjp_matmat = oadj.rbf_vjp_factory(x.astype(np.float64), theta0)
    want_val, want_grad = oadj.slq_grad_batched(matmat, vjp_matmat, 3, k, V)
    assert abs(float(val.detach()) - want_val) <= max(tol, 1e-10) * abs(want_val) * (1 if precision != "bf16" else 10)
    got = theta.grad.numpy()
    err = np.abs(got - want_grad) / np.maximum(np.abs(want_grad), 1e-3 * np.abs(want_grad).max())
    assert np.all(err < tol), (got, want_grad, err)


def test_rbf_logdet_gradient_matches_central_differences():
    # central differences (h = 1e-4) of the float64 GPU estimator itself
    n, k, p = 400, 16, 8
    x, V = _rbf_case(n, p, seed=7)
    theta0 = np.array([0.0, np.log(0.2), np.log(1e-2)])
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    xt, Vt = _t(x, torch.float32), _t(V)
    autodiff.rbf_logdet(xt, theta, Vt, k, precision="fp64").backward()
    h = 1e-4
    for i in range(3):
        e = np.zeros(3)
        e[i] = h
        fp = float(autodiff.rbf_logdet(xt, torch.tensor(theta0 + e), Vt, k, precision="fp64"))
        fm = float(autodiff.rbf_logdet(xt, torch.tensor(theta0 - e), Vt, k, precision="fp64"))
        fd = (fp - fm) / (2 * h)
        assert np.isclose(theta.grad[i].item(), fd, rtol=1e-5, atol=1e-6), (i, theta.grad[i].item(), fd)


def _callable_case(n=300, seed=4):
    rng = np.random.default_rng(seed)
    A0 = problems.dense_spd(n, seed=seed)
    E1 = rng.standard_normal((n, n))
    E2 = rng.standard_normal((n, n))
    E1, E2 = 0.01 * (E1 + E1.T), 0.01 * (E2 + E2.T)
    theta0 = np.array([0.3, -0.2])
    A = A0 + theta0[0] * E1 + theta0[1] * E2
    A0t, E1t, E2t = _t(A0), _t(E1), _t(E2)

    def matvec(v, theta):
        return A0t @ v + theta[0] * (E1t @ v) + theta[1] * (E2t @ v)

    def vjp_matmat(Qp, Lp):
        return Lp @ A, np.array([np.sum(Lp * (Qp @ E1.T)), np.sum(Lp * (Qp @ E2.T))])

    return A, theta0, matvec, vjp_matmat


def test_callable_matvec_logdet_gradient_matches_oracle():
    # a torch callable with a parameter that requires grad: the integrand runs
    # the Krylov loop, the eigensolver and the Hessenberg adjoint on the GPU
    n, k, p = 300, 20, 6
    A, theta0, matvec, vjp_matmat = _callable_case(n)
    V = np.random.default_rng(9).standard_normal((p, n))
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    theta = torch.tensor(theta0, dtype=torch.float64, device="cuda", requires_grad=True)
    val = integrand.batched(matvec, _t(V), theta).mean()
    val.backward()
    want_val, want_grad = oadj.slq_grad_batched(lambda X: X @ A.T, vjp_matmat, 2, k, V)
    assert abs(float(val.detach()) - want_val) <= 1e-9 * abs(want_val)
    np.testing.assert_allclose(theta.grad.cpu().numpy(), want_grad, rtol=1e-7, atol=1e-10)


def test_estimator_gradient_matches_central_differences():
    # estimator_monte_carlo(...)(matvec, key, theta).backward(), with an
    # arbitrary f whose derivative comes from autograd, against central
    # differences of the same estimator on the same probes
    n, k, num = 200, 12, 8
    _, theta0, matvec, _ = _callable_case(n, seed=6)
    x_like = torch.zeros(n, dtype=torch.float64, device="cuda")
    integrand = mf.funm.monte_carlo_funm_sym(mf.funm.dense_funm_sym_eigh(torch.sqrt),
                                             mf.decomp.tridiag_sym(k))
    estimate = mf.stochtrace.estimator_monte_carlo(
        integrand, mf.stochtrace.sampler_signs(x_like, num=num))
    key = mf.prng.prng_key(5)
    theta = torch.tensor(theta0, dtype=torch.float64, device="cuda", requires_grad=True)
    estimate(matvec, key, theta).backward()
    h = 1e-5
    for i in range(2):
        e = torch.zeros(2, dtype=torch.float64, device="cuda")
        e[i] = h
        with torch.no_grad():
            fp = float(estimate(matvec, key, torch.tensor(theta0, device="cuda") + e))
            fm = float(estimate(matvec, key, torch.tensor(theta0, device="cuda") - e))
        fd = (fp - fm) / (2 * h)
        assert abs(float(theta.grad[i]) - fd) <= 1e-6 * max(abs(fd), 1.0), (i, float(theta.grad[i]), fd)
