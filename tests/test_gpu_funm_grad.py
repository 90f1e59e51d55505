"""f(A) v by Lanczos on the device, and gradients through the decomposition.

* funm_lanczos_sym (matfree/funm.py:114-147), batched over vectors: the
  float64 path against the oracle's restatement on identical vectors, and
  matfree's own known-answer test (tests/test_funm/test_funm_lanczos_sym.py);
* the Hessenberg adjoint with a cotangent of the basis (dQ, through Pi_xi and
  Pi_gamma, matfree/decomp.py:505-506) against the oracle's adjoint, which is
  pinned by complex-step differentiation;
* the custom VJP of tridiag_sym (decomp.py:393-422) and the gradient of
  f(A) v, each against central differences of the float64 GPU path.
"""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import autodiff
from oracle import adjoint as oadj
from oracle import problems, slq

pytestmark = pytest.mark.gpu

DEV = "cuda"


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=DEV)


@pytest.mark.parametrize("name", ["log", "sin"])
def test_funm_lanczos_sym_batched_matches_oracle(name):
    n, k, p = 400, 30, 5
    A = problems.dense_spd(n, seed=6)
    V = np.random.default_rng(4).standard_normal((p, n))
    tf, nf = {"log": (torch.log, np.log), "sin": (torch.sin, np.sin)}[name]
    fn = mf.funm.funm_lanczos_sym(mf.funm.dense_funm_sym_eigh(tf), mf.decomp.tridiag_sym(k))
    got = fn.batched(mf.DenseOperator(_t(A), precision="fp64"), _t(V)).cpu().numpy()
    ofn = slq.funm_lanczos_sym(slq.dense_funm_sym_eigh(nf), k)
    for b in range(p):
        want = ofn(lambda x: A @ x, V[b])
        np.testing.assert_allclose(got[b], want, rtol=0, atol=1e-9 * np.abs(want).max())
    # the single-vector call is the batched call on one row
    one = fn(mf.DenseOperator(_t(A), precision="fp64"), _t(V[0])).cpu().numpy()
    np.testing.assert_allclose(one, got[0], rtol=0, atol=1e-12 * np.abs(got[0]).max())


@pytest.mark.parametrize("reortho", ["full", "none"])
def test_funm_lanczos_sym_reference_known_answer(reortho):
    # tests/test_funm/test_funm_lanczos_sym.py:7-37: pytree vector, matrix parameter
    n = 11
    v = np.random.default_rng(2).standard_normal(n)
    matrix = problems.hermitian_matrix_from_eigenvalues(np.linspace(0.01, 0.99, num=n),
                                                        np.random.default_rng(1))
    w, U = np.linalg.eigh(matrix)
    expected = U @ np.diag(np.sin(w)) @ U.T @ v

    def matvec(x, p):
        [(u,)] = x
        return [(p @ u,)]

    fn = mf.funm.funm_lanczos_sym(mf.funm.dense_funm_sym_eigh(torch.sin),
                                  mf.decomp.tridiag_sym(6, materialize=True, reortho=reortho))
    [(received,)] = fn(matvec, [(_t(v),)], _t(matrix))
    assert np.allclose(expected, received.cpu().numpy(), atol=1e-6)


def test_hessenberg_adjoint_with_dQ_matches_oracle():
    n, k, p = 150, 12, 3
    rng = np.random.default_rng(21)
    A = problems.dense_spd(n, seed=8)
    E = rng.standard_normal((n, n))
    V = rng.standard_normal((p, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    panel, ld = mf._panel.as_panel(_t(V), n, torch.float64)
    Q, H, R, c = autodiff._forward_panels(op, k, panel, ld)
    dQ = rng.standard_normal((p, k, n))
    dH = rng.standard_normal((p, k, k))
    dr = rng.standard_normal((p, n))
    dc = rng.standard_normal(p)
    dQp = torch.zeros_like(Q)
    dQp[:, :, :n] = _t(dQ)
    drp = torch.zeros_like(R)
    drp[:, :n] = _t(dr)
    Lam, dv = autodiff.hessenberg_adjoint(op, Q, H, R, c, _t(dH), dr=drp, dc=_t(dc), dQ=dQp)
    Qn = Q[:, :, :n].cpu().numpy()
    Ln = Lam[:, :, :n].cpu().numpy()
    for b in range(p):
        Qo, Ho, ro, co = slq.hessenberg_forward(lambda x: A @ x, k, V[b], reortho="full")

        def vjp_matvec(q, lam):
            return A.T @ lam, (np.outer(lam, q),)

        dvo, (dAo,) = oadj.hessenberg_adjoint(vjp_matvec, (A,), Q=Qo, H=Ho, r=ro, c=co, dQ=dQ[b].T,
                                              dH=dH[b], dr=dr[b], dc=dc[b], reortho="full")
        np.testing.assert_allclose(dv[b, :n].cpu().numpy(), dvo, rtol=1e-8, atol=1e-8 * np.abs(dvo).max())
        got = np.sum(Ln[b] * (Qn[b] @ E.T))
        np.testing.assert_allclose(got, np.sum(dAo * E), rtol=1e-8)


def _callable(n=120, seed=5):
    rng = np.random.default_rng(seed)
    A0 = problems.dense_spd(n, seed=seed)
    E1 = rng.standard_normal((n, n))
    E2 = rng.standard_normal((n, n))
    E1t, E2t, A0t = _t(0.01 * (E1 + E1.T)), _t(0.01 * (E2 + E2.T)), _t(A0)

    def matvec(v, theta):
        return A0t @ v + theta[0] * (E1t @ v) + theta[1] * (E2t @ v)

    return matvec


def test_tridiag_sym_custom_vjp_matches_central_differences():
    n, k = 120, 10
    matvec = _callable(n)
    rng = np.random.default_rng(7)
    v0 = _t(rng.standard_normal(n))
    theta0 = _t([0.3, -0.2])
    W1, W2 = _t(rng.standard_normal((k, n))), _t(rng.standard_normal((k, k)))
    w3, w4 = _t(rng.standard_normal(n)), float(rng.standard_normal())
    dec = mf.decomp.tridiag_sym(k)

    def loss(v, theta):
        Q, T, r, c = dec(matvec, v, theta)
        return (W1 * Q).sum() + (W2 * T).sum() + (w3 * r).sum() + w4 * c

    v = v0.clone().requires_grad_(True)
    theta = theta0.clone().requires_grad_(True)
    loss(v, theta).backward()
    h = 1e-6
    with torch.no_grad():
        for i in range(2):
            e = torch.zeros(2, dtype=torch.float64, device=DEV)
            e[i] = h
            fd = (loss(v0, theta0 + e) - loss(v0, theta0 - e)) / (2 * h)
            assert abs(float(theta.grad[i]) - float(fd)) <= 1e-6 * max(1.0, abs(float(fd))), (i, theta.grad[i], fd)
        t = _t(rng.standard_normal(n))
        fd = (loss(v0 + h * t, theta0) - loss(v0 - h * t, theta0)) / (2 * h)
        got = float((v.grad * t).sum())
        assert abs(got - float(fd)) <= 1e-6 * max(1.0, abs(float(fd))), (got, fd)


def test_funm_lanczos_sym_gradient_matches_central_differences():
    n, k = 120, 14
    matvec = _callable(n, seed=9)
    rng = np.random.default_rng(8)
    v0 = _t(rng.standard_normal(n))
    theta0 = _t([0.1, 0.25])
    w = _t(rng.standard_normal(n))
    fn = mf.funm.funm_lanczos_sym(mf.funm.dense_funm_sym_eigh(torch.log), mf.decomp.tridiag_sym(k))

    def loss(v, theta):
        return (w * fn(matvec, v, theta)).sum()

    v = v0.clone().requires_grad_(True)
    theta = theta0.clone().requires_grad_(True)
    loss(v, theta).backward()
    h = 1e-6
    with torch.no_grad():
        for i in range(2):
            e = torch.zeros(2, dtype=torch.float64, device=DEV)
            e[i] = h
            fd = (loss(v0, theta0 + e) - loss(v0, theta0 - e)) / (2 * h)
            assert abs(float(theta.grad[i]) - float(fd)) <= 1e-6 * max(1.0, abs(float(fd))), (i, theta.grad[i], fd)
        t = _t(rng.standard_normal(n))
        fd = (loss(v0 + h * t, theta0) - loss(v0 - h * t, theta0)) / (2 * h)
        got = float((v.grad * t).sum())
        assert abs(got - float(fd)) <= 1e-6 * max(1.0, abs(float(fd))), (got, fd)


def test_gradients_without_custom_vjp_are_refused():
    n, k = 50, 5
    matvec = _callable(n, seed=3)
    v = _t(np.ones(n)).requires_grad_(True)
    with pytest.raises(NotImplementedError, match="custom_vjp"):
        mf.decomp.tridiag_sym(k, custom_vjp=False)(matvec, v, _t([0.0, 0.0]))
