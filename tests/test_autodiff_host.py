"""Host logic of the differentiable SLQ integrand for callable matvecs
(``autodiff.callback_quadform``, the path ``monte_carlo_funm_sym`` takes when
a matvec parameter requires grad).  No GPU.

The three device calls -- the Krylov panels (``mfg_hessenberg``), the
eigendecomposition of T (``mfg_tridiag_eigh``) and the Hessenberg adjoint
(``mfg_hessenberg_adjoint``) -- are replaced by the oracle's float64
restatements.  What runs as in the library is the autograd plumbing: the
parameter leaves of a pytree, the Daleckii-Krein cotangent dH, and the one
batched VJP of the matvec that contracts Lambda with d(A q)/d params.  The
gradient is compared with the oracle's own assembly
(``oracle.adjoint.slq_grad_batched``: matfree/decomp.py:480-600 with
funm.py:226-241).
"""

import numpy as np
import pytest
import torch

from matfree_gb300 import autodiff
from matfree_gb300 import funm as mfunm
from oracle import adjoint as oadj
from oracle import problems, slq


@pytest.fixture
def oracle_device(monkeypatch):
    def forward_panels(op, k, panel, ld):
        V = panel.detach().double().numpy()
        Q, H, r, c = slq.hessenberg_forward_batched(
            lambda X: op._apply_rows(torch.as_tensor(X)).detach().double().numpy(), k, V)
        return (torch.as_tensor(Q), torch.as_tensor(H), torch.as_tensor(r), torch.as_tensor(c))

    def tridiag_eigh(H):
        d, e = slq.tridiag_from_hessenberg(H.numpy())
        k = d.shape[1]
        T = np.zeros_like(H.numpy())
        i = np.arange(k)
        T[:, i, i] = d
        T[:, i[:-1], i[1:]] = e
        T[:, i[1:], i[:-1]] = e
        w, S = np.linalg.eigh(T)
        return torch.as_tensor(w), torch.as_tensor(S)

    def hessenberg_adjoint(op, Q, H, R, c, dH, dr=None, dc=None):
        lams = []

        def vjp(q_panel, lam_panel):
            lams.append(lam_panel.copy())
            return op._apply_rows(torch.as_tensor(lam_panel)).detach().double().numpy(), np.zeros(1)

        dv, _ = oadj.hessenberg_adjoint_batched(vjp, 1, Q=Q.numpy(), H=H.numpy(), r=R.numpy(),
                                                dH=dH.numpy(), c=c.numpy())
        return torch.as_tensor(np.stack(lams[::-1], axis=1)), torch.as_tensor(dv)

    monkeypatch.setattr(autodiff, "_forward_panels", forward_panels)
    monkeypatch.setattr(autodiff, "as_panel", lambda x, n, dt: (x.to(dt), n))
    monkeypatch.setattr(autodiff, "hessenberg_adjoint", hessenberg_adjoint)
    monkeypatch.setattr(mfunm, "tridiag_eigh", tridiag_eigh)


def _problem(n=40, k=8, p=4, seed=0):
    rng = np.random.default_rng(seed)
    A0 = problems.dense_spd(n, seed=seed + 1)
    E1 = rng.standard_normal((n, n))
    E2 = rng.standard_normal((n, n))
    E1, E2 = 0.01 * (E1 + E1.T), 0.01 * (E2 + E2.T)
    V = rng.standard_normal((p, n))
    theta0 = np.array([0.3, -0.2])
    A = A0 + theta0[0] * E1 + theta0[1] * E2

    def vjp_matmat(Qp, Lp):
        return Lp @ A, np.array([np.sum(Lp * (Qp @ E1.T)), np.sum(Lp * (Qp @ E2.T))])

    return A0, E1, E2, V, theta0, A, vjp_matmat, k


@pytest.mark.parametrize("name,dense_funm,f,fprime", [
    ("log", mfunm.dense_funm_sym_eigh(torch.log), np.log, lambda x: 1.0 / x),
    ("sqrt via autograd", mfunm.dense_funm_sym_eigh(torch.sqrt), np.sqrt, lambda x: 0.5 / np.sqrt(x)),
    ("pow", mfunm.funm_pow(1.5), lambda x: x ** 1.5, lambda x: 1.5 * x ** 0.5),
])
def test_callback_quadform_gradient_matches_oracle(oracle_device, name, dense_funm, f, fprime):
    A0, E1, E2, V, theta0, A, vjp_matmat, k = _problem()
    A0t, E1t, E2t = (torch.as_tensor(M) for M in (A0, E1, E2))

    def matvec(v, theta):
        return A0t @ v + theta[0] * (E1t @ v) + theta[1] * (E2t @ v)

    theta = torch.tensor(theta0, requires_grad=True)
    n = V.shape[1]
    values = autodiff.callback_quadform(matvec, n, k, torch.as_tensor(V), dense_funm, (theta,))
    values.mean().backward()
    want_val, want_grad = oadj.slq_grad_batched(lambda X: X @ A.T, vjp_matmat, 2, k, V, f=f,
                                                fprime=fprime)
    assert abs(float(values.mean().detach()) - want_val) <= 1e-12 * abs(want_val)
    np.testing.assert_allclose(theta.grad.numpy(), want_grad, rtol=1e-9, atol=1e-12)


def test_callback_quadform_pytree_parameters(oracle_device):
    # parameters as a dict plus a non-tensor: each tensor leaf gets its own gradient
    A0, E1, E2, V, theta0, A, vjp_matmat, k = _problem(seed=3)
    A0t, E1t, E2t = (torch.as_tensor(M) for M in (A0, E1, E2))

    def matvec(v, params, scale):
        return scale * (A0t @ v + params["a"] * (E1t @ v) + params["b"] * (E2t @ v))

    a = torch.tensor(theta0[0], requires_grad=True)
    b = torch.tensor(theta0[1], requires_grad=True)
    n = V.shape[1]
    vals = autodiff.callback_quadform(matvec, n, k, torch.as_tensor(V),
                                      mfunm.dense_funm_sym_eigh(torch.log), ({"a": a, "b": b}, 1.0))
    vals.mean().backward()
    _, want = oadj.slq_grad_batched(lambda X: X @ A.T, vjp_matmat, 2, k, V)
    np.testing.assert_allclose([float(a.grad), float(b.grad)], want, rtol=1e-9)


def test_callback_quadform_k_zero_raises():
    with pytest.raises(ValueError, match="= 0"):
        autodiff.callback_quadform(lambda v: v, 3, 0, torch.ones((1, 3)),
                                   mfunm.dense_funm_sym_eigh(torch.log), ())


def test_params_require_grad_detection():
    t = torch.ones(2, requires_grad=True)
    assert autodiff.params_require_grad((t,))
    assert autodiff.params_require_grad(({"x": [1.0, t]},))
    assert not autodiff.params_require_grad((t.detach(), 2.0))
    with torch.no_grad():
        assert not autodiff.params_require_grad((t,))
