"""Golub-Kahan bidiagonalisation with full reorthogonalisation in two reads of
each basis per step, restated in float64 NumPy, against the oracle's CGS2
form (matfree/decomp.py:641-750, oracle/bidiag.py).  No GPU.

The reference projects each new left vector y_i = A v_i - beta_i u_{i-1} out
of U twice and each new right vector x_i = A^T u_i - alpha_i v_i out of V
twice, and keeps only the norms alpha_i, beta_{i+1} in B.  Here each side
keeps one vector pending after its first projection, and one sweep over a
basis does two things:

- the delayed second projection of that side's pending vector, which makes it
  final;
- the first projection of the operator applied to the OTHER side's pending
  vector, against the basis and the newly final vector, through the scalar
  (final vector) . w = (p.w - h.g) / rho.

The operator sees a vector before its second projection.  The missing term,
e.g. A V_i hv for the left side, lies in span(U_i), because
A v_m in span(U_m) for every finished m.  The first projection against U_i
removes it, so only the scale 1/rho carries over, and that scale enters alpha
and beta.  A sweep is therefore one pass for B^T p, B^T w and p.w and one
pass for the two subtractions.  That is the pattern of the two-vector stream
sweeps of the Arnoldi two-sweep step, against three passes per side per step
in the CGS2 form.
"""

import numpy as np
import pytest

from oracle import bidiag as ob


def _sweep(Bs, pend, w):
    """Finalise pend over the final rows Bs and first-project w; two passes over Bs."""
    h, g, c = Bs @ pend, Bs @ w, pend @ w  # pass 1
    r = pend - Bs.T @ h  # pass 2 (with w - Bs^T g)
    rho = np.linalg.norm(r)
    fin = r / rho
    z = w - Bs.T @ g - fin * ((c - h @ g) / rho)
    return fin, rho, z


def two_sweep_bidiag(A, v0, k):
    """Returns (U (k, m), B (k, k), V (k, n), residual (n,), 1/||v0||) like oracle.bidiag."""
    m, n = A.shape
    length = np.linalg.norm(v0)
    v = v0 / length
    v = v / np.linalg.norm(v)
    U, V = np.zeros((k, m)), np.zeros((k, n))
    alphas, betas = np.zeros(k), np.zeros(k)
    V[0] = v
    ut, su = A @ v, 1.0  # pending left vector; y_i' = su * ut
    vt = A.T @ ut - V[:1].T @ (V[:1] @ (A.T @ ut))  # pending right vector, true scale 1/rho_u
    for i in range(k):
        U[i], rho_u, zu = _sweep(U[:i], ut, A @ vt)
        alphas[i] = su * rho_u
        sv = 1.0 / rho_u
        vfin, rho_v, zv = _sweep(V[: i + 1], vt, A.T @ zu)
        beta = sv * rho_v
        if i + 1 == k:
            B = np.diag(alphas) + np.diag(betas[1:], 1)
            return U, B, V, beta * vfin, 1.0 / length
        V[i + 1], betas[i + 1] = vfin, beta
        ut, su, vt = zu, 1.0 / rho_v, zv
    raise AssertionError("unreachable")


@pytest.mark.parametrize("m,n,k", [(60, 40, 10), (200, 150, 30), (300, 120, 64), (50, 50, 49),
                                   (120, 300, 40), (90, 70, 1)])
def test_two_sweep_bidiag_equals_cgs2(m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((m, n))
    v0 = rng.standard_normal(n)
    Uo, Bo, Vo, ro, co = ob.bidiag(lambda v: A @ v, lambda u: A.T @ u, k, v0, m)
    U, B, V, r, c = two_sweep_bidiag(A, v0, k)
    np.testing.assert_allclose(B, Bo, atol=1e-12 * np.abs(Bo).max())
    np.testing.assert_allclose(U, Uo, atol=1e-11)
    np.testing.assert_allclose(V, Vo, atol=1e-11)
    np.testing.assert_allclose(r, ro, atol=1e-11 * max(np.abs(ro).max(), 1.0))
    assert c == co


def test_two_sweep_bidiag_product_logdet():
    # the product integrand ||v||^2 e1^T log(B^T B) e1 (funm.py:276-320) from either B
    rng = np.random.default_rng(5)
    A = rng.standard_normal((150, 100)) + 3.0 * np.eye(150, 100)
    v0 = rng.standard_normal(100)
    want = ob.product_quadform(A, v0, 20)
    _, B, _, _, _ = two_sweep_bidiag(A, v0, 20)
    _, S, Vt = np.linalg.svd(B)
    got = np.linalg.norm(v0) ** 2 * np.sum(np.log(S * S) * Vt.T[0, :] ** 2)
    assert abs(got - want) <= 1e-11 * abs(want)
