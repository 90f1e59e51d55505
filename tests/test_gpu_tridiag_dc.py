"""Batched tridiagonal eigensolve (divide and conquer for 16 <= k <= 2048, QL
otherwise) against numpy's eigh on hard spectra (needs a GPU).

Eigenvalues agree to 1e-12 of the spectral radius.  Eigenvector first
components are compared through quadratures sum_i g(lambda_i) s_1i^2, which
do not depend on the choice of basis inside a degenerate eigenspace; the
weights sum to one to 1e-12.  The full-eigenvector solver (mfg_tridiag_eigh)
is checked through S^T S = I and S diag(w) S^T = T to 1e-12 k.
"""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf

pytestmark = pytest.mark.gpu


def _lanczos_tridiagonal(rng, k):
    """Tridiagonal of k full-reorthogonalisation Lanczos steps on a matrix with
    a tight cluster and a wide log-spaced tail (the shape of SLQ on kernels)."""
    n = max(2 * k, 200)
    ev = np.concatenate([np.full(n // 2, 1e-2) + 1e-6 * rng.random(n // 2),
                         np.logspace(-2, 3, n - n // 2)])
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * ev) @ Q.T
    q = rng.choice([-1.0, 1.0], n)
    q /= np.linalg.norm(q)
    V = np.zeros((k, n))
    d = np.zeros(k)
    e = np.zeros(k - 1)
    for j in range(k):
        V[j] = q
        w = A @ q
        d[j] = q @ w
        for _ in range(2):
            w -= V[: j + 1].T @ (V[: j + 1] @ w)
        if j < k - 1:
            e[j] = np.linalg.norm(w)
            q = w / e[j]
    return d, e


def _case(kind, k, rng):
    if kind == "normal":
        return rng.standard_normal(k), rng.standard_normal(k - 1)
    if kind == "lanczos":
        return _lanczos_tridiagonal(rng, k)
    if kind == "tiny_couplings":
        return rng.standard_normal(k), rng.standard_normal(k - 1) * 10.0 ** rng.integers(-18, 0, k - 1)
    if kind == "wilkinson":
        return np.abs(np.arange(k) - k // 2).astype(float), np.ones(k - 1)
    if kind == "glued_wilkinson":
        d = np.resize(np.abs(np.arange(7) - 3).astype(float), k)
        e = np.ones(k - 1)
        e[6::7] = 1e-10
        return d, e
    if kind == "split_constant":
        e = np.zeros(k - 1)
        e[::3] = 1.0
        return np.ones(k), e
    if kind == "negative_couplings":
        return rng.uniform(1, 3, k), -rng.uniform(0.1, 0.5, k - 1)
    if kind == "zero":
        return np.zeros(k), np.zeros(k - 1)
    raise ValueError(kind)


KINDS = ["normal", "lanczos", "tiny_couplings", "wilkinson", "glued_wilkinson",
         "split_constant", "negative_couplings", "zero"]


def _stack(cases):
    p, k = len(cases), len(cases[0][0])
    H = np.zeros((p, k, k))
    idx = np.arange(k)
    for b, (d, e) in enumerate(cases):
        H[b, idx, idx] = d
        H[b, idx[:-1], idx[1:]] = e
        H[b, idx[1:], idx[:-1]] = e
    return H


@pytest.mark.parametrize("k", [12, 16, 17, 31, 32, 33, 64, 100, 128, 257])
def test_tridiag_eigh_first_hard_spectra(k):
    rng = np.random.default_rng(1000 + k)
    cases = [_case(kind, k, rng) for kind in KINDS for _ in range(3)]
    H = _stack(cases)
    lam, fsq = mf.funm.tridiag_eigh_first(torch.as_tensor(H, device="cuda"))
    lam, fsq = lam.cpu().numpy(), fsq.cpu().numpy()
    for b in range(len(cases)):
        w0, S0 = np.linalg.eigh(H[b])
        scale = max(np.max(np.abs(w0)), 1e-300)
        kind = KINDS[b // 3]
        np.testing.assert_allclose(lam[b], w0, rtol=0, atol=1e-12 * scale, err_msg=kind)
        np.testing.assert_allclose(fsq[b].sum(), 1.0, atol=1e-12, err_msg=kind)
        for g in (lambda x: np.exp(-x / scale), lambda x: (x / scale) ** 2, lambda x: np.sin(3 * x / scale)):
            want = np.sum(g(w0) * S0[0] ** 2)
            got = np.sum(g(lam[b]) * fsq[b])
            assert abs(got - want) <= 1e-12, (kind, got, want)


@pytest.mark.parametrize("k", [600, 2048])
def test_tridiag_eigh_first_large_k(k):
    rng = np.random.default_rng(k)
    cases = [_case(kind, k, rng) for kind in ("normal", "negative_couplings")]
    H = _stack(cases)
    lam, fsq = mf.funm.tridiag_eigh_first(torch.as_tensor(H, device="cuda"))
    lam, fsq = lam.cpu().numpy(), fsq.cpu().numpy()
    for b in range(len(cases)):
        w0, S0 = np.linalg.eigh(H[b])
        scale = np.max(np.abs(w0))
        np.testing.assert_allclose(lam[b], w0, rtol=0, atol=1e-12 * scale)
        g = np.exp(-w0 / scale)
        assert abs(np.sum(np.exp(-lam[b] / scale) * fsq[b]) - np.sum(g * S0[0] ** 2)) <= 1e-12


@pytest.mark.parametrize("k", [20, 64, 150])
def test_log_quadrature_of_lanczos_tridiagonals(k):
    rng = np.random.default_rng(7 + k)
    cases = [_lanczos_tridiagonal(rng, k) for _ in range(4)]
    H = _stack(cases)
    Ht = torch.as_tensor(H, device="cuda")
    lam, fsq = mf.funm.tridiag_eigh_first(Ht)
    got = (torch.log(lam) * fsq).sum(-1).cpu().numpy()
    for b in range(len(cases)):
        w0, S0 = np.linalg.eigh(H[b])
        want = np.sum(np.log(w0) * S0[0] ** 2)
        assert abs(got[b] - want) <= 1e-10 * max(abs(want), 1.0)


@pytest.mark.parametrize("k", [1, 2, 15, 16, 17, 32, 48, 64, 65, 100])
def test_tridiag_eigh_full_vectors(k):
    # mfg_tridiag_eigh: every eigenvector (the derivative of e1^T f(T) e1 uses them)
    rng = np.random.default_rng(2000 + k)
    kinds = KINDS if k > 2 else ["normal", "wilkinson", "zero"]
    cases = [_case(kind, k, rng) for kind in kinds] if k > 1 else [(rng.standard_normal(1), np.zeros(0))]
    H = _stack(cases)
    w, S = mf.funm.tridiag_eigh(torch.as_tensor(H, device="cuda"))
    w, S = w.cpu().numpy(), S.cpu().numpy()
    for b in range(len(cases)):
        T = H[b]
        scale = max(np.abs(np.linalg.eigvalsh(T)).max(), 1e-300)
        np.testing.assert_allclose(w[b], np.linalg.eigvalsh(T), rtol=0, atol=1e-12 * scale)
        np.testing.assert_allclose(S[b].T @ S[b], np.eye(k), atol=1e-12 * k)
        np.testing.assert_allclose((S[b] * w[b]) @ S[b].T, T, atol=1e-12 * k * scale)
