"""Pin the float64 oracle against the known-answer tests of matfree's own suite.

Each test names the matfree test it ports.  JAX keys are replaced by NumPy
generators; where matfree compares against JAX autodiff, central finite
differences of the forward pass stand in.
"""

import numpy as np
import pytest
import scipy.linalg

from oracle import adjoint, problems, slq


def _tol(dtype=np.float64):
    # matfree/test_util.py:80-84: 10 sqrt(eps), times 10 again in double precision
    tol = 10 * np.sqrt(np.finfo(dtype).eps)
    return tol * 10 if tol < 1e-6 else tol


# tests/test_decomp/test_tridiag_sym.py:7-38
def test_full_rank_reconstruction_is_exact():
    n = 12
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    A = problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))
    v = np.flip(np.arange(1.0, 1.0 + n))
    Q, T, _, _ = slq.tridiag_sym_full(lambda x: A @ x, n, v)
    assert np.allclose(Q.T @ T @ Q, A, atol=1e-5, rtol=1e-5)
    assert np.allclose(Q @ Q.T, np.eye(n), atol=_tol())
    assert np.allclose(Q.T @ Q, np.eye(n), atol=_tol())


# tests/test_decomp/test_tridiag_sym.py:43-65
@pytest.mark.parametrize("k", [1, 5, 11])
def test_mid_rank_reconstruction_satisfies_decomposition(k):
    n = 12
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    A = problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))
    v = np.flip(np.arange(1.0, 1.0 + n))
    Q, T, q, _ = slq.tridiag_sym_full(lambda x: A @ x, k, v)
    e_K = np.eye(k)[-1]
    assert np.allclose(A @ Q.T - Q.T @ T - np.outer(q, e_K), 0.0, atol=_tol())


# tests/test_decomp/test_hessenberg.py:7-41
@pytest.mark.parametrize("k", [0, 5, 9])
@pytest.mark.parametrize("reortho", ["none", "full"])
def test_hessenberg_decomposition_is_satisfied(k, reortho):
    rng = np.random.default_rng(1)
    n = 10
    A = rng.standard_normal((n, n))
    v = rng.standard_normal(n)
    Q, H, r, c = slq.hessenberg_forward(lambda x: A @ x, k, v, reortho=reortho)
    assert Q.shape == (n, k) and H.shape == (k, k) and r.shape == (n,) and np.shape(c) == ()
    ek = np.eye(k)[-1] if k else np.zeros(0)
    assert np.allclose(A @ Q - Q @ H - np.outer(r, ek), 0.0, atol=_tol())
    assert np.allclose(Q.T @ Q - np.eye(k), 0.0, atol=_tol())
    if k > 0:
        assert np.allclose(Q[:, 0], c * v, atol=_tol())


# tests/test_decomp/test_hessenberg.py:44-69 (Hilbert matrix needs reortho)
@pytest.mark.parametrize("k", [5, 9])
def test_reorthogonalisation_hilbert(k):
    n = 10
    A = scipy.linalg.hilbert(n)
    v = np.random.default_rng(2).standard_normal(n)
    Q, H, r, c = slq.hessenberg_forward(lambda x: A @ x, k, v, reortho="full")
    ek = np.eye(k)[-1]
    assert np.allclose(A @ Q - Q @ H - np.outer(r, ek), 0.0, atol=_tol())
    assert np.allclose(Q.T @ Q - np.eye(k), 0.0, atol=_tol())
    assert np.allclose(Q[:, 0], c * v, atol=_tol())


# tests/test_decomp/test_hessenberg.py:72-75
@pytest.mark.parametrize("wrong", [True, "full_with_sparsity", "None"])
def test_hessenberg_wrong_flag(wrong):
    with pytest.raises(TypeError, match="Unexpected input"):
        slq.hessenberg_forward(lambda x: x, 1, np.ones(3), reortho=wrong)


# tests/test_decomp/test_consistency.py:26-63
@pytest.mark.parametrize("k", [6, 13, 0])
def test_output_shapes(k):
    rng = np.random.default_rng(1)
    n = 13
    A = rng.standard_normal((n, n))
    v = rng.standard_normal(n)
    Q, T, r, c = slq.tridiag_sym_full(lambda x: A @ x, k, v)
    assert Q.shape == (k, n) and T.shape == (k, k) and r.shape == (n,) and np.shape(c) == ()


@pytest.mark.parametrize("k", [-1, 14])
def test_value_error_for_unusual_num_matvecs(k):
    n = 13
    with pytest.raises(ValueError, match="exceeds"):
        slq.tridiag_sym_full(lambda x: x, k, np.ones(n))


# tests/test_funm/test_monte_carlo_funm_sym_logdet.py:16-38
def test_logdet_spd():
    n = 200
    rng = np.random.default_rng(1)
    A = problems.make_A_logdet(n, 30, rng)
    samples = rng.standard_normal((10, n))
    integrand = slq.monte_carlo_funm_sym_logdet(10)
    received = slq.estimator_monte_carlo(integrand, lambda x: A @ x, samples)
    expected = np.linalg.slogdet(A)[1]
    assert np.allclose(received, expected, atol=1e-2, rtol=1e-2)


# tests/test_funm/test_monte_carlo_funm_sym_logdet.py:41-67
def test_logdet_exact_for_full_num_matvecs():
    n = 50
    A = problems.hermitian_matrix_from_eigenvalues(np.arange(1.0, 1.0 + n), np.random.default_rng(1))
    x = np.random.default_rng(1).standard_normal(n) + 10
    received = slq.monte_carlo_funm_sym_logdet(n - 1)(lambda v: A @ v, x)
    w, V = np.linalg.eigh(A)
    expected = x @ (V @ np.diag(np.log(w)) @ V.T) @ x
    assert np.allclose(received, expected)


def test_batched_matches_single_vector_path():
    """The probe-panel restatement runs the same arithmetic as the per-vector one."""
    rng = np.random.default_rng(3)
    n, k, p = 40, 12, 5
    A = problems.dense_spd(n, seed=4)
    V = rng.standard_normal((p, n))
    single = np.array([slq.monte_carlo_funm_sym_logdet(k)(lambda x: A @ x, v) for v in V])
    batched = slq.slq_batched(lambda X: X @ A.T, k, V)
    np.testing.assert_allclose(batched, single, rtol=1e-12)
    Qb, Hb, rb, cb = slq.hessenberg_forward_batched(lambda X: X @ A.T, k, V)
    for b in range(p):
        Q, H, r, c = slq.hessenberg_forward(lambda x: A @ x, k, V[b])
        np.testing.assert_allclose(Qb[b], Q.T, atol=1e-12)
        np.testing.assert_allclose(Hb[b], H, atol=1e-12)
        np.testing.assert_allclose(rb[b], r, atol=1e-12)
        np.testing.assert_allclose(cb[b], c, rtol=1e-14)


def test_mean_and_sem_matches_mean():
    """tests/test_stochtrace/test_monte_carlo/test_estimator_mean_and_std.py:7-28."""
    n = 30
    A = problems.dense_spd(n, seed=2)
    samples = np.random.default_rng(5).choice([-1.0, 1.0], size=(20, n))
    integrand = slq.monte_carlo_funm_sym_logdet(8)
    mean = slq.estimator_monte_carlo(integrand, lambda x: A @ x, samples)
    mean2, sem = slq.estimator_monte_carlo_mean_and_sem(integrand, lambda x: A @ x, samples)
    assert np.allclose(mean, mean2) and sem > 0


# tests/test_decomp/test_hessenberg_adjoint.py:5-40 (complex-step differentiation replaces autodiff)
def _fd_check_hessenberg_adjoint(A, v, k, seed, rtol):
    n = len(v)
    rng = np.random.default_rng(seed)

    def fwd(v_, A_):
        return slq.hessenberg_forward(lambda x: A_ @ x, k, v_, reortho="full")

    Q, H, r, c = fwd(v, A)
    dQ, dH, dr = rng.standard_normal(Q.shape), rng.standard_normal(H.shape), rng.standard_normal(r.shape)
    dc = rng.standard_normal()

    def vjp_matvec(q, lam):
        return A.T @ lam, (np.outer(lam, q),)

    dv, (dA,) = adjoint.hessenberg_adjoint(
        vjp_matvec, (A,), Q=Q, H=H, r=r, c=c, dQ=dQ, dH=dH, dr=dr, dc=dc, reortho="full"
    )

    def scalar(v_, A_):
        Q_, H_, r_, c_ = fwd(v_, A_)
        return np.sum(dQ * Q_) + np.sum(dH * H_) + np.sum(dr * r_) + dc * c_

    # complex-step differentiation: the forward pass is analytic (no conjugation),
    # so Im f(x + i h t) / h is the directional derivative to rounding accuracy
    h = 1e-30
    tv = rng.standard_normal(n)
    tA = rng.standard_normal(A.shape)
    fd_v = np.imag(scalar(v + 1j * h * tv, A)) / h
    fd_A = np.imag(scalar(v.astype(complex), A + 1j * h * tA)) / h
    assert np.isclose(fd_v, dv @ tv, rtol=rtol, atol=rtol)
    assert np.isclose(fd_A, np.sum(dA * tA), rtol=rtol, atol=rtol)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_hessenberg_adjoint_matches_finite_differences(seed):
    rng = np.random.default_rng(seed)
    n, k = 6, 4
    A = rng.standard_normal((n, n))
    v = rng.standard_normal(n)
    _fd_check_hessenberg_adjoint(A, v, k, seed + 10, rtol=1e-8)


# tests/test_decomp/test_hessenberg_adjoint.py:64-107 (Hilbert matrix, full reortho)
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_hessenberg_adjoint_hilbert(seed):
    n, k = 15, 10
    A = np.tril(scipy.linalg.hilbert(n))
    A = A - 0.5 * np.diag(np.diag(A))
    S = A + A.T
    v = np.random.default_rng(seed).standard_normal(n)
    _fd_check_hessenberg_adjoint(S, v, k, seed + 20, rtol=1e-3)  # matfree's tolerance


def test_hessenberg_adjoint_k_zero_raises():
    with pytest.raises(ValueError, match="= 0"):
        adjoint.hessenberg_adjoint(
            None, (), Q=np.zeros((3, 0)), H=np.zeros((0, 0)), r=np.zeros(3), c=1.0,
            dQ=np.zeros((3, 0)), dH=np.zeros((0, 0)), dr=np.zeros(3), dc=0.0,
        )


def test_batched_adjoint_matches_single():
    rng = np.random.default_rng(7)
    n, k, p = 9, 5, 3
    A = problems.dense_spd(n, seed=1)
    V = rng.standard_normal((p, n))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    Qb, Hb, rb, cb = slq.hessenberg_forward_batched(lambda X: X @ A.T, k, V)
    dH = rng.standard_normal((p, k, k))

    def vjp_matmat(Qp, Lp):
        return Lp @ A, np.array([np.sum(Lp * Qp)])

    dvb, dpb = adjoint.hessenberg_adjoint_batched(vjp_matmat, 1, Q=Qb, H=Hb, r=rb, dH=dH, c=cb)
    total = 0.0
    for b in range(p):
        dv, (dp,) = adjoint.hessenberg_adjoint(
            lambda q, lam: (A.T @ lam, (np.array(lam @ q),)), (0.0,),
            Q=Qb[b].T, H=Hb[b], r=rb[b], c=cb[b], dQ=np.zeros((n, k)), dH=dH[b],
            dr=np.zeros(n), dc=0.0,
        )
        np.testing.assert_allclose(dvb[b], dv, atol=1e-10)
        total += dp
    np.testing.assert_allclose(dpb[0], total, rtol=1e-10)


def test_slq_gradient_rbf_matches_central_differences():
    """d logdet / d theta for the RBF operator: adjoint vs central FD (h = 1e-4, float64)."""
    x = problems.rbf_points(60, seed=3)
    theta = np.array([0.0, np.log(0.2), np.log(1e-2)])
    V = np.random.default_rng(4).choice([-1.0, 1.0], size=(6, 60))
    k = 12

    def value(th):
        K, _, _ = adjoint.rbf_matrices(x, th)
        return slq.slq_batched(lambda X: X @ K.T, k, V).mean()

    matmat, vjp_matmat = adjoint.rbf_vjp_factory(x, theta)
    val, grad = adjoint.slq_grad_batched(matmat, vjp_matmat, 3, k, V)
    assert np.isclose(val, value(theta), rtol=1e-12)
    h = 1e-4
    for i in range(3):
        e = np.zeros(3)
        e[i] = h
        fd = (value(theta + e) - value(theta - e)) / (2 * h)
        assert np.isclose(grad[i], fd, rtol=1e-5, atol=1e-6), (i, grad[i], fd)


# tests/test_funm/test_funm_lanczos_sym.py:7-37 (sin, n = 11, k = 6, atol 1e-6)
def test_funm_lanczos_sym_matches_eigh_implementation():
    n = 11
    rng = np.random.default_rng(2)
    v = rng.standard_normal(n)
    A = problems.hermitian_matrix_from_eigenvalues(np.linspace(0.01, 0.99, num=n), np.random.default_rng(1))
    w, U = np.linalg.eigh(A)
    expected = U @ np.diag(np.sin(w)) @ U.T @ v
    fn = slq.funm_lanczos_sym(slq.dense_funm_sym_eigh(np.sin), 6)
    received = fn(lambda x: A @ x, v)
    assert np.allclose(expected, received, atol=1e-6)
