"""CUDA path vs the float64 oracle on identical inputs (needs a GPU).

Tolerances: float64 basis (precision "fp64") against the oracle to 1e-9;
float32 basis with float64 reductions to 1e-4 relative on log-determinants
(the bar for split-fp32 accuracy); the reference's own known-answer tests
with matfree's tolerances.
"""

import numpy as np
import pytest
import scipy.linalg
import torch

import matfree_gb300 as mf
from oracle import philox, problems, slq

pytestmark = pytest.mark.gpu

DEV = "cuda"


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=DEV)


# ----------------------------------------------------------------- samplers


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [1, 7, 1000, 4099])
def test_sampler_signs_bit_exact(dtype, n):
    key = mf.prng.prng_key(42)
    s = mf.stochtrace.sampler_signs(torch.ones(n, dtype=dtype, device=DEV), num=9)
    got = s(key).cpu().numpy()
    want = philox.rademacher(key, 9, n)
    np.testing.assert_array_equal(got, want)
    panel = s.panel(key)
    assert panel.stride(0) % 8 == 0


def test_sampler_normal_matches_oracle():
    key = mf.prng.prng_key(7)
    s = mf.stochtrace.sampler_normal(torch.ones(1003, device=DEV), num=17)
    got = s(key).double().cpu().numpy()
    want = philox.normal(key, 17, 1003)
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5)


def test_samplers_differ_per_key_and_are_deterministic():
    s = mf.stochtrace.sampler_signs(torch.ones(64, device=DEV), num=100)
    a = s(mf.prng.prng_key(1))
    assert torch.equal(a, s(mf.prng.prng_key(1)))
    assert not torch.equal(a, s(mf.prng.prng_key(2)))


# ---------------------------------------------------------- Arnoldi / CGS2


@pytest.mark.parametrize("n,k,p", [(50, 10, 3), (300, 25, 7), (2500, 40, 5)])
def test_hessenberg_fp64_matches_oracle(n, k, p):
    A = problems.dense_spd(n, seed=3)
    V = np.random.default_rng(5).standard_normal((p, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    Q, H, r, c = mf.decomp.run_hessenberg(op, k, _t(V))
    Qo, Ho, ro, co = slq.hessenberg_forward_batched(lambda X: X @ A.T, k, V)
    np.testing.assert_allclose(H.cpu().numpy(), Ho, atol=1e-9, rtol=1e-9)
    np.testing.assert_allclose(Q.cpu().numpy(), Qo, atol=1e-9)
    np.testing.assert_allclose(r.cpu().numpy(), ro, atol=1e-8)
    np.testing.assert_allclose(c.cpu().numpy(), co, rtol=1e-13)


@pytest.mark.parametrize("n,k,p", [(64, 16, 4), (5000, 30, 9)])
def test_hessenberg_fp32_matches_oracle(n, k, p):
    A = problems.dense_spd(n, seed=3)
    A32 = A.astype(np.float32).astype(np.float64)
    V = np.random.default_rng(5).standard_normal((p, n)).astype(np.float32)
    op = mf.DenseOperator(_t(A32, torch.float32), precision="fp32")
    _, H, _, _ = mf.decomp.run_hessenberg(op, k, _t(V, torch.float32))
    _, Ho, _, _ = slq.hessenberg_forward_batched(lambda X: X @ A32.T, k, V)
    d, e = slq.tridiag_from_hessenberg(H.cpu().numpy())
    do, eo = slq.tridiag_from_hessenberg(Ho)
    np.testing.assert_allclose(d, do, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(e, eo, rtol=1e-3, atol=1e-5)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_full_rank_reconstruction_is_exact(precision):
    # tests/test_decomp/test_tridiag_sym.py:7-38 through the CUDA path
    n = 12
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    A = problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))
    dt = torch.float64 if precision == "fp64" else torch.float32
    v = _t(np.flip(np.arange(1.0, 1.0 + n)).copy(), dt)
    op = mf.DenseOperator(_t(A, dt), precision=precision)
    Q, T, *_ = mf.decomp.tridiag_sym(n, reortho="full", materialize=True)(op, v)
    Q, T = Q.double().cpu().numpy(), T.double().cpu().numpy()
    assert np.allclose(Q.T @ T @ Q, A, atol=1e-5, rtol=1e-5)
    tol = 1e-6 if precision == "fp64" else 1e-5
    assert np.allclose(Q @ Q.T, np.eye(n), atol=tol)


@pytest.mark.parametrize("k", [1, 5, 11])
def test_mid_rank_reconstruction_satisfies_decomposition(k):
    # tests/test_decomp/test_tridiag_sym.py:43-65 (float64, matfree's double tolerance)
    n = 12
    eigvals = np.arange(1.0, 2.0, step=1 / n)
    A = problems.hermitian_matrix_from_eigenvalues(eigvals, np.random.default_rng(1))
    v = _t(np.flip(np.arange(1.0, 1.0 + n)).copy())
    Q, T, q, _ = mf.decomp.tridiag_sym(k)(mf.DenseOperator(_t(A), precision="fp64"), v)
    Q, T, q = (x.cpu().numpy() for x in (Q, T, q))
    e_K = np.eye(k)[-1]
    assert np.allclose(A @ Q.T - Q.T @ T - np.outer(q, e_K), 0.0, atol=1e-6)


@pytest.mark.parametrize("k", [5, 9])
def test_hessenberg_hilbert_needs_reortho(k):
    # tests/test_decomp/test_hessenberg.py:44-69
    n = 10
    A = scipy.linalg.hilbert(n)
    v = np.random.default_rng(2).standard_normal(n)
    Q, H, r, c = mf.decomp.hessenberg(k, reortho="full")(mf.DenseOperator(_t(A), precision="fp64"), _t(v))
    Q, H, r, c = (x.cpu().numpy() for x in (Q, H, r, c))
    ek = np.eye(k)[-1]
    assert np.allclose(A @ Q.T - Q.T @ H - np.outer(r, ek), 0.0, atol=1e-6)
    assert np.allclose(Q @ Q.T - np.eye(k), 0.0, atol=1e-6)
    assert np.allclose(Q.T[:, 0], c * v, atol=1e-6)


@pytest.mark.parametrize("k", [6, 13, 0])
def test_output_shapes(k):
    # tests/test_decomp/test_consistency.py:26-48
    n = 13
    rng = np.random.default_rng(1)
    A = rng.standard_normal((n, n))
    v0 = _t(rng.standard_normal(n), torch.float32)
    for alg in (mf.decomp.tridiag_sym(k), mf.decomp.hessenberg(k, reortho="full"),
                mf.decomp.hessenberg(k, reortho="none")):
        Us, B, res, ln = alg(lambda v: _t(A, torch.float32) @ v, v0)
        assert Us.shape == (k, n) and B.shape == (k, k) and res.shape == (n,) and ln.shape == ()


def test_hessenberg_without_reortho_matches_oracle():
    n, k = 40, 8
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, n))
    v = rng.standard_normal(n)
    Q, H, r, c = mf.decomp.hessenberg(k, reortho="none")(mf.DenseOperator(_t(A), precision="fp64"), _t(v))
    Qo, Ho, ro, co = slq.hessenberg_forward(lambda x: A @ x, k, v, reortho="none")
    np.testing.assert_allclose(H.cpu().numpy(), Ho, atol=1e-9)
    np.testing.assert_allclose(r.cpu().numpy(), ro, atol=1e-8)


def test_pytree_vector_and_callable_matvec():
    # the matvec protocol of tests/test_decomp/test_tridiag_sym.py:14-16 (pytree in/out)
    n = 12
    A = problems.dense_spd(n, seed=9)
    At = _t(A)
    vec = [(_t(np.arange(1.0, 1.0 + n)),)]

    def matvec(s, p):
        [(x,)] = s
        return [(p @ x,)]

    Q_tree, T, r_tree, c = mf.decomp.tridiag_sym(6)(matvec, vec, At)
    [(Q,)] = Q_tree
    Qo, To, ro, co = slq.tridiag_sym_full(lambda x: A @ x, 6, np.arange(1.0, 1.0 + n))
    np.testing.assert_allclose(Q.cpu().numpy(), Qo, atol=1e-9)
    np.testing.assert_allclose(T.cpu().numpy(), To, atol=1e-9)


# ----------------------------------------------------- quadrature and SLQ


@pytest.mark.parametrize("k", [1, 2, 17, 64, 100])
def test_tridiag_quadrature_matches_eigh(k):
    rng = np.random.default_rng(k)
    p = 33
    H = np.zeros((p, k, k))
    idx = np.arange(k)
    H[:, idx, idx] = rng.uniform(1, 3, size=(p, k))
    if k > 1:
        sub = rng.uniform(0.1, 0.5, size=(p, k - 1))
        sup = sub * (1 + 1e-3 * rng.standard_normal((p, k - 1)))
        H[:, idx[1:], idx[:-1]] = sub
        H[:, idx[:-1], idx[1:]] = sup
    lam, fsq = mf.funm.tridiag_eigh_first(_t(H))
    d, e = slq.tridiag_from_hessenberg(H)
    want = slq.quadrature_batched(d, e, np.log)
    got = (torch.log(lam) * fsq).sum(-1).cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-12)
    T = np.zeros((p, k, k))
    T[:, idx, idx] = d
    if k > 1:
        T[:, idx[:-1], idx[1:]] = e
        T[:, idx[1:], idx[:-1]] = e
    np.testing.assert_allclose(lam.cpu().numpy(), np.linalg.eigvalsh(T), atol=1e-12)


def test_logdet_spd_vs_slogdet():
    # tests/test_funm/test_monte_carlo_funm_sym_logdet.py:16-38 (10 normal probes)
    n = 200
    rng = np.random.default_rng(1)
    A = problems.make_A_logdet(n, 30, rng)
    op = mf.DenseOperator(_t(A, torch.float32), precision="fp32")
    sampler = mf.stochtrace.sampler_normal(torch.ones(n, device=DEV), num=10)
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(10))
    received = float(mf.stochtrace.estimator_monte_carlo(integrand, sampler)(op, mf.prng.prng_key(1)))
    expected = np.linalg.slogdet(A)[1]
    assert np.allclose(received, expected, atol=1e-2, rtol=1e-2)


def test_logdet_exact_for_full_num_matvecs():
    # tests/test_funm/test_monte_carlo_funm_sym_logdet.py:41-67 (float64 path)
    n = 50
    A = problems.hermitian_matrix_from_eigenvalues(np.arange(1.0, 1.0 + n), np.random.default_rng(1))
    x = np.random.default_rng(1).standard_normal(n) + 10
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(n - 1))
    received = float(integrand(mf.DenseOperator(_t(A), precision="fp64"), _t(x)))
    w, V = np.linalg.eigh(A)
    expected = x @ (V @ np.diag(np.log(w)) @ V.T) @ x
    assert np.allclose(received, expected)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-4)])
def test_slq_dense_config1_scale_vs_oracle(precision, tol):
    # dense SPD A = B B^T / n + I, n = 1000, k = 30, p = 100 Rademacher probes
    n, k, p = 1000, 30, 100
    A = problems.dense_spd(n, seed=0)
    key = mf.prng.prng_key(1)
    dt = torch.float64 if precision == "fp64" else torch.float32
    Ad = A if precision == "fp64" else A.astype(np.float32).astype(np.float64)
    op = mf.DenseOperator(_t(Ad, dt), precision=precision)
    sampler = mf.stochtrace.sampler_signs(torch.ones(n, dtype=dt, device=DEV), num=p)
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    mean, sem = mf.stochtrace.estimator_monte_carlo_mean_and_sem(integrand, sampler)(op, key)
    V = philox.rademacher(key, p, n)
    vals = slq.slq_batched(lambda X: X @ Ad.T, k, V)
    assert abs(float(mean) - vals.mean()) <= tol * abs(vals.mean())
    np.testing.assert_allclose(float(sem), vals.std() / np.sqrt(p), rtol=max(tol, 1e-8) * 100)
    exact = np.linalg.slogdet(A)[1]
    assert abs(float(mean) - exact) < 5 * float(sem) + 1e-3 * abs(exact)


def test_slq_csr_laplacian_vs_oracle():
    m, k, p = 64, 30, 16
    L = problems.laplacian_2d(m, shift=0.1)
    op = mf.CSROperator.from_scipy(L)
    key = mf.prng.prng_key(3)
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    sampler = mf.stochtrace.sampler_signs(torch.ones(m * m, device=DEV), num=p)
    got = float(mf.stochtrace.estimator_monte_carlo(integrand, sampler)(op, key))
    V = philox.rademacher(key, p, m * m)
    L64 = L.astype(np.float64)
    want = slq.slq_batched(lambda X: (L64 @ X.T).T, k, V).mean()
    assert abs(got - want) <= 1e-4 * abs(want)


def test_csr_shift_matches_explicit_diagonal():
    m = 20
    L0 = problems.laplacian_2d(m, shift=0.0)
    L1 = problems.laplacian_2d(m, shift=0.1)
    V = torch.randn(5, m * m, device=DEV)
    a = mf.CSROperator.from_scipy(L0, shift=0.1).matmat(V)
    b = mf.CSROperator.from_scipy(L1).matmat(V)
    torch.testing.assert_close(a, b, rtol=1e-6, atol=1e-5)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_rbf_build_matches_oracle(precision):
    n = 300
    x = problems.rbf_points(n, seed=2).astype(np.float32)
    op = mf.RBFKernelOperator(_t(x, torch.float32), precision=precision)
    K = problems.rbf_kernel(x.astype(np.float64))
    tol = 1e-12 if precision == "fp64" else 2e-7
    np.testing.assert_allclose(op.dense().cpu().numpy(), K, atol=tol)


def test_callback_operator_matches_dense():
    n, k, p = 300, 20, 8
    A = problems.dense_spd(n, seed=11)
    At = _t(A, torch.float32)
    V = torch.randn(p, n, device=DEV)
    cb = mf.CallbackOperator(lambda X: X @ At.T, n, batched=True)
    dense = mf.DenseOperator(At, precision="fp32")
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    a = integrand.batched(cb, V)
    b = integrand.batched(dense, V)
    torch.testing.assert_close(a, b, rtol=1e-5, atol=1e-5)


def test_general_matrix_function_exp():
    n, k, p = 200, 25, 6
    A = problems.dense_spd(n, seed=4) / 4
    V = np.random.default_rng(8).standard_normal((p, n))
    op = mf.DenseOperator(_t(A), precision="fp64")
    f = lambda x: torch.exp(-0.1 * x)  # noqa: E731  (arbitrary torch callable path)
    integrand = mf.funm.monte_carlo_funm_sym(mf.funm.dense_funm_sym_eigh(f), mf.decomp.tridiag_sym(k))
    got = integrand.batched(op, _t(V)).cpu().numpy()
    fused = mf.funm.monte_carlo_funm_sym(mf.funm.funm_exp(-0.1), mf.decomp.tridiag_sym(k))
    got2 = fused.batched(op, _t(V)).cpu().numpy()
    want = slq.slq_batched(lambda X: X @ A.T, k, V, matfun=lambda x: np.exp(-0.1 * x))
    np.testing.assert_allclose(got, want, rtol=1e-10)
    np.testing.assert_allclose(got2, want, rtol=1e-10)


def test_funm_lanczos_sym_logm_vector():
    n, k = 60, 59
    A = problems.hermitian_matrix_from_eigenvalues(np.linspace(1, 3, n), np.random.default_rng(2))
    v = np.random.default_rng(3).standard_normal(n)
    fn = mf.funm.funm_lanczos_sym(mf.funm.dense_funm_sym_eigh(torch.log), mf.decomp.tridiag_sym(k))
    got = fn(mf.DenseOperator(_t(A), precision="fp64"), _t(v)).cpu().numpy()
    w, U = np.linalg.eigh(A)
    want = U @ (np.log(w) * (U.T @ v))
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-8)


# ------------------------------------------------------- tensor-core apply


@pytest.mark.parametrize("precision,tol", [("bf16x3", 5e-5), ("bf16", 1.5e-2)])
@pytest.mark.parametrize("n,p", [(64, 16), (200, 1), (300, 100), (1000, 256), (777, 300),
                                 # CTA-pair (2-SM) form: even and ragged 256-row tiles,
                                 # one and two probe tiles, a probe tile of 64; the
                                 # first three also split K over two CTAs
                                 (1024, 256), (1500, 256), (2600, 300), (1300, 64), (1100, 40),
                                 # long K (one TMEM accumulator over K = 16384) and a
                                 # ragged split K over two CTAs
                                 (4608, 256), (16384, 256), (9000, 96),
                                 # GEMV form (p <= 8): ragged column tails, 5 and 8 probes
                                 (203, 1), (1001, 5), (4099, 8)])
def test_dense_tensor_core_apply(precision, tol, n, p):
    rng = np.random.default_rng(n + p)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    V = rng.standard_normal((p, n))
    op = mf.DenseOperator(_t(A, torch.float32), precision=precision, shift=0.5)
    W = op.matmat(_t(V, torch.float32)).double().cpu().numpy()
    A32 = A.astype(np.float32).astype(np.float64)
    V32 = V.astype(np.float32).astype(np.float64)
    want = V32 @ A32.T + 0.5 * V32
    err = np.abs(W - want).max() / np.abs(want).max()
    # the tensor pipe's fp32 accumulation truncates: the error of one output
    # grows with K (about 3e-5 of bias at K = 16384), so long K gets twice the
    # tolerance of the short cases
    assert err < tol * max(1.0, n / 8192), err


@pytest.mark.parametrize("precision,tol", [("bf16x3", 1e-4), ("fp32", 1e-4), ("bf16", 3e-3)])
def test_slq_rbf_precisions_vs_fp64(precision, tol):
    n, k, p = 2048, 40, 32
    x = problems.rbf_points(n, seed=0).astype(np.float32)
    op = mf.RBFKernelOperator(_t(x, torch.float32), precision=precision)
    key = mf.prng.prng_key(5)
    V = philox.rademacher(key, p, n)
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    got = float(integrand.batched(op, _t(V, torch.float32)).mean())
    if precision == "bf16":
        # Plain bf16 storage perturbs K by ~2^-9 per entry, far more than the
        # 1e-2 nugget tolerates; parity is checked against float64 SLQ of the
        # operator as stored (bf16 entries + exact nugget), on the same probes.
        K = op.dense().cpu().numpy()
    else:
        K = problems.rbf_kernel(x.astype(np.float64))
    want = slq.slq_batched(lambda X: X @ K, k, V).mean()
    assert abs(got - want) <= tol * abs(want), (got, want, abs(got - want) / abs(want))


# ------------------------------------------------------------ DLPack intake


class _DLPackOnly:
    """A CUDA array that exports its memory only through the DLPack protocol
    (as CuPy, JAX or Numba arrays do)."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, stream=None, **kwargs):
        return self._t.__dlpack__(stream=stream) if stream is not None else self._t.__dlpack__()

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_dlpack_inputs_give_the_torch_results():
    n, k, p = 700, 20, 12
    A = problems.dense_spd(n, seed=5)
    At = _t(A, torch.float32)
    V = _t(np.random.default_rng(3).standard_normal((p, n)), torch.float32)
    integrand = mf.funm.monte_carlo_funm_sym_logdet(mf.decomp.tridiag_sym(k))
    want = integrand.batched(mf.DenseOperator(At), V)
    op = mf.DenseOperator(_DLPackOnly(At))
    got = integrand.batched(op, _DLPackOnly(V))
    torch.testing.assert_close(got, want, rtol=0, atol=0)
    got2 = integrand.batched(op, torch.utils.dlpack.to_dlpack(V))
    torch.testing.assert_close(got2, want, rtol=0, atol=0)
    # the sampler's x_like and the RBF points may be DLPack producers as well
    s = mf.stochtrace.sampler_signs(_DLPackOnly(torch.ones(n, device=DEV)), num=p)
    key = mf.prng.prng_key(3)
    est = mf.stochtrace.estimator_monte_carlo(integrand, s)(op, key)
    np.testing.assert_allclose(float(est), float(integrand.batched(mf.DenseOperator(At), s(key)).mean()),
                               rtol=0, atol=0)
    x = _t(problems.rbf_points(300, seed=1), torch.float32)
    a = mf.RBFKernelOperator(_DLPackOnly(x), precision="fp32").dense()
    b = mf.RBFKernelOperator(x, precision="fp32").dense()
    assert torch.equal(a, b)


@pytest.mark.parametrize("bn,split", [(128, 1), (64, 1), (128, 2), (0, 2), (0, 1)])
def test_tensor_core_apply_under_tile_rules(bn, split):
    # every tile configuration the autotuner may install gives the same product
    from matfree_gb300 import _lib

    n, p = 4608, 256
    rng = np.random.default_rng(17)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    V = rng.standard_normal((p, n))
    lib = _lib.lib()
    try:
        assert lib.mfg_gemm_tuning_add(n, n, p, p, bn, split) == 0
        op = mf.DenseOperator(_t(A, torch.float32), precision="bf16x3", shift=0.5)
        W = op.matmat(_t(V, torch.float32)).double().cpu().numpy()
    finally:
        lib.mfg_gemm_tuning_clear()
    A32 = A.astype(np.float32).astype(np.float64)
    V32 = V.astype(np.float32).astype(np.float64)
    want = V32 @ A32.T + 0.5 * V32
    assert np.abs(W - want).max() / np.abs(want).max() < 5e-5


def test_autotuner_installs_rules_that_keep_the_product():
    from matfree_gb300 import _lib, tuning

    try:
        rules = tuning.autotune(ns=(1024, 2048), ps=(64, 256), reps=1)
        assert len(rules) == 4
        assert all(r["ms"] <= r["default_ms"] + 1e-9 for r in rules)
        n, p = 2048, 256
        rng = np.random.default_rng(3)
        A = rng.standard_normal((n, n)) / np.sqrt(n)
        V = rng.standard_normal((p, n))
        W = mf.DenseOperator(_t(A, torch.float32), precision="bf16x3").matmat(_t(V, torch.float32))
        want = V.astype(np.float32).astype(np.float64) @ A.astype(np.float32).astype(np.float64).T
        assert np.abs(W.double().cpu().numpy() - want).max() / np.abs(want).max() < 5e-5
    finally:
        _lib.lib().mfg_gemm_tuning_clear()


@pytest.mark.parametrize("precision", ["bf16x3", "bf16"])
@pytest.mark.parametrize("n,p", [(4608, 256),    # 18 tiles: each split in two halves on 36 pairs
                                 (16384, 256),   # 64 tiles on 76 pairs: 6 tails per spare pair
                                 (20000, 64),    # 79 tiles: a full wave, the rest unsplit (no mixed rows)
                                 (5000, 700),    # three probe tiles (256, 256, 188)
                                 (3000, 96)])
def test_persistent_pair_form_matches_float64_and_is_deterministic(precision, n, p):
    from matfree_gb300 import _lib

    rng = np.random.default_rng(n + p)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    V = rng.standard_normal((p, n))
    lib = _lib.lib()
    try:
        assert lib.mfg_gemm_tuning_add(n, n, p, p, 0, 3) == 0
        op = mf.DenseOperator(_t(A, torch.float32), precision=precision, shift=0.5)
        Vt = _t(V, torch.float32)
        W1 = op.matmat(Vt)
        W2 = op.matmat(Vt)
        lib.mfg_gemm_tuning_clear()
        assert lib.mfg_gemm_tuning_add(n, n, p, p, 0, 1) == 0
        W0 = op.matmat(Vt)
    finally:
        lib.mfg_gemm_tuning_clear()
    # two partial products per split tile: the sum does not depend on timing
    assert torch.equal(W1, W2)
    if precision == "bf16":
        A_s = op.dense().double().cpu().numpy() - 0.5 * np.eye(n)
        V_s = V.astype(np.float32).astype(np.float64)
        V_b = torch.tensor(V_s).to(torch.bfloat16).double().numpy()
        want = V_b @ A_s.T + 0.5 * V_s
    else:
        A32 = A.astype(np.float32).astype(np.float64)
        V32 = V.astype(np.float32).astype(np.float64)
        want = V32 @ A32.T + 0.5 * V32
    tol = 5e-5  # the tensor pipe's truncating fp32 accumulation, as in the apply tests
    W = W1.double().cpu().numpy()
    err = np.abs(W - want).max() / np.abs(want).max()
    assert err < tol * max(1.0, n / 8192), err
    # against one tile per pair: the same product up to the K split's rounding
    d = (W1.double() - W0.double()).abs().max().item() / np.abs(want).max()
    assert d < 2 * tol * max(1.0, n / 8192), d
