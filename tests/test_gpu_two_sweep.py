"""Full reorthogonalisation in two reads of the basis per step (reortho mode 3,
``mfg_slq_ex`` with MFG_SLQ_TWO_SWEEP) against the three-read form and the
oracle (needs a GPU).

Tolerances: the tridiagonal parts against the float64 oracle and against the
three-read form as for reortho="full" in float32 (1e-4 relative on the
diagonal, 1e-3 on the off-diagonal), bases and residuals to 1e-3; the two
GPU forms to 1e-5 relative on log-determinant values.  Near an invariant subspace the device
reports MFG_ERR_RETRY and the Python entry points repeat the solve with the
three-read form, whose results they then return bit for bit.
"""

import ctypes

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import _lib
from matfree_gb300._panel import Workspace
from matfree_gb300.decomp import run_hessenberg
from matfree_gb300.funm import slq_retry_needed, slq_values
from oracle import problems, slq

pytestmark = pytest.mark.gpu


def _t(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


@pytest.mark.parametrize("n,k,p", [(300, 2, 3), (300, 40, 5), (1000, 64, 4), (700, 65, 3),
                                   (700, 66, 2), (1500, 100, 3), (900, 129, 2)])
def test_two_sweep_hessenberg_matches_oracle_and_three_sweep(n, k, p):
    A = problems.dense_spd(n, seed=n + k)
    A32 = A.astype(np.float32).astype(np.float64)
    V = np.random.default_rng(k).standard_normal((p, n)).astype(np.float32)
    op = mf.DenseOperator(_t(A32, torch.float32), precision="fp32")
    Q2, H2, R2, c2 = run_hessenberg(op, k, _t(V, torch.float32), reortho="full-two-sweep")
    Q1, H1, R1, c1 = run_hessenberg(op, k, _t(V, torch.float32), reortho="full")
    # tridiagonal parts against the oracle, as for reortho="full" in float32
    _, Ho, _, _ = slq.hessenberg_forward_batched(lambda X: X @ A32.T, k, V)
    d, e = slq.tridiag_from_hessenberg(H2.cpu().numpy())
    do, eo = slq.tridiag_from_hessenberg(Ho)
    np.testing.assert_allclose(d, do, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(e, eo, rtol=1e-3, atol=1e-5)
    # and against the three-read form on the GPU
    d1, e1 = slq.tridiag_from_hessenberg(H1.cpu().numpy())
    np.testing.assert_allclose(d, d1, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(e, e1, rtol=1e-3, atol=1e-5)
    np.testing.assert_allclose(Q2.cpu().numpy(), Q1.cpu().numpy(), atol=1e-3)
    r1 = R1.cpu().numpy()
    np.testing.assert_allclose(R2.cpu().numpy(), r1, atol=1e-3 * np.abs(r1).max())
    np.testing.assert_allclose(c2.cpu().numpy(), c1.cpu().numpy(), rtol=1e-12)


def test_two_sweep_orthonormal_basis():
    n, k, p = 2000, 64, 3
    A = problems.dense_spd(n, seed=3)
    V = np.random.default_rng(5).standard_normal((p, n))
    op = mf.DenseOperator(_t(A, torch.float32), precision="fp32")
    Q, _, _, _ = run_hessenberg(op, k, _t(V, torch.float32), reortho="full-two-sweep")
    Q = Q.double()
    G = Q @ Q.transpose(1, 2)
    err = (G - torch.eye(k, dtype=torch.float64, device="cuda")).abs().max().item()
    assert err < 1e-5


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_two_sweep_slq_values_match_three_sweep(precision):
    rng = np.random.default_rng(11)
    x = torch.as_tensor(rng.random((2048, 3)), dtype=torch.float32, device="cuda")
    op = mf.RBFKernelOperator(x, s2=1.0, ell=0.2, tau=1e-2, precision=precision)
    V = mf.stochtrace.sampler_signs(torch.ones(2048, device="cuda"), num=16)(mf.prng.prng_key(3))
    v2 = slq_values(op, 64, V, _lib.MFG_FUN_LOG, 0.0, two_sweep=True)
    v1 = slq_values(op, 64, V, _lib.MFG_FUN_LOG, 0.0, two_sweep=False)
    np.testing.assert_allclose(v2.cpu().numpy(), v1.cpu().numpy(), rtol=1e-5)


def test_two_sweep_falls_back_near_an_invariant_subspace():
    # rank-10 operator plus 1e-8 I: the Krylov space is exhausted after ~10
    # steps, a vector is left inside the basis by one projection, and the
    # device asks for the three-read form
    n, k, p = 200, 30, 2
    rng = np.random.default_rng(0)
    U = rng.standard_normal((n, 10))
    A = U @ U.T + 1e-8 * np.eye(n)
    op = mf.DenseOperator(_t(A, torch.float32), precision="fp32")
    V = _t(rng.standard_normal((p, n)), torch.float32)
    ws = Workspace()
    slq_values(op, k, V, _lib.MFG_FUN_EXP, -1e-3, workspace=ws, two_sweep=True, check=False)
    assert slq_retry_needed(ws)
    got = slq_values(op, k, V, _lib.MFG_FUN_EXP, -1e-3, two_sweep=True)
    want = slq_values(op, k, V, _lib.MFG_FUN_EXP, -1e-3, two_sweep=False)
    assert torch.equal(got, want)
    Q2, H2, _, _ = run_hessenberg(op, k, V, reortho="full-two-sweep")
    Q1, H1, _, _ = run_hessenberg(op, k, V, reortho="full")
    assert torch.equal(H2, H1) and torch.equal(Q2, Q1)


def test_two_sweep_outside_its_range_is_the_three_sweep_form():
    # k = 130 and float64 bases run the three-read form unchanged
    n = 300
    A = problems.dense_spd(n, seed=1)
    V = np.random.default_rng(2).standard_normal((2, n))
    op = mf.DenseOperator(_t(A, torch.float32), precision="fp32")
    _, H2, _, _ = run_hessenberg(op, 130, _t(V, torch.float32), reortho="full-two-sweep")
    _, H1, _, _ = run_hessenberg(op, 130, _t(V, torch.float32), reortho="full")
    assert torch.equal(H2, H1)
    op64 = mf.DenseOperator(_t(A), precision="fp64")
    _, H2, _, _ = run_hessenberg(op64, 20, _t(V), reortho="full-two-sweep")
    _, H1, _, _ = run_hessenberg(op64, 20, _t(V), reortho="full")
    assert torch.equal(H2, H1)


def test_slq_ex_workspace_and_flags():
    n, k, p = 256, 16, 4
    op = mf.DenseOperator(_t(problems.dense_spd(n, seed=4), torch.float32), precision="fp32")
    s = op.c_struct()
    lib = _lib.lib()
    plain = lib.mfg_slq_workspace_bytes(ctypes.byref(s), k, p, n)
    two = lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, n, _lib.MFG_SLQ_TWO_SWEEP)
    assert two > plain
    assert lib.mfg_slq_ex_workspace_bytes(ctypes.byref(s), k, p, n, 0) == plain
    V = torch.zeros((p, n), device="cuda")
    vals = torch.zeros(p, dtype=torch.float64, device="cuda")
    ws = torch.empty(two, dtype=torch.uint8, device="cuda")
    st = lib.mfg_slq_ex(ctypes.byref(s), k, p, ctypes.c_void_p(V.data_ptr()), n, _lib.MFG_FUN_LOG,
                        0.0, ctypes.c_void_p(vals.data_ptr()), None, None, None, 4,
                        ctypes.c_void_p(ws.data_ptr()), two, None)
    assert st == _lib.MFG_ERR_BAD_ARG
    st = lib.mfg_slq_ex(ctypes.byref(s), k, p, ctypes.c_void_p(V.data_ptr()), n, _lib.MFG_FUN_LOG,
                        0.0, ctypes.c_void_p(vals.data_ptr()), None, None, None,
                        _lib.MFG_SLQ_TWO_SWEEP, ctypes.c_void_p(ws.data_ptr()), plain, None)
    assert st == _lib.MFG_ERR_WORKSPACE
