"""Shapes at kernel-configuration boundaries (launch limits, tile edges)."""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from oracle import problems, slq

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,k", [(torch.float32, 64), (torch.float64, 30)])
def test_fused_projection_across_the_default_shared_memory_limit(dtype, k):
    # the fused update+projection needs ~1 KB (float) / 2 KB (double) of shared
    # memory per basis vector: these depths cross the 48 KB default limit,
    # including the window just below it that the static shared memory eats
    n, p = 1000, 6
    A = problems.dense_spd(n, seed=5)
    V = np.random.default_rng(6).standard_normal((p, n))
    prec = "fp64" if dtype == torch.float64 else "fp32"
    Ad = A if dtype == torch.float64 else A.astype(np.float32).astype(np.float64)
    op = mf.DenseOperator(torch.tensor(Ad, dtype=dtype, device="cuda"), precision=prec)
    _, H, _, _ = mf.decomp.run_hessenberg(op, k, torch.tensor(V, dtype=dtype, device="cuda"))
    _, Ho, _, _ = slq.hessenberg_forward_batched(lambda X: X @ Ad.T, k, V.astype(
        np.float32 if dtype == torch.float32 else np.float64).astype(np.float64))
    d, e = slq.tridiag_from_hessenberg(H.cpu().numpy())
    do, eo = slq.tridiag_from_hessenberg(Ho)
    tol = 1e-9 if dtype == torch.float64 else 2e-4
    np.testing.assert_allclose(d, do, rtol=tol, atol=tol)


@pytest.mark.parametrize("n,p", [(64, 300), (1000, 257)])
def test_probe_tiles_beyond_256(n, p):
    # more probes than one tensor-core N tile (256): two probe tiles per row block
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) / np.sqrt(n)
    V = rng.standard_normal((p, n))
    op = mf.DenseOperator(torch.tensor(A, dtype=torch.float32, device="cuda"), precision="bf16x3")
    W = op.matmat(torch.tensor(V, dtype=torch.float32, device="cuda")).double().cpu().numpy()
    want = V.astype(np.float32).astype(np.float64) @ A.astype(np.float32).astype(np.float64).T
    assert np.abs(W - want).max() / np.abs(want).max() < 5e-5


@pytest.mark.parametrize("dtype,n,p,k", [
    (torch.float64, 3000, 2, 140),    # row segments; three- and two-buffer rings, unfused past 99
    (torch.float32, 4099, 3, 100),    # two-buffer ring past 66 float vectors; ragged last chunk
    (torch.float32, 1000, 400, 20),   # more probes than resident CTAs: one segment per probe
])
def test_fused_update_projection_variants(dtype, n, p, k):
    # the fused CGS2 step switches kernels with the vector count and splits
    # rows into segments when probes are few; every variant gives an
    # orthonormal basis, the Arnoldi relation and the oracle's tridiagonal
    A = problems.dense_spd(n, seed=11)
    V = np.random.default_rng(12).standard_normal((p, n))
    f64 = dtype == torch.float64
    Ad = A if f64 else A.astype(np.float32).astype(np.float64)
    Vd = V if f64 else V.astype(np.float32).astype(np.float64)
    op = mf.DenseOperator(torch.tensor(Ad, dtype=dtype, device="cuda"), precision="fp64" if f64 else "fp32")
    Q, H, r, _ = mf.decomp.run_hessenberg(op, k, torch.tensor(Vd, dtype=dtype, device="cuda"))
    Qc, Hc, rc = Q.double().cpu().numpy(), H.cpu().numpy(), r.double().cpu().numpy()
    G = Qc @ Qc.transpose(0, 2, 1)
    assert np.abs(G - np.eye(k)).max() < (1e-12 if f64 else 5e-5)
    AQ = Ad @ Qc.transpose(0, 2, 1)
    rel = AQ - Qc.transpose(0, 2, 1) @ Hc
    rel[:, :, -1] -= rc
    assert np.abs(rel).max() < (1e-10 if f64 else 1e-4) * np.abs(AQ).max()
    # the oracle's tridiagonal over the steps before rounding differences grow
    m = k if f64 else min(k, 30)
    _, Ho, _, _ = slq.hessenberg_forward_batched(lambda X: X @ Ad.T, m, Vd)
    d, e = slq.tridiag_from_hessenberg(Hc[:, :m, :m])
    do, eo = slq.tridiag_from_hessenberg(Ho)
    tol = 1e-9 if f64 else 5e-4
    np.testing.assert_allclose(d, do, rtol=tol, atol=tol)
    np.testing.assert_allclose(e, eo, rtol=tol, atol=tol)
