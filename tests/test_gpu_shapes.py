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
