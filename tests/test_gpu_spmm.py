"""The CSR SpMM kernel (csr_spmm_window_kernel) against scipy on every path:
the streamed-window path (banded matrices), the gather path (wide column
patterns), the warp-cooperative path for long rows, rows longer than the
entries held in registers, both register widths (6 and 12 entries), ragged
and empty rows, and CSR arrays at unaligned offsets."""

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from oracle import problems
from oracle.problems import random_csr as _random_csr

pytestmark = pytest.mark.gpu


def _check(A, p=5, shift=0.3, seed=0, op=None):
    n = A.shape[0]
    op = op or mf.CSROperator.from_scipy(A, shift=shift)
    V = np.random.default_rng(seed).standard_normal((p, n)).astype(np.float32)
    got = op.matmat(torch.from_numpy(V).cuda()).double().cpu().numpy()
    want = (A.astype(np.float64) @ V.astype(np.float64).T).T + shift * V.astype(np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5 * np.abs(want).max())


@pytest.mark.parametrize("case", ["laplace", "banded", "random", "long", "wide_rows", "dense_band", "empty_rows"])
def test_csr_spmm_paths_match_scipy(case):
    rng = np.random.default_rng(7)
    if case == "laplace":
        A = problems.laplacian_2d(300, shift=0.0)
    elif case == "banded":
        n = 20000
        A = _random_csr(n, rng, rng.integers(0, 9, size=n), band=1200)
    elif case == "random":
        n = 30000
        A = _random_csr(n, rng, rng.integers(0, 5, size=n))
    elif case == "long":
        n = 9000
        lens = rng.integers(1, 4, size=n)
        lens[[5, 1130, 4100, 8999]] = [70, 2000, 33, 900]
        A = _random_csr(n, rng, lens)
    elif case == "wide_rows":
        n = 3000
        A = _random_csr(n, rng, np.full(n, 40), band=1000)
    elif case == "dense_band":
        n = 20000
        A = _random_csr(n, rng, rng.integers(6, 16, size=n), band=1000)  # 12 entries in registers
    else:
        n = 5000
        lens = rng.integers(0, 4, size=n)
        lens[1000:3100] = 0
        A = _random_csr(n, rng, lens, band=500)
    A.sort_indices()
    _check(A.astype(np.float32), p=5)
    _check(A.astype(np.float32), p=67, seed=1)


def test_csr_spmm_unaligned_arrays_match_scipy():
    A = problems.laplacian_2d(100, shift=0.1)
    n = A.shape[0]
    # column indices and values one entry past a 16-byte boundary
    ci = torch.zeros(A.nnz + 1, dtype=torch.int32, device="cuda")
    va = torch.zeros(A.nnz + 1, dtype=torch.float32, device="cuda")
    ci[1:] = torch.from_numpy(A.indices.astype(np.int32)).cuda()
    va[1:] = torch.from_numpy(A.data.astype(np.float32)).cuda()
    rp = torch.from_numpy(A.indptr.astype(np.int32)).cuda()
    op = mf.CSROperator(rp, ci[1:], va[1:], n, shift=0.0)
    assert op.col_idx.data_ptr() % 16 != 0
    _check(A, p=9, shift=0.0, op=op)
