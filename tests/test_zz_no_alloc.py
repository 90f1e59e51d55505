"""The operator application that allocates nothing (mfg_operator_apply_noalloc).

Some callers cannot allocate device memory at all: code that runs inside
another framework's fixed memory pool, or on a host without a device
allocator of its own.  They still need W = (A + shift I) V, so the library
keeps the only scratch that product needs (the bf16 hi/lo copies of the
probe panel) in one fixed device array of its own.  This file checks,
through the C ABI, that two calls in a row give the float64 product of the
stored operator within the tolerances of the other apply tests, for every
operator form (the one-CTA and CTA-pair tensor-core GEMMs, the split-K pair
GEMM, the few-probe GEMV, fp32, and CSR), that they agree with the
workspace-based mfg_operator_apply, that the device status word reads back
as MFG_OK, and that the size limit sits exactly where the header states it.
It is collected last so that a stop at its first failure has already run
every other test.
"""

import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import torch

import matfree_gb300 as mf
from matfree_gb300 import _lib
from matfree_gb300._panel import Workspace, stream_ptr

pytestmark = pytest.mark.gpu

# relative to the largest entry, as in the tensor-core apply tests
TOL = {"bf16x3": 5e-5, "bf16": 1.5e-2, "fp32": 1e-5, "csr": 1e-6}
LIMIT = 32 * 1024 * 1024


def _apply_with_workspace(op, panel):
    lib = _lib.lib()
    p, ld = panel.shape
    out = torch.zeros_like(panel)
    s = op.c_struct()
    nbytes = lib.mfg_slq_workspace_bytes(ctypes.byref(s), 0, p, ld)
    ws, wsb = Workspace().get(nbytes, panel.device)
    st = lib.mfg_operator_apply(ctypes.byref(s), ctypes.c_void_p(panel.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), p, ld, ws, wsb, stream_ptr())
    assert st == _lib.MFG_OK, lib.mfg_status_string(st)
    return out


def _apply_noalloc(op, panel):
    lib = _lib.lib()
    p, ld = panel.shape
    out = torch.zeros_like(panel)
    s = op.c_struct()
    st = lib.mfg_operator_apply_noalloc(ctypes.byref(s), ctypes.c_void_p(panel.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), p, ld, stream_ptr())
    assert st == _lib.MFG_OK, lib.mfg_status_string(st)
    assert lib.mfg_operator_apply_noalloc_status(stream_ptr()) == _lib.MFG_OK
    return out


def _panel(rng, p, n):
    ld = (n + 7) // 8 * 8
    panel = torch.zeros((p, ld), dtype=torch.float32, device="cuda")
    panel[:, :n] = torch.tensor(rng.standard_normal((p, n)), dtype=torch.float32)
    return panel


@pytest.mark.parametrize("precision", ["bf16x3", "bf16", "fp32"])
@pytest.mark.parametrize("n,p", [(1000, 200),   # one-CTA tensor-core form
                                 (2048, 256),   # CTA-pair form
                                 (8192, 128),   # CTA-pair form with K split over two CTAs
                                 (4099, 5)])    # few-probe GEMV form
def test_noalloc_dense_apply_matches_float64_product_twice(precision, n, p):
    rng = np.random.default_rng(n + p)
    A = torch.tensor(rng.standard_normal((n, n)) / np.sqrt(n), dtype=torch.float32, device="cuda")
    op = mf.DenseOperator(A, precision=precision, shift=0.25)
    A64 = op.dense()  # the stored operator (bf16 parts, or fp32) plus the shift, in float64
    for _ in range(2):  # two calls in a row share (and reuse) the fixed scratch
        panel = _panel(rng, p, n)
        got = _apply_noalloc(op, panel)
        ref = _apply_with_workspace(op, panel)
        torch.cuda.synchronize()
        want = panel[:, :n].double() @ A64.T
        scale = float(want.abs().max())
        err = float((got[:, :n].double() - want).abs().max()) / scale
        assert err < TOL[precision], err
        torch.testing.assert_close(got[:, :n], ref[:, :n], rtol=TOL[precision],
                                   atol=TOL[precision] * scale)


def test_noalloc_csr_apply_matches_float64_product_twice():
    m = 200
    n = m * m
    rng0 = np.random.default_rng(3)
    rows = np.repeat(np.arange(n), 5)
    cols = rng0.integers(0, n, size=5 * n)
    L = sp.csr_matrix((rng0.standard_normal(5 * n).astype(np.float32), (rows, cols)), shape=(n, n))
    L = (L + sp.eye(n, dtype=np.float32)).tocsr()
    op = mf.CSROperator.from_scipy(L, shift=0.5)
    L64 = L.astype(np.float64)
    rng = np.random.default_rng(5)
    for _ in range(2):
        panel = _panel(rng, 24, m * m)
        got = _apply_noalloc(op, panel)[:, : m * m].double().cpu().numpy()
        V = panel[:, : m * m].double().cpu().numpy()
        want = (L64 @ V.T).T + 0.5 * V
        assert np.abs(got - want).max() / np.abs(want).max() < TOL["csr"]


def _status_noalloc(op, p, ld, buf_v, buf_w):
    s = op.c_struct()
    return _lib.lib().mfg_operator_apply_noalloc(ctypes.byref(s), ctypes.c_void_p(buf_v.data_ptr()),
                                                 ctypes.c_void_p(buf_w.data_ptr()), p, ld, stream_ptr())


def test_noalloc_limit_is_exactly_the_documented_condition():
    # 256 + copies * round_up(p * ld * 2, 256) <= 32 MiB, copies = 2 for bf16x3
    n = 1024
    A = torch.eye(n, dtype=torch.float32, device="cuda")
    op = mf.DenseOperator(A, precision="bf16x3")
    ld = n
    p_max = (LIMIT - 256) // (2 * ld * 2)  # p * 2048 bytes is already a multiple of 256
    assert 256 + 2 * p_max * ld * 2 <= LIMIT < 256 + 2 * (p_max + 1) * ld * 2
    V = torch.ones((p_max + 1, ld), dtype=torch.float32, device="cuda")
    W = torch.zeros_like(V)
    st = _status_noalloc(op, p_max + 1, ld, V, W)
    assert st == _lib.MFG_ERR_SCRATCH_LIMIT
    assert b"32 MiB" in _lib.lib().mfg_status_string(st)
    assert _status_noalloc(op, p_max, ld, V, W) == _lib.MFG_OK
    assert _lib.lib().mfg_operator_apply_noalloc_status(stream_ptr()) == _lib.MFG_OK
    torch.cuda.synchronize()
    # A = I and V = 1: the product of the accepted call is V itself
    assert torch.equal(W[:p_max], V[:p_max])
    # bf16 keeps one copy: 256 + round_up(p * ld * 2, 256) <= 32 MiB
    op1 = mf.DenseOperator(A, precision="bf16")
    p1 = (LIMIT - 256) // (ld * 2)
    V1 = torch.ones((p1 + 1, ld), dtype=torch.float32, device="cuda")
    W1 = torch.zeros_like(V1)
    assert _status_noalloc(op1, p1 + 1, ld, V1, W1) == _lib.MFG_ERR_SCRATCH_LIMIT
    assert _status_noalloc(op1, p1, ld, V1, W1) == _lib.MFG_OK
    # fp32 needs no copy and is never rejected for size
    op32 = mf.DenseOperator(A, precision="fp32")
    assert _status_noalloc(op32, p_max + 1, ld, V, W) == _lib.MFG_OK
    torch.cuda.synchronize()
