"""The operator application that allocates nothing (mfg_operator_apply_noalloc).

Some callers cannot allocate device memory at all: code that runs inside a
stream capture, inside another framework's fixed memory pool, or on a host
without an allocator of its own.  They still need W = (A + shift I) V, so the
library keeps the only scratch that product needs (the bf16 hi/lo copies of
the probe panel) in one fixed device array of its own.  This file checks,
through the C ABI, that two calls in a row give the same result as the
workspace-based mfg_operator_apply, within the tensor-core tolerance used by
the other apply tests, and that an oversized panel is rejected up front.
It is collected last so that a stop at its first failure has already run
every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import _lib
from matfree_gb300._panel import Workspace, stream_ptr

pytestmark = pytest.mark.gpu

TOL = 5e-5  # relative, as in the bf16x3 tensor-core apply tests


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
    return out


@pytest.mark.parametrize("precision", ["bf16x3", "bf16"])
def test_noalloc_apply_matches_workspace_apply_twice(precision):
    n, p = 1000, 200
    rng = np.random.default_rng(11)
    A = torch.tensor(rng.standard_normal((n, n)) / np.sqrt(n), dtype=torch.float32, device="cuda")
    op = mf.DenseOperator(A, precision=precision, shift=0.25)
    ld = (n + 7) // 8 * 8
    for call in range(2):  # two calls in a row share (and reuse) the fixed scratch
        panel = torch.zeros((p, ld), dtype=torch.float32, device="cuda")
        panel[:, :n] = torch.tensor(rng.standard_normal((p, n)), dtype=torch.float32)
        want = _apply_with_workspace(op, panel)
        got = _apply_noalloc(op, panel)
        torch.cuda.synchronize()
        scale = want[:, :n].abs().max()
        torch.testing.assert_close(got[:, :n], want[:, :n], rtol=TOL, atol=TOL * float(scale))


def test_noalloc_rejects_panels_beyond_the_fixed_scratch():
    n = 1000
    A = torch.eye(n, dtype=torch.float32, device="cuda")
    op = mf.DenseOperator(A, precision="bf16x3")
    ld = (n + 7) // 8 * 8
    p = 8400  # 8400 * 1000 * 2 copies * 2 bytes > 32 MiB
    s = op.c_struct()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = _lib.lib().mfg_operator_apply_noalloc(ctypes.byref(s), ctypes.c_void_p(buf.data_ptr()),
                                               ctypes.c_void_p(buf.data_ptr()), p, ld, stream_ptr())
    assert st == _lib.MFG_ERR_SCRATCH_LIMIT
    assert b"32 MiB" in _lib.lib().mfg_status_string(st)
