"""Failure detection on the device without a GPU fault (needs a GPU).

Every wait in the library's kernels is bounded: after its limit it gives up,
raises the CTA's failure flag and records MFG_ERR_TIMEOUT in a device status
word that the host reads.  ``mfg_wait_selftest`` runs that protocol on an
mbarrier nothing arrives on (no copies in flight, no tensor memory held), so
the wait runs out by construction.  The test checks the status the host reads,
that the polling waiter kept waiting for its limit, that the sleeping waiter
(the form idle roles use, with the 2 s production limit) left through the
failure flag well before its own limit, and that the context stays usable: a
tensor-core operator product right afterwards matches one taken before.
"""

import ctypes

import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import _lib
from matfree_gb300._panel import stream_ptr

pytestmark = pytest.mark.gpu

MFG_ERR_TIMEOUT = 7
MFG_ERR_BAD_ARG = 1


def _selftest(limit_ns):
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    times = torch.zeros(5, dtype=torch.int64, device="cuda")
    rc = _lib.lib().mfg_wait_selftest(limit_ns, ctypes.c_void_p(status.data_ptr()),
                                      ctypes.c_void_p(times.data_ptr()), stream_ptr())
    torch.cuda.synchronize()
    return rc, int(status.item()), [int(t) for t in times.cpu()]


@pytest.mark.parametrize("limit_ms", [1, 20])
def test_bounded_wait_times_out_and_reports_status(limit_ms):
    limit_ns = limit_ms * 1_000_000
    rc, status, (t0, ok0, t1, ok1, flag) = _selftest(limit_ns)
    assert rc == 0
    assert status == MFG_ERR_TIMEOUT
    assert ok0 == 0 and ok1 == 0 and flag == 1
    # the polling waiter waited its limit and not much longer
    assert limit_ns <= t0 <= limit_ns + 50_000_000, t0
    # the sleeping waiter (2 s limit) left through the failure flag
    assert t1 < 500_000_000, t1


def test_selftest_rejects_bad_limits():
    lib = _lib.lib()
    buf = torch.zeros(8, dtype=torch.int64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    assert lib.mfg_wait_selftest(0, p, p, stream_ptr()) == MFG_ERR_BAD_ARG
    assert lib.mfg_wait_selftest(3_000_000_000, p, p, stream_ptr()) == MFG_ERR_BAD_ARG
    assert lib.mfg_wait_selftest(1_000_000, None, p, stream_ptr()) == MFG_ERR_BAD_ARG


def test_context_usable_after_a_timeout():
    n, p = 2048, 64
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn((n, n), device="cuda", generator=g) / n ** 0.5
    op = mf.DenseOperator(A @ A.T + torch.eye(n, device="cuda"), precision="bf16x3")
    V = torch.randn((p, n), device="cuda", generator=g)
    before = op.matmat(V)
    rc, status, _ = _selftest(2_000_000)
    assert rc == 0 and status == MFG_ERR_TIMEOUT
    after = op.matmat(V)
    torch.cuda.synchronize()
    assert torch.equal(before, after)
