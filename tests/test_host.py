"""Host-side tests that need no GPU: the C ABI library, argument errors, keys."""

import ctypes
import os
import re

import numpy as np
import pytest
import torch

import matfree_gb300 as mf
from matfree_gb300 import _lib
from oracle import philox

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built_library():
    from matfree_gb300 import build

    build.build()
    yield


def _declared_symbols():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^MFG_API\s+[\w\s\*]+?\b(mfg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    names = _declared_symbols()
    assert len(names) >= 11
    handle = ctypes.CDLL(_lib.library_path())
    for name in names:
        assert hasattr(handle, name), name
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_version_and_status_strings():
    lib = _lib.lib()
    assert lib.mfg_version() >= 100
    assert b"exceeds" in lib.mfg_status_string(_lib.MFG_ERR_RANGE)
    assert lib.mfg_status_string(12345) == b"unknown status"


def test_workspace_size_grows_with_depth():
    A = _lib.MfgOperator()
    A.kind, A.precision, A.n, A.lda = _lib.MFG_OP_DENSE, _lib.MFG_PREC_FP32, 1000, 1000
    A.a = 4096  # never dereferenced by the size query
    lib = _lib.lib()
    s10 = lib.mfg_slq_workspace_bytes(ctypes.byref(A), 10, 64, 1000)
    s30 = lib.mfg_slq_workspace_bytes(ctypes.byref(A), 30, 64, 1000)
    assert 0 < s10 < s30
    # basis (p k ld fp32) + Hessenberg (p k k fp64) are part of the workspace
    assert s30 >= 64 * 30 * 1000 * 4 + 64 * 30 * 30 * 8
    assert lib.mfg_slq_workspace_bytes(ctypes.byref(A), 30, 64, 999) == 0  # ld < n
    A.lda = 1001
    assert lib.mfg_slq_workspace_bytes(ctypes.byref(A), 30, 64, 1000) == 0  # lda % 8


def test_argument_errors_without_gpu():
    lib = _lib.lib()
    A = _lib.MfgOperator()
    A.kind, A.precision, A.n, A.lda, A.a = _lib.MFG_OP_DENSE, _lib.MFG_PREC_FP32, 16, 16, 4096
    buf = ctypes.c_void_p(4096)
    # k out of range -> MFG_ERR_RANGE before any device work
    st = lib.mfg_hessenberg(ctypes.byref(A), 17, 1, buf, 16, 1, buf, buf, None, None, buf, 1 << 20, None)
    assert st == _lib.MFG_ERR_RANGE
    st = lib.mfg_hessenberg(ctypes.byref(A), 4, 1, buf, 16, 7, buf, buf, None, None, buf, 1 << 20, None)
    assert st == _lib.MFG_ERR_BAD_ARG
    st = lib.mfg_hessenberg(ctypes.byref(A), 4, 1, buf, 16, 1, buf, buf, None, None, buf, 16, None)
    assert st == _lib.MFG_ERR_WORKSPACE
    A.kind = 99
    assert lib.mfg_slq(ctypes.byref(A), 4, 1, buf, 16, 0, 0.0, buf, None, None, None, buf, 1 << 20, None) == _lib.MFG_ERR_BAD_ARG


# matfree/decomp.py:121-122 and :375-378
def test_decomposition_flag_errors():
    with pytest.raises(ValueError, match="unsupported"):
        mf.decomp.tridiag_sym(3, reortho="bogus")
    for wrong in [True, "full_with_sparsity", "None"]:
        with pytest.raises(TypeError, match="Unexpected input"):
            mf.decomp.hessenberg(1, reortho=wrong)


# tests/test_decomp/test_consistency.py:51-63
@pytest.mark.parametrize("k", [-1, 14])
def test_value_error_for_unusual_num_matvecs(k):
    v0 = torch.ones(13)
    with pytest.raises(ValueError, match="exceeds"):
        mf.decomp.tridiag_sym(k)(lambda v: v, v0)
    with pytest.raises(ValueError, match="exceeds"):
        mf.decomp.hessenberg(k, reortho="full")(lambda v: v, v0)


def test_cpu_tensors_are_rejected():
    with pytest.raises(TypeError, match="CUDA"):
        mf.decomp.tridiag_sym(3)(lambda v: v, torch.ones(8))


def test_prng_split_matches_oracle_philox():
    key = mf.prng.prng_key(123456789012)
    np.testing.assert_array_equal(key, philox.prng_key(123456789012))
    np.testing.assert_array_equal(mf.prng.split(key, 5), philox.split(key, 5))
    a, b = mf.prng.split(key)
    assert not np.array_equal(a, b)


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        got = philox.philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32))
        assert tuple(int(x) for x in got) == want
        assert mf.prng._philox(ctr, key) == want


def test_oracle_rademacher_moments():
    x = philox.rademacher(philox.prng_key(1), 2000, 50)
    assert set(np.unique(x)) == {-1.0, 1.0}
    assert abs(x.mean()) < 0.02
    z = philox.normal(philox.prng_key(2), 4000, 25)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02


def test_pytree_ravel_roundtrip():
    tree = {"a": torch.arange(3.0), "b": [torch.ones(2, 2), (torch.zeros(1),)]}
    flat, unravel = mf.tree.ravel_pytree(tree)
    assert flat.shape == (8,)
    back = unravel(flat)
    assert torch.equal(back["a"], tree["a"]) and torch.equal(back["b"][0], tree["b"][0])
    batched = unravel(torch.stack([flat, 2 * flat]))
    assert batched["b"][0].shape == (2, 2, 2)


def test_serve_footprint_grows_with_every_dimension():
    from matfree_gb300 import serve

    base = serve.footprint_bytes(4096, 32, 64, "bf16x3")
    assert base > 4 * 4096 * 4096  # at least the bf16 hi + lo operator (2 + 2 bytes)
    assert serve.footprint_bytes(8192, 32, 64, "bf16x3") > base
    assert serve.footprint_bytes(4096, 64, 64, "bf16x3") > base
    assert serve.footprint_bytes(4096, 32, 128, "bf16x3") > base
    assert serve.footprint_bytes(4096, 32, 64, "bf16") < base


def test_serve_request_stream_is_seeded():
    from matfree_gb300 import serve

    a = serve.synthetic_stream(20, rate=50.0, seed=3)
    b = serve.synthetic_stream(20, rate=50.0, seed=3)
    assert [(len(r.x), r.k, r.p, r.fun, r.arrival) for r in a] == \
        [(len(r.x), r.k, r.p, r.fun, r.arrival) for r in b]
    assert all(512 <= len(r.x) <= 32768 and r.k in (16, 32, 64, 96) for r in a)
    assert all(t1.arrival < t2.arrival for t1, t2 in zip(a, a[1:]))


def test_serve_function_names():
    from matfree_gb300 import _lib, serve

    assert serve._fun_code("log") == (_lib.MFG_FUN_LOG, 0.0)
    assert serve._fun_code("exp:-0.1") == (_lib.MFG_FUN_EXP, -0.1)
    with pytest.raises(ValueError, match="unknown matrix function"):
        serve._fun_code("sqrt")


def test_eigh_and_adjoint_argument_errors_without_gpu():
    lib = _lib.lib()
    buf = ctypes.c_void_p(4096)
    # mfg_tridiag_eigh: sizes and pointers are checked before any launch
    assert lib.mfg_tridiag_eigh(0, 1, buf, buf, buf, buf, None) == _lib.MFG_ERR_BAD_ARG
    assert lib.mfg_tridiag_eigh(4, 0, buf, buf, buf, buf, None) == _lib.MFG_ERR_BAD_ARG
    assert lib.mfg_tridiag_eigh(4, 1, None, buf, buf, buf, None) == _lib.MFG_ERR_BAD_ARG
    # mfg_hessenberg_adjoint: k = 0 is a range error (decomp.py:483-486), missing outputs bad args
    A = _lib.MfgOperator()
    A.kind, A.precision, A.n, A.lda, A.a = _lib.MFG_OP_DENSE, _lib.MFG_PREC_FP64, 16, 16, 4096
    args = (buf, buf, buf, buf, buf, None, None, buf, buf, buf, 1 << 20, None)
    assert lib.mfg_hessenberg_adjoint(ctypes.byref(A), 0, 1, 16, *args) == _lib.MFG_ERR_RANGE
    assert lib.mfg_hessenberg_adjoint(ctypes.byref(A), 17, 1, 16, *args) == _lib.MFG_ERR_RANGE
    bad = (None,) + args[1:]
    assert lib.mfg_hessenberg_adjoint(ctypes.byref(A), 4, 1, 16, *bad) == _lib.MFG_ERR_BAD_ARG
    small_ws = args[:-2] + (16, None)
    assert lib.mfg_hessenberg_adjoint(ctypes.byref(A), 4, 1, 16, *small_ws) == _lib.MFG_ERR_WORKSPACE


# ------------------------------------------------------------ DLPack intake


class _DLPackOnly:
    """An array that exports its memory only through the DLPack protocol."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, stream=None, **kwargs):
        return self._t.__dlpack__()

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_dlpack_producers_are_imported_without_copy():
    import torch

    from matfree_gb300._panel import as_tensor

    t = torch.arange(6.0)
    for obj in (_DLPackOnly(t), torch.utils.dlpack.to_dlpack(t), np.arange(6.0)):
        got = as_tensor(obj, "x")
        assert isinstance(got, torch.Tensor)
        np.testing.assert_array_equal(got.numpy(), np.arange(6.0))
    assert as_tensor(_DLPackOnly(t), "x").data_ptr() == t.data_ptr()


def test_host_arrays_and_unknown_objects_are_rejected():
    from matfree_gb300._panel import require_cuda

    with pytest.raises(TypeError, match="CUDA"):
        require_cuda(np.zeros(3), "x")  # a DLPack producer, but host memory
    with pytest.raises(TypeError, match="DLPack"):
        require_cuda([1.0, 2.0], "x")


def test_tuning_rule_ranges_tile_the_axis():
    from matfree_gb300 import tuning

    ns = tuning.DEFAULT_NS
    spans = [tuning._bounds(ns, i) for i in range(len(ns))]
    assert spans[0][0] == 0 and spans[-1][1] >= 1 << 40
    for (lo, hi), n in zip(spans, ns):
        assert lo <= n <= hi
    for (_, hi), (lo, _) in zip(spans, spans[1:]):
        assert lo == hi + 1


def test_tuning_keeps_the_built_in_form_within_the_margin():
    from matfree_gb300 import tuning

    # (ms, bn, split); the built-in choice is (0, 0)
    base = [(1.00, 0, 0), (0.99, 0, 3), (1.20, 128, 1)]
    assert tuning.pick(base, margin=0.03) == (1.00, (1.00, 0, 0))  # 1 % faster: noise
    faster = [(1.00, 0, 0), (0.95, 0, 2), (0.96, 128, 3)]
    assert tuning.pick(faster, margin=0.03) == (1.00, (0.95, 0, 2))
    assert tuning.pick(faster, margin=0.10) == (1.00, (1.00, 0, 0))
    slower = [(1.00, 0, 0), (1.10, 64, 1)]
    assert tuning.pick(slower) == (1.00, (1.00, 0, 0))


def test_gemm_tuning_rejects_bad_rules():
    lib = _lib.lib()
    assert lib.mfg_gemm_tuning_add(1024, 2048, 64, 64, 48, 0) == _lib.MFG_ERR_BAD_ARG  # not a multiple of 32
    assert lib.mfg_gemm_tuning_add(1024, 2048, 64, 64, 128, 4) == _lib.MFG_ERR_BAD_ARG
    assert lib.mfg_gemm_tuning_add(1024, 2048, 64, 64, 128, 3) == _lib.MFG_OK
    assert lib.mfg_gemm_tuning_add(2048, 1024, 64, 64, 128, 1) == _lib.MFG_ERR_BAD_ARG
    assert lib.mfg_gemm_tuning_add(1024, 2048, 64, 64, 128, 1) == _lib.MFG_OK
    assert lib.mfg_gemm_tuning_clear() == _lib.MFG_OK
