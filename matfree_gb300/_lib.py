"""ctypes binding of ``libmatfree_gb300.so`` (the C ABI in include/matfree_gb300.h).

Loading fails loudly when the library has not been built: there is no
fallback implementation of any entry point.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_size_t, c_uint32, c_void_p

from . import build as _build

MFG_OK = 0
MFG_ERR_BAD_ARG = 1
MFG_ERR_RANGE = 2
MFG_ERR_WORKSPACE = 3
MFG_ERR_CUDA = 4
MFG_ERR_UNSUPPORTED = 5
MFG_ERR_NO_CONVERGENCE = 6
MFG_ERR_TIMEOUT = 7
MFG_ERR_SCRATCH_LIMIT = 8
MFG_ERR_RETRY = 9
MFG_SLQ_TWO_SWEEP = 1

MFG_F32, MFG_F64 = 0, 1
MFG_OP_DENSE, MFG_OP_CSR, MFG_OP_CALLBACK = 0, 1, 2
MFG_PREC_FP32, MFG_PREC_BF16, MFG_PREC_BF16X3, MFG_PREC_FP64 = 0, 1, 2, 3
MFG_FUN_LOG, MFG_FUN_EXP, MFG_FUN_POW, MFG_FUN_NONE = 0, 1, 2, 3

PRECISIONS = {"fp32": MFG_PREC_FP32, "bf16": MFG_PREC_BF16, "bf16x3": MFG_PREC_BF16X3, "fp64": MFG_PREC_FP64}

APPLY_FN = ctypes.CFUNCTYPE(c_int, c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_int64, c_void_p)


class MfgOperator(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32),
        ("precision", c_int32),
        ("n", c_int64),
        ("a", c_void_p),
        ("a_lo", c_void_p),
        ("lda", c_int64),
        ("row_ptr", c_void_p),
        ("col_idx", c_void_p),
        ("values", c_void_p),
        ("nnz", c_int64),
        ("shift", c_double),
        ("apply", APPLY_FN),
        ("ctx", c_void_p),
    ]


# name -> (restype, argtypes); every symbol include/matfree_gb300.h declares
SIGNATURES = {
    "mfg_version": (c_int, []),
    "mfg_status_string": (ctypes.c_char_p, [c_int]),
    "mfg_last_error": (ctypes.c_char_p, []),
    "mfg_slq_workspace_bytes": (c_size_t, [POINTER(MfgOperator), c_int64, c_int64, c_int64]),
    "mfg_sampler_signs": (c_int, [POINTER(c_uint32), c_int64, c_int64, c_int64, c_int32, c_void_p, c_void_p]),
    "mfg_sampler_normal": (c_int, [POINTER(c_uint32), c_int64, c_int64, c_int64, c_int32, c_void_p, c_void_p]),
    "mfg_operator_apply": (c_int, [POINTER(MfgOperator), c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_size_t, c_void_p]),
    "mfg_hessenberg": (c_int, [POINTER(MfgOperator), c_int64, c_int64, c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_tridiag_quadrature": (c_int, [c_int64, c_int64, c_void_p, c_int32, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mfg_slq": (c_int, [POINTER(MfgOperator), c_int64, c_int64, c_void_p, c_int64, c_int32, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_slq_ex_workspace_bytes": (c_size_t, [POINTER(MfgOperator), c_int64, c_int64, c_int64, c_int32]),
    "mfg_slq_ex": (c_int, [POINTER(MfgOperator), c_int64, c_int64, c_void_p, c_int64, c_int32, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_size_t, c_void_p]),
    "mfg_workspace_status": (c_int, [c_void_p, c_void_p]),
    "mfg_tridiag_eigh": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mfg_rbf_build": (c_int, [c_void_p, c_int64, c_int32, c_double, c_double, c_int32, c_void_p, c_void_p, c_int64, c_void_p]),
    "mfg_rbf_build_dlogell": (c_int, [c_void_p, c_int64, c_int32, c_double, c_double, c_int32, c_void_p, c_void_p, c_int64, c_void_p]),
    "mfg_split_bf16": (c_int, [c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p, c_int64, c_void_p]),
    "mfg_cg_workspace_bytes": (c_size_t, [POINTER(MfgOperator), c_int64, c_int64]),
    "mfg_bidiag_workspace_bytes": (c_size_t, [POINTER(MfgOperator), POINTER(MfgOperator), c_int64, c_int64, c_int64]),
    "mfg_bidiag": (c_int, [POINTER(MfgOperator), POINTER(MfgOperator), c_int64, c_int64, c_void_p, c_int64, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_slq_product": (c_int, [POINTER(MfgOperator), POINTER(MfgOperator), c_int64, c_int64, c_void_p, c_int64,
                                c_int32, c_double, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_cg": (c_int, [POINTER(MfgOperator), c_int64, c_void_p, c_void_p, c_int64, c_double, c_double, c_int64,
                       c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_adjoint_workspace_bytes": (c_size_t, [POINTER(MfgOperator), c_int64, c_int64, c_int64]),
    "mfg_hessenberg_adjoint": (c_int, [POINTER(MfgOperator), c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_hessenberg_adjoint_ex": (c_int, [POINTER(MfgOperator), c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "mfg_gemm_tuning_add": (c_int, [c_int64, c_int64, c_int64, c_int64, c_int32, c_int32]),
    "mfg_gemm_tuning_clear": (c_int, []),
    "mfg_basis_combine": (c_int, [c_int32, c_int64, c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mfg_operator_apply_noalloc": (c_int, [POINTER(MfgOperator), c_void_p, c_void_p, c_int64, c_int64, c_void_p]),
    "mfg_operator_apply_noalloc_status": (c_int, [c_void_p]),
    "mfg_wait_selftest": (c_int, [ctypes.c_uint64, c_void_p, c_void_p, c_void_p]),
    "mfg_gemm_pair_schedule": (c_int64, [c_int64, c_int64, c_int32, c_int32, c_int32, c_void_p, c_int64]),
    "mfg_profile_enable": (c_int, [c_int]),
    "mfg_profile_read": (c_int, [c_int32, POINTER(c_double), POINTER(c_double), POINTER(c_double), POINTER(c_int64)]),
}

PROF_CLASSES = ["apply", "proj", "sub", "scale", "quad", "other", "subproj"]

_LIB = None


def library_path() -> str:
    return _build.LIB


def lib():
    """Load the CUDA library (once).  Raises if it is missing."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"matfree_gb300 CUDA library not found at {path}; build it with "
                "`python -m matfree_gb300.build` (nvcc, sm_103a)."
            )
        handle = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


class MatfreeGB300Error(RuntimeError):
    pass


def check(status: int, what: str) -> None:
    if status == MFG_OK:
        return
    text = lib().mfg_status_string(status).decode()
    if status == MFG_ERR_RANGE:
        raise ValueError(f"{what}: {text}")
    if status == MFG_ERR_BAD_ARG:
        raise ValueError(f"{what}: {text}")
    detail = lib().mfg_last_error().decode() if status == MFG_ERR_CUDA else ""
    raise MatfreeGB300Error(f"{what}: {text} (status {status}) {detail}".rstrip())
