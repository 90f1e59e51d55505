"""Device buffers in the library's probe-major panel layout.

A set of p vectors of length n lives in a (p, ld) tensor with ld = n rounded
up to a multiple of 8 elements, so that every row starts on a 16-byte (float)
or 32-byte boundary; the columns n..ld-1 are zero.  The user-facing views are
``panel[:, :n]``.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib


def padded_ld(n: int) -> int:
    return (int(n) + 7) // 8 * 8


def as_tensor(x, what: str):
    """A torch view of a torch tensor or of any array that exports its memory
    through DLPack (``__dlpack__``) or ``__cuda_array_interface__`` (CuPy, JAX,
    Numba, ...): no copy is made, the producer keeps ownership."""
    if isinstance(x, torch.Tensor):
        return x
    if hasattr(x, "__dlpack__"):
        try:
            return torch.from_dlpack(x)
        except Exception as err:  # noqa: BLE001  (producer-specific failures)
            raise TypeError(f"{what}: DLPack import failed ({err})") from err
    if hasattr(x, "__cuda_array_interface__"):
        return torch.as_tensor(x, device="cuda")
    if type(x).__name__ == "PyCapsule":
        return torch.utils.dlpack.from_dlpack(x)
    raise TypeError(f"{what} must be a CUDA tensor or a DLPack-capable CUDA array "
                    f"(matfree_gb300 runs on the GPU only); got {type(x).__name__}")


def require_cuda(t, what: str) -> torch.Tensor:
    """Return ``t`` as a torch CUDA tensor (DLPack producers are imported
    without a copy); raise TypeError for host arrays and unknown objects."""
    t = as_tensor(t, what)
    if not t.is_cuda:
        raise TypeError(f"{what} must be a CUDA tensor (matfree_gb300 runs on the GPU only)")
    return t


def stream_ptr() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def empty_panel(p: int, n: int, dtype, device="cuda") -> torch.Tensor:
    return torch.zeros((p, padded_ld(n)), dtype=dtype, device=device)


def is_panel(x: torch.Tensor, n: int) -> bool:
    """True if x is a (p, n) view of a panel the kernels can read in place."""
    if x.dim() != 2 or x.shape[1] != n or x.stride(1) != 1:
        return False
    ld = x.stride(0) if x.shape[0] > 1 else padded_ld(n)
    return ld % 8 == 0 and ld >= n and x.data_ptr() % 16 == 0


def as_panel(x: torch.Tensor, n: int, dtype) -> tuple[torch.Tensor, int]:
    """Return (panel tensor, ld) holding the rows of x (p, n) in panel layout.

    Reuses x's storage when its layout already qualifies and the padding
    columns are not read as data (the kernels mask every column >= n).
    """
    x = require_cuda(x, "probe/vector panel")
    if x.dtype == dtype and is_panel(x, n):
        ld = x.stride(0) if x.shape[0] > 1 else padded_ld(n)
        return x, ld
    out = empty_panel(x.shape[0], n, dtype, x.device)
    out[:, :n].copy_(x)
    return out, out.shape[1]


class Workspace:
    """Grow-only device scratch owned by one Python object (per stream use)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int, device) -> tuple[ctypes.c_void_p, int]:
        if self.buf is None or self.buf.numel() < nbytes or self.buf.device != torch.device(device):
            self.buf = torch.empty(int(nbytes), dtype=torch.uint8, device=device)
        return ctypes.c_void_p(self.buf.data_ptr()), self.buf.numel()


def dtype_code(dtype) -> int:
    if dtype == torch.float32:
        return _lib.MFG_F32
    if dtype == torch.float64:
        return _lib.MFG_F64
    raise TypeError(f"unsupported dtype {dtype}; use float32 or float64")


class CudaArray:
    """Minimal ``__cuda_array_interface__`` wrapper of a raw device pointer."""

    def __init__(self, ptr: int, shape, strides_elems, dtype: torch.dtype):
        typestr = {torch.float32: "<f4", torch.float64: "<f8"}[dtype]
        size = torch.tensor([], dtype=dtype).element_size()
        self.__cuda_array_interface__ = {
            "shape": tuple(int(s) for s in shape),
            "strides": tuple(int(s) * size for s in strides_elems),
            "typestr": typestr,
            "data": (int(ptr), False),
            "version": 3,
        }


def wrap_device(ptr: int, shape, strides_elems, dtype) -> torch.Tensor:
    return torch.as_tensor(CudaArray(ptr, shape, strides_elems, dtype), device="cuda")
