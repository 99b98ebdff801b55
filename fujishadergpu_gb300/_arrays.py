"""Device-array plumbing for the ctypes layer.

The reference passes ``cupy.ndarray`` blocks; this package accepts any CUDA
device array: torch tensors, objects exporting ``__cuda_array_interface__``
(CuPy, Numba) or ``__dlpack__``.  Results are returned as torch tensors, or
as CuPy arrays when the input was CuPy.  NumPy inputs are uploaded to the
current CUDA device first.  There is no host compute path.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional

import numpy as np


def _torch():
    import torch
    return torch


@dataclass
class DevView:
    tensor: Any          # torch tensor keeping the memory alive
    ptr: int
    h: int
    w: int
    ld: int              # row pitch in elements
    origin: str          # "torch" | "cupy" | "dlpack" | "numpy"


def require_cuda():
    torch = _torch()
    if not torch.cuda.is_available():
        from ._native import FsgError, FSG_ERR_UNSUPPORTED
        raise FsgError(FSG_ERR_UNSUPPORTED, "no CUDA device: fujishadergpu_gb300 has no CPU path")


def as_device_f32_2d(x, *, name: str = "block") -> DevView:
    """View ``x`` as a float32 2-D device array with unit column stride."""
    torch = _torch()
    require_cuda()
    origin = "torch"
    if isinstance(x, torch.Tensor):
        t = x
    elif isinstance(x, np.ndarray):
        origin = "numpy"
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda()
    elif hasattr(x, "__cuda_array_interface__"):
        origin = "cupy" if type(x).__module__.startswith("cupy") else "dlpack"
        t = torch.as_tensor(x, device="cuda")
    elif hasattr(x, "__dlpack__"):
        origin = "dlpack"
        t = torch.from_dlpack(x)
    else:
        raise TypeError(f"{name}: expected a CUDA device array, got {type(x).__name__}")
    if t.dim() != 2:
        raise ValueError(f"{name}: expected a 2-D array, got shape {tuple(t.shape)}")
    if not t.is_cuda:
        t = t.cuda()
    if t.dtype != torch.float32:
        t = t.to(torch.float32)
    if t.stride(1) != 1 or (t.shape[0] > 1 and t.stride(0) < t.shape[1]):
        t = t.contiguous()
    ld = t.stride(0) if t.shape[0] > 1 else max(1, t.shape[1])
    return DevView(t, t.data_ptr(), int(t.shape[0]), int(t.shape[1]), int(ld), origin)


def empty(h: int, w: int, dtype: str = "float32", device=None):
    torch = _torch()
    dt = {"float32": torch.float32, "uint8": torch.uint8, "int16": torch.int16}[dtype]
    return torch.empty((h, w), dtype=dt, device=device if device is not None else "cuda")


def wrap_result(t, origin: str):
    """Return ``t`` in the array family of the input."""
    if origin == "cupy":
        import cupy  # only reached when the caller passed CuPy arrays
        return cupy.asarray(t)
    return t


def current_stream_handle() -> int:
    torch = _torch()
    return int(torch.cuda.current_stream().cuda_stream)


def tensor_ptr(t) -> Optional[int]:
    return None if t is None else int(t.data_ptr())
