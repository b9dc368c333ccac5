"""Device-buffer plumbing: PyTorch tensors hold every device array.

NumPy inputs are copied to the current CUDA device (float64 / complex128,
C-contiguous); torch CUDA tensors pass through without a host round trip.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fluidlets_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def home(*arrays):
    """Where results go: None (NumPy in, NumPy out), or the torch device of the
    inputs ("cuda" if any input is a CUDA tensor, else "cpu")."""
    ts = [a for a in arrays if isinstance(a, torch.Tensor)]
    if not ts:
        return None
    return "cuda" if any(t.is_cuda for t in ts) else "cpu"


def is_torch(*arrays) -> bool:
    return any(isinstance(a, torch.Tensor) for a in arrays)


def stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def to_dev(a, dtype: torch.dtype) -> torch.Tensor:
    dev = require_cuda()
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous()
    arr = np.ascontiguousarray(np.asarray(a), dtype=torch_to_numpy(dtype))
    if not arr.flags.writeable:
        arr = arr.copy()
    return torch.from_numpy(arr).to(dev)


def workspace(nbytes: int) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=require_cuda())


def torch_to_numpy(dtype: torch.dtype):
    return {torch.float64: np.float64, torch.complex128: np.complex128, torch.float32: np.float32,
            torch.int64: np.int64, torch.int32: np.int32}[dtype]


def is_complex_value(a) -> bool:
    if isinstance(a, torch.Tensor):
        return a.is_complex()
    return np.iscomplexobj(a)


def to_host(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy()
