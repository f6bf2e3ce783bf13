"""Array-module interop at the operator boundary.

Mirrors mri-nufft's ``with_numpy_cupy`` / ``_to_interface`` contract
(``src/mrinufft/_array_compat.py:183-492``): whatever array type comes in
(numpy, torch CPU/CUDA, cupy or any ``__cuda_array_interface__`` /
DLPack producer) is what comes out, on the same device.  Device arrays
cross zero-copy through DLPack when they already are contiguous complex64
on the operator's GPU; host arrays are copied to the device once and the
result copied back once.

Host (numpy) results are returned in page-locked memory taken from torch's
caching host allocator (``PINNED_RESULTS``): the device-to-host copy then
runs at DMA speed, and a numpy result passed back in (``adj_op(op(x))``, the
iterations of a solver on host arrays) is copied to the device
asynchronously as a page-locked buffer.  The arrays are ordinary numpy
arrays; a freed one returns its block to the allocator's cache.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

# numpy results in page-locked host memory (False: pageable ``Tensor.cpu()``)
PINNED_RESULTS = True


@dataclass
class Interface:
    kind: str  # "numpy" | "torch" | "cupy" | "cai"
    device: object = None  # torch.device of a torch input


def module_name(x) -> str:
    return type(x).__module__.partition(".")[0]


def is_device_array(x) -> bool:
    if isinstance(x, torch.Tensor):
        return x.is_cuda
    return hasattr(x, "__cuda_array_interface__")


def interface_of(x) -> Interface:
    if isinstance(x, torch.Tensor):
        return Interface("torch", x.device)
    name = module_name(x)
    if name == "cupy":
        return Interface("cupy")
    if hasattr(x, "__cuda_array_interface__"):
        return Interface("cai")
    return Interface("numpy")


def to_tensor(x, device: torch.device, dtype: torch.dtype) -> torch.Tensor:
    """Any supported array -> contiguous torch tensor of ``dtype`` on ``device``."""
    if isinstance(x, torch.Tensor):
        t = x.detach()
    elif module_name(x) == "cupy" or hasattr(x, "__dlpack__") and is_device_array(x):
        t = torch.from_dlpack(x)
    elif hasattr(x, "__cuda_array_interface__"):
        t = torch.as_tensor(x, device=device)
    else:
        a = np.asarray(x)
        if a.dtype.kind == "c":
            a = a.astype(np.complex64, copy=False)
        elif a.dtype.kind in "fiub":
            a = a.astype(np.float32 if dtype != torch.complex64 else np.complex64, copy=False)
        t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype != dtype:
        t = t.to(dtype)
    if t.device != device:
        # pinned host memory copies asynchronously on the current stream
        t = t.to(device, non_blocking=t.device.type == "cpu" and t.is_pinned())
    return t.contiguous()


def from_tensor(t: torch.Tensor, like: Interface):
    """Torch CUDA tensor -> the caller's array interface."""
    if like.kind == "torch":
        return t if t.device == like.device else t.to(like.device)
    if like.kind == "cupy":
        import cupy as cp

        return cp.from_dlpack(t)
    if like.kind == "cai":
        return t
    if PINNED_RESULTS and t.is_cuda:
        out = pinned_empty(t.shape, t.dtype)
        if out is not None:
            out.copy_(t, non_blocking=True)
            torch.cuda.current_stream(t.device).synchronize()
            return out.numpy()
    return t.cpu().numpy()


def pinned_empty(shape, dtype):
    """A page-locked host tensor, or None when the host cannot lock that much
    memory (the caller then falls back to pageable memory)."""
    try:
        return torch.empty(shape, dtype=dtype, pin_memory=True)
    except RuntimeError:
        return None
