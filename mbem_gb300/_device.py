"""Device-array plumbing: numpy or torch in, CUDA float64 tensors to the C ABI.

Kernel drivers accept numpy arrays (the reference's types) or torch tensors.
Inputs are made C-contiguous float64 CUDA tensors; outputs come back as
numpy when the caller passed numpy (a drop-in for the reference's numba
drivers) and stay on the device when the caller passed torch tensors.
"""

from __future__ import annotations

import numpy as np
import torch


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("mbem_gb300 needs a CUDA device (sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def as_cuda(x, dtype=torch.float64) -> torch.Tensor:
    dev = require_cuda()
    if isinstance(x, torch.Tensor):
        t = x.to(device=dev, dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x), dtype=np.dtype(str(dtype).split(".")[-1])))
        t = t.to(dev, non_blocking=False)
    return t.contiguous()


def is_torch(*xs) -> bool:
    return any(isinstance(x, torch.Tensor) for x in xs)


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    return t.data_ptr() if t.numel() else None


def out_like(t: torch.Tensor, torch_in: bool):
    return t if torch_in else t.cpu().numpy()
