"""Many right-hand sides: the tensor-core product Y = A X (``mbem_gemm_bf16``)
that replaces one matvec per right-hand side by one GEMM per iteration.

The reference solves many right-hand sides by one LU factorisation and its
triangular solves (src/mbem/la/lu.py:110-258, the refinement product at
:210); here the operator stays in HBM once as BF16 and every product over
the whole block of right-hand sides reads it once.
"""

from __future__ import annotations

import torch

from .. import _native as nat
from .._device import ptr, stream_handle

MAX_RHS = 256


def gemm_bf16(A: torch.Tensor, Xt: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Y (M, n) FP32 = A (M, K) @ Xt (n, K)^T for BF16 CUDA tensors with
    unit column stride; n <= 256 (larger blocks: call per 256 columns)."""
    if A.dtype != torch.bfloat16 or Xt.dtype != torch.bfloat16 or not A.is_cuda:
        raise ValueError("A and Xt must be bfloat16 CUDA tensors")
    if A.stride(1) != 1 or Xt.stride(1) != 1 or A.shape[1] != Xt.shape[1]:
        raise ValueError("A (M, K) and Xt (n, K) need unit column strides and one K")
    M, K = A.shape
    n = Xt.shape[0]
    if not 1 <= n <= MAX_RHS:
        raise ValueError(f"1..{MAX_RHS} right-hand sides per product (got {n})")
    Y = out if out is not None else torch.empty((M, n), dtype=torch.float32, device=A.device)
    nat.call("mbem_gemm_bf16", ptr(A), A.stride(0), ptr(Xt), Xt.stride(0), M, K, n, ptr(Y), Y.stride(0),
             stream_handle())
    return Y


def gemm_check():
    """Synchronises and raises if a tensor-core pipeline wait gave up."""
    nat.call("mbem_gemm_bf16_check", stream_handle())
