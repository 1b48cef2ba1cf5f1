"""The tcgen05 multi-RHS GEMM against torch's FP32 product of the same BF16
operands. Tolerance: 1e-5 of the largest output entry (both accumulate in
FP32; the summation orders differ), 3e-5 for K = 4096."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ref(A, Xt):
    return A.float() @ Xt.float().T


@pytest.mark.parametrize("M,K,n", [(128, 64, 16), (300, 200, 37), (256, 1000, 256), (129, 72, 64), (64, 8, 5)])
def test_gemm_bf16_small(gpu, M, K, n):
    from mbem_gb300.la.multirhs import gemm_bf16, gemm_check
    g = torch.Generator(device="cuda").manual_seed(M * 1000 + K + n)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    Xt = torch.randn((n, K), generator=g, device="cuda").to(torch.bfloat16)
    Y = gemm_bf16(A, Xt)
    gemm_check()
    R = _ref(A, Xt)
    assert float((Y - R).abs().max() / R.abs().max()) < 1e-5


def test_gemm_bf16_large_and_strided(gpu):
    from mbem_gb300.la.multirhs import gemm_bf16, gemm_check
    g = torch.Generator(device="cuda").manual_seed(7)
    big = torch.randn((4100, 4104), generator=g, device="cuda").to(torch.bfloat16)
    A = big[:4096, :4096]                          # lda = 4104
    Xt = torch.randn((256, 4096), generator=g, device="cuda").to(torch.bfloat16)
    out = torch.full((4096, 260), 7.0, device="cuda")
    gemm_bf16(A, Xt, out=out[:, :256])
    gemm_check()
    R = _ref(A, Xt)
    assert float((out[:, :256] - R).abs().max() / R.abs().max()) < 3e-5
    assert torch.all(out[:, 256:] == 7.0)


@pytest.mark.parametrize("M,K,n", [(1000, 4096, 256), (20736, 1024, 64), (200, 640, 16)])
def test_gemm_split_k(gpu, M, K, n):
    """The K-split product (partial sums in slice order) equals the product."""
    from mbem_gb300.la.multirhs import gemm_bf16_t, gemm_check
    g = torch.Generator(device="cuda").manual_seed(M + K + n)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    Xt = torch.randn((n, K), generator=g, device="cuda").to(torch.bfloat16)
    out = torch.empty((n, M), device="cuda")
    gemm_bf16_t(A, Xt, K, out, split=True)
    gemm_check()
    ref = (A.float() @ Xt.float().T).T
    assert float((out - ref).abs().max() / ref.abs().max()) < 3e-5
