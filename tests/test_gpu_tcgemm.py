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


@pytest.mark.parametrize("M,N,K", [(300, 7, 384), (1000, 64, 384), (936, 64, 384), (520, 130, 384), (200, 256, 192),
                                   (777, 33, 64), (128, 16, 384), (1500, 300, 384)])
def test_gemm_sub_update(gpu, M, N, K):
    """C -= A Bt^T (the LU update) against FP64 products of the same BF16
    operands: FP32 accumulation, tolerance 1e-5 of max|A Bt^T|; rows and
    columns outside C untouched."""
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    g = torch.Generator(device="cpu").manual_seed(M + N)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    Bt = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    ldc = N + 5
    C0 = torch.randn(M + 3, ldc, generator=g).cuda()
    C = C0.clone()
    nat.call("mbem_gemm_bf16_sub", ptr(A), A.stride(0), ptr(Bt), Bt.stride(0), M, N, K, ptr(C), ldc, stream_handle())
    torch.cuda.synchronize()
    P = A.double() @ Bt.double().T
    ref = C0.double().clone()
    ref[:M, :N] -= P
    err = float((C.double() - ref).abs().max() / P.abs().max())
    assert err < 1e-5, err
    assert torch.equal(C[M:], C0[M:]) and torch.equal(C[:, N:], C0[:, N:])
