"""Many right-hand sides: the batched GMRES kernels against torch, and the
block solver (batched GMRES on the BF16 tensor-core operator inside
FP64-accurate refinement) against the single-RHS FGMRES of the same
operator.

Tolerances: kernels 1e-5 relative (FP32 vectors); solutions of the block
solver at true relative residual 1e-10 agree with the single-RHS solutions
to 1e-8 relative, and every true residual (recomputed here in FP64) is below
the target.
"""

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_gemm_transposed_output(gpu):
    from mbem_gb300.la.multirhs import gemm_bf16_t
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn((300, 264), generator=g, device="cuda").to(torch.bfloat16)
    Xt = torch.randn((40, 264), generator=g, device="cuda").to(torch.bfloat16)
    out = torch.zeros((40, 304), device="cuda")
    gemm_bf16_t(A, Xt, 264, out)
    ref = (A.float() @ Xt.float().T).T
    assert float((out[:, :300] - ref).abs().max() / ref.abs().max()) < 1e-5
    assert torch.all(out[:, 300:] == 0)


def test_batched_vector_kernels(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    g = torch.Generator(device="cuda").manual_seed(5)
    nv, k, n = 4, 7, 1003
    V = torch.randn((nv, k, n), generator=g, device="cuda")
    W = torch.randn((k, n), generator=g, device="cuda")
    H = torch.empty((nv, k), dtype=torch.float64, device="cuda")
    st = stream_handle()
    nat.call("mbem_batch_dots", ptr(V), nv, ptr(W), k, n, ptr(H), st)
    ref = torch.einsum("ikn,kn->ik", V.double(), W.double())
    assert rel_err(H.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    W2 = W.clone()
    nat.call("mbem_batch_axpy", ptr(W2), ptr(V), nv, ptr(H), -0.5, k, n, st)
    ref2 = W.double() - 0.5 * torch.einsum("ik,ikn->kn", H, V.double())
    assert rel_err(W2.cpu().numpy(), ref2.cpu().numpy()) < 1e-5
    norms = torch.empty(k, dtype=torch.float64, device="cuda")
    Vo = torch.empty((k, n), device="cuda")
    Vb = torch.empty((k, n), dtype=torch.bfloat16, device="cuda")
    nat.call("mbem_batch_normalize", ptr(W), 0, k, n, ptr(norms), ptr(Vo), ptr(Vb), st)
    assert rel_err(norms.cpu().numpy(), torch.linalg.vector_norm(W.double(), dim=1).cpu().numpy()) < 1e-6
    assert rel_err(Vo.cpu().numpy(), (W.double() / norms[:, None]).cpu().numpy()) < 1e-6
    assert torch.equal(Vb, Vo.to(torch.bfloat16))
    X = torch.randn((k, n), generator=g, device="cuda", dtype=torch.float64)
    X0 = X.clone()
    nat.call("mbem_batch_update", ptr(X), ptr(V), nv, ptr(H), k, n, st)
    assert rel_err(X.cpu().numpy(), (X0 + torch.einsum("ik,ikn->kn", H, V.double())).cpu().numpy()) < 1e-6
    rng = np.array([0, 300, 600, 303], dtype=np.int64)
    import ctypes
    Xp = X.clone()
    nat.call("mbem_batch_project", ptr(Xp), 1, k, n, rng.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 2, st)
    sel = torch.cat([torch.arange(0, 300), torch.arange(600, 903)]).cuda()
    for c in range(3):
        comp = sel[c::3]
        assert float(Xp[:, comp].mean(dim=1).abs().max()) < 1e-12
    untouched = torch.cat([torch.arange(300, 600), torch.arange(903, n)]).cuda()
    assert torch.equal(Xp[:, untouched], X[:, untouched])


def _cube(precision):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(8, 4)
    return DenseBackend(jump="calibrated", deflate=True, rtol=1e-12, precision=precision).assemble(
        generate_system(model), eps)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_block_solver_matches_single_rhs(gpu, precision):
    from mbem_gb300.la.multirhs import BlockSolver
    asm = _cube(precision)
    n = asm.b.shape[0]
    k = 12
    rng = np.random.default_rng(1)
    B = torch.from_numpy(rng.normal(size=(k, n))).cuda()
    B[0] = asm.b
    bs = BlockSolver(asm)
    X, rep = bs.solve(B, rtol=1e-10)
    assert rep.converged, rep
    A = asm.A if asm.A is not None else asm.op.dense64()
    Bp = bs.project(B.clone())
    R = Bp - (A @ X.T).T
    bs.project(R)
    assert float((torch.linalg.vector_norm(R, dim=1) / torch.linalg.vector_norm(Bp, dim=1)).max()) < 1e-10
    for r in (0, 5, 11):
        asm.b = B[r].clone()
        x1 = asm.solve_device(rtol=1e-12)
        assert rel_err(X[r].cpu().numpy(), x1.cpu().numpy()) < 1e-8


def test_block_residual_mixed_matches_fp64(gpu):
    from mbem_gb300.la.multirhs import BlockSolver
    asm = _cube("mixed")
    n = asm.b.shape[0]
    rng = np.random.default_rng(2)
    B = torch.from_numpy(rng.normal(size=(5, n))).cuda()
    X = torch.from_numpy(rng.normal(size=(5, n))).cuda()
    bs = BlockSolver(asm)
    R = bs.residual(B, X)
    ref = B - (asm.op.dense64() @ X.T).T
    bs.project(ref)
    assert rel_err(R.cpu().numpy(), ref.cpu().numpy()) < 1e-13


def test_slip_rhs_reproduces_the_system_rhs(gpu):
    from mbem_gb300.cases import gaussian_slips
    from mbem_gb300.la.multirhs import slip_rhs
    asm = _cube("fp64")
    fault = asm.system.model.regions[0].faults[0]
    own = np.broadcast_to(fault.value_array().reshape(-1, 3), (fault.n_dofs, 3))[None]
    slips = np.concatenate([own, gaussian_slips(fault, 3, seed0=4)])
    B = slip_rhs(asm, fault, slips)
    assert rel_err(B[0].cpu().numpy(), asm.b.cpu().numpy()) < 1e-13
    assert slips.shape == (4, fault.n_dofs, 3) and np.all(np.abs(slips[1:].std(axis=(1, 2)) - 1.0) < 0.6)
