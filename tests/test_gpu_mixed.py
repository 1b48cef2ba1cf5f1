"""Mixed-precision operator (FP32 quadrature far field + FP64 near blocks)
against the FP64 closed-form operator.

Stated tolerances (mixed mode): far entries within 1e-6 of the largest
far entry of the matrix, near entries equal to the FP64 operator's to 1e-13
of max|A|, the mixed matvec equal to the mixed operator applied in FP64 to
1e-13, and the mixed solution within 1e-5 of the FP64 solution.
"""

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(8, 4, 1.3, 1.95)
    system = generate_system(model)
    a64 = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12).assemble(system, eps)
    amx = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12, precision="mixed").assemble(system, eps)
    return a64, amx


def test_mixed_operator_entries(systems):
    a64, amx = systems
    A = a64.A.cpu().numpy()
    M = amx.op.dense64().cpu().numpy()
    nl = amx.op.near[0]
    near = np.zeros_like(A, dtype=bool)
    rp = nl.rowptr.cpu().numpy()
    f = np.repeat(np.arange(nl.n_field), np.diff(rp))
    s = nl.cols.cpu().numpy()
    for i in range(3):
        for j in range(3):
            near[3 * f + i, 3 * s + j] = True
    # the 3x3 diagonal blocks carry each operator's own calibration (the row
    # sums of that operator), so they are compared through the null space
    diag = np.zeros_like(near)
    for c in range(A.shape[0] // 3):
        diag[3 * c:3 * c + 3, 3 * c:3 * c + 3] = True
    scale = np.abs(A).max()
    near_err = np.abs(M - A)[near & ~diag].max() / scale
    far_err = np.abs(M - A)[~near].max() / np.abs(A[~near]).max()
    diag_err = np.abs(M - A)[diag].max() / scale
    print(f"near {near_err:.2e} far {far_err:.2e} diag {diag_err:.2e} near fraction {near.mean():.3f}")
    assert near_err < 1e-13
    assert far_err < 1e-6
    assert diag_err < 1e-6
    # every row has its self block, and the calibrated mixed operator
    # annihilates rigid translations exactly
    assert all(f0 in s[rp[f0]:rp[f0 + 1]] for f0 in range(nl.n_field))
    from mbem_gb300.backends.dense import translation_basis
    Z = translation_basis(amx.layout)
    assert np.abs(M @ Z).max() < 1e-13 * scale


@pytest.mark.parametrize("ns", [129, 200, 32])
def test_near_list_from_mask_equals_classification(gpu, ns):
    """The far kernel's ballot mask gives the same near list as the
    stand-alone classification pass (ragged source counts: partial words,
    a block with a single live warp)."""
    from mbem_gb300._device import as_cuda
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.mixed import far_near_block, near_list
    rng = np.random.default_rng(ns)
    c = rng.uniform(-1, 1, size=(ns, 3))
    tv = c[:, None, :] + rng.normal(scale=0.15, size=(ns, 3, 3))
    cr = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
    nrm = cr / np.linalg.norm(cr, axis=1)[:, None]
    x = rng.uniform(-1.2, 1.2, size=(97, 3))
    e = rng.uniform(0.02, 0.1, ns)
    X, T, N, E = as_cuda(x), as_cuda(tv), as_cuda(nrm), as_cuda(e)
    far = torch.empty((3 * 97, 3 * ns), dtype=torch.float32, device="cuda")
    nl = far_near_block("T", X, T, N, E, kb.t_coeffs(1.0, 1.0), 1.0, far)
    rowptr, cols = near_list(X, T, E)
    assert torch.equal(nl.rowptr, rowptr)
    assert torch.equal(nl.cols, cols)
    assert nl.nnz > 0


def test_mixed_matvec_is_exact_for_its_operator(systems):
    _, amx = systems
    x = torch.randn(amx.op.n, dtype=torch.float64, device="cuda")
    y = amx.op.matvec(x)
    ref = amx.op.dense64() @ x
    assert rel_err(y.cpu().numpy(), ref.cpu().numpy()) < 1e-13


def test_mixed_solution_against_fp64(systems):
    a64, amx = systems
    x64 = a64.solve_device()
    xmx = amx.solve_device()
    assert a64.report.converged and amx.report.converged
    err = float((xmx - x64).norm() / x64.norm())
    # the FP64 operator's residual of the mixed solution
    Pb = a64.b.clone()
    r = (a64.A @ xmx - a64.b)
    print(f"mixed vs fp64 solution {err:.2e}; its(fp64) {a64.report.iterations} "
          f"its(mixed) {amx.report.iterations}")
    assert err < 1e-5
    assert amx.report.true_relres < 1e-12
    del Pb, r


def test_bf16_matvec_against_rounded_operator(systems):
    """The BF16 inner operator equals bf16(A_far) x + near x, summed in FP32
    (tolerance 1e-5 of max|y|), and is within 2^-8 of the mixed operator."""
    from mbem_gb300.la.mixed import Bf16Inner
    _, amx = systems
    inner = Bf16Inner(amx.op, 4, amx.u_ranges())
    x = torch.randn(amx.op.n, dtype=torch.float64, device="cuda")
    y = inner.matvec(x)
    n = amx.op.n
    A16 = inner.A16[:, :n].to(torch.float64)
    ref = A16 @ x.to(torch.float32).to(torch.float64)
    for nb in amx.op.near:
        rp = nb.rowptr.cpu().numpy()
        f = torch.from_numpy(np.repeat(np.arange(nb.n_field), np.diff(rp))).to(x.device)
        v = nb.vals.view(-1, 3, 3)
        contrib = torch.einsum("kij,kj->ki", v, x[nb.col0:].view(-1, 3)[nb.cols])
        ref.view(-1, 3)[nb.row0 // 3:].index_add_(0, f, contrib)
    assert rel_err(y.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    y32 = amx.op.matvec(x)
    assert float((y - y32).norm() / y32.norm()) < 2.0 ** -8


def test_bf16_inner_preconditioned_solve(systems):
    """FGMRES on the mixed operator with the BF16 inner solve as flexible
    preconditioner: same convergence test (the mixed operator's true
    residual), the solution within 1e-9 of the unpreconditioned one, and
    fewer outer iterations."""
    _, amx = systems
    x0 = amx.solve_device(precond="none")
    its0 = amx.report.iterations
    x1 = amx.solve_device(precond=amx.bf16_inner(6))
    rep = amx.report
    assert rep.converged and rep.true_relres < 1e-12
    assert float((x1 - x0).norm() / x0.norm()) < 1e-9
    assert rep.iterations < its0


def test_fused_bf16_copy_equals_conversion(gpu):
    """precond="bf16_inner" makes the far-field assembly write the BF16 copy
    in the same pass: it equals the rounding of the FP32 far field bit for
    bit, and the preconditioned solve converges to the plain solution."""
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(8, 4, 1.3, 1.95)
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12, precision="mixed",
                       precond="bf16_inner").assemble(generate_system(model), eps)
    n = asm.op.n
    assert asm.op.A16 is not None
    ref = torch.empty_like(asm.op.A16)
    nat.call("mbem_to_bf16", ptr(asm.op.A32), 0, asm.op.A32.stride(0), n, n, ptr(ref), ref.stride(0),
             stream_handle())
    assert torch.equal(asm.op.A16[:, :n].view(torch.int16), ref[:, :n].view(torch.int16))
    x1 = asm.solve_device()
    assert asm.report.converged and asm.report.true_relres < 1e-12
    x0 = asm.solve_device(precond="none")
    assert float((x1 - x0).norm() / x0.norm()) < 1e-9


@pytest.mark.parametrize("order,n_face", [(1, 5), (2, 3)])
def test_mixed_nodal_operator(gpu, order, n_face):
    """The mixed operator of a P1/P2 cube (FP32 far quadrature weighted by
    the Lagrange shape functions, FP64 nodal near blocks, the calibrated
    diagonal spread by the collocation shape) against the FP64 nodal
    operator: near blocks to 1e-13 of max|A|, far entries to 1e-6 of the
    largest far entry, rigid translations annihilated, and the solution
    within 1e-5 of the FP64 solution."""
    from mbem_gb300.backends.dense import DenseBackend, translation_basis
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, 2, 1.3, 1.95, cube_order=order)
    system = generate_system(model)
    a64 = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12).assemble(system, eps)
    amx = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12, precision="mixed").assemble(system, eps)
    A = a64.A.cpu().numpy()
    M = amx.op.dense64().cpu().numpy()
    K = 3 if order == 1 else 6
    nl = amx.op.near[0]
    rp = nl.rowptr.cpu().numpy()
    f = np.repeat(np.arange(nl.n_field), np.diff(rp))
    s = nl.cols.cpu().numpy()
    near = np.zeros_like(A, dtype=bool)
    for i in range(3):
        for j in range(3):
            near[3 * f + i, 3 * s + j] = True
    # the blocks of each collocation point on its own element's nodes carry
    # each operator's own calibration: compared through the null space
    own = np.zeros_like(near)
    for c in range(A.shape[0] // 3):
        e = c // K
        own[3 * c:3 * c + 3, 3 * K * e:3 * K * e + 3 * K] = True
    scale = np.abs(A).max()
    near_err = np.abs(M - A)[near & ~own].max() / scale
    far_err = np.abs(M - A)[~near].max() / np.abs(A[~near]).max()
    own_err = np.abs(M - A)[own].max() / scale
    print(f"order {order}: near {near_err:.2e} far {far_err:.2e} own {own_err:.2e} near fraction {near.mean():.3f}")
    assert near_err < 1e-13
    assert far_err < 1e-6
    assert own_err < 1e-6
    Z = translation_basis(amx.layout)
    assert np.abs(M @ Z).max() < 1e-12 * scale
    x64 = a64.solve_device()
    xmx = amx.solve_device()
    assert a64.report.converged and amx.report.converged
    assert float((xmx - x64).norm() / x64.norm()) < 1e-5
