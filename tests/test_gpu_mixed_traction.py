"""FAULT_TRACTION systems on the mixed-precision operator: the fault's
traction rows are assembled in FP64, transformed (frame, drag, constraint,
locked rows) exactly as the FP64 system's, and split into FP32 far entries
(with their BF16 copy) and FP64 near blocks.

Stated tolerances: the traction rows (far pairs by the FP32 quadrature of
the point integrand, near pairs by the FP64 closed form) within 2e-6 of each
row's largest entry of the FP64 system's rows, their right-hand side equal
to 1e-13; the displacement rows as in test_gpu_mixed.py; the solutions
within 1e-5 of the FP64 solution, with the plain FGMRES, the BF16 inner solve
and the learned two-level preconditioner inside it."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[(90.0, None), (60.0, {"fault": 0.7})])
def pair(request, gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import fault_traction_model
    from mbem_gb300.model import generate_system
    dip, drag = request.param
    model, eps = fault_traction_model(10, 8, dip)
    system = generate_system(model)
    a64 = DenseBackend(jump="calibrated", deflate=True, rtol=1e-11, maxiter=800).assemble(system, eps,
                                                                                        fault_drag=drag)
    amx = DenseBackend(jump="calibrated", deflate=True, rtol=1e-11, maxiter=800, precision="mixed",
                       precond="bf16_inner").assemble(system, eps, fault_drag=drag)
    return system, a64, amx


def _fault_rows(system):
    (region, f), = system.traction_faults()
    s = system.layout.slot(f, "b")
    return s.offset, s.stop


def test_traction_rows_are_the_fp64_rows(pair):
    system, a64, amx = pair
    r0, r1 = _fault_rows(system)
    A = amx.op.dense64()
    T64 = a64.A[r0:r1]
    Tmx = A[r0:r1]
    scale = T64.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
    worst = float(((Tmx - T64).abs() / scale).max())
    print(f"traction rows: max entry error {worst:.2e} of the row's largest entry")
    assert worst < 2e-6
    assert float((amx.b[r0:r1] - a64.b[r0:r1]).abs().max()) <= 1e-13 * float(a64.b.abs().max()) + 1e-300
    # the rest of the system: the mixed operator's own tolerance
    other = torch.ones(A.shape[0], dtype=torch.bool, device=A.device)
    other[r0:r1] = False
    assert float((A[other] - a64.A[other]).abs().max()) < 1e-6 * float(a64.A[other].abs().max())


def test_mixed_traction_solutions(pair):
    system, a64, amx = pair
    x64 = a64.solve_device(precond="block_jacobi")
    assert a64.report.converged
    x0 = amx.solve_device(precond="block_jacobi")
    assert amx.report.converged and amx.report.true_relres < 1e-11
    assert float((x0 - x64).norm() / x64.norm()) < 1e-5
    for pc in ("bf16_inner", "bf16_learned"):
        x1 = amx.solve_device(precond=pc, maxiter=200)
        rep = amx.report
        print(f"{pc}: {rep.iterations} outer iterations, true relres {rep.true_relres:.2e}")
        assert rep.converged and rep.true_relres < 1e-11
        assert float((x1 - x64).norm() / x64.norm()) < 1e-5
