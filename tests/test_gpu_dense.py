"""The GPU dense backend and readout against the reference's own dense
backend (goldens made by the reference) and the C oracle.

Tolerances: system entries 1e-12 of max|A| (FP64 kernels, rewritten
contractions); solution 1e-10 relative (the deflated FGMRES runs to a true
relative residual of 1e-12, the reference solves by bordered LU); stress
readout 1e-10 relative (the GPU sums the eigenstress over every element,
the reference over its 20 (eps + h) near list).
"""

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _sub(g, tag):
    return {k[len(tag):]: v for k, v in g.items() if k.startswith(tag)} if tag else g


@pytest.mark.parametrize("tag", ["", "nu30_"])
def test_small_cube_system_and_solution(gpu, cube_small, tag):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.evaluate import evaluate_stress
    from mbem_gb300.model import generate_system
    g = _sub(cube_small, tag)
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12).assemble(generate_system(model), eps)
    assert rel_err(asm.A.cpu().numpy(), g["A"]) < 1e-12
    assert rel_err(asm.b.cpu().numpy(), g["b"]) < 1e-12
    assert rel_err(next(iter(asm.calib.values())).cpu().numpy(), g["calib"]) < 1e-12
    sol = asm.solve()
    assert asm.report.converged and asm.report.true_relres < 1e-12
    assert rel_err(sol["u:cube"].ravel(), g["x"]) < 1e-10
    sig, eig = evaluate_stress(model, "body", sol, g["points"], eps, parts=True, warn_near=False)
    assert rel_err(sig, g["stress"]) < 1e-10
    assert rel_err(eig, g["stress_eigen"]) < 1e-10


def test_c1_config_rows_solution_and_readout(gpu, c1_rows):
    """Config 1 (12x12 per face, fault 8x8, eps = h/2): sampled rows of A, b,
    the deflated solution, FGMRES(50) iteration counts and the stress
    readout against the reference."""
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.evaluate import evaluate_stress
    from mbem_gb300.model import generate_system
    g = c1_rows
    model, eps = cube_fault_model(12, 8)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    A = asm.A
    rows = torch.from_numpy(g["rows"]).cuda()
    assert rel_err(A[rows].cpu().numpy(), g["A_rows"]) < 1e-12
    assert rel_err(asm.b.cpu().numpy(), g["b"]) < 1e-12
    # FGMRES(50) to 1e-8 and 1e-10: the reference took 20 and 24 iterations
    for rtol, its_ref, _, _ in g["fgmres"]:
        asm.solve(rtol=rtol)
        assert asm.report.converged
        assert abs(asm.report.iterations - its_ref) <= 2
    sol = asm.solve(rtol=1e-12)
    assert rel_err(sol["u:cube"].ravel(), g["x"]) < 1e-10
    sig = evaluate_stress(model, "body", sol, g["points"], eps, warn_near=False)
    assert rel_err(sig, g["stress"]) < 1e-9


def test_gpu_system_matches_oracle_system(gpu, oracle):
    """A larger cube (n = 6: 432 + 32 elements) against the oracle assembly."""
    from oracle.cpu_system import assemble
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(6, 4, 1.3, 1.95)
    system = generate_system(model)
    A_ref, b_ref, _ = assemble(oracle, system, eps)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(system, eps)
    assert rel_err(asm.A.cpu().numpy(), A_ref) < 1e-12
    assert rel_err(asm.b.cpu().numpy(), b_ref) < 1e-12


def test_half_jump_and_anchor_rules(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(2, 2)
    with pytest.raises(ValueError):
        DenseBackend(jump="calibrated", deflate=False).assemble(generate_system(model), eps)
    asm = DenseBackend(jump="half", deflate=True).assemble(generate_system(model), eps)
    A = asm.A.cpu().numpy()
    B = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps).A.cpu().numpy()
    # the two differ only on the 3x3 diagonal blocks
    off = A - B
    for c in range(A.shape[0] // 3):
        off[3 * c:3 * c + 3, 3 * c:3 * c + 3] = 0.0
    assert np.abs(off).max() == 0.0


def test_fault_traction_system_and_solution(gpu, traction_small):
    """A FAULT_TRACTION fault (solved slip under a uniform shear-traction
    drop) in a 2x2-per-face cube: the whole system (traction rows through the
    nodal machinery at order 0, row frame, constraint rows) and the slip
    against the reference's bordered LU."""
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import BCType, generate_system
    g = traction_small
    model, eps = cube_fault_model(2, 2, fault_kind=BCType.FAULT_TRACTION, fault_value=g["drop"])
    assert eps == float(g["eps"])
    cube = model.regions[0].patches[0].mesh
    fault = model.regions[0].faults[0].mesh
    assert np.array_equal(cube.vertices, g["cube_vertices"])
    assert np.array_equal(fault.triangles, g["fault_triangles"])
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-13).assemble(generate_system(model), eps)
    assert rel_err(asm.A.cpu().numpy(), g["A"]) < 1e-12
    assert rel_err(asm.b.cpu().numpy(), g["b"]) < 1e-12
    sol = asm.solve()
    assert asm.report.converged
    assert rel_err(sol["u:cube"], g["x_u"]) < 1e-10
    assert rel_err(sol["b:fault"], g["x_b"]) < 1e-10
    # the constraint rows hold: no opening
    nrm = model.regions[0].faults[0].collocation_normals()
    assert np.abs(np.einsum("ij,ij->i", sol["b:fault"], nrm)).max() < 1e-12 * np.abs(sol["b:fault"]).max()


def test_rebuild_for_materials_equals_fresh_assembly(gpu):
    """rebuild_for_materials (dense.py:650-688): the same operator as a fresh
    assembly of the model with the new material (1e-14); unknown regions refused."""
    from mbem_gb300 import mesh as M
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(4, 2, 1.0, 1.0)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    new_mat = M.ElasticMaterial(mu=2.5, lam=1.7)
    re = asm.rebuild_for_materials({"body": new_mat})
    model2, _ = cube_fault_model(4, 2, 2.5, 1.7)
    fresh = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model2), eps)
    assert float((re.A - fresh.A).abs().max() / fresh.A.abs().max()) < 1e-14
    assert float((re.b - fresh.b).abs().max() / fresh.b.abs().max()) < 1e-14
    assert float((asm.A - fresh.A).abs().max()) > 0.0          # the original is untouched
    with pytest.raises(KeyError):
        asm.rebuild_for_materials({"nowhere": new_mat})
