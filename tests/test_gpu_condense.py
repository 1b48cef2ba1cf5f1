"""AssembledDense.condense (dense.py:580-646) on the GPU: the Schur
complement onto the FAULT_TRACTION slip coordinates against the same
algebra in FP64 torch (1e-10 of max|S|), and the condensed solution
x = x0 + X beta, beta = S^-1 (-L), equal to the direct solve of the whole
system (1e-8)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _anchored_model(n_face=4, n_fault=3):
    from mbem_gb300 import mesh as M
    from mbem_gb300.model import BCType, Patch, Region, RegionModel
    cube_p = Patch("cube", M.cube(n_face), BCType.PRESCRIBED_DISPLACEMENT, value=np.zeros(3))
    fault_p = Patch("fault", M.centre_fault(n_fault), BCType.FAULT_TRACTION, value=np.array([-1e-3, 0.0, 0.0]))
    region = Region("body", M.ElasticMaterial(mu=1.0, lam=1.0), [cube_p], np.zeros(3), faults=[fault_p])
    return RegionModel([region]), (4.0 / n_face) / 2.0


def test_condense_against_fp64_and_direct_solve(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.model import generate_system
    model, eps = _anchored_model()
    asm = DenseBackend(jump="calibrated", deflate=False, lu="gpu").assemble(generate_system(model), eps)
    c = asm.condense()
    f = model.regions[0].faults[0]
    assert c.n == 2 * f.n_dofs and len(c.faults) == 1 and c.faults[0].name == "fault"
    # the same algebra in FP64
    A, b = asm.A, asm.b
    N = A.shape[0]
    slot = asm.layout.slot(f, "b")
    on = np.zeros(N, bool)
    on[slot.offset:slot.stop] = True
    rest = torch.from_numpy(np.flatnonzero(~on)).cuda()
    fc = c.faults[0]
    rows = torch.from_numpy((slot.offset + 3 * fc.free[:, None] + np.arange(2)[None, :]).ravel()).cuda()
    E = torch.from_numpy(c.X[slot.offset:slot.stop]).cuda()
    AE = A[:, slot.offset:slot.stop] @ E
    Xr = -torch.linalg.solve(A[rest][:, rest], AE[rest])
    S_ref = AE[rows] + A[rows][:, rest] @ Xr
    x0r = torch.linalg.solve(A[rest][:, rest], b[rest])
    L_ref = -b[rows] + A[rows][:, rest] @ x0r
    assert np.abs(c.S - S_ref.cpu().numpy()).max() < 1e-10 * np.abs(c.S).max()
    assert np.abs(c.L - L_ref.cpu().numpy()).max() < 1e-10 * np.abs(c.L).max()
    # the condensed solution is the whole system's solution
    beta = np.linalg.solve(c.S, -c.L)
    x = c.x0 + c.X @ beta
    x_ref = asm.solve_device().cpu().numpy()
    assert np.abs(x - x_ref).max() < 1e-8 * np.abs(x_ref).max()
    # coordinates <-> Cartesian round trip on the free nodes
    v = np.random.default_rng(0).normal(size=fc.stop - fc.start)
    assert np.allclose(fc.coordinates(fc.cartesian(v)), v)
    assert c.dragged(1e3).shape == (c.n,)


def test_condense_refusals(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model, fault_traction_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(3, 2)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    with pytest.raises(ValueError, match="no FAULT_TRACTION"):
        asm.condense()
    model, eps = fault_traction_model(3, 2)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    with pytest.raises(ValueError, match="deflate"):
        asm.condense()


def test_drag_solve_equals_condensed_drag(gpu):
    """An operator built with a fault drag kappa solves for the slip that the
    drag-free condensed body gives by (kappa - S) beta = L (dense.py:333-340)."""
    from mbem_gb300.backends.dense import AssembledDense
    from mbem_gb300.model import generate_system
    model, eps = _anchored_model()
    system = generate_system(model)
    c = AssembledDense(system, eps, jump="calibrated", deflate=False, lu="gpu").condense()
    kappa = 0.7
    dr = AssembledDense(system, eps, jump="calibrated", deflate=False, lu="gpu", fault_drag={"fault": kappa})
    x = dr.solve_device().cpu().numpy()
    fc = c.faults[0]
    slot = system.layout.slot(model.regions[0].faults[0], "b")
    beta_solve = fc.coordinates(x[slot.offset:slot.stop].reshape(-1, 3))
    beta = c.dragged(kappa)
    assert np.abs(beta_solve - beta).max() < 1e-8 * np.abs(beta).max()
    with pytest.raises(ValueError, match="drag"):
        dr.condense()
    with pytest.raises(KeyError):
        AssembledDense(system, eps, jump="calibrated", deflate=False, fault_drag={"cube": 1.0})


@pytest.mark.parametrize("tag", ["tangential", "opening"])
def test_condense_against_reference_golden(gpu, condense_small, tag):
    """The reference's own ``AssembledDense.condense()`` (dense.py:580-646)
    on an anchored 3x3-per-face cube with a 3x3 FAULT_TRACTION fault
    (tests/golden/condense_small.npz): strike and dip with locked elements,
    and all three components without. The free nodes, frame rows and
    coordinate ranges equal the reference's exactly; S, L, X and x0 agree to
    1e-10 of their largest entries; the condensed slip equals the reference's
    solve."""
    from mbem_gb300 import mesh as M
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.model import BCType, Patch, Region, RegionModel, generate_system
    g = condense_small
    cube = M.cube(3)
    fault = M.centre_fault(3)
    assert np.array_equal(cube.vertices, g["cube_vertices"]) and np.array_equal(cube.triangles, g["cube_triangles"])
    assert np.array_equal(fault.vertices, g["fault_vertices"])
    locked = g["locked"] if tag == "tangential" else None
    cube_p = Patch("cube", cube, BCType.PRESCRIBED_DISPLACEMENT, value=np.zeros(3))
    fault_p = Patch("fault", fault, BCType.FAULT_TRACTION, value=g[f"{tag}_value"],
                    allow_opening=tag == "opening", locked=locked)
    model = RegionModel([Region("body", M.ElasticMaterial(1.0, 1.0), [cube_p], np.zeros(3), faults=[fault_p])])
    eps = float(g["eps"])
    asm = DenseBackend(jump="calibrated", deflate=False, lu="gpu").assemble(generate_system(model), eps)
    c = asm.condense()
    (fc,) = c.faults
    assert np.array_equal(fc.free, g[f"{tag}_free"])
    assert [fc.start, fc.stop] == list(g[f"{tag}_range"])
    assert np.abs(fc.frame - g[f"{tag}_frame"]).max() < 1e-15
    for key, got in (("S", c.S), ("L", c.L), ("X", c.X), ("x0", c.x0)):
        ref = g[f"{tag}_{key}"]
        assert got.shape == ref.shape, key
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max(), key
    beta = np.linalg.solve(c.S, -c.L)
    slip = fc.cartesian(beta)
    assert np.abs(slip - g[f"{tag}_x"]).max() < 1e-9 * np.abs(g[f"{tag}_x"]).max()
