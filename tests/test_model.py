"""Host-side model logic on the CPU: meshes, layout, orientation, the block
terms and the calibrated system, checked against the reference's goldens
through the C oracle (no GPU)."""

import numpy as np
import pytest

from conftest import rel_err
from oracle.cpu_system import assemble, deflated_solve
from mbem_gb300 import mesh as M
from mbem_gb300.backends.dense import require_anchor_or_deflate, translation_basis
from mbem_gb300.cases import cube_fault_model
from mbem_gb300.kernels import basis as kb
from mbem_gb300.model import BCType, Patch, Region, RegionModel, generate_system


def test_meshes_match_reference(cube_small):
    g = cube_small
    c = M.cube(int(g["n_face"]))
    f = M.centre_fault(int(g["n_fault"]))
    assert np.array_equal(c.vertices, g["cube_vertices"])
    assert np.array_equal(c.triangles, g["cube_triangles"])
    assert np.array_equal(f.vertices, g["fault_vertices"])
    assert np.array_equal(f.triangles, g["fault_triangles"])


def test_layout_and_orientation():
    model, eps = cube_fault_model(3, 2)
    system = generate_system(model)
    lay = system.layout
    assert lay.n_unknowns == 3 * 108
    assert [s.name for s in lay.slots] == ["u:cube"]
    r = model.regions[0]
    assert model.orientation(r, r.patches[0]) == 1           # outward normals
    assert model.orientation(r, r.faults[0]) == -1           # the fault convention
    assert len(system.terms) == 1 and system.terms[0].diag == 0.5
    assert len(system.rhs_terms) == 1 and system.rhs_terms[0].scale == 1.0


def test_reversed_cube_gets_negative_orientation():
    cube = M.cube(2)
    cube.triangles = cube.triangles[:, [0, 2, 1]]
    model = RegionModel([Region("b", M.ElasticMaterial(1.0, 1.0),
                                [Patch("cube", cube, BCType.FREE_TRACTION)], np.zeros(3))])
    assert model.orientation(model.regions[0], model.regions[0].patches[0]) == -1


@pytest.mark.parametrize("tag", ["", "nu30_"])
def test_cpu_system_matches_reference(oracle, cube_small, tag):
    g = {k[len(tag):]: v for k, v in cube_small.items() if k.startswith(tag)} if tag else cube_small
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    assert eps == float(g["eps"])
    system = generate_system(model)
    A, b, calib = assemble(oracle, system, eps)
    C = next(iter(calib.values()))
    assert rel_err(C, g["calib"]) < 1e-13
    assert rel_err(A, g["A"]) < 1e-13
    assert rel_err(b, g["b"]) < 1e-13
    x = deflated_solve(A, b, system.layout)
    assert rel_err(x, g["x"]) < 1e-10


def test_translation_basis_is_null_space_of_calibrated_operator(oracle):
    model, eps = cube_fault_model(2, 2)
    system = generate_system(model)
    A, _, _ = assemble(oracle, system, eps)
    Z = translation_basis(system.layout)
    assert np.abs(A @ Z).max() < 1e-13 * np.abs(A).max()


def test_errors_like_the_reference():
    with pytest.raises(ValueError):
        kb.as_eps_array(0.0, 4)
    with pytest.raises(ValueError):
        kb.as_eps_array(np.array([0.1, -0.1]), 2)
    with pytest.raises(ValueError):
        kb.as_eps_array(np.ones(3), 4)
    bad = M.TriMesh(np.array([[0.0, 0, 0], [1, 0, 0], [2, 0, 0]]), np.array([[0, 1, 2]]))
    with pytest.raises(ValueError):
        Patch("bad", bad, BCType.FREE_TRACTION)
    with pytest.raises(ValueError):
        Patch("p", M.cube(1), BCType.FREE_TRACTION, order=3)
    model, _ = cube_fault_model(2, 2)
    with pytest.raises(ValueError):
        require_anchor_or_deflate(generate_system(model), "calibrated", False)


def test_coefficients_from_mu_lam():
    c = kb.t_coeffs(1.0, 1.0)
    g = kb.u_coeffs(1.3, 1.95)
    nu = 1.95 / (2 * (1.95 + 1.3))
    assert abs(nu - 0.3) < 1e-15
    C1 = 1.0 / (16 * np.pi * 1.3 * (1 - nu))
    assert np.allclose(g, [(3 - 4 * nu) * C1, 1 / (8 * np.pi * 1.3), C1], rtol=1e-15)
    assert c.shape == (6,)


def test_cluster_leaves_partition_and_bound():
    """Principal-axis bisection (la/cluster.py:56-75): the leaves partition
    the points, none exceeds the bound, and each is spatially compact."""
    from mbem_gb300.la.precond import cluster_leaves
    from mbem_gb300.mesh import cube
    pts = cube(12, 4.0).centroids()
    leaves = cluster_leaves(pts, 75)
    allidx = np.sort(np.concatenate(leaves))
    assert np.array_equal(allidx, np.arange(pts.shape[0]))
    assert max(l.size for l in leaves) <= 75 and min(l.size for l in leaves) >= 75 // 2 - 1
    span = max(np.ptp(pts[l], axis=0).max() for l in leaves)
    assert span < 2.5
    coincident = cluster_leaves(np.zeros((10, 3)), 3)
    assert sorted(np.concatenate(coincident).tolist()) == list(range(10))
    assert max(l.size for l in coincident) <= 3
