"""The volume sampler on the GPU against the reference's own outputs
(``tests/golden/volume_small.npz``) and the numpy oracle: the solid-angle
closure sums and region codes, exact distances, on-patch flags,
clearances, the sampled fields, and region codes of a 110,592-point grid
over the 27,648-triangle cube against the box test."""

import numpy as np
import pytest
import torch

from conftest import rel_err
from mbem_gb300 import geometry as G
from mbem_gb300 import volume as V
from mbem_gb300.cases import cube_fault_model
from oracle import geometry_oracle as go

pytestmark = pytest.mark.gpu

# FP32 far pairs: a closure sum within this of the FP64 sum (steradian); the
# classifier's band is 1e-6 x 4 pi = 1.26e-5
SOLID_ANGLE_ATOL = 2e-6
DIST_ATOL = 1e-13


def _tv(g, name):
    return g[f"{name}_vertices"][g[f"{name}_triangles"]]


def _solution(g):
    return {"u:cube": g["x"]}


def test_closure_sums_and_inside_flags_match_reference(gpu, volume_small):
    g = volume_small
    model, _ = cube_fault_model(3, 2)
    inside, total = model.point_in_region(model.regions[0], g["sc_points"], closure=True)
    assert np.abs(total - g["sc_total"]).max() < SOLID_ANGLE_ATOL
    assert np.array_equal(inside, g["sc_inside"])
    # numpy in, numpy out; torch in, CUDA out
    t = model.point_in_region("body", torch.from_numpy(g["sc_points"]))
    assert t.is_cuda and torch.equal(t.cpu(), torch.from_numpy(g["sc_inside"]))


def test_solid_angle_against_oracle_on_a_larger_mesh(gpu):
    """Cube 24 (6,912 triangles) from 4,096 points, 512 of them within
    1e-4 .. 0.3 h of a face on either side."""
    model, _ = cube_fault_model(24, 4)
    tv = model.regions[0].patches[0].tri_verts()
    rng = np.random.default_rng(3)
    pts = rng.uniform(-2.6, 2.6, size=(3584, 3))
    face = rng.uniform(-1.9, 1.9, size=(512, 3))
    ax = rng.integers(0, 3, 512)
    side = rng.choice([-2.0, 2.0], 512)
    off = rng.choice([-1.0, 1.0], 512) * 10.0 ** rng.uniform(-4, np.log10(0.3), 512) * (4.0 / 24)
    face[np.arange(512), ax] = side + off
    pts = np.concatenate([pts, face])
    total = G.solid_angle_batch(model.regions[0].patches[0].mesh, pts)
    ref = go.solid_angle_sum(tv, pts)
    assert np.abs(total - ref).max() < SOLID_ANGLE_ATOL
    inside = model.point_in_region("body", pts)
    assert np.array_equal(inside, go.closure([(tv, 1.0)], pts)[0])
    box = (np.abs(pts) < 2.0).all(axis=1)
    assert np.array_equal(inside, box)


def test_distances_match_reference_and_oracle(gpu, volume_small):
    g = volume_small
    model, _ = cube_fault_model(3, 2)
    r = model.regions[0]
    for name, patch in (("cube", r.patches[0]), ("fault", r.faults[0])):
        d, i = G.distance_to_mesh(g["all_points"], patch.mesh)
        assert np.abs(d - g[f"d_{name}"]).max() < DIST_ATOL
        tv = _tv(g, name)
        # the same triangle, or one at the same distance (a tie)
        alt = go.point_triangle_distance(g["all_points"], tv[i, 0], tv[i, 1], tv[i, 2])
        assert np.abs(alt - g[f"d_{name}"]).max() < DIST_ATOL
    # a larger mesh against the oracle
    big, _ = cube_fault_model(16, 8)
    rng = np.random.default_rng(5)
    pts = rng.uniform(-3.0, 3.0, size=(2048, 3))
    for patch in (big.regions[0].patches[0], big.regions[0].faults[0]):
        d, i = G.distance_to_mesh(pts, patch.mesh)
        tv = patch.tri_verts()
        dr, _ = go.distance_to_mesh(pts, tv)
        assert np.abs(d - dr).max() < DIST_ATOL
        alt = go.point_triangle_distance(pts, tv[i, 0], tv[i, 1], tv[i, 2])
        assert np.abs(alt - dr).max() < DIST_ATOL


def test_on_patch_classify_and_clearance_match_reference(gpu, volume_small):
    g = volume_small
    model, eps = cube_fault_model(3, 2)
    assert np.array_equal(V.on_patch(g["all_points"], model.regions[0].patches[0]), g["on_patch"])
    grid = V.make_grid(model, 1.0, pad=1.0)
    code = V.classify(model, grid)
    assert code.dtype == np.int8 and np.array_equal(code, g["code"])
    c_h, c_eps, c_fault = V.clearance(model, grid, eps)
    assert rel_err(c_h, g["c_h"]) < 1e-13
    assert rel_err(c_eps, g["c_eps"]) < 1e-13
    assert rel_err(c_fault, g["c_fault"]) < 1e-13


def test_sample_matches_reference(gpu, volume_small):
    g = volume_small
    model, eps = cube_fault_model(3, 2)
    grid = V.make_grid(model, 1.0, pad=1.0)
    code = g["code"]
    seen = []
    fields = V.sample(model, _solution(g), eps, grid, code, chunk=40,
                      progress=lambda name, done, total: seen.append((name, done, total)))
    assert seen[-1] == ("body", 64, 64) and len(seen) == 2
    inside = code > 0
    for k, v in fields.items():
        ref = g[f"f_{k}"]
        assert v.shape == ref.shape, k
        assert np.array_equal(np.isnan(v), np.isnan(ref)), k
        assert rel_err(v[inside], ref[inside]) < 1e-9, k
    mixed = V.sample(model, _solution(g), eps, grid, code, eigenstress=False, precision="mixed")
    assert "eigenstress" not in mixed
    assert rel_err(mixed["sigma"][inside], g["f_sigma"][inside]) < 1e-5
    with pytest.raises(NotImplementedError):
        V.sample(model, _solution(g), eps, grid, code, near=object())
    with pytest.raises(ValueError):
        V.sample(model, _solution(g), eps, grid, code[:-1])
    with pytest.raises(ValueError):
        G.distance_to_mesh(np.array([[0.0, np.nan, 0.0]]), model.regions[0].patches[0].mesh)


def test_region_codes_of_a_large_grid(gpu):
    """Cube 48 (27,648 triangles), a 48^3 grid half a cell off every face:
    every code equals the box test and every closure sum is 0 or 4 pi."""
    model, _ = cube_fault_model(48, 8)
    grid = V.make_grid(model, 4.0 / 44, pad=4.0 / 44 * 2)
    assert grid.points.shape[0] > 100_000
    code = V.classify(model, grid)
    box = (np.abs(grid.points) < 2.0).all(axis=1)
    assert np.array_equal(code > 0, box)
    pts = torch.from_numpy(grid.points).cuda()
    _, total = model.point_in_region("body", pts, closure=True)
    total = total.cpu().numpy()
    assert np.abs(np.where(box, total - 4.0 * np.pi, total)).max() < SOLID_ANGLE_ATOL


# the mixed displacement readout: FP32-far quadrature against the FP64
# contraction, relative to the largest displacement of the set
DISP_MIXED_TOL = 2e-6


def test_mixed_displacement_readout_against_fp64(gpu):
    """Cube 24 (6,912 triangles) + fault 16 (512): 8,192 observers, a
    quarter within 0.02 .. 0.5 h of a face, both double layers."""
    from mbem_gb300.evaluate import evaluate_displacement
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.kernels import tri_nodal as tn
    model, eps = cube_fault_model(24, 16)
    rng = np.random.default_rng(9)
    pts = rng.uniform(-1.95, 1.95, size=(8192, 3))
    h = 4.0 / 24
    k = rng.integers(0, 3, 2048)
    pts[:2048][np.arange(2048), k] = rng.choice([-2.0, 2.0], 2048) * (1.0 - rng.uniform(0.02, 0.5, 2048) * h / 2.0)
    c = kb.t_coeffs(1.0, 1.0)
    for patch in (model.regions[0].patches[0], model.regions[0].faults[0]):
        tv = patch.tri_verts()
        nrm, _ = patch.mesh.normals_and_areas()
        e = np.full(tv.shape[0], eps)
        d = rng.normal(size=(tv.shape[0], 3))
        ref = tn.t_disp_contract(pts, tv, nrm, e, d, *c)
        got = tn.t_disp_readout(pts, tv, nrm, e, d, *c)
        assert rel_err(got, ref) < DISP_MIXED_TOL
        acc = tn.t_disp_readout(pts, tv, nrm, e, d, *c, out=torch.from_numpy(ref).cuda(), alpha=-1.0,
                                accumulate=True)
        assert np.abs(acc.cpu().numpy()).max() < DISP_MIXED_TOL * np.abs(ref).max()
    sol = {"u:cube": rng.normal(size=(6912, 3)) * 1e-2}
    u64 = evaluate_displacement(model, "body", sol, pts, eps, warn_near=False)
    u32 = evaluate_displacement(model, "body", sol, pts, eps, warn_near=False, precision="mixed")
    assert rel_err(u32, u64) < DISP_MIXED_TOL


def test_mixed_sample_matches_reference(gpu, volume_small):
    g = volume_small
    model, eps = cube_fault_model(3, 2)
    grid = V.make_grid(model, 1.0, pad=1.0)
    inside = g["code"] > 0
    f = V.sample(model, _solution(g), eps, grid, g["code"], precision="mixed")
    assert rel_err(f["u"][inside], g["f_u"][inside]) < DISP_MIXED_TOL
    assert rel_err(f["sigma"][inside], g["f_sigma"][inside]) < 1e-5
    assert np.isnan(f["u"][~inside]).all()


def test_two_region_codes_and_clearances_match_reference(gpu, volume_regions):
    """Host cube + inclusion behind an INTERFACE patch (the reference's own
    volume module wrote the codes): points on the interface, on its edge and
    corner, 1e-6 either side of it, on the outer surface."""
    from volume_models import two_region_model
    g = volume_regions
    model, _, _ = two_region_model(g)
    grid = V.Grid(origin=(0.0, 0.0, 0.0), spacing=(0.5,) * 3, dims=(g["points"].shape[0], 1, 1),
                  points=g["points"])
    code = V.classify(model, grid)
    assert np.array_equal(code, g["code"])
    c_h, c_eps, c_fault = V.clearance(model, grid, 0.1)
    assert rel_err(c_h, g["c_h"]) < 1e-13 and rel_err(c_eps, g["c_eps"]) < 1e-13
    assert np.isinf(c_fault).all()
    # closure sums off the surfaces (on a surface the sum is rounding's choice)
    off = (g["c_h"] > 1e-6)
    for r, reg in enumerate(model.regions):
        _, total = model.point_in_region(reg, g["points"], closure=True)
        assert np.abs(total[off] - g["totals"][r][off]).max() < SOLID_ANGLE_ATOL
