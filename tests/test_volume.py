"""The volume sampler's oracle and host logic on the CPU (no GPU): the numpy
restatement of the reference's geometry pinned to the golden fixture that
the reference's own ``volume`` module wrote, and the grid, strain, scalar,
difference and VTI bookkeeping of ``mbem_gb300.volume`` against it."""

import numpy as np
import torch

from conftest import rel_err
from mbem_gb300 import volume as V
from mbem_gb300.cases import cube_fault_model
from oracle import geometry_oracle as go
from volume_models import two_region_model


def _tv(g, name):
    return g[f"{name}_vertices"][g[f"{name}_triangles"]]


def test_oracle_closure_sums_match_reference(volume_small):
    g = volume_small
    inside, total = go.closure([(_tv(g, "cube"), 1.0)], g["sc_points"])
    assert np.abs(total - g["sc_total"]).max() < 1e-12
    assert np.array_equal(inside, g["sc_inside"])


def test_oracle_distances_match_reference(volume_small):
    g = volume_small
    for name in ("cube", "fault"):
        d, i = go.distance_to_mesh(g["all_points"], _tv(g, name))
        assert np.abs(d - g[f"d_{name}"]).max() < 1e-14
        # a different index only at an exact tie of distances
        tv = _tv(g, name)
        alt = go.point_triangle_distance(g["all_points"], tv[g[f"i_{name}"], 0], tv[g[f"i_{name}"], 1],
                                         tv[g[f"i_{name}"], 2])
        assert np.abs(alt - d).max() < 1e-14


def test_oracle_classify_on_patch_and_clearance_match_reference(volume_small):
    g = volume_small
    cube, fault = _tv(g, "cube"), _tv(g, "fault")
    assert np.array_equal(go.on_patch(g["all_points"], cube), g["on_patch"])
    assert np.array_equal(go.classify([[(cube, 1.0)]], g["grid_points"]), g["code"])
    eps = float(g["eps"])
    c_h, c_eps, c_fault = go.clearance(g["grid_points"], [(cube, np.full(len(cube), eps))],
                                       [(fault, np.full(len(fault), eps))])
    assert rel_err(c_h, g["c_h"]) < 1e-14
    assert rel_err(c_eps, g["c_eps"]) < 1e-14
    assert rel_err(c_fault, g["c_fault"]) < 1e-14


def test_grids_match_reference(volume_small):
    g = volume_small
    model, _ = cube_fault_model(3, 2)
    grid = V.make_grid(model, 1.0, pad=1.0)
    assert np.array_equal(grid.points, g["grid_points"])
    assert np.allclose(grid.origin, g["grid_origin"]) and tuple(grid.dims) == tuple(g["grid_dims"])
    sec = V.section_grid(model, "y", 0.1, 0.5)
    assert np.array_equal(sec.points, g["section_points"])
    assert np.allclose(sec.origin, g["section_origin"]) and tuple(sec.dims) == tuple(g["section_dims"])
    assert grid.fold(grid.points).shape == (6, 6, 6, 3)
    for bad in (("w", 0.1), ("y", 2.0), ("z", -2.5)):
        try:
            V.section_grid(model, bad[0], bad[1], 0.5)
        except ValueError:
            continue
        raise AssertionError(f"section {bad} was not refused")


def test_strain_and_scalars_match_reference(volume_small):
    g = volume_small
    inside = g["code"] > 0
    sig = torch.from_numpy(g["f_sigma"][inside])
    e = V._strain(sig, 1.0, 1.0).numpy()
    assert rel_err(e, g["f_strain"][inside]) < 1e-14
    assert rel_err(e, go.strain(g["f_sigma"][inside], 1.0, 1.0)) < 1e-15
    d = V._derived(torch.from_numpy(g["f_u"][inside]), sig, torch.from_numpy(e))
    for k, v in d.items():
        assert rel_err(v.numpy(), g[f"f_{k}"][inside]) < 1e-13, k
    assert np.isnan(g["f_von_mises"][~inside]).all()


def test_difference_and_vti_arrays_match_reference(volume_small):
    g = volume_small
    fields = {k[2:]: g[k] for k in g if k.startswith("f_")}
    half = {k: 0.5 * fields[k] for k in V.PRIMARY}
    diff = V.difference(fields, half, g["code"] > 0)
    for k, v in diff.items():
        ref = g[f"d_{k}"]
        assert np.array_equal(np.isnan(v), np.isnan(ref)), k
        ok = ~np.isnan(ref)
        assert rel_err(v[ok], ref[ok]) < 1e-13, k
    model, _ = cube_fault_model(3, 2)
    grid = V.make_grid(model, 1.0, pad=1.0)
    vti = V.as_vti_arrays(grid, fields, g["code"], g["c_h"], g["c_eps"], g["c_fault"])
    assert sorted(vti) == list(g["vti_keys"])
    assert np.array_equal(vti["sigma_xy"], g["vti_sigma_xy"], equal_nan=True)
    assert np.array_equal(vti["u"], g["vti_u"], equal_nan=True)


def test_eigenvalues_3x3_match_lapack():
    """The Jacobi eigenvalues behind max_shear: within a few eps of ||A|| of
    LAPACK's, for well-separated, near-double and near-triple spectra and
    at extreme scales."""
    rng = np.random.default_rng(0)
    n = 4000
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    ones = np.ones(n)
    spectra = [rng.normal(size=(n, 3)),
               np.stack([ones, ones + 10 ** rng.uniform(-14, -2, n), 3 * rng.normal(size=n)], 1),
               np.stack([ones, ones - 10 ** rng.uniform(-14, -2, n), ones + 10 ** rng.uniform(-14, -2, n)], 1),
               rng.normal(size=(n, 3)) * 1e-3 + 100.0,
               np.stack([rng.normal(size=n), 0 * ones, 0 * ones], 1),
               rng.normal(size=(n, 3)) * 10.0 ** rng.uniform(-200, 200, (n, 1))]
    for lam in spectra:
        A = np.einsum("nij,nj,nkj->nik", Q, lam, Q)
        A = 0.5 * (A + A.transpose(0, 2, 1))
        got = V.eigvalsh3(torch.from_numpy(A)).numpy()
        ref = np.linalg.eigvalsh(A)
        assert (np.abs(got - ref).max(1) / np.abs(A).reshape(n, -1).max(1)).max() < 2e-14
    Z = np.zeros((2, 3, 3))
    Z[1] = np.diag([3.0, 1.0, 2.0])
    assert np.array_equal(V.eigvalsh3(torch.from_numpy(Z)).numpy(), [[0, 0, 0], [1, 2, 3]])


def test_mixed_displacement_readout_is_p0_only():
    from mbem_gb300.kernels import tri_nodal as tn
    import pytest
    with pytest.raises(NotImplementedError):
        tn.t_disp_readout(np.zeros((1, 3)), np.zeros((1, 3, 3)), np.zeros((1, 3)), np.ones(1), np.zeros((3, 3)),
                          1, 1, 1, 1, 1, 1, order=1)


def test_two_region_oracle_and_orientation_match_reference(volume_regions):
    """Region codes with an interface: points ON it go to the first region
    that owns it; the orientation signs of the interface are opposite."""
    g = volume_regions
    model, host_p, iface = two_region_model(g)
    host, incl = model.regions
    sig = [model.orientation(host, host_p), model.orientation(host, iface), model.orientation(incl, iface)]
    assert sig == list(g["orientation"])
    outer = _tv(g, "outer")
    inner = _tv(g, "inner")
    regions = [[(outer, sig[0]), (inner, sig[1])], [(inner, sig[2])]]
    assert np.array_equal(go.classify(regions, g["points"]), g["code"])
    for r, patches in enumerate(regions):
        assert np.abs(go.closure(patches, g["points"])[1] - g["totals"][r]).max() < 1e-12
    c_h, c_eps, c_f = go.clearance(g["points"], [(outer, np.full(len(outer), 0.1)), (inner, np.full(len(inner), 0.1)),
                                                 (inner, np.full(len(inner), 0.1))], [])
    assert rel_err(c_h, g["c_h"]) < 1e-14 and rel_err(c_eps, g["c_eps"]) < 1e-14
    assert np.isinf(g["c_fault"]).all() and np.isinf(c_f).all()
