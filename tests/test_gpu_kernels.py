"""CUDA P0 kernels against the reference's golden vectors and the C oracle.

Tolerance: FP64 throughout; entries agree to 1e-12 of the largest entry of
each output (observed ~1e-15: the CUDA formulation rewrites the moment
contractions, so agreement is to rounding, not bitwise).
"""

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def tk(gpu):
    from mbem_gb300.kernels import tri_kernels
    return tri_kernels


def test_basis_stacks(tk, p0_pairs):
    g = p0_pairs
    assert rel_err(tk.t_basis_matrices(g["x_field"], g["tri_verts"], g["normals"], g["eps"]),
                   g["t_basis"]) < TOL
    assert rel_err(tk.u_basis_matrices(g["x_field"], g["tri_verts"], g["eps"]), g["u_basis"]) < TOL


@pytest.mark.parametrize("m", [0, 1])
def test_matrices(tk, p0_pairs, m):
    g = p0_pairs
    T = tk.t_matrix_direct(g["x_field"], g["tri_verts"], g["normals"], g["eps"], *g[f"t_coeffs_{m}"])
    U = tk.u_matrix_direct(g["x_field"], g["tri_verts"], g["eps"], *g[f"u_coeffs_{m}"])
    assert rel_err(T, g[f"t_matrix_{m}"]) < TOL
    assert rel_err(U, g[f"u_matrix_{m}"]) < TOL
    s = g["tri_verts"].shape[0] - 1          # degenerate source -> zero columns
    assert np.all(T[:, 3 * s:3 * s + 3] == 0.0)


@pytest.mark.parametrize("m", [0, 1])
def test_contractions(tk, p0_pairs, m):
    g = p0_pairs
    x, tv, n, e, d = g["x_field"], g["tri_verts"], g["normals"], g["eps"], g["density"]
    mu, lam = g["materials"][m]
    assert rel_err(tk.t_disp_contract(x, tv, n, e, d, *g[f"t_coeffs_{m}"]), g[f"t_disp_{m}"]) < TOL
    assert rel_err(tk.u_disp_contract(x, tv, e, d, *g[f"u_coeffs_{m}"]), g[f"u_disp_{m}"]) < TOL
    assert rel_err(tk.dd_stress_contract(x, tv, n, e, d, mu, lam), g[f"dd_stress_{m}"]) < TOL
    assert rel_err(tk.kelvin_stress_contract(x, tv, e, d, mu, lam), g[f"kelvin_stress_{m}"]) < TOL
    assert rel_err(tk.eigenstress_contract(x, tv, n, e, d, mu, lam), g[f"eigenstress_{m}"]) < TOL


def test_elastic_stress_is_dd_minus_eigen(tk, p0_pairs):
    from mbem_gb300.kernels import tri_nodal as tn
    g = p0_pairs
    x, tv, n, e, d = g["x_field"], g["tri_verts"], g["normals"], g["eps"], g["density"]
    el = tn.elastic_stress_contract(x, tv, n, e, d, 1.3, 1.95)
    assert rel_err(el, g["dd_stress_1"] - g["eigenstress_1"]) < TOL


def test_contraction_equals_matrix_times_density(tk, oracle):
    """Matrix-free contraction == assembled matrix @ density (the reference's
    verify_disp_contract gate), on a random cloud larger than one tile."""
    rng = np.random.default_rng(5)
    tv = rng.normal(size=(200, 3, 3))
    cr = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
    n = cr / np.linalg.norm(cr, axis=1)[:, None]
    e = rng.uniform(0.05, 0.2, 200)
    x = rng.normal(size=(300, 3)) * 2.0
    d = rng.normal(size=(200, 3))
    from mbem_gb300.kernels import basis as kb
    c = kb.t_coeffs(1.0, 1.5)
    T = tk.t_matrix_direct(x, tv, n, e, *c)
    u = tk.t_disp_contract(x, tv, n, e, d, *c)
    assert rel_err(u.ravel(), T @ d.ravel()) < 1e-13
    assert rel_err(T, oracle.matrix("t", x, tv, n, e, c)) < TOL


def test_block_written_in_place_with_scale_and_offset(tk, p0_pairs):
    from mbem_gb300.kernels import tri_nodal as tn
    g = p0_pairs
    x, tv, n, e = g["x_field"], g["tri_verts"], g["normals"], g["eps"]
    rows, cols = 3 * x.shape[0], 3 * tv.shape[0]
    big = torch.full((rows + 6, cols + 9), 7.0, dtype=torch.float64, device="cuda")
    view = big[3:3 + rows, 6:6 + cols]
    tn.t_matrix_direct(x, tv, n, e, *g["t_coeffs_0"], 0, out=view, alpha=-2.0, accumulate=True)
    got = big.cpu().numpy()
    assert rel_err(got[3:3 + rows, 6:6 + cols], 7.0 - 2.0 * g["t_matrix_0"]) < TOL
    assert np.all(got[:3] == 7.0) and np.all(got[:, :6] == 7.0)
    assert np.all(got[3 + rows:] == 7.0) and np.all(got[:, 6 + cols:] == 7.0)


def test_torch_inputs_stay_on_device(tk, p0_pairs):
    g = p0_pairs
    x = torch.from_numpy(g["x_field"]).cuda()
    out = tk.u_matrix_direct(x, g["tri_verts"], g["eps"], *g["u_coeffs_0"])
    assert isinstance(out, torch.Tensor) and out.is_cuda


def test_empty_and_bad_inputs(tk, p0_pairs):
    g = p0_pairs
    out = tk.t_matrix_direct(np.zeros((0, 3)), g["tri_verts"], g["normals"], g["eps"], *g["t_coeffs_0"])
    assert out.shape == (0, 3 * g["tri_verts"].shape[0])
    with pytest.raises(ValueError):
        tk.t_matrix_direct(g["x_field"], g["tri_verts"], g["normals"], g["eps"][:-1], *g["t_coeffs_0"])
    from mbem_gb300.kernels import tri_nodal as tn
    with pytest.raises(ValueError):
        tn.t_matrix_direct(g["x_field"], g["tri_verts"], g["normals"], g["eps"], *g["t_coeffs_0"], 3)
