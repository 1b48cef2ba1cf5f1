"""The C oracle against golden vectors produced by the reference itself.

The oracle restates the reference's P0 kernels (tri_kernels.py) in C; these
tests pin it to the reference's own outputs (tests/golden/, made by
make_golden.py), entry by entry, before it is trusted to check the
CUDA path at sizes the reference cannot reach here.
"""

import numpy as np
import pytest

from conftest import rel_err

TOL = 1e-13      # relative to the largest entry; observed ~3e-16


def test_oracle_basis_stacks(oracle, p0_pairs):
    g = p0_pairs
    assert rel_err(oracle.matrix("t_basis", g["x_field"], g["tri_verts"], g["normals"], g["eps"]),
                   g["t_basis"]) < TOL
    assert rel_err(oracle.matrix("u_basis", g["x_field"], g["tri_verts"], None, g["eps"]),
                   g["u_basis"]) < TOL


@pytest.mark.parametrize("m", [0, 1])
def test_oracle_matrices(oracle, p0_pairs, m):
    g = p0_pairs
    args = (g["x_field"], g["tri_verts"])
    assert rel_err(oracle.matrix("t", *args, g["normals"], g["eps"], g[f"t_coeffs_{m}"]),
                   g[f"t_matrix_{m}"]) < TOL
    assert rel_err(oracle.matrix("u", *args, None, g["eps"], g[f"u_coeffs_{m}"]),
                   g[f"u_matrix_{m}"]) < TOL


@pytest.mark.parametrize("m", [0, 1])
def test_oracle_contractions(oracle, p0_pairs, m):
    g = p0_pairs
    x, tv, n, e, d = g["x_field"], g["tri_verts"], g["normals"], g["eps"], g["density"]
    mu, lam = g["materials"][m]
    assert rel_err(oracle.contract("t_disp", x, tv, n, e, d, g[f"t_coeffs_{m}"]), g[f"t_disp_{m}"]) < TOL
    assert rel_err(oracle.contract("u_disp", x, tv, None, e, d, g[f"u_coeffs_{m}"]),
                   g[f"u_disp_{m}"]) < TOL
    assert rel_err(oracle.contract("dd", x, tv, n, e, d, mu=mu, lam=lam), g[f"dd_stress_{m}"]) < TOL
    assert rel_err(oracle.contract("kelvin", x, tv, None, e, d, mu=mu, lam=lam),
                   g[f"kelvin_stress_{m}"]) < TOL
    assert rel_err(oracle.contract("eigen", x, tv, n, e, d, mu=mu, lam=lam),
                   g[f"eigenstress_{m}"]) < TOL


def test_oracle_degenerate_source_gives_zero_columns(oracle, p0_pairs):
    g = p0_pairs
    A = oracle.matrix("t", g["x_field"], g["tri_verts"], g["normals"], g["eps"], g["t_coeffs_0"])
    s = g["tri_verts"].shape[0] - 1            # the collinear triangle
    assert np.all(A[:, 3 * s:3 * s + 3] == 0.0)


def test_oracle_source_range_matches_full(oracle, p0_pairs):
    g = p0_pairs
    args = (g["x_field"], g["tri_verts"], g["normals"], g["eps"], g["t_coeffs_0"])
    full = oracle.matrix("t", *args)
    part = oracle.matrix("t", *args, src_range=(3, 9))
    assert np.array_equal(part[:, 9:27], full[:, 9:27])
    assert np.all(part[:, :9] == 0.0)
