"""P0 kernel drivers with the signatures of ``src/mbem/kernels/tri_kernels.py``
(:451-591 matrices, :976-1260 contractions), on the GPU.

Thin order-0 views of :mod:`mbem_gb300.kernels.tri_nodal`; the pair code is
the CUDA P0 kernel (``csrc/p0_kernels.cu``).
"""

from __future__ import annotations

from . import tri_nodal as _tn


def u_basis_matrices(x_field, tri_verts, eps_arr):
    return _tn.u_basis_matrices(x_field, tri_verts, eps_arr, 0)


def t_basis_matrices(x_field, tri_verts, normals, eps_arr):
    return _tn.t_basis_matrices(x_field, tri_verts, normals, eps_arr, 0)


def u_matrix_direct(x_field, tri_verts, eps_arr, g1, g2, g3):
    return _tn.u_matrix_direct(x_field, tri_verts, eps_arr, g1, g2, g3, 0)


def t_matrix_direct(x_field, tri_verts, normals, eps_arr, c1, c2, c3, c4, c5, c6):
    return _tn.t_matrix_direct(x_field, tri_verts, normals, eps_arr, c1, c2, c3, c4, c5, c6, 0)


def u_disp_contract(x_field, tri_verts, eps_arr, density, g1, g2, g3):
    return _tn.u_disp_contract(x_field, tri_verts, eps_arr, density, g1, g2, g3, 0)


def t_disp_contract(x_field, tri_verts, normals, eps_arr, density, c1, c2, c3, c4, c5, c6):
    return _tn.t_disp_contract(x_field, tri_verts, normals, eps_arr, density, c1, c2, c3, c4, c5, c6, 0)


def kelvin_stress_contract(x_field, tri_verts, eps_arr, density, mu, lam):
    return _tn.kelvin_stress_contract(x_field, tri_verts, eps_arr, density, mu, lam, 0)


def dd_stress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam):
    return _tn.dd_stress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam, 0)


def eigenstress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam):
    return _tn.eigenstress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam, 0)
