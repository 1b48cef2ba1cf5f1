"""Kernel identifiers and the kernel API (``src/mbem/kernels/__init__.py``)."""

KERNEL_T = "H"     # displacement jump (slip / u_p) -> displacement
KERNEL_U = "G"     # traction -> displacement
KERNEL_HT = "Ht"   # displacement jump -> elastic traction (eigenstress removed)
KERNEL_GT = "Gt"   # traction -> traction (Kelvin single layer)
KERNELS = (KERNEL_T, KERNEL_U, KERNEL_HT, KERNEL_GT)
DISPLACEMENT_KERNELS = (KERNEL_T, KERNEL_U)

from .basis import (  # noqa: E402
    TBasis,
    UBasis,
    assemble_t_basis,
    assemble_t_matrix,
    assemble_traction_matrix,
    assemble_u_basis,
    assemble_u_matrix,
    identity_ids,
    n_nodes,
    t_coeffs,
    u_coeffs,
)


def kernel_n_basis(kernel: str) -> int:
    if kernel == KERNEL_T:
        return 6
    if kernel == KERNEL_U:
        return 3
    if kernel in (KERNEL_HT, KERNEL_GT):
        raise ValueError(f"kernel {kernel!r} (a traction kernel) has no basis stack")
    raise ValueError(f"unknown kernel {kernel!r}; expected one of {KERNELS}")


def kernel_coeffs(kernel: str, material):
    if kernel == KERNEL_T:
        return t_coeffs(material.mu, material.lam)
    if kernel == KERNEL_U:
        return u_coeffs(material.mu, material.lam)
    if kernel in (KERNEL_HT, KERNEL_GT):
        raise ValueError(f"kernel {kernel!r} (a traction kernel) has no coefficient vector")
    raise ValueError(f"unknown kernel {kernel!r}; expected one of {KERNELS}")


__all__ = ["KERNEL_T", "KERNEL_U", "KERNEL_HT", "KERNEL_GT", "KERNELS", "DISPLACEMENT_KERNELS",
           "kernel_n_basis", "kernel_coeffs", "UBasis", "TBasis", "assemble_u_basis",
           "assemble_t_basis", "assemble_u_matrix", "assemble_t_matrix", "assemble_traction_matrix",
           "identity_ids", "u_coeffs", "t_coeffs", "n_nodes"]
