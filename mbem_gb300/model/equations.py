"""Block-equation generation (``src/mbem/model/equations.py``).

THE sign rule, for region R, collocation patch q and sigma(R, p):

    A[row(R,q), u_p] += sigma(R,p) H_qp + D_q delta_qp
    A[row(R,q), t_p] += -sigma(R,p) G_qp
    b[row(R,q)]      -= sum_f sigma(R,f) H_qf @ slip_f   (+ prescribed columns)

with the traction rows of a FAULT_TRACTION fault f (elastic traction, the
eigenstress removed; no free term):

    A[b_f, u_p] += -sigma_p Ht    A[b_f, t_p] += +sigma_p Gt
    A[b_f, b_g] += -sigma_g Ht    b[b_f] += +sigma_p Ht u_p - sigma_p Gt t_p
                                            + sigma_g Ht slip_g + dt

This module builds the same ``BlockSystem`` terms as the reference's
``generate_system`` (:212-386) for the models of the dense hot path, the
calibrated diagonal (:512-537) and the fault-row transform (:443-507); the
backend applies them to device arrays.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .. import defaults
from ..kernels import KERNEL_GT, KERNEL_HT, KERNEL_T, KERNEL_U
from .core import BCType, Patch, Region, RegionModel
from .layout import Slot, UnknownLayout

COLLOCATION_JUMP = 0.5


@dataclass(frozen=True)
class BlockTerm:
    row: Slot
    col: Slot
    kernel: str
    field_patch: Patch
    source_patch: Patch
    region: Region
    scale: float
    diag: float = 0.0


@dataclass(frozen=True)
class RhsTerm:
    row: Slot
    kernel: str
    field_patch: Patch
    source_patch: Patch
    region: Region
    scale: float
    vector: np.ndarray
    add_half_of_vector: bool = False
    scale_half: float = 0.0


@dataclass(frozen=True)
class RhsValue:
    row: Slot
    vector: np.ndarray


@dataclass
class BlockSystem:
    model: RegionModel
    layout: UnknownLayout
    terms: list = field(default_factory=list)
    rhs_terms: list = field(default_factory=list)
    rhs_values: list = field(default_factory=list)

    def traction_faults(self) -> list:
        return sorted(self.model.solved_faults(), key=lambda rf: self.layout.slot(rf[1], "b").offset)


def generate_system(model: RegionModel) -> BlockSystem:
    layout = UnknownLayout(model)
    system = BlockSystem(model=model, layout=layout)
    for region in model.regions:
        for q in region.patches:
            row = layout.row_slot(region, q)
            for p in region.patches:
                sigma = float(model.orientation(region, p))
                if layout.has_slot(p, "u"):
                    system.terms.append(BlockTerm(row, layout.slot(p, "u"), KERNEL_T, q, p, region,
                                                  sigma, COLLOCATION_JUMP if p is q else 0.0))
                else:
                    u_bar = model.value_of(p).ravel()
                    if np.any(u_bar):
                        system.rhs_terms.append(RhsTerm(row, KERNEL_T, q, p, region, -sigma, u_bar,
                                                        add_half_of_vector=(p is q),
                                                        scale_half=-COLLOCATION_JUMP))
                if layout.has_slot(p, "t"):
                    system.terms.append(BlockTerm(row, layout.slot(p, "t"), KERNEL_U, q, p, region,
                                                  -sigma))
                else:
                    t_bar = model.value_of(p).ravel()
                    if np.any(t_bar):
                        system.rhs_terms.append(RhsTerm(row, KERNEL_U, q, p, region, sigma, t_bar))
            for f in region.faults:
                sigma = float(model.orientation(region, f))
                if f.bc is BCType.FAULT_TRACTION:
                    system.terms.append(BlockTerm(row, layout.slot(f, "b"), KERNEL_T, q, f, region,
                                                  sigma))
                    continue
                slip = f.value_array().ravel()
                if np.any(slip):
                    system.rhs_terms.append(RhsTerm(row, KERNEL_T, q, f, region, -sigma, slip))
        for f in region.faults:
            if f.bc is not BCType.FAULT_TRACTION:
                continue
            row = layout.slot(f, "b")
            for p in region.patches:
                sigma = float(model.orientation(region, p))
                if layout.has_slot(p, "u"):
                    system.terms.append(BlockTerm(row, layout.slot(p, "u"), KERNEL_HT, f, p, region,
                                                  -sigma))
                else:
                    u_bar = model.value_of(p).ravel()
                    if np.any(u_bar):
                        system.rhs_terms.append(RhsTerm(row, KERNEL_HT, f, p, region, sigma, u_bar))
                if layout.has_slot(p, "t"):
                    system.terms.append(BlockTerm(row, layout.slot(p, "t"), KERNEL_GT, f, p, region,
                                                  sigma))
                else:
                    t_bar = model.value_of(p).ravel()
                    if np.any(t_bar):
                        system.rhs_terms.append(RhsTerm(row, KERNEL_GT, f, p, region, -sigma, t_bar))
            for g in region.faults:
                sigma = float(model.orientation(region, g))
                if g.bc is BCType.FAULT_TRACTION:
                    system.terms.append(BlockTerm(row, layout.slot(g, "b"), KERNEL_HT, f, g, region,
                                                  -sigma))
                else:
                    slip = g.value_array().ravel()
                    if np.any(slip):
                        system.rhs_terms.append(RhsTerm(row, KERNEL_HT, f, g, region, sigma, slip))
            system.rhs_values.append(RhsValue(row, f.value_array().ravel()))
    return system


def calibrated_diagonal(system: BlockSystem, rowsum) -> dict:
    """{(id(region), id(q)): C (q.n_nodes, 3, 3)} with
    C_c = -sum_p sigma(R,p) rowsum(R, q, p)[c]: constant displacement over all
    of dR is annihilated exactly (equations.py:512-537). ``rowsum`` returns
    an (n_nodes, 3, 3) array (numpy or torch) of the applied H block."""
    model = system.model
    calib: dict = {}
    for region in model.regions:
        for q in region.patches:
            C = None
            for p in region.patches:
                term = float(model.orientation(region, p)) * rowsum(region, q, p)
                C = -term if C is None else C - term
            calib[(id(region), id(q))] = C
    return calib


def term_diagonal(term: BlockTerm, calib: dict | None):
    """The per-collocation-point (n_nodes, 3, 3) diagonal of a term, or None."""
    if not term.diag:
        return None
    if calib is not None:
        return calib[(id(term.region), id(term.field_patch))]
    return np.broadcast_to(term.diag * np.eye(3), (term.field_patch.n_nodes, 3, 3))


def traction_row_frame(fault: Patch) -> np.ndarray:
    """(n_dofs, 3, 3) rows [strike; dip; normal] per node (identity with
    allow_opening) (equations.py:423-440)."""
    n = np.asarray(fault.collocation_normals(), float)
    if fault.allow_opening:
        return np.ascontiguousarray(np.broadcast_to(np.eye(3), (n.shape[0], 3, 3)))
    s = np.cross(np.array([0.0, 0.0, 1.0]), n)
    length = np.linalg.norm(s, axis=1)
    flat = length <= defaults.FRAME_FLAT_TOL
    s[flat] = [1.0, 0.0, 0.0]
    s[~flat] /= length[~flat, None]
    d = np.cross(n, s)
    d /= np.linalg.norm(d, axis=1)[:, None]
    return np.ascontiguousarray(np.stack([s, d, n], axis=1))
