"""The body as its solved faults see it: ``AssembledDense.condense``
(src/mbem/backends/dense.py:580-646), on the GPU.

Every unknown but the FAULT_TRACTION faults' slip is eliminated: with the
faults' enforced rows (strike, dip, and normal with ``allow_opening``) of the
free nodes, E the unit slip of each coordinate in Cartesian components and
r the remaining unknowns,

    S = A_ff E - A_fr A_rr^-1 A_rf E        L = -(b_f - A_fr A_rr^-1 b_r)

so the traction the fault rows hold to zero is S beta + L and the whole
unknown vector is x = x0 + X beta (x0 = A_rr^-1 b_r on r, X = -A_rr^-1 A_rf E
on r and E on the faults' slots). A_rr is factored once by the project's GPU
LU (FP32 factors); the coordinate columns and b_r are solved together as one
block and refined in FP64 (la/lu.py); the products with A_fr are FP64.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from ..model.equations import traction_row_frame


@dataclass
class FaultCoordinates:
    """One FAULT_TRACTION fault's share of the condensed unknowns
    (dense.py:275-302). Entries ``start`` to ``stop`` of a condensed vector
    belong to this fault: for each dof node in ``free`` (the nodes that are
    not locked), in order, its slip measured along each row of ``frame`` for
    that node. The rows are strike and dip, plus the normal when the fault may
    open."""
    name: str
    free: np.ndarray            # (n_free,) dof nodes
    frame: np.ndarray           # (n_free, n_comp, 3)
    start: int
    stop: int
    n_dofs: int

    def cartesian(self, v) -> np.ndarray:
        """Coordinates (stop - start,) -> Cartesian vectors (n_dofs, 3), zero at a locked node."""
        out = np.zeros((self.n_dofs, 3))
        out[self.free] = np.einsum("fi,fij->fj", np.asarray(v, float).reshape(self.frame.shape[:2]), self.frame)
        return out

    def coordinates(self, vectors) -> np.ndarray:
        """Cartesian vectors at the dof nodes -> coordinates (the components along the frame's rows)."""
        return np.einsum("fij,fj->fi", self.frame, np.asarray(vectors, float)[self.free]).ravel()


@dataclass
class Condensed:
    """traction = S @ beta + L, x = x0 + X @ beta (dense.py:305-345)."""
    S: np.ndarray
    L: np.ndarray
    X: np.ndarray
    x0: np.ndarray
    faults: tuple
    layout: object
    cond_estimate: float

    @property
    def n(self) -> int:
        return self.S.shape[0]

    def dragged(self, kappa) -> np.ndarray:
        """The slip (coordinates) of faults that drag with ``kappa``."""
        k = np.broadcast_to(np.asarray(kappa, float), (self.n,))
        return np.linalg.solve(np.diag(k) - self.S, self.L)

    def split(self, v) -> dict:
        return {f.name: np.asarray(v)[f.start:f.stop].reshape(f.frame.shape[:2]) for f in self.faults}


def condense(asm, refine: bool = True) -> Condensed:
    """The Schur complement of an assembled FP64 system onto its traction
    faults' slip coordinates (see the module docstring)."""
    from ..la.lu import Factor, _many, solve_many
    system = asm.system
    faults = system.traction_faults()
    if not faults:
        raise ValueError("condense: the model has no FAULT_TRACTION fault, so there is nothing to condense onto")
    if getattr(asm, "fault_drag", None):
        raise ValueError("condense: this operator was built with a drag; its fault rows already carry a law")
    if asm.deflate:
        raise ValueError("condense: not with deflate (a bordered system)")
    if asm.A is None:
        raise ValueError("condense needs the FP64 operator (precision='fp64')")
    A, b = asm.A, asm.b
    dev = A.device
    N = A.shape[0]
    on_fault = np.zeros(N, bool)
    coords, rows, start = [], [], 0
    for region, f in faults:
        slot = asm.layout.slot(f, "b")
        free = np.flatnonzero(~np.asarray(f.locked_mask(region.patches), bool))
        n_comp = 3 if f.allow_opening else 2
        on_fault[slot.offset:slot.stop] = True
        rows.append((slot.offset + 3 * free[:, None] + np.arange(n_comp)[None, :]).ravel())
        coords.append(FaultCoordinates(f.name, free, traction_row_frame(f)[free, :n_comp, :], start,
                                       start + n_comp * free.size, f.n_dofs))
        start += n_comp * free.size
    n = start
    rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    # AE: the columns of a unit of each coordinate; X on the faults' slots: E
    AE = torch.empty((N, n), dtype=torch.float64, device=dev)
    X = torch.zeros((N, n), dtype=torch.float64, device=dev)
    for (_region, f), c in zip(faults, coords):
        slot = asm.layout.slot(f, "b")
        cols = A[:, slot.offset:slot.stop].reshape(N, f.n_dofs, 3)
        fr = torch.from_numpy(np.ascontiguousarray(c.frame)).to(dev)
        free = torch.from_numpy(c.free).to(dev)
        AE[:, c.start:c.stop] = torch.einsum("rfj,fij->rfi", cols[:, free, :], fr).reshape(N, -1)
        k = c.start + c.frame.shape[1] * np.arange(c.free.size)
        for i in range(c.frame.shape[1]):
            for j in range(3):
                X[torch.from_numpy(slot.offset + 3 * c.free + j).to(dev),
                  torch.from_numpy(k + i).to(dev)] = fr[:, i, j]
    rest = torch.from_numpy(np.flatnonzero(~on_fault)).to(dev)
    rows_d = torch.from_numpy(rows).to(dev)
    x0 = torch.zeros(N, dtype=torch.float64, device=dev)
    S = AE[rows_d].clone()
    L = -b[rows_d].clone()
    cond = 1.0
    if rest.numel():
        A_rr = A[rest][:, rest].contiguous()
        fac = Factor(A_rr)
        rhs = torch.cat([AE[rest], b[rest][:, None]], dim=1).contiguous()
        sol = solve_many(fac, rhs) if refine else _many(fac, rhs)
        X[rest] = -sol[:, :n]
        x0[rest] = sol[:, n]
        A_fr = A[rows_d][:, rest]
        S = S + A_fr @ X[rest]
        L = L + A_fr @ x0[rest]
        asm.lu_report = dict(fac.report)
        cond = fac.cond()
        del fac, A_rr
    # the eliminated block's condition estimate in the report, as the
    # reference's condense leaves it (dense.py:641)
    from .dense import DenseSolveReport
    asm.report = DenseSolveReport(converged=True, iterations=0, true_relres=float("nan"),
                                  arnoldi_relres=float("nan"), cond_estimate=cond,
                                  lu=getattr(asm, "lu_report", None))
    return Condensed(S=S.cpu().numpy(), L=L.cpu().numpy(), X=X.cpu().numpy(), x0=x0.cpu().numpy(),
                     faults=tuple(coords), layout=asm.layout, cond_estimate=cond)
