"""The row frame, drag, constraint and locked rows of FAULT_TRACTION faults,
applied in place to the device system (src/mbem/model/equations.py:443-506
``apply_fault_rows``).

Per traction fault f (rows r0 .. r0 + 3 n of A, every column):

* rows of node c -> F_c times themselves, F the strike/dip/normal frame
  (``traction_row_frame``; identity with ``allow_opening``), A and b alike
  (the CUDA row-triple kernel);
* ``scale`` = mean |diagonal| of the fault's tangential self-rows over its
  free nodes (1 when there are none or it is 0);
* a drag kappa >= 0 (number or one per node, ``inf`` allowed) divides every
  enforced row of a free node by 1 + kappa / scale and subtracts
  kappa / (1 + kappa / scale) times the frame row from its own slip columns;
* without ``allow_opening`` a free node's third row becomes the constraint
  scale * n_c . b_c = 0;
* a locked node's three rows become scale * b_c = 0.
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _native as nat
from .._device import ptr, stream_handle
from ..model.equations import traction_row_frame


def apply_fault_rows(A: torch.Tensor, b: torch.Tensor, system, drag: dict | None = None) -> None:
    """In place on the CUDA system (A (n, n) row-major, b (n,))."""
    for region, f in system.traction_faults():
        r0 = system.layout.slot(f, "b").offset
        n = f.n_dofs
        fault_rows_one(A[r0:r0 + 3 * n], b[r0:r0 + 3 * n], region, f, r0, drag)


def fault_rows_one(R: torch.Tensor, bf: torch.Tensor, region, f, c0: int, drag: dict | None = None) -> None:
    """One fault's transformation in place on its own rows: R (3 n, n_cols)
    (every column of the system), bf (3 n,), the fault's slip columns at
    c0 .. c0 + 3 n (its row and column slots coincide)."""
    n_cols = R.shape[1]
    n = f.n_dofs
    F_np = traction_row_frame(f)
    F = torch.from_numpy(np.ascontiguousarray(F_np)).to(R.device)
    nat.call("mbem_rotate_row_triples", ptr(R), R.stride(0), n_cols, ptr(bf), n, ptr(F), stream_handle())
    lock = np.asarray(f.locked_mask(region.patches), bool)
    free = np.flatnonzero(~lock)
    free_d = torch.from_numpy(free).to(R.device)
    if free.size:
        rr = 3 * free_d
        cc = c0 + 3 * free_d
        diag = torch.cat([R[rr, cc], R[rr + 1, cc + 1]])
        scale = float(diag.abs().mean())
    else:
        scale = 1.0
    if scale == 0.0:
        scale = 1.0
    kappa = None if drag is None else drag.get(f.name)
    if kappa is not None and free.size:
        k = np.broadcast_to(np.asarray(kappa, float), (n,))[free]
        if np.any(k < 0.0) or np.any(np.isnan(k)):
            raise ValueError(f"fault '{f.name}': drag must be >= 0")
        inf = np.isinf(k)
        kf = np.where(inf, 0.0, k)
        w = np.where(inf, 0.0, scale / (scale + kf))
        wk = np.where(inf, scale, w * kf)
        w_d = torch.from_numpy(w).to(R.device)
        wk_d = torch.from_numpy(wk).to(R.device)
        F_free = F[free_d]
        for i in range(3 if f.allow_opening else 2):
            rows = 3 * free_d + i
            R[rows, :] *= w_d[:, None]
            bf[rows] *= w_d
            for j in range(3):
                R[rows, c0 + 3 * free_d + j] -= wk_d * F_free[:, i, j]
    if not f.allow_opening and free.size:
        nrm = torch.from_numpy(np.asarray(f.collocation_normals(), float)[free]).to(R.device)
        rows = 3 * free_d + 2
        R[rows, :] = 0.0
        for j in range(3):
            R[rows, c0 + 3 * free_d + j] = scale * nrm[:, j]
        bf[rows] = 0.0
    locked = np.flatnonzero(lock)
    if locked.size:
        locked_d = torch.from_numpy(locked).to(R.device)
        for i in range(3):
            rows = 3 * locked_d + i
            R[rows, :] = 0.0
            R[rows, c0 + rows] = scale
            bf[rows] = 0.0
