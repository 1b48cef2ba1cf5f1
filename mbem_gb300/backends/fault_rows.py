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
    n_cols = A.shape[1]
    for region, f in system.traction_faults():
        slot = system.layout.slot(f, "b")
        r0 = slot.offset
        n = f.n_dofs
        F_np = traction_row_frame(f)
        F = torch.from_numpy(np.ascontiguousarray(F_np)).to(A.device)
        nat.call("mbem_rotate_row_triples", ptr(A[r0:]), A.stride(0), n_cols, ptr(b[r0:]), n, ptr(F),
                 stream_handle())
        lock = np.asarray(f.locked_mask(region.patches), bool)
        free = np.flatnonzero(~lock)
        free_d = torch.from_numpy(free).to(A.device)
        if free.size:
            rr = r0 + 3 * free_d
            diag = torch.cat([A[rr, rr], A[rr + 1, rr + 1]])
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
            w_d = torch.from_numpy(w).to(A.device)
            wk_d = torch.from_numpy(wk).to(A.device)
            F_free = F[free_d]
            for i in range(3 if f.allow_opening else 2):
                rows = r0 + 3 * free_d + i
                A[rows, :] *= w_d[:, None]
                b[rows] *= w_d
                for j in range(3):
                    A[rows, r0 + 3 * free_d + j] -= wk_d * F_free[:, i, j]
        if not f.allow_opening and free.size:
            nrm = torch.from_numpy(np.asarray(f.collocation_normals(), float)[free]).to(A.device)
            rows = r0 + 3 * free_d + 2
            A[rows, :] = 0.0
            for j in range(3):
                A[rows, r0 + 3 * free_d + j] = scale * nrm[:, j]
            b[rows] = 0.0
        locked = np.flatnonzero(lock)
        if locked.size:
            locked_d = torch.from_numpy(locked).to(A.device)
            for i in range(3):
                rows = r0 + 3 * locked_d + i
                A[rows, :] = 0.0
                A[rows, rows] = scale
                b[rows] = 0.0
