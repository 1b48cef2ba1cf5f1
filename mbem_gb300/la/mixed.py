"""Mixed-precision operator: FP32 far field (dense, quadrature) plus FP64 near
field (closed form, 3x3 blocks in CSR by field point).

``far_near_block`` assembles one kernel block both ways; ``MixedOperator``
holds the blocks of a system and applies it (far part in double-float
arithmetic, near part in FP64) through the C ABI.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import ptr, stream_handle


@dataclass
class NearList:
    row0: int               # first row of the block in the system (3 per field point)
    col0: int               # first column of the block in the system
    n_field: int
    rowptr: torch.Tensor    # (n_field + 1,) int64
    cols: torch.Tensor      # (nnz,) int64
    vals: torch.Tensor      # (nnz, 9) float64

    @property
    def nnz(self) -> int:
        return int(self.cols.numel())


_KERNEL_ID = {"T": 0, "U": 1}


def near_list(x_field: torch.Tensor, tri_verts: torch.Tensor, eps: torch.Tensor,
              near_factor: float = defaults.MIXED_NEAR_RADIUS_FACTOR):
    """(rowptr, cols) of the near pairs, sources in increasing order."""
    nf, ns = x_field.shape[0], tri_verts.shape[0]
    dev = x_field.device
    rowptr = torch.empty(nf + 1, dtype=torch.int64, device=dev)
    work = torch.empty(int(nat.lib().mbem_near_list_workspace_size(nf)), dtype=torch.uint8, device=dev)
    nnz = ctypes.c_int64(0)
    nat.call("mbem_near_count", ptr(x_field), nf, ptr(tri_verts), ptr(eps), ns, float(near_factor),
             ptr(rowptr), ptr(work), work.numel(), ctypes.byref(nnz), stream_handle())
    cols = torch.empty(max(nnz.value, 1), dtype=torch.int64, device=dev)[:nnz.value]
    nat.call("mbem_near_fill", ptr(x_field), nf, ptr(tri_verts), ptr(eps), ns, float(near_factor),
             ptr(rowptr), ptr(cols), stream_handle())
    return rowptr, cols


def far_near_block(kernel: str, x_field, tri_verts, normals, eps, coeffs, alpha: float,
                   far_out: torch.Tensor, row0: int = 0, col0: int = 0,
                   near_factor: float = defaults.MIXED_NEAR_RADIUS_FACTOR, timer=None,
                   far16_out: torch.Tensor | None = None, order: int = 0) -> NearList:
    """Writes alpha * (far part) into ``far_out`` (FP32 (3Nf, 3 K Ns) view,
    zeros at near pairs; K = 1, 3, 6 nodes per source for order 0, 1, 2) and
    returns the near blocks alpha * (closed form; the nodal closed form at
    order 1/2) in FP64, listed by field point over source nodes.
    ``far16_out``: an optional BF16 view of the same shape that receives the
    far part rounded to BF16 in the same pass."""
    return near_blocks(far_launch(kernel, x_field, tri_verts, normals, eps, coeffs, alpha, far_out, row0, col0,
                                  near_factor, timer, far16_out, order))


@dataclass
class FarLaunch:
    """A far-field block whose kernel is enqueued and whose near list is not
    read yet (``near_blocks`` reads it: the count is one wait on the stream)."""
    kernel: int
    order: int
    x_field: torch.Tensor
    tri_verts: torch.Tensor
    normals: torch.Tensor
    eps: torch.Tensor
    coeffs: object
    alpha: float
    row0: int
    col0: int
    mask: torch.Tensor


def far_launch(kernel: str, x_field, tri_verts, normals, eps, coeffs, alpha: float,
               far_out: torch.Tensor, row0: int = 0, col0: int = 0,
               near_factor: float = defaults.MIXED_NEAR_RADIUS_FACTOR, timer=None,
               far16_out: torch.Tensor | None = None, order: int = 0) -> FarLaunch:
    """The far half of ``far_near_block``: enqueues the far-field kernel
    (which also votes the near pairs into a bit mask) and returns at once."""
    k = _KERNEL_ID[kernel]
    nf, ns = x_field.shape[0], tri_verts.shape[0]
    K = {0: 1, 1: 3, 2: 6}[int(order)]
    if far_out.dtype != torch.float32 or far_out.stride(1) != 1 or tuple(far_out.shape) != (3 * nf, 3 * K * ns):
        raise ValueError("far_out must be a float32 (3Nf, 3 K Ns) view with unit column stride")
    c = nat.dbl_array(coeffs)
    ev = None
    if timer is not None:
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev[0].record()
    # the far kernel votes the near pairs into a bit mask (one word per warp of
    # sources), from which the near list is read without a second pass over
    # all pairs
    n_words = (ns + 31) // 32
    mask = torch.empty((nf, n_words), dtype=torch.int32, device=x_field.device)
    if far16_out is not None:
        if far16_out.dtype != torch.bfloat16 or far16_out.stride(1) != 1 or far16_out.shape != far_out.shape:
            raise ValueError("far16_out must be a bfloat16 view shaped like far_out with unit column stride")
    nat.call("mbem_far_matrix_nodal", k, int(order), ptr(x_field), nf, ptr(tri_verts), ptr(normals), ptr(eps), ns,
             c, float(near_factor), float(alpha), ptr(far_out), far_out.stride(0),
             ptr(far16_out) if far16_out is not None else None,
             far16_out.stride(0) if far16_out is not None else 0, ptr(mask), stream_handle())
    if ev is not None:
        ev[1].record()
        timer.append(("far_" + kernel, nf, ns, ev[0], ev[1]))
    return FarLaunch(k, int(order), x_field, tri_verts, normals, eps, c, float(alpha), row0, col0, mask)


def near_blocks(fl: FarLaunch) -> NearList:
    """The near half of ``far_near_block``: the near list read from the far
    kernel's mask and the near blocks evaluated in FP64."""
    k, c, x_field, tri_verts, normals, eps, alpha = (fl.kernel, fl.coeffs, fl.x_field, fl.tri_verts, fl.normals,
                                                     fl.eps, fl.alpha)
    mask, row0, col0 = fl.mask, fl.row0, fl.col0
    nf, ns = x_field.shape[0], tri_verts.shape[0]
    K = {0: 1, 1: 3, 2: 6}[fl.order]
    order = fl.order
    fl.mask = None
    rowptr = torch.empty(nf + 1, dtype=torch.int64, device=x_field.device)
    work = torch.empty(int(nat.lib().mbem_near_list_workspace_size(nf)), dtype=torch.uint8,
                       device=x_field.device)
    nnz = ctypes.c_int64(0)
    nat.call("mbem_near_mask_count", ptr(mask), nf, ns, ptr(rowptr), ptr(work), work.numel(),
             ctypes.byref(nnz), stream_handle())
    cols = torch.empty(max(nnz.value, 1), dtype=torch.int64, device=x_field.device)[:nnz.value]
    nat.call("mbem_near_mask_fill", ptr(mask), nf, ns, ptr(rowptr), ptr(cols), stream_handle())
    del mask
    nnz = cols.numel()
    vals = torch.empty((max(K * nnz, 1), 9), dtype=torch.float64, device=x_field.device)[:K * nnz]
    if K == 1:
        nat.call("mbem_near_eval", k, ptr(x_field), nf, ptr(tri_verts), ptr(normals), ptr(eps), ptr(rowptr),
                 ptr(cols), nnz, c, float(alpha), ptr(vals), stream_handle())
        return NearList(row0, col0, nf, rowptr, cols, vals)
    nat.call("mbem_near_eval_nodal", k, int(order), ptr(x_field), nf, ptr(tri_verts), ptr(normals), ptr(eps),
             ptr(rowptr), ptr(cols), nnz, c, float(alpha), ptr(vals), stream_handle())
    # the list by source nodes: pair q's node k is entry K q + k, column K s + k
    node_cols = (cols.view(-1, 1) * K + torch.arange(K, device=cols.device)).reshape(-1).contiguous()
    return NearList(row0, col0, nf, (rowptr * K).contiguous(), node_cols, vals)


class MixedOperator:
    """A = A32 (FP32 dense far field) + sum of near-block lists (FP64)."""

    def __init__(self, A32: torch.Tensor, near: list[NearList], A16: torch.Tensor | None = None):
        self.A32 = A32
        self.near = near
        self.A16 = A16          # optional BF16 copy of A32 (n, ld16), made by the assembly
        self._keep = None

    @property
    def n(self) -> int:
        return int(self.A32.shape[0])

    def struct(self, n_rows=None, n_cols=None) -> nat.MixedOperator:
        arr = (nat.NearBlocks * max(len(self.near), 1))()
        for i, nb in enumerate(self.near):
            arr[i] = nat.NearBlocks(nb.row0, nb.col0, nb.n_field, ptr(nb.rowptr), ptr(nb.cols), ptr(nb.vals))
        self._keep = arr
        return nat.MixedOperator(self.A32.shape[0] if n_rows is None else n_rows,
                                 self.A32.shape[1] if n_cols is None else n_cols, ptr(self.A32),
                                 self.A32.stride(0), len(self.near), arr)

    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        x = x.to(torch.float64).contiguous()
        y = out if out is not None else torch.empty(self.A32.shape[0], dtype=torch.float64, device=x.device)
        work = torch.empty(2 * x.numel() * 4 + 64, dtype=torch.uint8, device=x.device)
        op = self.struct()
        nat.call("mbem_mixed_matvec", ctypes.byref(op), ptr(x), ptr(y), ptr(work), work.numel(),
                 stream_handle())
        return y

    def rowsum3(self, row0: int, rows: int, col0: int, cols: int, near: NearList) -> torch.Tensor:
        """(rows/3, 3, 3) calibration row sums of one block (far + its near list)."""
        out = torch.empty((rows // 3, 3, 3), dtype=torch.float64, device=self.A32.device)
        view = self.A32[row0:row0 + rows, col0:col0 + cols]
        nat.call("mbem_mixed_rowsum3", ptr(view), view.stride(0), rows, cols // 3, ptr(near.rowptr),
                 ptr(near.vals), ptr(out), stream_handle())
        return out

    def dense64(self) -> torch.Tensor:
        """The operator as an FP64 dense matrix (tests and small systems only)."""
        A = self.A32.to(torch.float64)
        for nb in self.near:
            rp = nb.rowptr.cpu().numpy()
            f = torch.from_numpy(np.repeat(np.arange(nb.n_field), np.diff(rp))).to(A.device)
            for i in range(3):
                for j in range(3):
                    A[nb.row0 + 3 * f + i, nb.col0 + 3 * nb.cols + j] += nb.vals[:, 3 * i + j]
        return A


class Bf16Inner:
    """The mixed solve's inner preconditioner: GMRES from zero on the
    deflated operator with the far field rounded to BF16 (2 bytes per entry)
    and the near blocks in FP64, for at most ``iterations`` steps or until
    its residual estimate falls below ``rtol`` (0: always all steps). Used as a flexible right
    preconditioner of FGMRES on the accurate mixed operator (FP32 far field,
    double-float sums), whose true residual decides convergence."""

    PRECOND_KIND = 3

    def __init__(self, op: MixedOperator, iterations: int = defaults.MIXED_INNER_ITERATIONS,
                 u_ranges=(), rtol: float = defaults.MIXED_INNER_RTOL):
        if not 1 <= iterations <= nat.INNER_MAX_ITERS:
            raise ValueError(f"iterations must be in [1, {nat.INNER_MAX_ITERS}] (got {iterations})")
        if not 0.0 <= rtol < 1.0:
            raise ValueError(f"rtol must be in [0, 1) (got {rtol})")
        n = op.n
        self.rtol = float(rtol)
        self.op = op
        self.iterations = int(iterations)
        if op.A16 is not None:
            self.A16 = op.A16
            self.ld16 = op.A16.stride(0)
        else:
            self.ld16 = (n + 7) // 8 * 8
            self.A16 = torch.empty((n, self.ld16), dtype=torch.bfloat16, device=op.A32.device)
            nat.call("mbem_to_bf16", ptr(op.A32), 0, op.A32.stride(0), n, n, ptr(self.A16), self.ld16,
                     stream_handle())
        self.u_ranges = np.asarray(u_ranges, dtype=np.int64).reshape(-1, 2)
        self.work = None
        self.precond = None
        self.set_iterations(iterations)
        self.built = True
        self._keep = None

    def set_preconditioner(self, precond) -> None:
        """A fixed right preconditioner M of the inner GMRES (None: none):
        ``la.precond.BlockJacobi`` or ``la.learned.LearnedPreconditioner``
        built on this operator; the inner steps then multiply A16 by M."""
        kind = getattr(precond, "PRECOND_KIND", None) if precond is not None else 0
        if kind not in (0, 1, 2):
            raise TypeError(f"the inner solve takes a block-Jacobi or learned preconditioner, not "
                            f"{type(precond).__name__}")
        self.precond = precond

    def set_iterations(self, iterations: int) -> None:
        """Changes the inner step count (and grows the workspace to match)."""
        if not 1 <= iterations <= nat.INNER_MAX_ITERS:
            raise ValueError(f"iterations must be in [1, {nat.INNER_MAX_ITERS}] (got {iterations})")
        size = int(nat.lib().mbem_inner_bf16_workspace_size(self.n, iterations))
        if self.work is None or self.work.numel() < size:
            self.work = torch.empty(size, dtype=torch.uint8, device=self.op.A32.device)
        self.iterations = int(iterations)

    @property
    def n(self) -> int:
        return self.op.n

    def struct(self) -> nat.InnerBf16:
        arr = (nat.NearBlocks * max(len(self.op.near), 1))()
        for i, nb in enumerate(self.op.near):
            arr[i] = nat.NearBlocks(nb.row0, nb.col0, nb.n_field, ptr(nb.rowptr), ptr(nb.cols), ptr(nb.vals))
        ur = np.ascontiguousarray(self.u_ranges.ravel())
        kind, state = 0, None
        if self.precond is not None:
            kind = self.precond.PRECOND_KIND
            pst = self.precond.struct()
            state = ctypes.cast(ctypes.byref(pst), ctypes.c_void_p)
        self._keep = (arr, ur, state, pst if self.precond is not None else None)
        return nat.InnerBf16(self.n, ptr(self.A16), self.ld16, len(self.op.near), arr, self.iterations,
                             self.rtol, len(self.u_ranges), ur.ctypes.data if ur.size else None, ptr(self.work),
                             self.work.numel(), kind, state)

    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """(A16 + near) x: the inner operator itself."""
        x = x.to(torch.float64).contiguous()
        y = out if out is not None else torch.empty(self.n, dtype=torch.float64, device=x.device)
        arr = self.struct()
        work = torch.empty(4 * x.numel() + 64, dtype=torch.uint8, device=x.device)
        nat.call("mbem_bf16_matvec", ptr(self.A16), self.ld16, self.n, self.n, arr.n_near, arr.near, ptr(x),
                 ptr(y), ptr(work), work.numel(), stream_handle())
        return y

    def apply(self, r: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        r = r.to(torch.float64).contiguous()
        z = out if out is not None else torch.empty_like(r)
        st = self.struct()
        nat.call("mbem_inner_bf16_apply", ctypes.byref(st), ptr(r), ptr(z), stream_handle())
        return z


def inner_stats(timing: bool = False) -> tuple[int, int, float]:
    """(inner steps, inner solves, device ms of their BF16 products when they
    were timed) since the last call; ``timing`` switches the timing of the
    following inner solves on or off."""
    a, b, t = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_double(0.0)
    nat.lib().mbem_inner_bf16_stats(int(timing), ctypes.byref(a), ctypes.byref(b), ctypes.byref(t))
    return int(a.value), int(b.value), float(t.value)
