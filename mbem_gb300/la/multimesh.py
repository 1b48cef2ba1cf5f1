"""Many unevenly sized meshes solved together (one persistent launch per
operator application, one CUDA graph per restart cycle).

``MeshBatch`` takes assembled mixed-precision systems (``DenseBackend(...,
precision="mixed").assemble``), lays their unknowns out one after another in
batch vectors (segments rounded up to 512 entries) and solves all of them by
deflated GMRES(restart) in lockstep on the device: the same iteration as the
single-system FGMRES (la/solver.py:115-245 with backends/hmat.py:678-690
deflation) per mesh, with each mesh's convergence judged on its own true
residual.
"""

from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as nat
from .._device import ptr, stream_handle


@dataclass
class BatchReport:
    iterations: list          # Arnoldi steps per mesh
    relres: list              # true relative residual per mesh at the last check
    converged: list
    cycles: int               # restart cycles run

    @property
    def all_converged(self) -> bool:
        return all(self.converged)


def _merged_near(op):
    """One CSR by field point over the whole system of a mixed operator
    (its near-block lists, each placed at its row/column offset)."""
    n_nodes = op.n // 3
    if len(op.near) == 1:
        nl = op.near[0]
        if nl.row0 == 0 and nl.col0 == 0 and nl.n_field == n_nodes:
            return nl.rowptr, nl.cols, nl.vals
    dev = op.A32.device
    rows, cols, vals = [], [], []
    for nl in op.near:
        f = torch.repeat_interleave(torch.arange(nl.n_field, device=dev), torch.diff(nl.rowptr))
        rows.append(nl.row0 // 3 + f)
        cols.append(nl.col0 // 3 + nl.cols)
        vals.append(nl.vals)
    if not rows:
        return (torch.zeros(n_nodes + 1, dtype=torch.int64, device=dev),
                torch.zeros(1, dtype=torch.int64, device=dev), torch.zeros((1, 9), dtype=torch.float64, device=dev))
    r = torch.cat(rows)
    order = torch.argsort(r, stable=True)
    rowptr = torch.zeros(n_nodes + 1, dtype=torch.int64, device=dev)
    rowptr[1:] = torch.cumsum(torch.bincount(r, minlength=n_nodes), 0)
    return rowptr, torch.cat(cols)[order].contiguous(), torch.cat(vals)[order].contiguous()


class MeshBatch:
    """A batch of assembled mixed-precision systems solved together."""

    def __init__(self, systems: list, restart: int = 50):
        if not systems:
            raise ValueError("no systems")
        if not 1 <= restart <= nat.MM_MAX_RESTART:
            raise ValueError(f"restart must be in [1, {nat.MM_MAX_RESTART}] (got {restart})")
        self.systems = list(systems)
        self.restart = int(restart)
        n_mesh = len(self.systems)
        meshes = (nat.MmMesh * n_mesh)()
        self._keep = []
        self.offsets, self.sizes = [], []
        off = 0
        for i, asm in enumerate(self.systems):
            op = getattr(asm, "op", None)
            if op is None:
                raise ValueError("MeshBatch needs mixed-precision systems (precision='mixed')")
            ur = asm.u_ranges()
            if len(ur) > 1:
                raise ValueError("MeshBatch deflates at most one u-slot range per mesh")
            u_off, u_len = ur[0] if ur else (0, 0)
            rowptr, cols, vals = _merged_near(op)
            self._keep.append((rowptr, cols, vals))
            n = op.n
            A16 = op.A16
            meshes[i] = nat.MmMesh(ptr(op.A32), op.A32.stride(0), n, off, ptr(rowptr), ptr(cols), ptr(vals),
                                   int(u_off), int(u_len), ptr(A16) if A16 is not None else None,
                                   A16.stride(0) if A16 is not None else 0)
            self.offsets.append(off)
            self.sizes.append(n)
            off += -(-n // nat.MM_SEGMENT) * nat.MM_SEGMENT
        self.n_total = off
        self._meshes = meshes
        size = int(nat.lib().mbem_mm_workspace_size(meshes, n_mesh, self.restart))
        if size == 0:
            raise ValueError("invalid mesh batch layout")
        dev = self.systems[0].op.A32.device
        self.device = dev
        self.work = torch.empty(size, dtype=torch.uint8, device=dev)
        # graph capture needs a stream of its own (not the legacy default)
        self.stream = torch.cuda.Stream(device=dev)
        handle = ctypes.c_void_p()
        with torch.cuda.stream(self.stream):
            nat.call("mbem_mm_create", meshes, n_mesh, self.restart, ptr(self.work), size, stream_handle(),
                     ctypes.byref(handle))
        self._handle = handle
        self._finalizer = weakref.finalize(self, nat.lib().mbem_mm_destroy, handle)

    @property
    def n_mesh(self) -> int:
        return len(self.systems)

    def gather(self, vectors) -> torch.Tensor:
        """Batch vector (zero padding) from one vector per mesh."""
        out = torch.zeros(self.n_total, dtype=torch.float64, device=self.device)
        for o, n, v in zip(self.offsets, self.sizes, vectors):
            out[o:o + n] = torch.as_tensor(v, dtype=torch.float64, device=self.device).reshape(-1)
        return out

    def scatter(self, X: torch.Tensor) -> list:
        """Per-mesh views of a batch vector."""
        return [X[o:o + n] for o, n in zip(self.offsets, self.sizes)]

    def _run(self, fn):
        cur = torch.cuda.current_stream(self.device)
        self.stream.wait_stream(cur)
        with torch.cuda.stream(self.stream):
            out = fn()
        cur.wait_stream(self.stream)
        return out

    def matvec(self, X: torch.Tensor) -> torch.Tensor:
        X = X.to(torch.float64).contiguous()
        Y = torch.zeros_like(X)
        self._run(lambda: nat.call("mbem_mm_matvec", self._handle, ptr(X), ptr(Y), stream_handle()))
        return Y

    @property
    def has_bf16(self) -> bool:
        """Every mesh carries the BF16 copy of its far field (assembled with
        precond="bf16_inner"): the mixed solve is available."""
        return all(a.op.A16 is not None for a in self.systems)

    def solve_mixed(self, B: torch.Tensor | None = None, rtol: float = 1e-8, inner_rtol: float = 1e-5,
                    max_outer: int = 6, max_cycles: int = 4, graph: bool = True):
        """(X, BatchReport): refinement on the accurate operators whose
        corrections are lockstep GMRES solves on the BF16 far fields (2 bytes
        an entry) to ``inner_rtol`` of each residual. BatchReport.cycles:
        refinement steps; iterations: the inner steps of each mesh."""
        if not self.has_bf16:
            raise ValueError("the mixed batch solve needs every system assembled with precond='bf16_inner'")
        if B is None:
            B = self.gather([asm.b for asm in self.systems])
        B = B.to(torch.float64).contiguous()
        X = torch.empty_like(B)
        nm = self.n_mesh
        its = (ctypes.c_int * nm)()
        rel = (ctypes.c_double * nm)()
        conv = (ctypes.c_int * nm)()
        rep = nat.MmReport(its, rel, conv, 0)
        self._run(lambda: nat.call("mbem_mm_solve_mixed", self._handle, ptr(B), ptr(X), float(rtol),
                                   float(inner_rtol), int(max_outer), int(max_cycles), int(bool(graph)),
                                   ctypes.byref(rep), stream_handle()))
        return X, BatchReport(list(its), list(rel), [bool(c) for c in conv], int(rep.cycles))

    def solve(self, B: torch.Tensor | None = None, rtol: float = 1e-8, max_cycles: int = 40,
              graph: bool = True):
        """(X, BatchReport): every mesh's deflated solution (batch vector) to
        ``rtol`` on its own true residual. B defaults to each system's b."""
        if B is None:
            B = self.gather([asm.b for asm in self.systems])
        B = B.to(torch.float64).contiguous()
        X = torch.empty_like(B)
        nm = self.n_mesh
        its = (ctypes.c_int * nm)()
        rel = (ctypes.c_double * nm)()
        conv = (ctypes.c_int * nm)()
        rep = nat.MmReport(its, rel, conv, 0)
        self._run(lambda: nat.call("mbem_mm_solve", self._handle, ptr(B), ptr(X), float(rtol), int(max_cycles),
                                   int(bool(graph)), ctypes.byref(rep), stream_handle()))
        return X, BatchReport(list(its), list(rel), [bool(c) for c in conv], int(rep.cycles))


def random_cube_batch(n_mesh: int = 64, lo: int = 8, hi: int = 32, seed: int = 7) -> list[tuple[int, int]]:
    """(per-face grid, fault grid) of ``n_mesh`` cubes with per-face grids
    drawn uniformly in [lo, hi] (seeded); each fault grid is two thirds of
    the face grid (at least 2), as in the single-cube workloads."""
    rng = np.random.default_rng(seed)
    faces = rng.integers(lo, hi + 1, size=n_mesh)
    return [(int(f), max(2, int(round(2 * f / 3)))) for f in faces]
