"""The calibrated dense backend on one GB300 (``src/mbem/backends/dense.py``).

Same API as the reference: ``DenseBackend(jump=..., deflate=...).assemble(
system, eps)`` returns an ``AssembledDense`` with ``.A``, ``.b``, ``.calib``,
``.layout``, ``.solve() -> {slot_name: (n, 3)}`` and ``.report``.

Where the reference builds ``A`` block by block with numba on the host and
factors it with LAPACK (dense.py:480-571), this backend assembles every
block with the CUDA pair kernels straight into a device-resident FP64 ``A``
(each block written at its offset, scaled by its sign, no host copy), takes
the calibration row sums from the blocks in place (a fixed-order reduction),
contracts the right-hand side matrix-free, and solves with deflated FGMRES
on the device (the hmat.py:678-690 wiring). The solution agrees with the
reference's bordered-LU solution to the solver tolerance.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import as_cuda, ptr, require_cuda, stream_handle
from ..kernels import KERNEL_GT, KERNEL_HT, KERNEL_T, KERNEL_U
from ..kernels import basis as kb
from ..kernels import tri_nodal as tn
from ..la.solver import SolveReport, fgmres_dense, fgmres_mixed
from ..model.core import BCType
from ..model.equations import BlockSystem, calibrated_diagonal, term_diagonal


class DenseBackend:
    """``jump="calibrated"`` sets each collocation diagonal so that constant
    displacement fields are annihilated exactly; ``"half"`` adds 1/2 I. On an
    all-Neumann model the calibrated operator has the rigid translations as
    an exact null space, which ``deflate=True`` projects out."""

    def __init__(self, mode: str = "direct", jump: str = "calibrated", deflate: bool = False,
                 lu: str | None = None, rtol: float = 1e-10, restart: int = 50,
                 maxiter: int = defaults.GMRES_MAXITER, precision: str = "fp64",
                 near_factor: float = defaults.MIXED_NEAR_RADIUS_FACTOR, precond: str | None = None):
        """``precond``: None (plain FGMRES, the reference's dense-backend
        solve), "block_jacobi" (la/preconditioner.py:421-470 cluster
        block-Jacobi, built on first solve) or, with ``precision="mixed"``,
        "bf16_inner" (a few GMRES steps on the far field rounded to BF16 as a
        flexible preconditioner; the outer FGMRES keeps the FP32 operator).
        "bf16_learned" adds to that inner solve, as its right preconditioner,
        the learned two-level preconditioner (block-Jacobi with the learned
        coarse space, ``la.learned``) set up on the BF16 inner operator.
        ``precision="fp64"``: every entry by the FP64 closed form, the
        reference's operator. ``"mixed"``: pairs beyond near_factor *
        max(eps, h) of the source by FP32 quadrature (stored FP32), the near
        pairs by the FP64 closed form (stored as 3x3 blocks); the solve's
        residuals are those of that operator."""
        if mode not in ("direct", "basis", "legacy"):
            raise ValueError(mode)
        if jump not in ("half", "calibrated"):
            raise ValueError(jump)
        if lu not in (None, "gpu", "single"):
            raise ValueError(f"lu must be None (FGMRES), 'gpu' or 'single' (FP32 factors on the GPU, refined "
                             f"in FP64); got {lu!r}")
        if lu is not None and precision != "fp64":
            raise ValueError("lu= factors the FP64 operator (precision='fp64')")
        self.lu = lu
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed' (got {precision!r})")
        self.mode = "direct"
        self.jump = jump
        self.deflate = deflate
        self.rtol = rtol
        self.restart = restart
        self.maxiter = maxiter
        self.precision = precision
        self.near_factor = near_factor
        if precond not in (None, "block_jacobi", "bf16_inner", "bf16_learned"):
            raise ValueError(f"precond must be None, 'block_jacobi', 'bf16_inner' or 'bf16_learned' "
                             f"(got {precond!r})")
        if precond in ("bf16_inner", "bf16_learned") and precision != "mixed":
            raise ValueError(f"precond={precond!r} needs precision='mixed'")
        self.precond = precond

    def assemble(self, system: BlockSystem, eps, arrays: dict | None = None,
                 timer: list | None = None, fault_drag: dict | None = None) -> "AssembledDense":
        """``arrays``: an optional caller-held dict of per-patch device arrays,
        reused across assemblies of the same model (no host-to-device copy
        when it is already filled). ``timer``: an optional list that receives
        (start, end) CUDA events around every kernel-block launch."""
        return AssembledDense(system, eps, jump=self.jump, deflate=self.deflate, rtol=self.rtol,
                              restart=self.restart, maxiter=self.maxiter, arrays=arrays, timer=timer,
                              precision=self.precision, near_factor=self.near_factor, precond=self.precond,
                              lu=self.lu, fault_drag=fault_drag)


def _checked_drag(system: BlockSystem, drag) -> dict:
    """``{fault name: kappa}`` naming only FAULT_TRACTION faults of the model
    (dense.py:247-257: a drag on a prescribed slip would be silently nothing)."""
    drag = dict(drag or {})
    known = {f.name for _r, f in system.traction_faults()}
    unknown = set(drag) - known
    if unknown:
        raise KeyError(f"fault_drag names {sorted(unknown)}, which are not FAULT_TRACTION faults of the model "
                       f"(those are {sorted(known)})")
    return drag


# one high-priority side stream per device for the assembly warnings
_SIDE_STREAMS: dict = {}


def _f32_matrix(rows: int, cols: int, dev, zero: bool = False) -> torch.Tensor:
    """An FP32 (rows, cols) matrix whose rows start on 16-byte boundaries
    (leading dimension rounded up to 4), as the streaming matvecs need."""
    ld = (cols + 3) // 4 * 4
    return (torch.zeros if zero else torch.empty)((rows, ld), dtype=torch.float32, device=dev)[:, :cols]


def require_anchor_or_deflate(system: BlockSystem, jump: str, deflate: bool):
    """The calibrated jump on an un-anchored model needs deflation
    (dense.py:101-121)."""
    if jump == "calibrated" and not deflate and not system.model.is_anchored() \
            and system.layout.has_kind("u"):
        raise ValueError("jump='calibrated' on an all-Neumann model (no PRESCRIBED_DISPLACEMENT "
                         "patch): rigid translations are an EXACT null space of the calibrated "
                         "operator. Pass deflate=True (projected solve) or prescribe displacement "
                         "on a patch.")


def translation_basis(layout) -> np.ndarray:
    """Orthonormal rigid-translation basis Z (n, 3) on the u-slots
    (dense.py:190-208); (n, 0) when there is no u-slot."""
    if not layout.has_kind("u"):
        return np.zeros((layout.n_unknowns, 0))
    Z = np.zeros((layout.n_unknowns, 3))
    for slot in layout.slots:
        if slot.kind == "u":
            for k in range(3):
                Z[slot.offset + k:slot.stop:3, k] = 1.0
    Z /= np.linalg.norm(Z, axis=0, keepdims=True)
    return Z


@dataclass
class DenseSolveReport(SolveReport):
    """The report of a dense GPU solve: ``SolveReport`` fields, and for an LU
    solve the 1-norm condition estimate of the factored operator
    (dense.py:260-271 ``cond_estimate``; NaN for an FGMRES solve) and the
    factorisation's report (``lu``)."""
    cond_estimate: float = float("nan")
    lu: dict | None = None


def warn_condition(cond: float) -> None:
    """The reference's warning above COND_WARN_THRESHOLD (dense.py:555-562)."""
    if cond > defaults.COND_WARN_THRESHOLD:
        warnings.warn(f"dense solve: condition estimate {cond:.2e} exceeds {defaults.COND_WARN_THRESHOLD:.0e}; "
                      f"the solution may miss the {defaults.SOLUTION_RTOL:.0e} accuracy target (thin panels, "
                      f"near-fluid material, un-anchored calibrated jump, or discretization resonance)")


class AssembledDense:
    def __init__(self, system: BlockSystem, eps, mode: str = "direct", jump: str = "calibrated",
                 deflate: bool = False, rtol: float = 1e-10, restart: int = 50,
                 maxiter: int = defaults.GMRES_MAXITER, arrays: dict | None = None,
                 timer: list | None = None, precision: str = "fp64",
                 near_factor: float = defaults.MIXED_NEAR_RADIUS_FACTOR, precond: str | None = None,
                 lu: str | None = None, fault_drag: dict | None = None):
        if jump not in ("half", "calibrated"):
            raise ValueError(jump)
        require_anchor_or_deflate(system, jump, deflate)
        require_cuda()
        from .diagnostics import warn_assembly
        # the mixed assembly runs them once its far-field kernels are enqueued
        self._warn_pending = precision == "mixed"
        if not self._warn_pending:
            warn_assembly(system, eps, jump)
        self.fault_drag = _checked_drag(system, fault_drag)
        self.lu = lu
        self._factor = None
        self._arrays_in = arrays
        self._timer = timer
        self.precision = precision
        self.near_factor = near_factor
        self.precond = precond
        self._bj = None
        self._inner = None
        self.op = None
        self.system = system
        self.layout = system.layout
        self.eps = eps
        self.mode = "direct"
        self.jump = jump
        self.deflate = deflate
        self.rtol, self.restart, self.maxiter = rtol, restart, maxiter
        self.materials = {r.name: r.material for r in system.model.regions}
        self.report = None
        self.A = None
        self.b = None
        self._x = None
        self._build()

    # -- per-patch device arrays, built once per assembly --------------
    def _patch_arrays(self, patch):
        key = id(patch)
        v = self._arrays.get(key)
        if v is None:
            tv, normals, coll, coll_n = patch.geometry()
            eps_arr = kb.resolve_patch_eps(self.eps, patch)
            v = dict(tv=as_cuda(tv), normals=as_cuda(normals), eps=as_cuda(eps_arr),
                     coll=as_cuda(coll), coll_n=as_cuda(coll_n))
            self._arrays[key] = v
        return v

    def _block_into(self, out, field_patch, source_patch, kernel, material, alpha, accumulate):
        """Assemble one kernel block into ``out`` (a (rows, cols) view)."""
        f = self._patch_arrays(field_patch)
        s = self._patch_arrays(source_patch)
        order = source_patch.order
        ev = None
        if self._timer is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        if kernel == KERNEL_T:
            c = kb.t_coeffs(material.mu, material.lam)
            tn.t_matrix_direct(f["coll"], s["tv"], s["normals"], s["eps"], *c, order, out=out,
                               alpha=alpha, accumulate=accumulate)
        elif kernel == KERNEL_U:
            g = kb.u_coeffs(material.mu, material.lam)
            tn.u_matrix_direct(f["coll"], s["tv"], s["eps"], *g, order, out=out, alpha=alpha,
                               accumulate=accumulate)
        else:
            which = "slip" if kernel == KERNEL_HT else "force"
            ids = kb.identity_ids(order, source_patch.n_triangles)
            if not accumulate:
                out.zero_()          # the traction rows are always accumulated
            tn.traction_matrix(f["coll"], f["coll_n"], s["tv"], s["normals"], s["eps"], ids, ids.size,
                               material.mu, material.lam, order, which, out=out, alpha=alpha)
        if ev is not None:
            ev[1].record()
            self._timer.append((kernel, out.shape[0] // 3, out.shape[1] // 3, ev[0], ev[1]))

    def _rowsum(self, out_rows, block):
        """(rows/3, 3, 3) calibration row sums of a (rows, 3 n) block view."""
        rows, cols = block.shape
        res = torch.empty((rows, 3), dtype=torch.float64, device=block.device)
        nat.call("mbem_block_rowsum3", ptr(block), block.stride(0), rows, cols // 3, 1.0, 0, ptr(res),
                 stream_handle())
        return res.reshape(rows // 3, 3, 3)

    # -- mixed precision: FP32 far field + FP64 near blocks -------------
    def _mixed_block(self, far_out, q, p, kernel, material, alpha, row0, col0, far16_out=None):
        from ..la.mixed import near_blocks
        return near_blocks(self._mixed_launch(far_out, q, p, kernel, material, alpha, row0, col0, far16_out))

    def _mixed_launch(self, far_out, q, p, kernel, material, alpha, row0, col0, far16_out=None):
        """Enqueues one block's far-field kernel; ``near_blocks`` of the
        result reads its near list."""
        from ..la.mixed import far_launch
        if kernel not in (KERNEL_T, KERNEL_U):
            raise NotImplementedError("traction rows are not in the mixed-precision operator")
        f = self._patch_arrays(q)
        s = self._patch_arrays(p)
        name = "T" if kernel == KERNEL_T else "U"
        coeffs = (kb.t_coeffs if kernel == KERNEL_T else kb.u_coeffs)(material.mu, material.lam)
        return far_launch(name, f["coll"], s["tv"], s["normals"], s["eps"], coeffs, alpha, far_out, row0, col0,
                          self.near_factor, self._timer, far16_out, p.order)

    @staticmethod
    def _side_stream():
        dev = torch.cuda.current_device()
        side = _SIDE_STREAMS.get(dev)
        if side is None:
            side = _SIDE_STREAMS[dev] = torch.cuda.Stream(priority=-1)
        return side

    def _warn_on_side_stream(self):
        """The assembly warnings (their distance kernels and reads) on a
        high-priority side stream, so that they overlap the kernels already
        enqueued on the current one."""
        from .diagnostics import warn_assembly
        if not self._warn_pending:
            return
        self._warn_pending = False
        side = self._side_stream()
        with torch.cuda.stream(side):
            warn_assembly(self.system, self.eps, self.jump)
        side.synchronize()

    def _learned_geometry_on_side_stream(self, arrays_ready):
        """The learned preconditioner's mesh-only setup (the block-Jacobi
        chunks, the node features, the network's coarse vectors) on the side
        stream, behind the device mesh arrays (``arrays_ready``) but beside
        the far-field kernels; ``block_jacobi`` and ``bf16_learned`` make
        the current stream wait for it."""
        from ..la.learned import LearnedGeometry
        from ..la.precond import MAX_NODES, BlockJacobi
        from ..la.train_learned import load_default
        main = torch.cuda.current_stream()
        side = self._side_stream()
        side.wait_event(arrays_ready)
        with torch.cuda.stream(side):
            groups = [(s_.offset, self._patch_arrays(s_.patch)["coll"].view(-1, 3)) for s_ in self.layout.slots]
            bj = BlockJacobi.from_device_points(self.layout.n_unknowns, groups, MAX_NODES)
            geo = LearnedGeometry(self, bj, load_default())
            done = torch.cuda.Event()
            done.record(side)
        # made on the side stream, used and freed behind the current one
        for t in (bj._ptr, bj._dofs, bj._local, bj._chunk_of, bj.inv, *geo.tensors()):
            t.record_stream(main)
        self._pending_geometry = (bj, geo, done)

    def _build_mixed(self):
        from ..la.mixed import MixedOperator, near_blocks
        dev = require_cuda()
        n = self.layout.n_unknowns
        self._arrays = self._arrays_in if self._arrays_in is not None else {}
        counts = {}
        for t in self.system.terms:
            counts[(t.row.offset, t.col.offset)] = counts.get((t.row.offset, t.col.offset), 0) + 1
        if any(v > 1 for v in counts.values()):
            raise NotImplementedError("mixed precision: two terms on one block")
        covered = sum(t.row.size * t.col.size for t in self.system.terms)
        alloc = torch.empty if covered == n * n else torch.zeros
        A32 = _f32_matrix(n, n, dev, zero=covered != n * n)
        # the BF16 inner operator's copy, written by the same far-field pass
        A16 = (alloc((n, (n + 7) // 8 * 8), dtype=torch.bfloat16, device=dev)
               if self.precond in ("bf16_inner", "bf16_learned") else None)
        op = MixedOperator(A32, [], A16)
        placed = {}
        # FAULT_TRACTION rows are assembled in FP64 (their kernels have no FP32
        # quadrature here), transformed like the FP64 system's, then split
        # into FP32 / BF16 far entries and FP64 near blocks (_traction_rows)
        trac = {self.layout.slot(f, "b").offset: (region, f) for region, f in self.system.traction_faults()}
        for r0, (_, f) in trac.items():
            if f.order:
                raise NotImplementedError("mixed precision: FAULT_TRACTION rows of an order > 0 fault")
        terms = [t for t in self.system.terms if t.row.offset not in trac]
        trac_terms = [t for t in self.system.terms if t.row.offset in trac]
        # every far-field kernel is enqueued first; the assembly warnings (and,
        # for the learned preconditioner, its mesh-only setup) run on a side
        # stream while they work, then the near lists are read
        for s_ in self.layout.slots:
            self._patch_arrays(s_.patch)
        arrays_ready = torch.cuda.Event()
        arrays_ready.record()
        launched = []
        for t in terms:
            mat = self.materials[t.region.name]
            view = A32[t.row.offset:t.row.stop, t.col.offset:t.col.stop]
            view16 = None if A16 is None else A16[t.row.offset:t.row.stop, t.col.offset:t.col.stop]
            launched.append(self._mixed_launch(view, t.field_patch, t.source_patch, t.kernel, mat, t.scale,
                                               t.row.offset, t.col.offset, view16))
        self._warn_on_side_stream()
        self._pending_geometry = None
        if self.precond == "bf16_learned":
            self._learned_geometry_on_side_stream(arrays_ready)
        for t, fl in zip(terms, launched):
            nl = near_blocks(fl)
            op.near.append(nl)
            placed[(id(t.field_patch), id(t.source_patch), t.kernel, id(self.materials[t.region.name]))] = (t, nl)
        del launched

        temp = {}

        def block(q, p, kernel, region):
            mat = self.materials[region.name]
            key = (id(q), id(p), kernel, id(mat))
            if key in placed:
                t, nl = placed[key]
                return MixedOperator(A32[t.row.offset:t.row.stop, t.col.offset:t.col.stop], [
                    type(nl)(0, 0, nl.n_field, nl.rowptr, nl.cols, nl.vals)]), t.scale
            if key not in temp:
                far = _f32_matrix(3 * q.n_dofs, 3 * p.n_nodes, dev)
                nl = self._mixed_block(far, q, p, kernel, mat, 1.0, 0, 0)
                temp[key] = (MixedOperator(far, [nl]), 1.0)
            return temp[key]

        self.calib = None
        if self.jump == "calibrated":
            def rowsum(region, q, p):
                bop, scale = block(q, p, KERNEL_T, region)
                rs = bop.rowsum3(0, bop.A32.shape[0], 0, bop.A32.shape[1], bop.near[0])
                return rs if scale == 1.0 else rs * (1.0 / scale)
            self.calib = calibrated_diagonal(self.system, rowsum)
        missing = torch.zeros(1, dtype=torch.int32, device=dev)
        for t, nl in zip(terms, op.near):
            D = term_diagonal(t, self.calib)
            if D is None:
                continue
            Dd = (as_cuda(np.ascontiguousarray(D)) if not isinstance(D, torch.Tensor) else D.contiguous())
            shape = np.ascontiguousarray(t.field_patch.collocation_shape(), dtype=float)
            if shape.shape[0] == 1:
                nat.call("mbem_near_add_diagonal", ptr(nl.rowptr), ptr(nl.cols), ptr(nl.vals), nl.n_field,
                         ptr(Dd), ptr(missing), stream_handle())
            else:
                # the free term on the element's own nodes by the collocation shape
                nat.call("mbem_near_add_diagonal_nodal", ptr(nl.rowptr), ptr(nl.cols), ptr(nl.vals), nl.n_field,
                         ptr(Dd), shape.shape[0], nat.dbl_array(shape.ravel()), ptr(missing), stream_handle())
        if int(missing.item()) != 0:
            raise RuntimeError("mixed precision: a collocation row has no self block in its near list")
        b = torch.zeros(n, dtype=torch.float64, device=dev)
        for rt in self.system.rhs_terms:
            if rt.kernel in (KERNEL_HT, KERNEL_GT) and not np.any(np.asarray(rt.vector, float)):
                continue                        # a zero density adds nothing (e.g. a traction-free patch)
            dens = as_cuda(np.asarray(rt.vector, float))
            if rt.kernel in (KERNEL_HT, KERNEL_GT):
                tmp = torch.zeros((3 * rt.field_patch.n_dofs, 3 * rt.source_patch.n_nodes), dtype=torch.float64,
                                  device=dev)
                self._block_into(tmp, rt.field_patch, rt.source_patch, rt.kernel, self.materials[rt.region.name],
                                 1.0, True)
                b[rt.row.offset:rt.row.stop] += rt.scale * (tmp @ dens)
                del tmp
                continue
            bop, _ = block(rt.field_patch, rt.source_patch, rt.kernel, rt.region)
            y = bop.matvec(dens)
            b[rt.row.offset:rt.row.stop] += rt.scale * y
        for rv in self.system.rhs_values:
            b[rv.row.offset:rv.row.stop] += as_cuda(np.asarray(rv.vector, float))
        for rt in self.system.rhs_terms:
            if not rt.add_half_of_vector:
                continue
            u_c = as_cuda(rt.field_patch.collocation_values(rt.vector)).reshape(-1, 3)
            bview = b[rt.row.offset:rt.row.stop].view(-1, 3)
            if self.calib is None:
                bview += rt.scale_half * u_c
            else:
                bview -= torch.einsum("nij,nj->ni", self.calib[(id(rt.region), id(rt.field_patch))], u_c)
        for r0, (region, f) in trac.items():
            self._traction_rows(op, r0, region, f, [t for t in trac_terms if t.row.offset == r0], b)
        self._arrays = None
        self.op = op
        self.A = None
        self.b = b

    def _traction_rows(self, op, r0, region, f, trac_terms, b):
        """One FAULT_TRACTION fault's rows of the mixed operator: assembled in
        FP64 over every column, their free terms added, the fault-row
        transformation applied (``fault_rows_one``: frame, drag, constraint
        and locked rows, as the FP64 system gets them), then split by the
        mixed operator's near rule per source slot: near pairs as FP64 blocks
        in the near lists, the rest into the FP32 far field and its BF16 copy."""
        from ..la.mixed import NearList, near_list
        from .fault_rows import fault_rows_one
        n = self.layout.n_unknowns
        m = 3 * f.n_dofs
        dev = op.A32.device
        R = torch.zeros((m, n), dtype=torch.float64, device=dev)
        fa = self._patch_arrays(f)
        xf = fa["coll"]
        near = {}       # column slot offset -> its near list (rowptr, cols)
        for slot in self.layout.slots:
            if slot.size == 0:
                continue
            if slot.patch.order:
                raise NotImplementedError("mixed precision: FAULT_TRACTION rows over an order > 0 patch")
            sp = self._patch_arrays(slot.patch)
            near[slot.offset] = near_list(xf, sp["tv"], sp["eps"], self.near_factor)
        for t in trac_terms:
            mat = self.materials[t.region.name]
            if t.kernel == KERNEL_HT and t.source_patch.order == 0 and t.col.offset in near:
                # FP32 far quadrature + FP64 near pairs, straight into the FP64 rows
                sp = self._patch_arrays(t.source_patch)
                rowptr, cols = near[t.col.offset]
                blk = R[:, t.col.offset:t.col.stop]
                nat.call("mbem_traction_matrix_mixed", ptr(xf), ptr(fa["coll_n"]), xf.shape[0], ptr(sp["tv"]),
                         ptr(sp["normals"]), ptr(sp["eps"]), t.source_patch.n_triangles, float(mat.mu),
                         float(mat.lam), float(self.near_factor), float(t.scale), ptr(rowptr), ptr(cols),
                         int(cols.numel()), ptr(blk), R.stride(0), stream_handle())
            else:
                self._block_into(R[:, t.col.offset:t.col.stop], t.field_patch, t.source_patch, t.kernel, mat,
                                 t.scale, True)
            D = term_diagonal(t, self.calib)
            if D is not None:
                Dd = as_cuda(np.ascontiguousarray(D)) if not isinstance(D, torch.Tensor) else D.contiguous()
                shape = np.ascontiguousarray(t.field_patch.collocation_shape(), dtype=float)
                nat.call("mbem_add_block_diagonal", ptr(R[:, t.col.offset:]), R.stride(0), ptr(Dd),
                         t.field_patch.n_nodes, shape.shape[0], nat.dbl_array(shape.ravel()), stream_handle())
        fault_rows_one(R, b[r0:r0 + m], region, f, r0, self.fault_drag)
        A32 = op.A32[r0:r0 + m, :n]
        A32.copy_(R)
        A16 = None if op.A16 is None else op.A16[r0:r0 + m, :n]
        if A16 is not None:
            A16.copy_(R)
        three = torch.arange(3, device=dev)
        for slot in self.layout.slots:
            if slot.offset not in near:
                continue
            rowptr, cols = near[slot.offset]
            nnz = int(cols.numel())
            if nnz == 0:
                continue
            fidx = torch.repeat_interleave(torch.arange(xf.shape[0], device=dev), rowptr[1:] - rowptr[:-1])
            rr = (3 * fidx[:, None] + three)[:, :, None].expand(nnz, 3, 3)
            cc = (slot.offset + 3 * cols[:, None] + three)[:, None, :].expand(nnz, 3, 3)
            vals = R[rr, cc].reshape(nnz, 9).contiguous()
            A32[rr, cc] = 0.0
            if A16 is not None:
                A16[rr, cc] = 0.0
            op.near.append(NearList(r0, slot.offset, xf.shape[0], rowptr, cols, vals))
        del R

    def _build(self):
        if self.precision == "mixed":
            return self._build_mixed()
        dev = require_cuda()
        lay = self.layout
        n = lay.n_unknowns
        self._arrays = self._arrays_in if self._arrays_in is not None else {}
        placed = {}      # (id q, id p, kernel, id material) -> (view, scale)
        written = {}     # (row offset, col offset) -> count of terms
        for t in self.system.terms:
            written[(t.row.offset, t.col.offset)] = written.get((t.row.offset, t.col.offset), 0) + 1
        # blocks with one writer are written, not accumulated; when such
        # blocks tile all of A it needs no zero fill (55 GB at 83k unknowns)
        single = sum(t.row.size * t.col.size for t in self.system.terms
                     if written[(t.row.offset, t.col.offset)] == 1)
        A = (torch.empty if single == n * n else torch.zeros)((n, n), dtype=torch.float64, device=dev)
        b = torch.zeros(n, dtype=torch.float64, device=dev)
        for t in self.system.terms:
            mat = self.materials[t.region.name]
            view = A[t.row.offset:t.row.stop, t.col.offset:t.col.stop]
            one = written[(t.row.offset, t.col.offset)] == 1
            self._block_into(view, t.field_patch, t.source_patch, t.kernel, mat, t.scale, not one)
            if one:
                placed[(id(t.field_patch), id(t.source_patch), t.kernel, id(mat))] = (view, t.scale)

        temp_cache = {}

        def block(q, p, kernel, region):
            mat = self.materials[region.name]
            key = (id(q), id(p), kernel, id(mat))
            if key in placed:
                return placed[key]
            if key not in temp_cache:
                rows = 3 * q.n_dofs
                cols = 3 * p.n_nodes
                tmp = torch.empty((rows, cols), dtype=torch.float64, device=dev)
                self._block_into(tmp, q, p, kernel, mat, 1.0, False)
                temp_cache[key] = (tmp, 1.0)
            return temp_cache[key]

        self.calib = None
        if self.jump == "calibrated":
            def rowsum(region, q, p):
                view, scale = block(q, p, KERNEL_T, region)
                rs = self._rowsum(None, view)
                return rs if scale == 1.0 else rs * (1.0 / scale)
            self.calib = calibrated_diagonal(self.system, rowsum)

        for t in self.system.terms:
            D = term_diagonal(t, self.calib)
            if D is None:
                continue
            Dd = as_cuda(D) if not isinstance(D, torch.Tensor) else D.contiguous()
            shape = np.ascontiguousarray(t.field_patch.collocation_shape(), dtype=float)
            K = shape.shape[0]
            nat.call("mbem_add_block_diagonal", ptr(A[t.row.offset:, t.col.offset:]), A.stride(0),
                     ptr(Dd), t.field_patch.n_nodes, K, nat.dbl_array(shape.ravel()), stream_handle())

        for rt in self.system.rhs_terms:
            if rt.kernel in (KERNEL_HT, KERNEL_GT) and not np.any(np.asarray(rt.vector, float)):
                continue                        # a zero density adds nothing (e.g. a traction-free patch)
            mat = self.materials[rt.region.name]
            bview = b[rt.row.offset:rt.row.stop].view(-1, 3)
            f = self._patch_arrays(rt.field_patch)
            s = self._patch_arrays(rt.source_patch)
            dens = as_cuda(np.asarray(rt.vector, float).reshape(-1, 3))
            order = rt.source_patch.order
            key = (id(rt.field_patch), id(rt.source_patch), rt.kernel, id(mat))
            if key in temp_cache or rt.kernel in (KERNEL_HT, KERNEL_GT):
                view, _ = block(rt.field_patch, rt.source_patch, rt.kernel, rt.region)
                nat.call("mbem_dgemv", ptr(view), view.stride(0), view.shape[0], view.shape[1], ptr(dens),
                         float(rt.scale), 1.0, ptr(bview), stream_handle())
            elif rt.kernel == KERNEL_T:
                c = kb.t_coeffs(mat.mu, mat.lam)
                tn.t_disp_contract(f["coll"], s["tv"], s["normals"], s["eps"], dens, *c, order,
                                   out=bview, alpha=rt.scale, accumulate=True)
            else:
                g = kb.u_coeffs(mat.mu, mat.lam)
                tn.u_disp_contract(f["coll"], s["tv"], s["eps"], dens, *g, order, out=bview,
                                   alpha=rt.scale, accumulate=True)
        for rv in self.system.rhs_values:
            b[rv.row.offset:rv.row.stop] += as_cuda(np.asarray(rv.vector, float))
        # prescribed-displacement rows: the free term moves to the RHS
        for rt in self.system.rhs_terms:
            if not rt.add_half_of_vector:
                continue
            u_c = as_cuda(rt.field_patch.collocation_values(rt.vector)).reshape(-1, 3)
            bview = b[rt.row.offset:rt.row.stop].view(-1, 3)
            if self.calib is None:
                bview += rt.scale_half * u_c
            else:
                C = self.calib[(id(rt.region), id(rt.field_patch))]
                bview -= torch.einsum("nij,nj->ni", C, u_c)
        if self.system.traction_faults():
            from .fault_rows import apply_fault_rows
            apply_fault_rows(A, b, self.system, self.fault_drag)
        self._arrays = None
        self.A = A
        self.b = b

    # -- solve -----------------------------------------------------------
    def u_ranges(self):
        if not self.deflate:
            return []
        return [(s.offset, s.size) for s in self.layout.slots if s.kind == "u"]

    def block_jacobi(self, max_nodes: int | None = None):
        """The cluster block-Jacobi preconditioner of this system (built once);
        the chunks are made on the device from the device mesh arrays
        (``BlockJacobi.from_device_points``)."""
        from ..la.precond import MAX_NODES, BlockJacobi
        pend = getattr(self, "_pending_geometry", None)
        if self._bj is None and pend is not None and max_nodes in (None, MAX_NODES) and self.op is not None:
            bj, _, done = pend
            torch.cuda.current_stream().wait_event(done)
            self._bj_nodes = MAX_NODES
            self._bj = bj.build_mixed(self.op)
        if self._bj is None or (max_nodes is not None and max_nodes != self._bj_nodes):
            self._bj_nodes = MAX_NODES if max_nodes is None else max_nodes
            groups = [(s.offset, self.device_patch_arrays(s.patch)["coll"].view(-1, 3)) for s in self.layout.slots]
            bj = BlockJacobi.from_device_points(self.layout.n_unknowns, groups, self._bj_nodes)
            self._bj = bj.build_mixed(self.op) if self.op is not None else bj.build_dense(self.A)
        return self._bj

    def device_patch_arrays(self, patch) -> dict:
        """The device mesh arrays of one patch (tv, normals, eps, coll,
        coll_n): the caller's ``arrays`` dict when one was given, else made
        once and kept with this assembly."""
        saved = self._arrays
        if saved is None:
            if self._arrays_in is None:
                self._arrays_in = {}
            self._arrays = self._arrays_in
        try:
            return self._patch_arrays(patch)
        finally:
            self._arrays = saved

    def bf16_inner(self, iterations: int | None = None, rtol: float | None = None):
        """The BF16 inner-solve preconditioner of the mixed operator (the
        BF16 copy of the far field is made once)."""
        from ..la.mixed import Bf16Inner
        if self.op is None:
            raise ValueError("the BF16 inner solve needs the mixed-precision operator")
        it = defaults.MIXED_INNER_ITERATIONS if iterations is None else iterations
        tol = defaults.MIXED_INNER_RTOL if rtol is None else rtol
        if self._inner is None:
            self._inner = Bf16Inner(self.op, it, self.u_ranges(), tol)
        self._inner.set_iterations(it)
        if not 0.0 <= tol < 1.0:
            raise ValueError(f"rtol must be in [0, 1) (got {tol})")
        self._inner.rtol = float(tol)
        return self._inner

    def bf16_learned(self, params=None):
        """The BF16 inner solve with the learned two-level preconditioner of
        its operator as right preconditioner (set up once per assembly)."""
        from ..la.learned import LearnedPreconditioner
        from ..la.train_learned import load_default
        inner = self.bf16_inner()
        if getattr(self, "_learned", None) is None or params is not None:
            pend = getattr(self, "_pending_geometry", None)
            if params is None and pend is not None:
                bj = self.block_jacobi()
                geo = pend[1] if bj is pend[0] else None
                self._learned = LearnedPreconditioner(self, load_default(), bj=bj, geometry=geo)
            else:
                self._learned = LearnedPreconditioner(self, load_default() if params is None else params)
        inner.set_preconditioner(self._learned)
        return inner

    def rebuild_for_materials(self, material_map: dict, fault_drag: dict | None = None) -> "AssembledDense":
        """A new AssembledDense of the same model with updated region
        materials (dense.py:650-688): ``material_map`` maps region name ->
        material; ``fault_drag`` replaces the faults' drag (``{}`` removes
        it), ``None`` keeps this one's. The geometry arrays of this assembly
        are reused; the blocks are re-assembled (direct mode)."""
        new = AssembledDense.__new__(AssembledDense)
        new.__dict__.update(self.__dict__)
        new.materials = dict(self.materials)
        for name, mat in material_map.items():
            if name not in new.materials:
                raise KeyError(f"unknown region '{name}'")
            new.materials[name] = mat
        new.fault_drag = self.fault_drag if fault_drag is None else _checked_drag(self.system, fault_drag)
        new.report = None
        new.A = new.b = new.op = new._x = None
        new._bj = new._inner = new._factor = new._learned = None
        new.calib = None
        new._build()
        return new

    def condense(self, refine: bool = True):
        """Every unknown but the FAULT_TRACTION faults' slip eliminated
        (dense.py:580-646): a ``backends.condense.Condensed``."""
        from .condense import condense
        return condense(self, refine)

    def factor(self):
        """The FP32 GPU LU of this operator (the bordered one [[A, Z], [Z^T, 0]]
        with deflation, backends/dense.py:538-566), refined against the FP64
        operator; built once."""
        from ..la.lu import Factor
        if self._factor is not None:
            return self._factor
        if self.A is None:
            raise ValueError("lu= needs the FP64 operator (precision='fp64')")
        A = self.A
        n = A.shape[0]
        Z = translation_basis(self.layout) if self.deflate else np.zeros((n, 0))
        m = Z.shape[1]
        if m == 0:
            self._factor = Factor(A)
            return self._factor
        Zd = as_cuda(np.ascontiguousarray(Z))
        B32 = torch.zeros((n + m, n + m), dtype=torch.float32, device=A.device)
        B32[:n, :n] = A
        B32[:n, n:] = Zd
        B32[n:, :n] = Zd.T

        def bordered(x):
            y = torch.empty_like(x)
            nat.call("mbem_dgemv", ptr(A), A.stride(0), n, n, ptr(x), 1.0, 0.0, ptr(y), stream_handle())
            y[:n] += Zd @ x[n:]
            y[n:] = Zd.T @ x[:n]
            return y
        self._factor = Factor(None, bordered, lu32=B32)
        return self._factor

    def _solve_lu(self) -> torch.Tensor:
        f = self.factor()
        n = self.A.shape[0]
        rhs = torch.zeros(f.n, dtype=torch.float64, device=self.A.device)
        rhs[:n] = self.b
        x = f.solve(rhs)[:n].contiguous()
        # the deflated true residual |P (b - A x)| / |P b|, as FGMRES reports it
        r = self.b - self.A @ x
        pb = self.b.clone()
        for off, size in self.u_ranges():
            r[off:off + size].view(-1, 3).sub_(r[off:off + size].view(-1, 3).mean(dim=0))
            pb[off:off + size].view(-1, 3).sub_(pb[off:off + size].view(-1, 3).mean(dim=0))
        rel = float(r.norm() / pb.norm()) if float(pb.norm()) > 0 else 0.0
        cond = f.cond()
        self.report = DenseSolveReport(converged=rel < max(self.rtol, 1e-12), iterations=int(f.report["passes"]),
                                       true_relres=rel, arnoldi_relres=float(f.report["left"]), cond_estimate=cond,
                                       lu=dict(f.report))
        warn_condition(cond)
        self._x = x
        return x

    def solve_device(self, rtol: float | None = None, restart: int | None = None,
                     maxiter: int | None = None, x0=None, time_matvec: bool = False,
                     precond=None) -> torch.Tensor:
        """FGMRES on the device; returns the solution vector as a CUDA tensor
        and leaves ``self.report``. ``precond``: None (the backend's
        default), "none", "block_jacobi", or a preconditioner object
        (``la.precond.BlockJacobi``, ``la.learned.LearnedPreconditioner``)."""
        if self.lu is not None and precond is None:
            return self._solve_lu()
        precond = self.precond if precond is None else precond
        if precond == "none":
            precond = None
        elif precond == "block_jacobi":
            precond = self.block_jacobi()
        elif precond == "bf16_inner":
            precond = self.bf16_inner()
            precond.set_preconditioner(None)
        elif precond == "bf16_learned":
            precond = self.bf16_learned()
        kw = dict(x0=x0, rtol=self.rtol if rtol is None else rtol,
                  restart=self.restart if restart is None else restart,
                  maxiter=self.maxiter if maxiter is None else maxiter, u_ranges=self.u_ranges(),
                  time_matvec=time_matvec, precond=precond)
        if self.op is not None:
            x, rep = fgmres_mixed(self.op, self.b, **kw)
        else:
            x, rep = fgmres_dense(self.A, self.b, **kw)
        self.report = rep
        if not rep.converged:
            warnings.warn(f"dense GPU solve: {rep}")
        self._x = x
        return x

    def solve(self, rtol: float | None = None, restart: int | None = None,
              maxiter: int | None = None, x0=None, precond=None) -> dict:
        """FGMRES on the device; returns {slot_name: (n, 3) ndarray} and
        leaves ``self.report`` (a SolveReport)."""
        xh = self.solve_device(rtol, restart, maxiter, x0, precond=precond).cpu().numpy()
        return {s.name: xh[s.offset:s.stop].reshape(-1, 3) for s in self.layout.slots}

    @property
    def x(self) -> torch.Tensor | None:
        return self._x

    def release(self):
        self.A = None
        torch.cuda.empty_cache()
