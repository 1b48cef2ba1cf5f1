"""Region-model API of the dense hot path: ``BCType``, ``Patch``, ``Region``,
``RegionModel`` and the one fault sign convention.

Same names, fields and semantics as the reference's
``src/mbem/model/core.py`` (BCType :72-77, FAULT_ORIENTATION :100, Patch
:103-497, Region :500-513, RegionModel :702-1107) for what the dense backend
and the stress readout consume: boundary patches that are FREE_TRACTION,
PRESCRIBED_DISPLACEMENT or INTERFACE (order 0/1/2, discontinuous layout),
and faults that are FAULT (prescribed slip, order 0/1/2) or FAULT_TRACTION
(solved slip, order 0). Gravity, far-field walls, interfaces that slip and
continuous (shared-node) layouts are outside this hot path and are refused.

Orientation sigma(R, p) = +1 iff p's stored normals point out of R, inferred
from the signed solid angle of p seen from the region's probe point, as the
reference does; faults answer FAULT_ORIENTATION.
"""

from __future__ import annotations

import enum
from dataclasses import dataclass, field

import numpy as np

from .. import defaults
from ..kernels.basis import lagrange_nodes, lagrange_shape
from ..kernels.tri_nodal import n_nodes


class BCType(enum.Enum):
    FREE_TRACTION = "free_traction"
    PRESCRIBED_DISPLACEMENT = "prescribed_displacement"
    INTERFACE = "interface"
    FAULT = "fault"
    FAULT_TRACTION = "fault_traction"


FAULT_KINDS = (BCType.FAULT, BCType.FAULT_TRACTION)

# A fault is interior to its region, so its sigma is a convention: with -1
# the coefficient -sigma is +1 on the fault source and the value is the
# Burgers vector b = u(+n side) - u(-n side), n the stored normal.
FAULT_ORIENTATION = -1


@dataclass(eq=False)
class Patch:
    """A named triangulated boundary piece with a boundary condition.

    ``value``: traction (FREE_TRACTION), displacement (PRESCRIBED_DISPLACEMENT),
    slip b (FAULT) or the prescribed traction change (FAULT_TRACTION); a (3,)
    constant, an (N_tri, 3) per-element array, an (n_dofs, 3) nodal array or
    a callable of the dof nodes; None means zeros.
    """
    name: str
    mesh: object
    bc: BCType
    value: object = None
    order: int = 0
    layout: str = "discontinuous"
    allow_opening: bool = False
    locked: object = None
    slip: object = None

    def __post_init__(self):
        if self.order != int(self.order):
            raise ValueError(f"patch '{self.name}': order must be an integer 0, 1 or 2 "
                             f"(got {self.order!r})")
        self.order = int(self.order)
        n_nodes(self.order)
        if self.layout != "discontinuous":
            raise NotImplementedError(f"patch '{self.name}': only the discontinuous layout is on "
                                      f"the GPU dense path")
        if self.slip is not None:
            raise NotImplementedError(f"patch '{self.name}': interfaces that slip are not on the "
                                      f"GPU dense path")
        if self.bc is BCType.FAULT_TRACTION and self.order != 0:
            raise ValueError(f"patch '{self.name}': a discontinuous FAULT_TRACTION fault is "
                             f"order 0 (got order {self.order})")
        if self.bc is not BCType.FAULT_TRACTION and (self.allow_opening or self.locked is not None):
            raise ValueError(f"patch '{self.name}': allow_opening and locked apply to a "
                             f"FAULT_TRACTION fault only")
        self._refuse_degenerate()

    def _refuse_degenerate(self) -> None:
        tv = np.asarray(self.mesh.vertices, float)[np.asarray(self.mesh.triangles)]
        edges = tv[:, [1, 2, 0], :] - tv
        L = np.linalg.norm(edges, axis=2).max(axis=1)
        two_area = np.linalg.norm(np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]), axis=1)
        h_over_L = two_area / np.where(L > 0.0, L, 1.0) ** 2
        bad = np.nonzero(h_over_L <= defaults.MIN_TRIANGLE_HEIGHT_OVER_L)[0]
        if bad.size:
            worst = int(bad[np.argmin(h_over_L[bad])])
            raise ValueError(f"patch '{self.name}': {bad.size} of {tv.shape[0]} elements are "
                             f"degenerate (height / longest edge at or below "
                             f"{defaults.MIN_TRIANGLE_HEIGHT_OVER_L:g}; worst "
                             f"{h_over_L[worst]:.1e} at element {worst})")

    # ---- sizes and node tables ----
    @property
    def n_triangles(self) -> int:
        return self.mesh.n_triangles

    @property
    def n_nodes(self) -> int:
        return n_nodes(self.order) * self.mesh.n_triangles

    @property
    def n_dofs(self) -> int:
        return self.n_nodes

    @property
    def continuous(self) -> bool:
        return False

    @property
    def solves_slip(self) -> bool:
        return self.bc is BCType.FAULT_TRACTION

    def column_ids(self):
        return None

    def expand(self, values) -> np.ndarray:
        v = np.asarray(values, float)
        if v.shape != (self.n_nodes, 3):
            raise ValueError(f"patch '{self.name}': values must be ({self.n_nodes}, 3), got {v.shape}")
        return np.ascontiguousarray(v)

    def tri_verts(self) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(self.mesh.vertices, float)[np.asarray(self.mesh.triangles)])

    def _points(self, lam) -> np.ndarray:
        return np.einsum("kv,svc->skc", lam, self.tri_verts()).reshape(-1, 3)

    def nodes(self) -> np.ndarray:
        if self.order == 0:
            return np.asarray(self.mesh.centroids(), float)
        return self._points(lagrange_nodes(self.order))

    def collocation_points(self) -> np.ndarray:
        t = defaults.COLLOCATION_SHRINK_BY_ORDER[self.order]
        if t == 0.0:
            return self.nodes()
        return self._points(lagrange_nodes(self.order, t))

    def collocation_normals(self) -> np.ndarray:
        normals, _ = self.mesh.normals_and_areas()
        return np.ascontiguousarray(np.repeat(np.asarray(normals, float), n_nodes(self.order), axis=0))

    def collocation_shape(self) -> np.ndarray:
        t = defaults.COLLOCATION_SHRINK_BY_ORDER[self.order]
        return lagrange_shape(self.order, lagrange_nodes(self.order, t))

    def value_array(self) -> np.ndarray:
        """The prescribed datum at the dof nodes (n_dofs, 3)."""
        K = n_nodes(self.order)
        if self.value is None:
            v = np.zeros((self.n_nodes, 3))
        elif callable(self.value):
            normals, _ = self.mesh.normals_and_areas()
            try:
                v = self.value(self.nodes(), np.repeat(normals, K, axis=0))
            except TypeError:
                v = self.value(self.nodes())
            v = np.asarray(v, dtype=float)
            if v.shape != (self.n_nodes, 3):
                raise ValueError(f"patch '{self.name}': callable value returned {v.shape}, "
                                 f"expected {(self.n_nodes, 3)}")
        else:
            v = np.asarray(self.value, dtype=float)
            if not (K > 1 and v.shape == (self.n_nodes, 3)):
                v = np.broadcast_to(v, (self.n_triangles, 3))
                if K > 1:
                    v = np.repeat(v, K, axis=0)
        v = np.ascontiguousarray(v)
        if self.bc is BCType.FAULT_TRACTION and not self.allow_opening:
            scale = float(np.max(np.abs(v))) if v.size else 0.0
            if scale:
                nn = np.abs(np.einsum("ij,ij->i", v, self.collocation_normals())).max()
                if nn > defaults.TRACTION_VALUE_NORMAL_TOL * scale:
                    raise ValueError(f"fault '{self.name}': the traction value has a normal "
                                     f"component ({nn:.2e} against |value| {scale:.2e}) but "
                                     f"allow_opening=False enforces the tangential components only")
        return v

    def density(self) -> np.ndarray:
        if self.bc is BCType.FAULT_TRACTION:
            raise ValueError(f"fault '{self.name}' is a FAULT_TRACTION fault: its slip is solved, "
                             f"not prescribed -- read solution['b:{self.name}']")
        return self.expand(self.value_array())

    def collocation_values(self, nodal) -> np.ndarray:
        K = n_nodes(self.order)
        v = np.asarray(nodal, float).reshape(self.n_triangles, K, 3)
        return np.einsum("ck,skj->scj", self.collocation_shape(), v).reshape(-1, 3)

    def locked_mask(self, patches=()) -> np.ndarray:
        if not self.solves_slip:
            raise ValueError(f"patch '{self.name}': locked nodes are a notion of a solved slip")
        n = self.n_dofs
        if self.locked is None:
            return np.zeros(n, bool)
        if callable(self.locked):
            m = np.asarray(self.locked(self.collocation_points()), bool).reshape(-1)
        else:
            m = np.asarray(self.locked, bool).reshape(-1)
        if m.shape != (n,):
            raise ValueError(f"patch '{self.name}': locked mask must have {n} entries, got {m.shape}")
        return m


@dataclass(eq=False)
class Region:
    name: str
    material: object
    patches: list
    probe_point: np.ndarray
    faults: list = field(default_factory=list)
    orientation_overrides: dict = field(default_factory=dict)

    @property
    def is_full_space(self) -> bool:
        return len(self.patches) == 0


def solid_angle_sum(mesh, x) -> float:
    """Sum over the triangles of the van Oosterom signed solid angle seen from x."""
    tv = np.asarray(mesh.vertices, float)[np.asarray(mesh.triangles)] - np.asarray(x, float)
    r1, r2, r3 = tv[:, 0], tv[:, 1], tv[:, 2]
    R1, R2, R3 = (np.linalg.norm(r, axis=1) for r in (r1, r2, r3))
    numer = np.einsum("ij,ij->i", r1, np.cross(r2, r3))
    denom = (R1 * R2 * R3 + R3 * np.einsum("ij,ij->i", r1, r2) + R1 * np.einsum("ij,ij->i", r2, r3)
             + R2 * np.einsum("ij,ij->i", r1, r3))
    return float(np.sum(2.0 * np.arctan2(numer, denom)))


_CLOSED_THRESHOLD = 2.0 * np.pi
_OPEN_FLOOR = 1e-3
_CLOSURE_TOL = 1e-6
# a point this close to a patch, in units of the nearest element's mean
# edge, lies ON it (core.py:89)
_ON_PATCH_TOL = 1e-9


class RegionModel:
    def __init__(self, regions: list, gravity=None, far_field=None):
        if gravity is not None or far_field is not None:
            raise NotImplementedError("gravity and far-field walls are not on the GPU dense path")
        self.regions = regions
        self.gravity = None
        self.far_field = None
        self._sigma: dict = {}
        self.validate()

    def _infer_sigma(self, region: Region, patch: Patch) -> int:
        if patch.name in region.orientation_overrides:
            return int(region.orientation_overrides[patch.name])
        omega = solid_angle_sum(patch.mesh, region.probe_point)
        if abs(omega) > _CLOSED_THRESHOLD or abs(omega) > _OPEN_FLOOR:
            return 1 if omega > 0 else -1
        omega_in = solid_angle_sum(patch.mesh, np.asarray(patch.mesh.vertices).mean(axis=0))
        if abs(omega_in) < _CLOSED_THRESHOLD:
            raise ValueError(f"cannot infer orientation of patch '{patch.name}' for region "
                             f"'{region.name}'; supply orientation_overrides")
        return -1 if omega_in > 0 else 1

    def orientation(self, region: Region, patch: Patch) -> int:
        """sigma(region, patch): inferred for boundary patches,
        FAULT_ORIENTATION for faults."""
        if patch.bc in FAULT_KINDS:
            if not any(f is patch for f in region.faults):
                raise ValueError(f"patch '{patch.name}' is a {patch.bc.name} but is not a fault of "
                                 f"region '{region.name}'")
            return FAULT_ORIENTATION
        return self._sigma[(region.name, patch.name)]

    def validate(self) -> None:
        names = [r.name for r in self.regions]
        if len(set(names)) != len(names):
            raise ValueError("region names must be unique")
        incidence: dict = {}
        for r in self.regions:
            if r.is_full_space and not r.faults:
                raise ValueError(f"region '{r.name}' has neither boundary patches nor faults")
            for p in r.patches:
                if p.bc in FAULT_KINDS:
                    raise ValueError(f"patch '{p.name}' is a fault; list it in Region.faults")
                incidence.setdefault(id(p), []).append(r)
            for f in r.faults:
                if f.bc not in FAULT_KINDS:
                    raise ValueError(f"fault '{f.name}' must be FAULT or FAULT_TRACTION")
        for r in self.regions:
            total = 0.0
            for p in r.patches:
                s = self._infer_sigma(r, p)
                self._sigma[(r.name, p.name)] = s
                total += s * solid_angle_sum(p.mesh, r.probe_point)
            if r.patches and abs(total - 4.0 * np.pi) > 1e-3 * 4.0 * np.pi:
                raise ValueError(f"region '{r.name}': boundary does not close around its probe "
                                 f"point (sum sigma Omega = {total:.6f}, expected 4 pi)")
        for pid, regs in incidence.items():
            p = next(q for r in regs for q in r.patches if id(q) == pid)
            if p.bc is BCType.INTERFACE:
                if len(regs) != 2:
                    raise ValueError(f"interface '{p.name}' must bound exactly two regions")
                if self._sigma[(regs[0].name, p.name)] != -self._sigma[(regs[1].name, p.name)]:
                    raise ValueError(f"interface '{p.name}' gets the same sign from both regions")
            elif len(regs) != 1:
                raise ValueError(f"patch '{p.name}' ({p.bc.name}) is shared by {len(regs)} regions")

    def value_of(self, patch: Patch) -> np.ndarray:
        return patch.value_array()

    def far_field_patches(self) -> list:
        return []

    def buoyancy(self, region, patch):
        return None

    def point_in_region(self, region, points, closure: bool = False):
        """Which of ``points`` lie strictly inside ``region``: ``(N,) bool``
        (core.py:994-1025). The Gauss closure identity read as a classifier,
        sum_p sigma(R, p) Omega_p(x) = 4 pi iff x is inside R, within
        _CLOSURE_TOL x 4 pi; the solid angles are summed on the GPU.
        ``closure=True`` also returns the sum. A full-space region holds every
        point. Numpy in, numpy out; torch in, CUDA tensors out."""
        import torch

        from .._device import as_cuda, is_torch, out_like
        from ..geometry import MeshGeometry

        region = region if not isinstance(region, str) else next(r for r in self.regions if r.name == region)
        torch_in = is_torch(points)
        pts = as_cuda(points).reshape(-1, 3)
        if region.is_full_space:
            total = torch.full((pts.shape[0],), 4.0 * np.pi, dtype=torch.float64, device=pts.device)
        else:
            total = torch.zeros(pts.shape[0], dtype=torch.float64, device=pts.device)
            for p in region.patches:
                MeshGeometry(p.mesh).solid_angle(pts, float(self._sigma[(region.name, p.name)]), out=total,
                                                 accumulate=True)
        inside = (total - 4.0 * np.pi).abs() <= _CLOSURE_TOL * 4.0 * np.pi
        if closure:
            return out_like(inside, torch_in), out_like(total, torch_in)
        return out_like(inside, torch_in)

    def is_anchored(self) -> bool:
        return any(p.bc is BCType.PRESCRIBED_DISPLACEMENT for r in self.regions for p in r.patches)

    def interface_regions(self, patch: Patch) -> list:
        return [r for r in self.regions if any(q is patch for q in r.patches)]

    def solved_faults(self) -> list:
        return [(r, f) for r in self.regions for f in r.faults if f.bc is BCType.FAULT_TRACTION]

    def with_materials(self, material_map: dict) -> "RegionModel":
        from dataclasses import replace
        new = RegionModel.__new__(RegionModel)
        new.regions = [replace(r, material=material_map.get(r.name, r.material)) for r in self.regions]
        new.gravity = None
        new.far_field = None
        new._sigma = self._sigma
        return new
