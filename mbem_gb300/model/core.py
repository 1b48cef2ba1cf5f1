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
from ..mesh import centroids_of, normals_and_areas_of


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
        """Collapsed elements are a mesher failure (core.py:227-254): their
        height over longest edge, 2 area / L_max^2, must exceed
        MIN_TRIANGLE_HEIGHT_OVER_L, or the kernels have no frame to integrate
        over and "auto" eps no size."""
        v = np.asarray(self.mesh.vertices, float)
        t = np.asarray(self.mesh.triangles)
        p0, p1, p2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
        e0, e1, e2 = p1 - p0, p2 - p1, p0 - p2
        longest2 = np.maximum(np.maximum(np.einsum("ij,ij->i", e0, e0), np.einsum("ij,ij->i", e1, e1)),
                              np.einsum("ij,ij->i", e2, e2))
        # |e0 x (p2 - p0)| = twice the area
        f = p2 - p0
        cx = e0[:, 1] * f[:, 2] - e0[:, 2] * f[:, 1]
        cy = e0[:, 2] * f[:, 0] - e0[:, 0] * f[:, 2]
        cz = e0[:, 0] * f[:, 1] - e0[:, 1] * f[:, 0]
        twice_area = np.sqrt(cx * cx + cy * cy + cz * cz)
        quality = twice_area / np.where(longest2 > 0.0, longest2, 1.0)
        limit = defaults.MIN_TRIANGLE_HEIGHT_OVER_L
        flat = np.flatnonzero(quality <= limit)
        if flat.size:
            k = int(flat[quality[flat].argmin()])
            raise ValueError(f"patch '{self.name}' has {flat.size} degenerate element(s) among {quality.size}: "
                             f"height over longest edge must exceed {limit:g}, element {k} has {quality[k]:.1e}")

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

    def _points(self, lam, tv=None) -> np.ndarray:
        tv = self.tri_verts() if tv is None else tv
        return np.einsum("kv,svc->skc", lam, tv).reshape(-1, 3)

    def nodes(self, tv=None) -> np.ndarray:
        if self.order == 0:
            return centroids_of(self.tri_verts() if tv is None else tv)
        return self._points(lagrange_nodes(self.order), tv)

    def collocation_points(self, tv=None) -> np.ndarray:
        t = defaults.COLLOCATION_SHRINK_BY_ORDER[self.order]
        if t == 0.0:
            return self.nodes(tv)
        return self._points(lagrange_nodes(self.order, t), tv)

    def collocation_normals(self, normals=None) -> np.ndarray:
        if normals is None:
            normals, _ = self.mesh.normals_and_areas()
        return np.ascontiguousarray(np.repeat(np.asarray(normals, float), n_nodes(self.order), axis=0))

    def geometry(self):
        """(corners (n, 3, 3), unit normals (n, 3), collocation points,
        collocation normals) from one gather of the corners."""
        tv = self.tri_verts()
        normals, _ = normals_and_areas_of(tv)
        return tv, normals, self.collocation_points(tv), self.collocation_normals(normals)

    def collocation_shape(self) -> np.ndarray:
        t = defaults.COLLOCATION_SHRINK_BY_ORDER[self.order]
        return lagrange_shape(self.order, lagrange_nodes(self.order, t))

    def value_array(self) -> np.ndarray:
        """The prescribed datum at the dof nodes (n_dofs, 3) (core.py:355-419):
        None is zero; a callable is asked at the nodes (with their normals
        when it takes them); an array is one vector for the patch, one per
        element (repeated over its nodes) or, at order 1/2, one per node."""
        v = self._node_values()
        if self.bc is BCType.FAULT_TRACTION and not self.allow_opening:
            self._check_tangential(v)
        return v

    def _node_values(self) -> np.ndarray:
        K = n_nodes(self.order)
        want = (self.n_nodes, 3)
        if self.value is None:
            return np.zeros(want)
        if callable(self.value):
            normals = np.repeat(self.mesh.normals_and_areas()[0], K, axis=0)
            try:
                got = self.value(self.nodes(), normals)
            except TypeError:                 # a callable of the points alone
                got = self.value(self.nodes())
            got = np.asarray(got, dtype=float)
            if got.shape != want:
                raise ValueError(f"patch '{self.name}': its value callable gave an array of shape {got.shape}; "
                                 f"one vector per dof node, {want}, is needed")
            return np.ascontiguousarray(got)
        given = np.asarray(self.value, dtype=float)
        if K > 1 and given.shape == want:
            return np.ascontiguousarray(given)
        per_element = np.broadcast_to(given, (self.n_triangles, 3))
        return np.ascontiguousarray(np.repeat(per_element, K, axis=0))

    def _check_tangential(self, v: np.ndarray) -> None:
        """Without allow_opening only strike and dip are enforced, so a
        traction value with a normal part would be dropped unseen: refused."""
        size = float(np.abs(v).max()) if v.size else 0.0
        if size == 0.0:
            return
        normal_part = float(np.abs((v * self.collocation_normals()).sum(axis=1)).max())
        if normal_part > defaults.TRACTION_VALUE_NORMAL_TOL * size:
            raise ValueError(f"fault '{self.name}': allow_opening=False enforces only the tangential traction, "
                             f"but the value has a normal part {normal_part:.2e} (largest entry {size:.2e}); "
                             f"remove it or set allow_opening=True")

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
    rel = np.asarray(mesh.vertices, float) - np.asarray(x, float)
    R = np.sqrt(np.einsum("ij,ij->i", rel, rel))
    # the triple product per vertex-relative vector, by its cofactors
    t = np.asarray(mesh.triangles)
    a, b, c = t[:, 0], t[:, 1], t[:, 2]
    r1, r2, r3 = rel[a], rel[b], rel[c]
    R1, R2, R3 = R[a], R[b], R[c]
    numer = (r1[:, 0] * (r2[:, 1] * r3[:, 2] - r2[:, 2] * r3[:, 1])
             + r1[:, 1] * (r2[:, 2] * r3[:, 0] - r2[:, 0] * r3[:, 2])
             + r1[:, 2] * (r2[:, 0] * r3[:, 1] - r2[:, 1] * r3[:, 0]))
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

    def _infer_sigma(self, region: Region, patch: Patch, seen: float | None = None) -> int:
        """The sign rule (core.py:713-729): +1 when the patch is seen from
        the region's probe point with a positive solid angle (outward
        normals), -1 when negative. A closed patch that does not enclose the
        probe bounds a cavity: its sign is the opposite of the solid angle it
        subtends at its own vertex centroid. An override wins. ``seen`` is
        the patch's solid angle at the probe point when already summed."""
        if patch.name in region.orientation_overrides:
            return int(region.orientation_overrides[patch.name])
        if seen is None:
            seen = solid_angle_sum(patch.mesh, region.probe_point)
        if abs(seen) > _OPEN_FLOOR:
            return int(np.sign(seen))
        from_inside = solid_angle_sum(patch.mesh, np.asarray(patch.mesh.vertices, float).mean(axis=0))
        if abs(from_inside) >= _CLOSED_THRESHOLD:
            return -int(np.sign(from_inside))
        raise ValueError(f"patch '{patch.name}' of region '{region.name}': its orientation cannot be inferred "
                         f"({seen:.3e} sr from the probe point, and it does not enclose its own vertex centroid); "
                         f"give it in orientation_overrides")

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
        """The model's consistency (core.py:751-820): unique region names,
        faults only in Region.faults, every region with something to solve,
        each boundary patch in one region and each interface in two with
        opposite signs, and every bounded region closed around its probe."""
        if len({r.name for r in self.regions}) != len(self.regions):
            raise ValueError("two regions share a name; region names must be unique")
        owners: dict = {}
        for r in self.regions:
            if r.is_full_space and not r.faults:
                raise ValueError(f"region '{r.name}' has no boundary patch and no fault: nothing to solve")
            for p in r.patches:
                if p.bc in FAULT_KINDS:
                    raise ValueError(f"'{p.name}' is a fault ({p.bc.name}): list it in Region.faults")
                owners.setdefault(id(p), (p, []))[1].append(r)
            for f in r.faults:
                if f.bc not in FAULT_KINDS:
                    raise ValueError(f"'{f.name}' is listed as a fault of '{r.name}' but is {f.bc.name}")
        for r in self.regions:
            if r.is_full_space:
                continue
            closure = 0.0
            for p in r.patches:
                seen = solid_angle_sum(p.mesh, r.probe_point)
                self._sigma[(r.name, p.name)] = self._infer_sigma(r, p, seen)
                closure += self._sigma[(r.name, p.name)] * seen
            if abs(closure / (4.0 * np.pi) - 1.0) > 1e-3:
                raise ValueError(f"region '{r.name}' is not closed around its probe point: the signed solid "
                                 f"angles sum to {closure:.6f} sr, not 4 pi")
        for p, regs in owners.values():
            if p.bc is not BCType.INTERFACE:
                if len(regs) != 1:
                    raise ValueError(f"{p.bc.name} patch '{p.name}' belongs to {len(regs)} regions; it must "
                                     f"belong to one")
                continue
            if len(regs) != 2:
                raise ValueError(f"interface '{p.name}' belongs to {len(regs)} regions; it must belong to two")
            a, b = (self._sigma[(q.name, p.name)] for q in regs)
            if a != -b:
                raise ValueError(f"interface '{p.name}' has the same orientation in both of its regions")

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
