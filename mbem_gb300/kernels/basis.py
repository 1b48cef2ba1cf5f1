"""Material coefficients, eps resolution, Lagrange nodes and the assembly entry
points, with the API of ``src/mbem/kernels/basis.py``.

Binding rules kept from the reference: coefficients come from (mu, lam)
directly, never through 1/(1-2 nu) (basis.py:14-17); eps is an (N_src,)
per-source-element array everywhere, a scalar being promoted (:187-204).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .. import defaults
from . import tri_nodal as tn
from .tri_nodal import n_nodes  # noqa: F401


def _material_pair(material=None, mu=None, lam=None):
    """(mu, lam) from a material, or the pair given directly."""
    pair = (material.mu, material.lam) if material is not None else (mu, lam)
    if None in pair:
        raise ValueError("a basis combination needs a material or both Lame parameters (mu, lam)")
    return pair


def u_coeffs(mu, lam) -> np.ndarray:
    """Coefficients (3,) of the U basis [I1 d, eps^2 I3 d, T2[3]] (basis.py:46-55)."""
    nu = lam / (2.0 * (lam + mu))
    one_minus_nu = (lam + 2.0 * mu) / (2.0 * (lam + mu))
    C1 = 1.0 / (16.0 * np.pi * mu * one_minus_nu)
    return np.array([(3.0 - 4.0 * nu) * C1, 1.0 / (8.0 * np.pi * mu), C1])


def t_coeffs(mu, lam) -> np.ndarray:
    """Coefficients (6,) of the T basis [N1, N2, N3, R1, R2, R3] (basis.py:58-72):
    lam C1 on the trace (N) blocks, mu C1 on the R blocks."""
    nu = lam / (2.0 * (lam + mu))
    one_minus_nu = (lam + 2.0 * mu) / (2.0 * (lam + mu))
    C1 = 1.0 / (16.0 * np.pi * mu * one_minus_nu)
    c34 = 3.0 - 4.0 * nu
    cL, cM = lam * C1, mu * C1
    blob = 6.0 * one_minus_nu
    return np.array([c34 * cL, -cL, blob * cL, c34 * cM, -cM, blob * cM])


class MeshArrays:
    """Arrays derived from meshes and patches, computed once per object for
    the life of ONE assembly (the reference's rule, basis.py:91-146): keyed
    by ``id()``, so an instance must not outlive the meshes it has seen, and
    is never a module-level cache."""

    def __init__(self):
        self._memo: dict = {}

    def _get(self, kind: str, obj, make):
        key = (kind, id(obj))
        if key not in self._memo:
            self._memo[key] = make()
        return self._memo[key]

    def source_arrays(self, mesh_source):
        """(tri_verts (N, 3, 3), normals (N, 3)), both C-contiguous FP64."""
        def make():
            corners = np.take(np.asarray(mesh_source.vertices, float), np.asarray(mesh_source.triangles), axis=0)
            return np.ascontiguousarray(corners), np.ascontiguousarray(mesh_source.normals_and_areas()[0])
        return self._get("src", mesh_source, make)

    def field_points(self, mesh_or_points):
        """A mesh's centroids, or an (N, 3) point array as given."""
        if hasattr(mesh_or_points, "centroids"):
            return self._get("pts", mesh_or_points, lambda: np.ascontiguousarray(mesh_or_points.centroids()))
        return np.ascontiguousarray(np.asarray(mesh_or_points, dtype=float))

    def collocation_points(self, patch):
        return self._get("coll", patch, lambda: np.ascontiguousarray(patch.collocation_points()))

    def collocation_normals(self, patch):
        return self._get("colln", patch, lambda: np.ascontiguousarray(patch.collocation_normals()))


# Barycentric coordinates of the Lagrange nodes in the kernels' node order:
# P0 the centroid; P1 the vertices v1 v2 v3; P2 the vertices, then the edge
# midpoints m12 m23 m31 (node k of element s is density row K s + k).
_NODE_BARY = {
    0: np.full((1, 3), 1.0 / 3.0),
    1: np.eye(3),
    2: np.vstack([np.eye(3), 0.5 * (np.eye(3) + np.roll(np.eye(3), -1, axis=0))]),
}
# the vertex pairs of the P2 midpoint nodes
_MID_PAIRS = ((0, 1), (1, 2), (2, 0))


def lagrange_nodes(order: int, shrink: float = 0.0) -> np.ndarray:
    """(K, 3) barycentric node coordinates, each moved toward the centroid
    by the fraction ``shrink`` (a collocation point; 0 leaves the nodes)."""
    if order not in _NODE_BARY:
        raise ValueError(f"order must be 0, 1 or 2 (got {order!r})")
    t = float(shrink)
    return _NODE_BARY[order] * (1.0 - t) + t / 3.0


def lagrange_shape(order: int, lam) -> np.ndarray:
    """(M, K) values of the element's shape functions at barycentric points
    ``lam`` (M, 3): 1 at P0; the coordinates themselves at P1; at P2
    l_i (2 l_i - 1) on the vertices and 4 l_a l_b on the midpoints."""
    L = np.atleast_2d(np.asarray(lam, float))
    if order == 0:
        return np.ones((L.shape[0], 1))
    if order == 1:
        return L.copy()
    vertex = L * (2.0 * L - 1.0)
    mid = np.column_stack([4.0 * L[:, i] * L[:, j] for i, j in _MID_PAIRS])
    return np.hstack([vertex, mid])


def as_eps_array(eps, n_source: int) -> np.ndarray:
    """One eps per source element (N_src,): a scalar is repeated. Refused:
    another length, and any entry that is not a finite positive number (the
    kernels use eps^2, so a negative eps would pass as |eps| while the
    eigenstress term that tests eps > 0 vanished; eps = 0 divides by zero
    in the closed form)."""
    given = np.asarray(eps, dtype=float)
    if given.ndim != 0 and given.shape != (n_source,):
        raise ValueError(f"eps has shape {given.shape}; expected a scalar or ({n_source},), one per source element")
    arr = np.ascontiguousarray(np.broadcast_to(given, (n_source,)), dtype=float)
    ok = np.isfinite(arr) & (arr > 0.0)
    if not ok.all():
        raise ValueError(f"eps must be finite and > 0 for every source element: {int((~ok).sum())} of "
                         f"{arr.size} are not (smallest {arr.min()})")
    return arr


def element_sizes(mesh) -> np.ndarray:
    """(N_src,) size of each triangle: the mean of its three edge lengths."""
    v = np.asarray(mesh.vertices, float)
    t = np.asarray(mesh.triangles)
    c0, c1, c2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]

    def length(e):
        return np.sqrt(e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1] + e[:, 2] * e[:, 2])

    return (length(c1 - c0) + length(c2 - c1) + length(c0 - c2)) / 3.0


def resolve_eps(eps, mesh) -> np.ndarray:
    """(N_src,) eps of one mesh from a spec: a scalar, one value per
    element, or "auto" (EPS_OVER_H times each element's size, so eps / h
    stays fixed under grading and refinement)."""
    if not isinstance(eps, str):
        return as_eps_array(eps, mesh.n_triangles)
    if eps == "auto":
        return np.ascontiguousarray(defaults.EPS_OVER_H * element_sizes(mesh))
    raise ValueError(f"eps spec {eps!r} is not understood: give a number, an array or 'auto'")


def resolve_patch_eps(spec, patch) -> np.ndarray:
    """(N_src,) eps of one patch or fault. A dict spec maps patch names to
    specs and must hold this patch. On a fault "auto" means ONE width for the
    whole fault, FAULT_EPS_OVER_H times its smallest element size (a uniform
    slip smeared unequally would be a source of its own)."""
    from ..model.core import FAULT_KINDS

    if isinstance(spec, dict):
        try:
            spec = spec[patch.name]
        except KeyError:
            raise ValueError(f"the eps dict names {sorted(spec)} but not patch {patch.name!r}") from None
    if patch.bc in FAULT_KINDS and isinstance(spec, str) and spec == "auto":
        width = defaults.FAULT_EPS_OVER_H * float(element_sizes(patch.mesh).min())
        return np.full(patch.mesh.n_triangles, width)
    return resolve_eps(spec, patch.mesh)


def identity_ids(order: int, n_source: int) -> np.ndarray:
    """(N_src, K) column ids of the discontinuous layout: element s, node k
    owns column K s + k, the kernels' own order."""
    K = n_nodes(order)
    return np.ascontiguousarray(np.add.outer(K * np.arange(n_source, dtype=np.int64), np.arange(K, dtype=np.int64)))


@dataclass
class UBasis:
    """Geometry-only U basis stack (3, 3 N_f, 3 K N_s)."""
    stack: object

    def combine(self, material=None, mu=None, lam=None):
        c = u_coeffs(*_material_pair(material, mu, lam))
        return sum(float(ci) * self.stack[i] for i, ci in enumerate(c))


@dataclass
class TBasis:
    """Geometry-only T basis stack (6, 3 N_f, 3 K N_s)."""
    stack: object

    def combine(self, material=None, mu=None, lam=None):
        c = t_coeffs(*_material_pair(material, mu, lam))
        return sum(float(ci) * self.stack[i] for i, ci in enumerate(c))


def assemble_u_basis(mesh_field, mesh_source, eps, arrays=None, order: int = 0) -> UBasis:
    a = arrays if arrays is not None else MeshArrays()
    x_field = a.field_points(mesh_field)
    tri_verts, _ = a.source_arrays(mesh_source)
    return UBasis(tn.u_basis_matrices(x_field, tri_verts, as_eps_array(eps, tri_verts.shape[0]), order))


def assemble_t_basis(mesh_field, mesh_source, eps, arrays=None, order: int = 0) -> TBasis:
    a = arrays if arrays is not None else MeshArrays()
    x_field = a.field_points(mesh_field)
    tri_verts, normals = a.source_arrays(mesh_source)
    return TBasis(tn.t_basis_matrices(x_field, tri_verts, normals,
                                      as_eps_array(eps, tri_verts.shape[0]), order))


def assemble_u_matrix(mesh_field, mesh_source, material, eps, arrays=None, order: int = 0, ids=None,
                      n_cols=None, out=None, alpha=1.0, accumulate=False):
    """Real-material U matrix (3 N_f, 3 K N_s) (basis.py:372-386). Shared-node
    columns (``ids``) are not part of the dense hot path and are refused."""
    if ids is not None:
        raise NotImplementedError("shared-node (continuous) columns are not built on the GPU path")
    a = arrays if arrays is not None else MeshArrays()
    x_field = a.field_points(mesh_field)
    tri_verts, _ = a.source_arrays(mesh_source)
    g = u_coeffs(material.mu, material.lam)
    return tn.u_matrix_direct(x_field, tri_verts, as_eps_array(eps, tri_verts.shape[0]), *g, order,
                              out=out, alpha=alpha, accumulate=accumulate)


def assemble_t_matrix(mesh_field, mesh_source, material, eps, arrays=None, order: int = 0, ids=None,
                      n_cols=None, out=None, alpha=1.0, accumulate=False):
    """Real-material T matrix (3 N_f, 3 K N_s) (basis.py:389-403)."""
    if ids is not None:
        raise NotImplementedError("shared-node (continuous) columns are not built on the GPU path")
    a = arrays if arrays is not None else MeshArrays()
    x_field = a.field_points(mesh_field)
    tri_verts, normals = a.source_arrays(mesh_source)
    c = t_coeffs(material.mu, material.lam)
    return tn.t_matrix_direct(x_field, tri_verts, normals, as_eps_array(eps, tri_verts.shape[0]), *c,
                              order, out=out, alpha=alpha, accumulate=accumulate)


def assemble_traction_matrix(x_field, n_field, mesh_source, material, eps, arrays=None, order: int = 0,
                             kind: str = "slip", ids=None, n_cols=None, out=None, alpha=1.0):
    """Traction rows (3 N_f, 3 n_cols) (basis.py:406-427)."""
    a = arrays if arrays is not None else MeshArrays()
    tri_verts, normals = a.source_arrays(mesh_source)
    eps_arr = as_eps_array(eps, tri_verts.shape[0])
    if ids is None:
        ids = identity_ids(order, tri_verts.shape[0])
        n_cols = ids.size
    return tn.traction_matrix(np.asarray(x_field, float), np.asarray(n_field, float), tri_verts, normals,
                              eps_arr, ids, int(n_cols), material.mu, material.lam, order, kind,
                              out=out, alpha=alpha)
