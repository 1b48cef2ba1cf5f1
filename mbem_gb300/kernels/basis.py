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


def _mu_lam(material=None, mu=None, lam=None):
    if material is not None:
        return material.mu, material.lam
    if mu is None or lam is None:
        raise ValueError("provide either material or (mu, lam)")
    return mu, lam


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


def _source_arrays(mesh_source):
    tri_verts = np.asarray(mesh_source.vertices, float)[np.asarray(mesh_source.triangles)]
    normals, _ = mesh_source.normals_and_areas()
    return np.ascontiguousarray(tri_verts), np.ascontiguousarray(normals)


def _field_points(mesh_or_points):
    if hasattr(mesh_or_points, "centroids"):
        return np.ascontiguousarray(mesh_or_points.centroids())
    return np.ascontiguousarray(np.asarray(mesh_or_points, dtype=float))


class MeshArrays:
    """Assembly-scoped memo of mesh-derived arrays keyed by ``id()`` (the
    reference's basis.py:91-146 scope rule: never a module cache)."""

    def __init__(self):
        self._src: dict = {}
        self._pts: dict = {}
        self._coll: dict = {}

    def source_arrays(self, mesh_source):
        key = id(mesh_source)
        if key not in self._src:
            self._src[key] = _source_arrays(mesh_source)
        return self._src[key]

    def field_points(self, mesh_or_points):
        if not hasattr(mesh_or_points, "centroids"):
            return _field_points(mesh_or_points)
        key = id(mesh_or_points)
        if key not in self._pts:
            self._pts[key] = _field_points(mesh_or_points)
        return self._pts[key]

    def collocation_points(self, patch):
        key = id(patch)
        if key not in self._coll:
            self._coll[key] = np.ascontiguousarray(patch.collocation_points())
        return self._coll[key]

    def collocation_normals(self, patch):
        key = ("n", id(patch))
        if key not in self._coll:
            self._coll[key] = np.ascontiguousarray(patch.collocation_normals())
        return self._coll[key]


def lagrange_nodes(order: int, shrink: float = 0.0) -> np.ndarray:
    """Barycentric node coordinates (K, 3) in the kernels' node order (P0
    centroid; P1 v1 v2 v3; P2 v1 v2 v3 m12 m23 m31), pulled toward the
    centroid by ``shrink`` (basis.py lagrange_nodes)."""
    K = n_nodes(order)
    if order == 0:
        lam = np.full((1, 3), 1.0 / 3.0)
    elif order == 1:
        lam = np.eye(3)
    else:
        lam = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0],
                        [0.5, 0.5, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5]])
    t = float(shrink)
    if t:
        lam = (1.0 - t) * lam + t / 3.0
    assert lam.shape == (K, 3)
    return lam


def lagrange_shape(order: int, lam) -> np.ndarray:
    """Shape functions N_k (M, K) at barycentric points (M, 3)."""
    lam = np.atleast_2d(np.asarray(lam, float))
    l1, l2, l3 = lam[:, 0], lam[:, 1], lam[:, 2]
    if n_nodes(order) == 1:
        return np.ones((lam.shape[0], 1))
    if order == 1:
        return np.stack([l1, l2, l3], axis=1)
    return np.stack([l1 * (2.0 * l1 - 1.0), l2 * (2.0 * l2 - 1.0), l3 * (2.0 * l3 - 1.0),
                     4.0 * l1 * l2, 4.0 * l2 * l3, 4.0 * l3 * l1], axis=1)


def as_eps_array(eps, n_source: int) -> np.ndarray:
    """Promote scalar eps to (N_src,); refuse wrong shapes and non-positive or
    non-finite entries (basis.py:187-204)."""
    arr = np.asarray(eps, dtype=float)
    if arr.ndim == 0:
        arr = np.full(n_source, float(arr))
    elif arr.shape != (n_source,):
        raise ValueError(f"eps array shape {arr.shape} != ({n_source},)")
    bad = ~(np.isfinite(arr) & (arr > 0.0))
    if bad.any():
        raise ValueError(f"eps must be finite and > 0: {int(bad.sum())} bad of {arr.size}, "
                         f"min = {arr.min()}")
    return np.ascontiguousarray(arr)


def element_sizes(mesh) -> np.ndarray:
    """Per-triangle size: mean edge length (N_src,)."""
    tv = np.asarray(mesh.vertices, float)[np.asarray(mesh.triangles)]
    e = np.stack([tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 1], tv[:, 0] - tv[:, 2]])
    return np.linalg.norm(e, axis=2).mean(axis=0)


def resolve_eps(eps, mesh) -> np.ndarray:
    """An eps spec (scalar, (N_src,) array or "auto") for one mesh."""
    if isinstance(eps, str):
        if eps != "auto":
            raise ValueError(f"unknown eps spec {eps!r} (only 'auto')")
        return np.ascontiguousarray(defaults.EPS_OVER_H * element_sizes(mesh))
    return as_eps_array(eps, mesh.n_triangles)


def resolve_patch_eps(spec, patch) -> np.ndarray:
    """The eps spec of one patch (a dict is keyed by patch name); on a fault
    "auto" is the single value FAULT_EPS_OVER_H * min(h) (basis.py:234-258)."""
    from ..model.core import FAULT_KINDS

    if isinstance(spec, dict):
        if patch.name not in spec:
            raise ValueError(f"eps dict has no entry for patch {patch.name!r} (keys: {sorted(spec)})")
        spec = spec[patch.name]
    if isinstance(spec, str) and spec == "auto" and patch.bc in FAULT_KINDS:
        h = element_sizes(patch.mesh)
        return np.full(h.size, defaults.FAULT_EPS_OVER_H * float(h.min()))
    return resolve_eps(spec, patch.mesh)


def identity_ids(order: int, n_source: int) -> np.ndarray:
    """Element-major column ids (N_s, K): ids[s, k] = K s + k."""
    K = n_nodes(order)
    return np.ascontiguousarray(np.arange(K * n_source, dtype=np.int64).reshape(n_source, K))


@dataclass
class UBasis:
    """Geometry-only U basis stack (3, 3 N_f, 3 K N_s)."""
    stack: object

    def combine(self, material=None, mu=None, lam=None):
        c = u_coeffs(*_mu_lam(material, mu, lam))
        return sum(float(ci) * self.stack[i] for i, ci in enumerate(c))


@dataclass
class TBasis:
    """Geometry-only T basis stack (6, 3 N_f, 3 K N_s)."""
    stack: object

    def combine(self, material=None, mu=None, lam=None):
        c = t_coeffs(*_mu_lam(material, mu, lam))
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
