"""Triangle meshes, materials and the tensor-grid generators of the configs.

``TriMesh`` and ``ElasticMaterial`` carry the fields and derived quantities of
the reference's ``src/mollified_bem.py:31-45, :183-219``. The generators
produce the same vertex arrays and triangulations as the reference's
``src/local_box_mesh.py`` (rectangles, box walls, vertical faults; N x N
squares split into two triangles with the 4-fold mirror-symmetric diagonal
pattern), so a model built here is element-for-element the reference's.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class ElasticMaterial:
    """Isotropic material by (mu, lam); nu is derived, never the other way."""
    mu: float
    lam: float

    @property
    def nu(self) -> float:
        return self.lam / (2.0 * (self.lam + self.mu))

    @property
    def E(self) -> float:
        return self.mu * (3.0 * self.lam + 2.0 * self.mu) / (self.lam + self.mu)


@dataclass
class TriMesh:
    vertices: np.ndarray    # (n_verts, 3)
    triangles: np.ndarray   # (n_tris, 3) int

    @property
    def n_triangles(self) -> int:
        return int(self.triangles.shape[0])

    @property
    def n_vertices(self) -> int:
        return int(self.vertices.shape[0])

    def tri_verts(self) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(self.vertices, float)[np.asarray(self.triangles)])

    def centroids(self) -> np.ndarray:
        return centroids_of(self.tri_verts())

    def normals_and_areas(self):
        return normals_and_areas_of(self.tri_verts())


def centroids_of(tv: np.ndarray) -> np.ndarray:
    """(n, 3) centroids of the corners ``tv`` (n, 3, 3): (c0 + c1 + c2) / 3,
    the same sums as a mean over the corner axis."""
    return (tv[:, 0] + tv[:, 1] + tv[:, 2]) / 3.0


def normals_and_areas_of(tv: np.ndarray):
    """Unit normals (n, 3) and areas (n,) of the corners ``tv`` (n, 3, 3):
    the normal is (c1 - c0) x (c2 - c0) over its length, the area half
    that length. Written by components, the products and sums of a cross
    product and a Euclidean norm in the same order."""
    a = tv[:, 1] - tv[:, 0]
    b = tv[:, 2] - tv[:, 0]
    cross = np.empty_like(a)
    cross[:, 0] = a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1]
    cross[:, 1] = a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2]
    cross[:, 2] = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
    area2 = np.sqrt(cross[:, 0] * cross[:, 0] + cross[:, 1] * cross[:, 1] + cross[:, 2] * cross[:, 2])
    return cross / area2[:, None], 0.5 * area2


def grid_triangles(nx: int, ny: int, flip: bool, symmetric: bool = True) -> np.ndarray:
    """Two triangles per cell of an (nx+1) x (ny+1) vertex grid (vertex (i, j)
    at j (nx+1) + i). The symmetric pattern takes the (v00, v11) diagonal in
    the (+,+) and (-,-) quadrants and (v10, v01) in the others, which keeps
    the triangulation invariant under both mirrors; ``flip`` reverses the
    winding."""
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i = i.ravel()
    j = j.ravel()
    row = nx + 1
    v00 = j * row + i
    v10 = v00 + 1
    v01 = v00 + row
    v11 = v01 + 1
    if symmetric:
        main = ((2 * i + 1) < nx) == ((2 * j + 1) < ny)
    else:
        main = np.ones_like(i, bool)
    a = np.where(main[:, None], np.stack([v00, v10, v11], 1), np.stack([v00, v10, v01], 1))
    b = np.where(main[:, None], np.stack([v00, v11, v01], 1), np.stack([v10, v11, v01], 1))
    if flip:
        a = a[:, [0, 2, 1]]
        b = b[:, [0, 2, 1]]
    out = np.empty((2 * a.shape[0], 3), dtype=int)
    out[0::2] = a
    out[1::2] = b
    return out


def rectangle(x_range, y_range, z_level, nx, ny, normal_up=True) -> TriMesh:
    """Flat rectangle at fixed z (the reference's make_rectangular_patch)."""
    xs = np.linspace(x_range[0], x_range[1], nx + 1)
    ys = np.linspace(y_range[0], y_range[1], ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    verts = np.column_stack([X.ravel(), Y.ravel(), np.full(X.size, z_level)])
    return TriMesh(verts, grid_triangles(nx, ny, flip=not normal_up))


def wall(axis, fixed_coord, tangent_range, z_range, nt, nz, outward_sign) -> TriMesh:
    """Vertical box wall at constant x or y whose normals point along
    ``outward_sign`` times that axis (the reference's make_vertical_panel)."""
    if axis not in ("x", "y"):
        raise ValueError("axis must be 'x' or 'y'")
    ts = np.linspace(tangent_range[0], tangent_range[1], nt + 1)
    zs = np.linspace(z_range[0], z_range[1], nz + 1)
    T, Z = np.meshgrid(ts, zs, indexing="xy")
    fixed = np.full(T.size, fixed_coord)
    verts = (np.column_stack([fixed, T.ravel(), Z.ravel()]) if axis == "x"
             else np.column_stack([T.ravel(), fixed, Z.ravel()]))
    mesh = TriMesh(verts, grid_triangles(nt, nz, flip=False))
    n, _ = mesh.normals_and_areas()
    want = np.zeros(3)
    want[0 if axis == "x" else 1] = float(outward_sign)
    if np.dot(n[0], want) < 0:
        mesh.triangles = mesh.triangles[:, [0, 2, 1]]
    return mesh


def concatenate(meshes) -> TriMesh:
    """One mesh from several, vertices not merged."""
    verts, tris, off = [], [], 0
    for m in meshes:
        verts.append(m.vertices)
        tris.append(m.triangles + off)
        off += m.n_vertices
    return TriMesh(np.vstack(verts), np.vstack(tris))


def vertical_fault(strike_length, depth_range, n_along, n_down, center_xy=(0.0, 0.0),
                   strike_azimuth_deg=0.0):
    """Vertical rectangular fault; returns (mesh, n_hat, s_hat) with the stored
    normal along n_hat (the reference's make_vertical_fault_xy)."""
    z_bot, z_top = depth_range
    if not (z_bot < z_top <= 0):
        raise ValueError("Expected z_bot < z_top <= 0 in depth_range")
    theta = np.radians(strike_azimuth_deg)
    s_hat = np.array([np.sin(theta), np.cos(theta), 0.0])
    n_hat = np.array([np.cos(theta), -np.sin(theta), 0.0])
    ss = np.linspace(-strike_length / 2, strike_length / 2, n_along + 1)
    zs = np.linspace(z_bot, z_top, n_down + 1)
    Z, S = np.meshgrid(zs, ss, indexing="ij")
    S = S.ravel()
    verts = np.column_stack([center_xy[0] + S * s_hat[0], center_xy[1] + S * s_hat[1], Z.ravel()])
    mesh = TriMesh(verts, grid_triangles(n_along, n_down, flip=False))
    n, _ = mesh.normals_and_areas()
    if np.dot(n[0], n_hat) < 0:
        mesh.triangles = mesh.triangles[:, [0, 2, 1]]
    return mesh, n_hat, s_hat


def cube(n_face: int, side: float = 4.0) -> TriMesh:
    """Closed cube centred at the origin, n_face x n_face squares per face,
    outward normals: top, bottom, +x, -x, +y, -y walls in that order."""
    a = side / 2.0
    faces = [
        rectangle((-a, a), (-a, a), a, n_face, n_face, normal_up=True),
        rectangle((-a, a), (-a, a), -a, n_face, n_face, normal_up=False),
        wall("x", a, (-a, a), (-a, a), n_face, n_face, +1),
        wall("x", -a, (-a, a), (-a, a), n_face, n_face, -1),
        wall("y", a, (-a, a), (-a, a), n_face, n_face, +1),
        wall("y", -a, (-a, a), (-a, a), n_face, n_face, -1),
    ]
    return concatenate(faces)


def centre_fault(n_fault: int, length: float = 1.0) -> TriMesh:
    """Vertical fault of side ``length`` in the plane y = 0, centred at the
    origin, striking along x (stored normal -y)."""
    mesh, _, _ = vertical_fault(length, (-length, 0.0), n_fault, n_fault, strike_azimuth_deg=90.0)
    mesh.vertices = mesh.vertices + np.array([0.0, 0.0, length / 2.0])
    return mesh
