"""Numpy restatement of the reference's mesh geometry and volume-sampler
bookkeeping (TEST INFRASTRUCTURE, not the product).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
use this module, to check the CUDA path. It follows, step by step:

- ``solid_angle_sum``: the van Oosterom signed solid angle summed over a
  mesh (src/mbem/geometry.py:8-47), chunked over the points;
- ``point_triangle_distance`` / ``distance_to_mesh``: the Voronoi-region
  closest point and the search over the ``k`` nearest centroids
  (src/mbem/geometry.py:60-105);
- ``closure`` / ``classify``: RegionModel.point_in_region's closure sum and
  the sampler's region codes with the on-patch rule
  (src/mbem/model/core.py:994-1025, src/mbem/volume.py:199-252);
- ``clearance``: the boundary and fault clearances (src/mbem/volume.py:255-301);
- ``strain`` / ``derived``: Hooke inverted and the render scalars
  (src/mbem/volume.py:304-328).

``tests/test_volume.py`` pins it to ``tests/golden/volume_small.npz``,
which the reference's own ``volume`` module wrote. Meshes are passed as
(n_tri, 3, 3) vertex arrays.
"""

from __future__ import annotations

import numpy as np

CLOSURE_TOL = 1e-6          # src/mbem/model/core.py:621
ON_PATCH_TOL = 1e-9         # src/mbem/model/core.py:89


def solid_angle_sum(tv: np.ndarray, points: np.ndarray, chunk: int = 4096) -> np.ndarray:
    tv = np.asarray(tv, float)
    pts = np.asarray(points, float).reshape(-1, 3)
    out = np.zeros(pts.shape[0])
    for s in range(0, pts.shape[0], chunk):
        p = pts[s:s + chunk, None, :]
        a, b, c = tv[None, :, 0] - p, tv[None, :, 1] - p, tv[None, :, 2] - p
        ra, rb, rc = (np.sqrt((v * v).sum(-1)) for v in (a, b, c))
        numer = (a[..., 0] * (b[..., 1] * c[..., 2] - b[..., 2] * c[..., 1])
                 + a[..., 1] * (b[..., 2] * c[..., 0] - b[..., 0] * c[..., 2])
                 + a[..., 2] * (b[..., 0] * c[..., 1] - b[..., 1] * c[..., 0]))
        denom = ra * rb * rc + rc * (a * b).sum(-1) + ra * (b * c).sum(-1) + rb * (a * c).sum(-1)
        out[s:s + chunk] = (2.0 * np.arctan2(numer, denom)).sum(axis=1)
    return out


def point_triangle_distance(p, a, b, c) -> np.ndarray:
    ab, ac = b - a, c - a
    ap, bp, cp = p - a, p - b, p - c
    d1, d2 = (ab * ap).sum(-1), (ac * ap).sum(-1)
    d3, d4 = (ab * bp).sum(-1), (ac * bp).sum(-1)
    d5, d6 = (ab * cp).sum(-1), (ac * cp).sum(-1)
    va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
    with np.errstate(divide="ignore", invalid="ignore"):
        s = va + vb + vc
        q = a + ab * (vb / s)[..., None] + ac * (vc / s)[..., None]
        regions = [
            ((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * (d1 / (d1 - d3))[..., None]),
            ((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * (d2 / (d2 - d6))[..., None]),
            ((va <= 0) & (d4 >= d3) & (d5 >= d6), b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[..., None]),
        ]
        for cond, val in regions:
            q = np.where(cond[..., None], val, q)
    for cond, val in (((d1 <= 0) & (d2 <= 0), a), ((d3 >= 0) & (d4 <= d3), b), ((d6 >= 0) & (d5 <= d6), c)):
        q = np.where(cond[..., None], val, q)
    return np.linalg.norm(p - q, axis=-1)


def distance_to_mesh(points, tv, k: int = 32):
    from scipy.spatial import cKDTree

    pts = np.asarray(points, float).reshape(-1, 3)
    tv = np.asarray(tv, float)
    k = min(k, tv.shape[0])
    _, idx = cKDTree(tv.mean(axis=1)).query(pts, k=k)
    idx = np.asarray(idx).reshape(pts.shape[0], k)
    d = point_triangle_distance(pts[:, None, :], tv[idx, 0], tv[idx, 1], tv[idx, 2])
    j = d.argmin(axis=1)
    rows = np.arange(pts.shape[0])
    return d[rows, j], idx[rows, j]


def element_sizes(tv) -> np.ndarray:
    e = np.stack([tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 1], tv[:, 0] - tv[:, 2]])
    return np.linalg.norm(e, axis=2).mean(axis=0)


def closure(patches, points):
    """``(inside, total)`` for one region: patches = [(tv, sigma), ...]."""
    pts = np.asarray(points, float).reshape(-1, 3)
    total = np.zeros(pts.shape[0])
    for tv, sigma in patches:
        total += sigma * solid_angle_sum(tv, pts)
    return np.abs(total - 4.0 * np.pi) <= CLOSURE_TOL * 4.0 * np.pi, total


def on_patch(points, tv) -> np.ndarray:
    d, j = distance_to_mesh(points, tv)
    return d < ON_PATCH_TOL * element_sizes(np.asarray(tv, float))[j]


def classify(regions, points) -> np.ndarray:
    """regions = [[(tv, sigma), ...] per region]."""
    pts = np.asarray(points, float).reshape(-1, 3)
    code = np.zeros(pts.shape[0], np.int8)
    for i, patches in enumerate(regions, start=1):
        hit = closure(patches, pts)[0] & (code == 0)
        code[hit] = i
    settled = np.zeros(pts.shape[0], bool)
    for i, patches in enumerate(regions, start=1):
        for tv, _ in patches:
            on = on_patch(pts, tv) & ~settled
            code[on] = i
            settled |= on
    return code


def clearance(points, patches, faults):
    """patches = [(tv, eps (n_tri,))], faults likewise."""
    pts = np.asarray(points, float).reshape(-1, 3)
    n = pts.shape[0]
    c_h, c_eps, c_fault = np.full(n, np.inf), np.full(n, np.inf), np.full(n, np.inf)
    for tv, eps in patches:
        d, idx = distance_to_mesh(pts, tv)
        c_h = np.minimum(c_h, d / element_sizes(np.asarray(tv, float))[idx])
        c_eps = np.minimum(c_eps, d / np.asarray(eps, float)[idx])
    for tv, eps in faults:
        d, idx = distance_to_mesh(pts, tv)
        c_fault = np.minimum(c_fault, d / np.asarray(eps, float)[idx])
    return c_h, c_eps, c_fault


def strain(sig: np.ndarray, mu: float, lam: float) -> np.ndarray:
    tr_e = np.trace(sig, axis1=1, axis2=2) / (2.0 * mu + 3.0 * lam)
    e = sig.copy()
    for k in range(3):
        e[:, k, k] -= lam * tr_e
    return e / (2.0 * mu)


def derived(u: np.ndarray, sig: np.ndarray, e: np.ndarray) -> dict:
    tr = np.trace(sig, axis1=1, axis2=2)
    dev = sig - (tr / 3.0)[:, None, None] * np.eye(3)
    w = np.linalg.eigvalsh(sig)
    return {"u_mag": np.linalg.norm(u, axis=1),
            "von_mises": np.sqrt(1.5 * np.einsum("nij,nij->n", dev, dev)),
            "mean_stress": tr / 3.0,
            "max_shear": 0.5 * (w[:, 2] - w[:, 0]),
            "dilatation": np.trace(e, axis1=1, axis2=2)}
