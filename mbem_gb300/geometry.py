"""Exact mesh geometry for batches of points on the GPU (``src/mbem/geometry.py``).

- ``solid_angle_batch(mesh, points)``: the signed solid angle the mesh
  subtends at each point (geometry.py:8-57), the quantity
  ``RegionModel.point_in_region`` sums to classify points (core.py:994-1025);
- ``distance_to_mesh(points, mesh)``: the exact distance to the nearest
  triangle and its index (geometry.py:90-105).

Both run the CUDA kernels of ``csrc/geometry.cu`` through the C ABI
(``mbem_solid_angle_sum``, ``mbem_mesh_distance``): far (point, triangle)
pairs in FP32 on hi/lo split coordinates, near pairs in the reference's FP64
arithmetic. ``MeshGeometry`` keeps one mesh's device records for repeated
queries (the volume sampler asks the same mesh several questions).
Points and results follow the ``_device`` rule: numpy in, numpy out; torch
in, CUDA tensors out.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from ._device import as_cuda, is_torch, out_like, ptr, stream_handle


class MeshGeometry:
    """Device copy of one triangle mesh and its per-triangle records."""

    def __init__(self, mesh):
        tv = np.asarray(mesh.vertices, float)[np.asarray(mesh.triangles)]
        self.n_tri = int(tv.shape[0])
        self.tv = as_cuda(tv.reshape(-1, 9))
        edges = np.stack([tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 1], tv[:, 0] - tv[:, 2]])
        self.max_edge = float(np.linalg.norm(edges, axis=2).max()) if self.n_tri else 0.0
        nbytes = int(nat.lib().mbem_geom_record_bytes(self.n_tri))
        # float32 storage: 16-byte aligned by the caching allocator
        self.records = torch.empty(max(nbytes // 4, 4), dtype=torch.float32, device=self.tv.device)
        nat.call("mbem_geom_prepare", ptr(self.tv), self.n_tri, ptr(self.records), stream_handle())

    def solid_angle(self, points: torch.Tensor, weight: float = 1.0, out: torch.Tensor | None = None,
                    accumulate: bool = False) -> torch.Tensor:
        """``out (+)= weight * Omega(points)`` for (N, 3) CUDA float64 points."""
        pts = points.reshape(-1, 3).contiguous()
        if out is None:
            out = torch.zeros(pts.shape[0], dtype=torch.float64, device=pts.device)
            accumulate = False
        nat.call("mbem_solid_angle_sum", ptr(self.records), ptr(self.tv), self.n_tri, ptr(pts), pts.shape[0],
                 float(weight), int(bool(accumulate)), ptr(out), stream_handle())
        return out

    def distance(self, points: torch.Tensor):
        """``(d, idx)``: CUDA float64 and int64 tensors of shape (N,)."""
        if self.n_tri == 0:
            raise ValueError("the distance to a mesh needs at least one triangle")
        pts = points.reshape(-1, 3).contiguous()
        if not bool(torch.isfinite(pts).all()):
            raise ValueError("the distance to a mesh needs finite points")
        d = torch.empty(pts.shape[0], dtype=torch.float64, device=pts.device)
        idx = torch.empty(pts.shape[0], dtype=torch.int64, device=pts.device)
        nat.call("mbem_mesh_distance", ptr(self.records), ptr(self.tv), self.n_tri, ptr(pts), pts.shape[0],
                 self.max_edge, ptr(d), ptr(idx), stream_handle())
        return d, idx


def solid_angle_batch(mesh, points):
    """``(N,)`` signed solid angle subtended by ``mesh`` at each point
    (geometry.py:50-57)."""
    pts = as_cuda(points).reshape(-1, 3)
    return out_like(MeshGeometry(mesh).solid_angle(pts), is_torch(points))


def distance_to_mesh(points, mesh, k: int | None = None):
    """``(d, idx)``: exact distance from each point to the mesh and the index
    of the nearest triangle (geometry.py:90-105). The reference searches the
    ``k = 32`` triangles with the nearest centroids; this searches every
    triangle, so ``k`` is accepted and unused."""
    del k
    pts = as_cuda(points).reshape(-1, 3)
    d, idx = MeshGeometry(mesh).distance(pts)
    torch_in = is_torch(points)
    return out_like(d, torch_in), out_like(idx, torch_in)
