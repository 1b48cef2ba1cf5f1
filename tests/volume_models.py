"""Models the volume-sampler tests share (test infrastructure)."""

from __future__ import annotations

import numpy as np


def two_region_model(g):
    """Host cube with an inclusion bounded by an INTERFACE patch of both
    regions, built from the ``volume_regions`` fixture's own meshes; returns
    (model, host outer patch, interface patch)."""
    from mbem_gb300.mesh import ElasticMaterial, TriMesh
    from mbem_gb300.model import BCType, Patch, Region, RegionModel
    outer = TriMesh(g["outer_vertices"], g["outer_triangles"])
    inner = TriMesh(g["inner_vertices"], g["inner_triangles"])
    host_p = Patch("outer", outer, BCType.FREE_TRACTION)
    iface = Patch("iface", inner, BCType.INTERFACE)
    host = Region("host", ElasticMaterial(1.0, 1.0), [host_p, iface], np.array([1.5, 1.5, 1.5]))
    incl = Region("incl", ElasticMaterial(2.0, 3.0), [iface], np.zeros(3))
    return RegionModel([host, incl]), host_p, iface
