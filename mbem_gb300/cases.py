"""The cube-with-fault models of the benchmark workloads, built through the
region-model API.

A traction-free cube of side 4 centred at the origin (n x n squares per face,
two triangles each, outward normals) with an embedded vertical planar fault
of side 1 in the plane y = 0 at the centre (m x m squares), prescribed
uniform slip (FAULT) or solved slip under a prescribed traction change
(FAULT_TRACTION).
"""

from __future__ import annotations

import numpy as np

from . import mesh as M
from .model import BCType, Patch, Region, RegionModel


def cube_fault_model(n_face: int, n_fault: int, mu: float = 1.0, lam: float = 1.0,
                     cube_order: int = 0, fault_order: int = 0, slip=(1.0, 0.0, 0.0),
                     fault_kind: BCType = BCType.FAULT, fault_value=None, side: float = 4.0):
    """Returns (model, eps) with eps = half the cube grid spacing, one scalar
    for every patch."""
    cube = M.cube(n_face, side)
    fault = M.centre_fault(n_fault)
    mat = M.ElasticMaterial(mu=mu, lam=lam)
    cube_p = Patch("cube", cube, BCType.FREE_TRACTION, order=cube_order)
    if fault_kind is BCType.FAULT:
        fault_p = Patch("fault", fault, BCType.FAULT, value=np.asarray(slip, float), order=fault_order)
    else:
        fault_p = Patch("fault", fault, BCType.FAULT_TRACTION, value=fault_value, order=0)
    region = Region("body", mat, [cube_p], np.zeros(3), faults=[fault_p])
    eps = (side / n_face) / 2.0
    return RegionModel([region]), eps


def readout_grid(n: int = 64, y: float = 0.1, half: float = 2.0) -> np.ndarray:
    """n x n cell-centre grid on the plane y = const over x, z in [-half, half]."""
    g = (np.arange(n) + 0.5) / n * (2.0 * half) - half
    X, Z = np.meshgrid(g, g, indexing="xy")
    return np.column_stack([X.ravel(), np.full(X.size, y), Z.ravel()])


def fault_traction_model(n_face: int, n_fault: int, dip_deg: float = 90.0, mu: float = 1.0, lam: float = 1.0,
                         drop: float = 1e-3, side: float = 4.0):
    """The cube with a FAULT_TRACTION fault (slip solved under a uniform
    shear-traction drop of ``drop * mu`` along strike, no normal component)
    whose plane is the centre fault rotated about its strike (the x axis)
    to dip ``dip_deg`` (90: vertical). Returns (model, eps), eps = half the
    cube grid spacing."""
    cube = M.cube(n_face, side)
    fault = M.centre_fault(n_fault)
    th = np.deg2rad(90.0 - dip_deg)
    c, s = np.cos(th), np.sin(th)
    R = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    fault.vertices = np.ascontiguousarray(fault.vertices @ R.T)
    mat = M.ElasticMaterial(mu=mu, lam=lam)
    cube_p = Patch("cube", cube, BCType.FREE_TRACTION)
    fault_p = Patch("fault", fault, BCType.FAULT_TRACTION, value=np.array([-drop * mu, 0.0, 0.0]))
    region = Region("body", mat, [cube_p], np.zeros(3), faults=[fault_p])
    return RegionModel([region]), (side / n_face) / 2.0


def gaussian_slips(fault: Patch, n_rhs: int, length: float = 0.3, seed0: int = 0) -> np.ndarray:
    """(n_rhs, n_dofs, 3) smooth random slip patterns on a fault's collocation
    points: a Gaussian random field with squared-exponential covariance of
    ``length`` and unit variance per component, Cholesky factor with 1e-10
    jitter, one ``np.random.default_rng(seed0 + i)`` draw per pattern."""
    pts = np.asarray(fault.collocation_points(), float)
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    C = np.exp(-0.5 * d2 / (length * length))
    L = np.linalg.cholesky(C + 1e-10 * np.eye(pts.shape[0]))
    out = np.empty((n_rhs, pts.shape[0], 3))
    for i in range(n_rhs):
        out[i] = L @ np.random.default_rng(seed0 + i).normal(size=(pts.shape[0], 3))
    return out
