"""The clearance warnings' bounding-box cull (backends/diagnostics.py
``_clearance``): points farther from a mesh's bounding box than the limit
times the largest eps cannot fall inside it, so they never reach the exact
(device) distance; with none left the count is 0 and no GPU is touched."""

import numpy as np

from mbem_gb300 import defaults
from mbem_gb300 import mesh as M
from mbem_gb300.backends import diagnostics as D


def test_far_points_are_culled_without_a_distance_call(monkeypatch):
    fault = M.centre_fault(8)
    eps = np.full(fault.n_triangles, 0.01)
    rng = np.random.default_rng(0)
    pts = rng.uniform(2.0, 3.0, size=(500, 3))      # well outside the fault's box
    import mbem_gb300.geometry as G

    def no_distance(*args, **kwargs):
        raise AssertionError("the exact distance was asked for culled points")

    monkeypatch.setattr(G, "distance_to_mesh", no_distance)
    assert D._clearance(pts, fault, eps) == (0, np.inf)


def test_only_candidates_reach_the_distance(monkeypatch):
    fault = M.centre_fault(8)
    eps = np.full(fault.n_triangles, 0.05)
    limit = defaults.COLLOCATION_FAULT_CLEARANCE_EPS * 0.05
    v = np.asarray(fault.vertices, float)
    lo, hi = v.min(axis=0), v.max(axis=0)
    near = (lo + hi) / 2
    far = hi + 10.0 * max(limit, 1e-3)
    pts = np.array([near, far, far + 1.0])
    seen = {}

    def fake_distance(points, mesh, k=None):
        seen["n"] = len(points)
        return np.zeros(len(points)), np.zeros(len(points), dtype=np.int64)

    import mbem_gb300.geometry as G
    monkeypatch.setattr(G, "distance_to_mesh", fake_distance)
    count, worst = D._clearance(pts, fault, eps)
    assert seen["n"] == 1 and count == 1 and worst == 0.0
