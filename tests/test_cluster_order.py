"""The level-by-level bisection (``cluster_order_device``) against the
recursive one (``cluster_leaves``, the reference's la/cluster.py:56-75 rule):
the same leaves in the same tree order on point clouds without degenerate
principal axes, and a valid partition with leaves of at most max_nodes where
projections coincide (runs on the CPU with CPU tensors)."""

import numpy as np
import pytest
import torch

from mbem_gb300.la.precond import cluster_leaves, cluster_order_device


@pytest.mark.parametrize("m, max_nodes, seed", [(1, 75, 0), (75, 75, 1), (76, 75, 2), (1000, 75, 3),
                                                (5000, 25, 4), (777, 10, 5)])
def test_same_leaves_as_the_recursive_bisection(m, max_nodes, seed):
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(m, 3)) * np.array([3.0, 1.5, 0.7])        # distinct principal axes
    ref = cluster_leaves(pts, max_nodes)
    order, sizes = cluster_order_device(torch.from_numpy(pts), max_nodes)
    got = np.split(order.numpy(), np.cumsum(sizes)[:-1])
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert np.array_equal(np.sort(a), np.sort(b))


def test_coincident_points_still_partition():
    pts = np.zeros((300, 3))
    pts[150:] = 1.0
    order, sizes = cluster_order_device(torch.from_numpy(pts), 40)
    assert sorted(order.tolist()) == list(range(300))
    assert sizes.sum() == 300 and sizes.max() <= 40
