"""The level-by-level bisection (``cluster_order_device`` with torch
ops, ``cluster_order_cuda`` with the CUDA level kernels) against the
recursive one (``cluster_leaves``, the reference's la/cluster.py:56-75 rule):
the same leaves in the same tree order on point clouds without degenerate
principal axes, and a valid partition with leaves of at most max_nodes where
projections coincide (runs on the CPU with CPU tensors)."""

import numpy as np
import pytest
import torch

from mbem_gb300.la.precond import cluster_leaves, cluster_order_device, next_segments


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


@pytest.mark.gpu
@pytest.mark.parametrize("m, max_nodes, seed", [(1, 75, 0), (75, 75, 1), (76, 75, 2), (1000, 75, 3),
                                                (5000, 25, 4), (777, 10, 5), (30000, 75, 6)])
def test_cuda_levels_same_leaves_as_the_recursive_bisection(gpu, m, max_nodes, seed):
    """``cluster_order_cuda`` (the level kernels) makes the recursive rule's
    leaves in its tree order."""
    from mbem_gb300.la.precond import cluster_order_cuda
    rng = np.random.default_rng(seed)
    pts = rng.normal(size=(m, 3)) * np.array([3.0, 1.5, 0.7])
    ref = cluster_leaves(pts, max_nodes)
    order, sizes = cluster_order_cuda(torch.from_numpy(pts).cuda(), max_nodes)
    got = np.split(order.cpu().numpy(), np.cumsum(sizes)[:-1])
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert np.array_equal(np.sort(a), np.sort(b))


@pytest.mark.gpu
def test_cuda_levels_coincident_points_split_by_rank(gpu):
    from mbem_gb300.la.precond import cluster_order_cuda
    pts = np.zeros((300, 3))
    pts[150:] = 1.0
    order, sizes = cluster_order_cuda(torch.from_numpy(pts).cuda(), 40)
    assert sorted(order.cpu().tolist()) == list(range(300))
    assert sizes.sum() == 300 and sizes.max() <= 40
    ref = cluster_leaves(pts, 40)
    got = np.split(order.cpu().numpy(), np.cumsum(sizes)[:-1])
    assert [np.sort(a).tolist() for a in got] == [np.sort(b).tolist() for b in ref]


def test_next_segments_splits_in_place():
    """The level bookkeeping of the CUDA bisection: split segments become
    (left, right) where they stood, leaves stay, starts follow the sizes."""
    sizes = np.array([100, 40, 77, 3])
    big = sizes > 50
    nl = np.array([50, 40, 38, 3])
    starts, new = next_segments(sizes, nl, big)
    assert new.tolist() == [50, 50, 40, 38, 39, 3]
    assert starts.tolist() == [0, 50, 100, 140, 178, 217]
    assert new.sum() == sizes.sum()
