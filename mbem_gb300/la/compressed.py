"""Compressed pair operator on the GPU: the far field of a (field mesh,
source mesh, kernel) block in low-rank form, the near field dense
(``src/mbem/la/hop.py`` ``PairCompressed``, ``la/cluster.py``, ``la/aca.py``).

The partition follows the reference's rules: a cluster tree of each mesh's
element centroids by principal-axis bisection at the median (leaves of at
most CLUSTER_MIN_LEAF elements; a split that leaves one side empty makes a
leaf), axis-aligned bounding boxes, and block pairs admissible when
``min(diam_f, diam_s) < eta * dist(box_f, box_s)`` (eta = 2), neither side
above MAX_ADMISSIBLE_BLOCK elements; admissible pairs smaller than
ACA_MIN_BLOCK on a side, and pairs of leaves that are not admissible, are
dense.

Every admissible block is compressed on the device by cross approximation
with 3 x 3 element pivots (``mbem_aca_compress``: one CTA a block, the
block's rows and columns evaluated by the FP64 closed form of the pair
kernel, stopped when the newest rank-3 term is below half the tolerance of
the running Frobenius norm), then certified on 3 random element rows and 3
random element columns evaluated exactly: a block whose estimated relative
Frobenius error exceeds ACA_CERTIFY_FACTOR x tol is compressed again at
tol / ACA_RETRY_TOL_FACTOR, and applied exactly (dense) if it fails again or
reaches the rank cap (a third of its element rank). The matvec applies all
low-rank blocks and all dense blocks in two launches each over the flat
arrays. Unlike the reference, which compresses the geometry-only basis
stack once and recombines it per material, a view here is compressed per
material directly (the material's coefficients enter the pair kernel).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import as_cuda, ptr, stream_handle


# ---------------------------------------------------------------------------
# cluster tree and partition (host)
# ---------------------------------------------------------------------------
@dataclass
class Cluster:
    indices: np.ndarray          # element indices
    lo: np.ndarray               # bounding box
    hi: np.ndarray
    children: tuple = ()

    @property
    def n(self) -> int:
        return int(self.indices.size)

    @property
    def leaf(self) -> bool:
        return not self.children

    def diameter(self) -> float:
        return float(np.linalg.norm(self.hi - self.lo))

    def gap(self, other: "Cluster") -> float:
        d = np.maximum(0.0, np.maximum(self.lo - other.hi, other.lo - self.hi))
        return float(np.linalg.norm(d))


def cluster_tree(centroids: np.ndarray, min_leaf: int = defaults.CLUSTER_MIN_LEAF) -> Cluster:
    """The bisection tree of la/cluster.py:56-76 over element centroids."""
    pts = np.asarray(centroids, float)

    def node(idx):
        p = pts[idx]
        return Cluster(idx, p.min(axis=0), p.max(axis=0))

    root = node(np.arange(pts.shape[0]))
    todo = [root]
    while todo:
        c = todo.pop()
        if c.n <= min_leaf:
            continue
        p = pts[c.indices]
        d = p - p.mean(axis=0)
        axis = np.linalg.eigh(d.T @ d)[1][:, -1]
        proj = d @ axis
        left = proj < np.median(proj)
        if left.all() or not left.any():
            continue
        c.children = (node(c.indices[left]), node(c.indices[~left]))
        todo.extend(c.children)
    return root


def partition(tree_f: Cluster, tree_s: Cluster, eta: float = defaults.ADMISSIBILITY_ETA,
              max_admissible: int = defaults.MAX_ADMISSIBLE_BLOCK, min_aca: int = defaults.ACA_MIN_BLOCK):
    """(admissible, dense): lists of (field element indices, source element
    indices) blocks covering every (field, source) pair once
    (la/cluster.py:95-124)."""
    adm, dense = [], []
    todo = [(tree_f, tree_s)]
    while todo:
        cf, cs = todo.pop()
        small = cf.n <= max_admissible and cs.n <= max_admissible
        if small and min(cf.diameter(), cs.diameter()) < eta * cf.gap(cs):
            (dense if min(cf.n, cs.n) < min_aca else adm).append((cf.indices, cs.indices))
        elif cf.leaf and cs.leaf:
            dense.append((cf.indices, cs.indices))
        else:
            fs = cf.children if not cf.leaf else (cf,)
            ss = cs.children if not cs.leaf else (cs,)
            # pushed in reverse so that blocks come out in the tree order
            for a in reversed(fs):
                for b in reversed(ss):
                    todo.append((a, b))
    return adm, dense


def _flat(blocks):
    """Flat int32 row / column index arrays and int64 offsets of a block list."""
    rows = np.concatenate([r for r, _ in blocks]).astype(np.int32) if blocks else np.zeros(0, np.int32)
    cols = np.concatenate([c for _, c in blocks]).astype(np.int32) if blocks else np.zeros(0, np.int32)
    rp = np.concatenate([[0], np.cumsum([len(r) for r, _ in blocks])]).astype(np.int64)
    cp = np.concatenate([[0], np.cumsum([len(c) for _, c in blocks])]).astype(np.int64)
    return rows, cols, rp, cp
