"""Cluster block-Jacobi preconditioner on the GPU
(``src/mbem/la/preconditioner.py:421-470``, the "block_jacobi" rung).

The chunks are the leaves of the principal-axis bisection tree of the
node centroids of each slot (``src/mbem/la/cluster.py:56-75``
``build_cluster_tree``: split at the median of the projection on the
covariance's leading eigenvector, ``proj < median`` to the left). A
leaf holds at most ``max_nodes`` nodes (3 DOF each, at most
``MBEM_BJ_MAX_DOF`` = 225 DOF), so that the CUDA build inverts it in one
CTA's shared memory; the reference's default chunk is 9000 DOF, factored
by LAPACK on the host.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _native as nat
from .._device import ptr, stream_handle

MAX_NODES = nat.BJ_MAX_DOF // 3


def cluster_leaves(points: np.ndarray, max_nodes: int) -> list:
    """Index arrays of the leaves of the bisection tree over ``points``
    (n, 3), each with at most ``max_nodes`` entries, in tree order."""
    points = np.asarray(points, float)
    leaves = []
    stack = [np.arange(points.shape[0])]
    while stack:
        idx = stack.pop()
        if idx.size <= max_nodes:
            leaves.append(idx)
            continue
        pts = points[idx]
        mean = pts.mean(axis=0)
        cov = (pts - mean).T @ (pts - mean)
        _, vecs = np.linalg.eigh(cov)
        proj = (pts - mean) @ vecs[:, -1]
        left = proj < np.median(proj)
        if left.all() or not left.any():
            # coincident projections: halve by position
            order = np.argsort(proj, kind="stable")
            left = np.zeros(idx.size, bool)
            left[order[:idx.size // 2]] = True
        # right pushed first so the left subtree is emitted first
        stack.append(idx[~left])
        stack.append(idx[left])
    return leaves


def _segment_sums(v: torch.Tensor, ends: torch.Tensor) -> torch.Tensor:
    """Sums of v (m,) or (m, q) over consecutive segments ending (exclusive)
    at ``ends``: prefix sums along the contiguous dimension of v^T (a scan
    down the rows of a tall, narrow matrix is slow on the device)."""
    t = v.reshape(v.shape[0], -1).T.contiguous()
    c = torch.cumsum(t, dim=1)
    c = torch.cat([torch.zeros_like(c[:, :1]), c], dim=1)
    starts = torch.cat([torch.zeros_like(ends[:1]), ends[:-1]])
    out = (c[:, ends] - c[:, starts]).T
    return out.reshape((ends.shape[0],) + tuple(v.shape[1:]))


def cluster_order_device(points: torch.Tensor, max_nodes: int):
    """The bisection tree of ``cluster_leaves`` built level by level on the
    device: returns (order (m,) int64 CUDA, leaf sizes (L,) host int64), the
    leaves as consecutive runs of ``order`` in the tree order of
    ``cluster_leaves``. Each split is the one ``cluster_leaves`` makes
    (median of the projection on the leading principal axis, ``proj <
    median`` to the left, halves by rank when the projections coincide).
    A level costs one small copy each way: the segments' sizes and 3 x 3
    covariances to the host, whose eigenproblems are solved together there,
    and their principal axes back. Where the two leading principal axes are
    degenerate the axis, and so the split, may differ from the host's."""
    dev = points.device
    m = int(points.shape[0])
    order = torch.arange(m, dtype=torch.int64, device=dev)
    sizes = torch.tensor([m], dtype=torch.int64, device=dev)
    pos = torch.arange(m, device=dev)
    while m:
        S = int(sizes.numel())
        ends = torch.cumsum(sizes, 0)
        starts = ends - sizes
        is_start = torch.zeros(m + 1, dtype=torch.int64, device=dev)
        is_start[starts] = 1
        seg = torch.cumsum(is_start[:m], 0) - 1
        P = points[order]
        cnt = sizes.to(torch.float64)
        mean = _segment_sums(P, ends) / cnt[:, None]
        X = P - mean[seg]
        cov = _segment_sums((X[:, :, None] * X[:, None, :]).reshape(m, 9), ends)
        host = torch.cat([cnt[:, None], cov], dim=1).cpu().numpy()
        sz_h = host[:, 0].astype(np.int64)
        big = sz_h > max_nodes
        if not big.any():
            break
        axis = np.zeros((S, 3))
        _, vecs = np.linalg.eigh(host[big, 1:].reshape(-1, 3, 3))
        axis[big] = vecs[:, :, -1]
        proj = (X * torch.from_numpy(axis).to(dev)[seg]).sum(dim=1)
        # projections sorted within each segment (stable: ties keep the current order)
        by_proj = torch.argsort(proj, stable=True)
        srt = by_proj[torch.argsort(seg[by_proj], stable=True)]
        sproj = proj[srt]
        median = 0.5 * (sproj[starts + (sizes - 1) // 2] + sproj[starts + sizes // 2])
        bigd = torch.from_numpy(big).to(dev)
        left = (proj < median[seg]) & bigd[seg]
        nl = _segment_sums(left.long(), ends)
        flat = bigd & ((nl == 0) | (nl == sizes))
        # coincident projections: the lower half by rank goes left
        rank = torch.empty(m, dtype=torch.int64, device=dev)
        rank[srt] = pos - starts[seg[srt]]
        left = torch.where(flat[seg], rank < (sizes // 2)[seg], left)
        nl = torch.where(flat, sizes // 2, nl)
        # stable partition: each segment's left part, then its right part
        key = 2 * seg + (~left).long() * bigd[seg].long()
        order = order[torch.argsort(key, stable=True)]
        # the new segment list: a big segment becomes (left, right)
        n_new = 1 + bigd.long()
        new_start = torch.cumsum(n_new, 0) - n_new
        new_sizes = torch.empty(int(S + big.sum()), dtype=torch.int64, device=dev)
        new_sizes[new_start] = torch.where(bigd, nl, sizes)
        bi = new_start[bigd] + 1
        new_sizes[bi] = (sizes - nl)[bigd]
        sizes = new_sizes
    return order, sizes.cpu().numpy()


def cluster_order_cuda(points: torch.Tensor, max_nodes: int):
    """``cluster_order_device``'s tree by the CUDA level kernels
    (``mbem_cluster_stats`` / ``mbem_cluster_split``: a CTA a segment, the
    median by an exact radix select, a stable partition): returns the same
    (order (m,) int64 CUDA, leaf sizes (L,) host int64). A level costs one
    small copy each way: the segments' sizes and covariances to the host,
    whose 3 x 3 eigenproblems numpy solves together (so the axes are the
    host rule's), and their axes back; a segment whose projections coincide
    at the median is split by rank on the host (the rule's fallback)."""
    if points.device.type != "cuda":
        raise ValueError("cluster_order_cuda needs CUDA points")
    dev = points.device
    pts = points.to(torch.float64).contiguous()
    m = int(pts.shape[0])
    order = torch.arange(m, dtype=torch.int64, device=dev)
    if m == 0:
        return order, np.zeros(0, np.int64)
    other = torch.empty_like(order)
    proj = torch.empty(m, dtype=torch.float64, device=dev)
    starts_h = np.zeros(1, np.int64)
    sizes_h = np.array([m], np.int64)
    st = stream_handle()
    while True:
        S = int(sizes_h.size)
        starts = torch.from_numpy(starts_h).to(dev)
        sizes = torch.from_numpy(sizes_h).to(dev)
        mean = torch.empty((S, 3), dtype=torch.float64, device=dev)
        stats = torch.empty((S, 10), dtype=torch.float64, device=dev)
        nat.call("mbem_cluster_stats", ptr(pts), ptr(order), ptr(starts), ptr(sizes), S, int(max_nodes), ptr(mean),
                 ptr(stats), st)
        host = stats.cpu().numpy()
        big = sizes_h > max_nodes
        if not big.any():
            break
        axis = np.zeros((S, 3))
        _, vecs = np.linalg.eigh(host[big, 1:].reshape(-1, 3, 3))
        axis[big] = vecs[:, :, -1]
        nl = torch.empty(S, dtype=torch.int64, device=dev)
        nat.call("mbem_cluster_split", ptr(pts), ptr(order), ptr(other), ptr(starts), ptr(sizes), S, int(max_nodes),
                 ptr(mean), ptr(torch.from_numpy(axis).to(dev)), ptr(proj), ptr(nl), st)
        order, other = other, order
        nl_h = nl.cpu().numpy()
        for s_ in np.flatnonzero(nl_h < 0):
            # coincident projections: the lower half by rank goes left
            a, n_s = int(starts_h[s_]), int(sizes_h[s_])
            cur = order[a:a + n_s].cpu().numpy()
            rank_order = np.argsort(proj[a:a + n_s].cpu().numpy(), kind="stable")
            left = np.zeros(n_s, bool)
            left[rank_order[:n_s // 2]] = True
            order[a:a + n_s] = torch.from_numpy(np.concatenate([cur[left], cur[~left]])).to(dev)
            nl_h[s_] = n_s // 2
        starts_h, sizes_h = next_segments(sizes_h, nl_h, big)
    return order, sizes_h


def next_segments(sizes: np.ndarray, nl: np.ndarray, big: np.ndarray):
    """The segment list of the next tree level: a split segment (``big``)
    becomes its left part of ``nl`` points and its right part, in place; a
    leaf stays. Returns (starts, sizes), int64."""
    sizes = np.asarray(sizes, np.int64)
    n_new = 1 + np.asarray(big, bool).astype(np.int64)
    new_sizes = np.empty(int(n_new.sum()), np.int64)
    pos = np.cumsum(n_new) - n_new
    new_sizes[pos] = np.where(big, nl, sizes)
    new_sizes[pos[big] + 1] = (sizes - nl)[big]
    starts = np.concatenate([[0], np.cumsum(new_sizes)[:-1]]).astype(np.int64)
    return starts, new_sizes


class BlockJacobi:
    """M^-1 = blockdiag(A[c, c]^-1) over spatial chunks c of every slot.

    ``groups``: [(dof_offset, node_points (n_nodes, 3)), ...] covering the
    unknowns 0..n-1, each node owning DOFs offset + 3 i + (0, 1, 2)."""

    PRECOND_KIND = 1

    def __init__(self, n: int, groups, max_nodes: int = MAX_NODES, device="cuda"):
        if not 1 <= max_nodes <= MAX_NODES:
            raise ValueError(f"max_nodes must be in [1, {MAX_NODES}]")
        chunks = []
        for off, pts in groups:
            for leaf in cluster_leaves(pts, max_nodes):
                leaf = np.sort(leaf)
                chunks.append((off + 3 * leaf[:, None] + np.arange(3)[None, :]).ravel())
        dofs = np.concatenate(chunks) if chunks else np.zeros(0, np.int64)
        if dofs.size != n or not np.array_equal(np.sort(dofs), np.arange(n)):
            raise ValueError("the slots' nodes do not partition the unknowns")
        sizes = np.array([c.size for c in chunks], np.int64)
        ptr_h = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        local = np.empty(n, np.int32)
        chunk_of = np.empty(n, np.int32)
        for c, d in enumerate(chunks):
            local[d] = np.arange(d.size, dtype=np.int32)
            chunk_of[d] = c
        self.n = int(n)
        self.n_chunks = len(chunks)
        self.m_max = int(sizes.max()) if sizes.size else 1
        self.chunk_sizes = sizes
        self._chunks = chunks
        self.device = torch.device(device)
        self._ptr = torch.from_numpy(ptr_h).to(self.device)
        self._dofs = torch.from_numpy(dofs.astype(np.int64)).to(self.device)
        self._local = torch.from_numpy(local).to(self.device)
        self._chunk_of = torch.from_numpy(chunk_of).to(self.device)
        nbytes = nat.lib().mbem_bj_inverse_bytes(self.n_chunks, self.m_max)
        self.inv = torch.zeros(nbytes // 4, dtype=torch.float32, device=self.device)
        self._struct = nat.BlockJacobi(n=self.n, n_chunks=self.n_chunks, m_max=self.m_max,
                                       chunk_ptr=ptr(self._ptr), dofs=ptr(self._dofs), local=ptr(self._local),
                                       chunk_of=ptr(self._chunk_of), inv=ptr(self.inv))
        self.built = False

    @classmethod
    def from_device_points(cls, n: int, groups, max_nodes: int = MAX_NODES):
        """As the constructor, with the slots' node points as CUDA tensors and
        the chunks made by ``cluster_order_cuda`` (no host pass over the
        nodes)."""
        if not 1 <= max_nodes <= MAX_NODES:
            raise ValueError(f"max_nodes must be in [1, {MAX_NODES}]")
        self = cls.__new__(cls)
        dev = groups[0][1].device
        dof_parts, sizes_all = [], []
        for off, pts in groups:
            order, sizes = cluster_order_cuda(pts, max_nodes)
            # each leaf's nodes ascending, as the host constructor sorts them
            leaf = torch.repeat_interleave(torch.arange(sizes.size, device=dev), torch.from_numpy(sizes).to(dev))
            order = order[torch.argsort(leaf * (pts.shape[0] + 1) + order)]
            dof_parts.append((off + 3 * order[:, None] + torch.arange(3, device=dev)).reshape(-1))
            sizes_all.append(3 * sizes)
        dofs = torch.cat(dof_parts) if dof_parts else torch.zeros(0, dtype=torch.int64, device=dev)
        sizes = np.concatenate(sizes_all) if sizes_all else np.zeros(0, np.int64)
        if dofs.numel() != n or int(sizes.sum()) != n:
            raise ValueError("the slots' nodes do not partition the unknowns")
        ptr_h = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        chunk = torch.repeat_interleave(torch.arange(sizes.size, device=dev, dtype=torch.int32),
                                        torch.from_numpy(sizes).to(dev))
        start = torch.from_numpy(ptr_h[:-1]).to(dev)
        local = torch.empty(n, dtype=torch.int32, device=dev)
        chunk_of = torch.empty(n, dtype=torch.int32, device=dev)
        pos = torch.arange(n, device=dev)
        local[dofs] = (pos - start[chunk.long()]).to(torch.int32)
        chunk_of[dofs] = chunk
        self.n = int(n)
        self.n_chunks = int(sizes.size)
        self.m_max = int(sizes.max()) if sizes.size else 1
        self.chunk_sizes = sizes
        self._chunks = None
        self.device = dev
        self._ptr = torch.from_numpy(ptr_h).to(dev)
        self._dofs = dofs.contiguous()
        self._local = local
        self._chunk_of = chunk_of
        nbytes = nat.lib().mbem_bj_inverse_bytes(self.n_chunks, self.m_max)
        self.inv = torch.zeros(nbytes // 4, dtype=torch.float32, device=dev)
        self._struct = nat.BlockJacobi(n=self.n, n_chunks=self.n_chunks, m_max=self.m_max,
                                       chunk_ptr=ptr(self._ptr), dofs=ptr(self._dofs), local=ptr(self._local),
                                       chunk_of=ptr(self._chunk_of), inv=ptr(self.inv))
        self.built = False
        return self

    @classmethod
    def for_layout(cls, layout, max_nodes: int = MAX_NODES, device="cuda"):
        """Chunks over every slot of an ``UnknownLayout``, nodes at the
        slot patch's collocation points."""
        groups = [(s.offset, np.asarray(s.patch.collocation_points(), float)) for s in layout.slots]
        return cls(layout.n_unknowns, groups, max_nodes, device)

    def struct(self):
        return self._struct

    def chunk_nodes(self) -> list:
        """Node indices (unknowns 3i..3i+2) of every chunk, in chunk order."""
        if self._chunks is None:
            d = self._dofs.cpu().numpy()
            p = self._ptr.cpu().numpy()
            self._chunks = [d[p[c]:p[c + 1]] for c in range(self.n_chunks)]
        return [d[::3] // 3 for d in self._chunks]

    def chunk_of_node(self) -> torch.Tensor:
        """(n / 3,) int64 CUDA: the chunk of every node."""
        return self._chunk_of[0::3].long()

    def build_dense(self, A: torch.Tensor):
        if A.dtype != torch.float64 or A.stride(1) != 1 or A.shape[0] != self.n:
            raise ValueError("A must be the (n, n) FP64 system with unit column stride")
        self._build("mbem_bj_build_dense", ptr(A), A.stride(0))
        return self

    def build_mixed(self, op):
        s = op.struct()
        self._build("mbem_bj_build_mixed", ctypes.byref(s))
        return self

    def _build(self, name, *args):
        try:
            nat.call(name, *args, ctypes.byref(self._struct), stream_handle())
        except nat.MbemError as err:
            # a singular chunk: its inverse is the identity, the rest stand
            self.built = err.code == nat.ERR_NUMERIC
            raise
        self.built = True

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        if not self.built:
            raise RuntimeError("block-Jacobi preconditioner applied before a build")
        r = r.to(dtype=torch.float64, device=self.device).contiguous()
        z = torch.empty_like(r)
        nat.call("mbem_bj_apply", ctypes.byref(self._struct), ptr(r), ptr(z), stream_handle())
        return z

    def dense_blocks_host(self, A: np.ndarray) -> list:
        """(dofs, A[dofs, dofs]) per chunk from a host matrix (for checks)."""
        ptr_h = self._ptr.cpu().numpy()
        dofs = self._dofs.cpu().numpy()
        return [(dofs[ptr_h[c]:ptr_h[c + 1]], A[np.ix_(dofs[ptr_h[c]:ptr_h[c + 1]], dofs[ptr_h[c]:ptr_h[c + 1]])])
                for c in range(self.n_chunks)]
