"""Compressed pair operator on the GPU: one (field mesh, source mesh,
kernel) pair with P0 sources, its far field in low-rank form and its near
field dense (``src/mbem/la/hop.py:137`` ``PairCompressed``, ``:489``
``matvec``; ``la/cluster.py``; ``la/aca.py``; ``la/flatview.py``).

The partition follows the reference's rules (``la/cluster.py:56-124``): a
cluster tree of each mesh's element centroids by principal-axis bisection at
the median (leaves of at most CLUSTER_MIN_LEAF elements; a split that leaves
one side empty makes a leaf), axis-aligned bounding boxes, and block pairs
admissible when ``min(diam_f, diam_s) < eta * dist(box_f, box_s)`` (eta = 2)
with neither side above MAX_ADMISSIBLE_BLOCK elements; admissible pairs with a
side below ACA_MIN_BLOCK, and pairs of leaves that are not admissible, are
dense.

Elements are renumbered so that every block is a pair of contiguous ranges
(``laminar_order``: the blocks' row sets, and their column sets, nest or are
disjoint, so a depth-first walk of their containment tree lists each set
contiguously). Every admissible block is compressed on the device by cross
approximation with 3 x 3 element pivots (``mbem_aca_compress``: one CTA a
block; stopped on the true residual of a 10 x 10 element sample; certified on
3 exact element rows and 3 exact element columns; a failed certificate reruns
the block at tol / 10; a second failure, or the rank cap, leaves the block
exact). Dense blocks are evaluated into one flat FP32 buffer, each transposed
(``mbem_pair_dense_blocks``). The product (``mbem_compressed_matvec``) runs
three kernels: the gather of x into tree order, the projections
``w_i = V_i^T x`` of every low-rank block, and one CTA per field-row strip
whose warps stream the strip's blocks (rows of U^T times w, rows of D^T
times x) and add their sums in warp order, so no row has two writers and the
result is bitwise repeatable.

What differs from the reference. A view is compressed per material directly
(the material's coefficients enter the pair kernel), where the reference
compresses the geometry-only basis stack once, folds it into a shared
subspace and recombines it per material; the matvec of a view is the same
operator either way, to the block tolerance. The factors are certified as
stored and not recompressed by a QR + SVD, so their ranks are those of the
cross approximation. Entries are the mixed operator's: the FP32 far
quadrature for far pairs (<= ~1.5e-7 relative), the FP64 closed form for near
ones.
"""

from __future__ import annotations

import ctypes
import time
from collections import OrderedDict

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import as_cuda, is_torch, out_like, ptr, require_cuda, stream_handle
from ..kernels import KERNEL_T, KERNEL_U, kernel_n_basis
from ..kernels import basis as kb


# ---------------------------------------------------------------------------
# cluster tree and partition (host)
# ---------------------------------------------------------------------------
class Cluster:
    """A cluster-tree node: element indices (increasing), the axis-aligned
    bounding box of their centroids, children, and (after ``tree_order``)
    the first position of its elements in the tree order."""

    __slots__ = ("indices", "lo", "hi", "children", "n", "diam", "start")

    def __init__(self, indices: np.ndarray, lo: np.ndarray, hi: np.ndarray):
        self.indices = indices
        self.lo = lo
        self.hi = hi
        self.children = ()
        self.n = int(indices.size)
        self.diam = float(np.linalg.norm(hi - lo))     # la/cluster.py:47-48, evaluated once
        self.start = -1

    @property
    def leaf(self) -> bool:
        return not self.children

    def diameter(self) -> float:
        return self.diam

    def gap(self, other: "Cluster") -> float:
        d = np.maximum(0.0, np.maximum(self.lo - other.hi, other.lo - self.hi))
        return float(np.linalg.norm(d))


def cluster_tree(centroids: np.ndarray, min_leaf: int = defaults.CLUSTER_MIN_LEAF) -> Cluster:
    """The bisection tree of la/cluster.py:56-76 over element centroids:
    split at the median of the projection on the principal axis (``proj <
    median`` goes left), stop at ``min_leaf`` elements or when a side would
    be empty. The same numpy expressions as the reference, so that the same
    centroids give the same tree."""
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
        mean = p.mean(axis=0)
        cov = (p - mean).T @ (p - mean)
        axis = np.linalg.eigh(cov)[1][:, -1]
        proj = (p - mean) @ axis
        left = proj < np.median(proj)
        if left.sum() == 0 or (~left).sum() == 0:
            continue
        c.children = (node(c.indices[left]), node(c.indices[~left]))
        todo.extend(c.children)
    return root


def tree_order(root: Cluster) -> np.ndarray:
    """Position -> element: the leaves depth first, left child first; sets
    every node's ``start`` so that its elements sit at [start, start + n)."""
    out = []
    pos = 0
    stack = [root]
    while stack:
        c = stack.pop()
        c.start = pos
        if c.leaf:
            out.append(c.indices)
            pos += c.n
        else:
            stack.extend(reversed(c.children))
    # interior nodes start where their first leaf does: the stack visits a
    # node before its first child, at the same position
    return np.concatenate(out) if out else np.zeros(0, np.int64)


def partition_nodes(tree_f: Cluster, tree_s: Cluster, eta: float = defaults.ADMISSIBILITY_ETA,
                    max_admissible: int = defaults.MAX_ADMISSIBLE_BLOCK, min_aca: int = defaults.ACA_MIN_BLOCK):
    """(admissible, dense): lists of (field cluster, source cluster) pairs
    covering every (field, source) pair once, in the reference's recursion
    order (la/cluster.py:95-124): admissible when neither side exceeds
    ``max_admissible`` and ``min(diam_f, diam_s) < eta * dist``, dense when
    admissible with a side below ``min_aca`` or when both are leaves."""
    adm, dense = [], []
    todo = [(tree_f, tree_s)]
    while todo:
        cf, cs = todo.pop()
        small = cf.n <= max_admissible and cs.n <= max_admissible
        if small and min(cf.diam, cs.diam) < eta * cf.gap(cs):
            (dense if min(cf.n, cs.n) < min_aca else adm).append((cf, cs))
        elif cf.leaf and cs.leaf:
            dense.append((cf, cs))
        else:
            fs = cf.children if not cf.leaf else (cf,)
            ss = cs.children if not cs.leaf else (cs,)
            # pushed in reverse so that blocks come out in the recursion order
            for a in reversed(fs):
                for b in reversed(ss):
                    todo.append((a, b))
    return adm, dense


def partition_blocks(tree_f: Cluster, tree_s: Cluster, eta: float = defaults.ADMISSIBILITY_ETA,
                     max_admissible: int = defaults.MAX_ADMISSIBLE_BLOCK, min_aca: int = defaults.ACA_MIN_BLOCK):
    """The partition as (field element indices, source element indices)
    lists, the reference's ``BlockPartition`` form."""
    adm, dense = partition_nodes(tree_f, tree_s, eta, max_admissible, min_aca)
    return ([(a.indices, b.indices) for a, b in adm], [(a.indices, b.indices) for a, b in dense])


def _flat(blocks):
    """Flat int32 row / column index arrays and int64 offsets of a block list."""
    rows = np.concatenate([r for r, _ in blocks]).astype(np.int32) if blocks else np.zeros(0, np.int32)
    cols = np.concatenate([c for _, c in blocks]).astype(np.int32) if blocks else np.zeros(0, np.int32)
    rp = np.concatenate([[0], np.cumsum([len(r) for r, _ in blocks])]).astype(np.int64)
    cp = np.concatenate([[0], np.cumsum([len(c) for _, c in blocks])]).astype(np.int64)
    return rows, cols, rp, cp


# ---------------------------------------------------------------------------
# tree order and row strips (host)
# ---------------------------------------------------------------------------
def laminar_order(n: int, sets) -> np.ndarray:
    """An order of ``range(n)`` (position -> element) in which every set of
    ``sets`` is contiguous. The sets must be laminar (any two nest or are
    disjoint), as the clusters of one tree are; a depth-first walk of their
    containment tree lists each set contiguously (children by their smallest
    element, then the node's own elements in increasing order)."""
    uniq = {}
    for s in sets:
        a = np.unique(np.asarray(s, dtype=np.int64))
        if a.size:
            uniq.setdefault(a.tobytes(), a)
    nodes = sorted(uniq.values(), key=lambda a: (-a.size, int(a[0])))
    label = np.full(n, -1, dtype=np.int64)
    parent = np.empty(len(nodes), dtype=np.int64)
    for k, a in enumerate(nodes):
        if a[0] < 0 or a[-1] >= n:
            raise ValueError(f"block index out of range [0, {n})")
        lab = label[a]
        if (lab != lab[0]).any():
            raise ValueError("block index sets are not laminar (they do not come from one cluster tree)")
        parent[k] = lab[0]
        label[a] = k
    children = [[] for _ in range(len(nodes) + 1)]   # slot len(nodes): the root
    for k in range(len(nodes)):
        children[parent[k] if parent[k] >= 0 else len(nodes)].append(k)
    own_sorted = np.argsort(label, kind="stable")
    own_lab = label[own_sorted]
    bounds = np.searchsorted(own_lab, np.arange(-1, len(nodes) + 1))

    def own(k):     # elements whose smallest set is k (k = -1: in no set)
        return own_sorted[bounds[k + 1]:bounds[k + 2]]

    out = []
    stack = [(len(nodes), False)]
    while stack:
        k, done = stack.pop()
        node = -1 if k == len(nodes) else k
        if done:
            out.append(own(node))
            continue
        stack.append((k, True))
        for c in sorted(children[k], key=lambda c: -int(nodes[c][0])):
            stack.append((c, False))
    order = np.concatenate(out) if out else np.zeros(0, np.int64)
    if order.size != n:
        raise ValueError("laminar_order: lost elements")
    return order


def block_ranges(blocks, pos_f: np.ndarray, pos_s: np.ndarray):
    """(r0, nr, c0, nc) int32 arrays of element-range blocks in tree order;
    raises if a block is not contiguous there."""
    nb = len(blocks)
    r0 = np.empty(nb, np.int64)
    nr = np.empty(nb, np.int64)
    c0 = np.empty(nb, np.int64)
    nc = np.empty(nb, np.int64)
    for i, (rows, cols) in enumerate(blocks):
        pr, pc = pos_f[np.asarray(rows)], pos_s[np.asarray(cols)]
        r0[i], nr[i], c0[i], nc[i] = pr.min(), pr.size, pc.min(), pc.size
        if pr.max() - r0[i] + 1 != nr[i] or pc.max() - c0[i] + 1 != nc[i]:
            raise ValueError(f"block {i} is not contiguous in the tree order")
    return (r0.astype(np.int32), nr.astype(np.int32), c0.astype(np.int32), nc.astype(np.int32))


def row_strips(n_rows: int, r0: np.ndarray, nr: np.ndarray):
    """The field rows cut at every block boundary: strip starts and sizes,
    and for each strip the blocks covering it in block order (CSR)."""
    r0 = np.asarray(r0, np.int64)
    r1 = r0 + np.asarray(nr, np.int64)
    bounds = np.unique(np.concatenate([[0, n_rows], r0, r1]))
    s0 = np.searchsorted(bounds, r0)
    s1 = np.searchsorted(bounds, r1)
    cnt = s1 - s0
    tot = int(cnt.sum())
    first = np.repeat(np.cumsum(cnt) - cnt, cnt)
    strip = np.repeat(s0, cnt) + (np.arange(tot) - first)
    item = np.repeat(np.arange(r0.size), cnt)
    o = np.argsort(strip, kind="stable")
    ptr_ = np.concatenate([[0], np.cumsum(np.bincount(strip, minlength=bounds.size - 1))])
    return (bounds[:-1].astype(np.int32), np.diff(bounds).astype(np.int32), ptr_.astype(np.int64),
            item[o].astype(np.int32))


def strip_units(sptr: np.ndarray, items: np.ndarray, rows_of_item: np.ndarray, unit: int = nat.COMPRESSED_UNIT):
    """Each strip's blocks cut into work units of at most ``unit`` factor
    rows, in item order: (unit_ptr, unit_item, unit_k0). ``rows_of_item``:
    the factor rows of every block id (rank, or 3 nc for a dense block)."""
    k = np.asarray(rows_of_item, np.int64)[items]
    nu = np.maximum(1, (k + unit - 1) // unit)
    tot = int(nu.sum())
    item = np.repeat(items, nu).astype(np.int32)
    first = np.repeat(np.cumsum(nu) - nu, nu)
    k0 = ((np.arange(tot) - first) * unit).astype(np.int32)
    cs = np.concatenate([[0], np.cumsum(nu)])
    uptr = cs[np.asarray(sptr, np.int64)].astype(np.int64)
    return uptr, item, k0


def _pad4(n):
    return (np.asarray(n, np.int64) + 3) // 4 * 4


def _exclusive(sizes) -> np.ndarray:
    sizes = np.asarray(sizes, np.int64)
    return np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64) if sizes.size else sizes


def rank_caps(nr, nc) -> np.ndarray:
    """The cross approximation's rank cap in element pivots (aca.py:618-620)."""
    m = np.minimum(np.asarray(nr, np.int64), np.asarray(nc, np.int64))
    return np.minimum(np.maximum(8, (m * defaults.ACA_MAX_RANK_FRACTION).astype(np.int64)), m).astype(np.int32)


# ---------------------------------------------------------------------------
# the operator
# ---------------------------------------------------------------------------
class _View:
    """The flat operator of one material: device arrays and the C view."""

    def __init__(self):
        self.keep = []          # tensors the C view points into
        self.arrays = {}        # the same, by field name of the C view
        self.struct = nat.CompressedView()
        self.work = None
        self.work_bytes = 0
        self.stats = {}
        self.nbytes = 0

    def dev(self, a, dtype) -> torch.Tensor:
        t = torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(require_cuda())
        self.keep.append(t)
        return t


def _i32(v: _View, a, name: str | None = None):
    t = v.dev(a, torch.int32)
    if name:
        v.arrays[name] = t
    return ptr(t)


def _i64(v: _View, a, name: str | None = None):
    t = v.dev(a, torch.int64)
    if name:
        v.arrays[name] = t
    return ptr(t)


class PairCompressed:
    """Compressed (field mesh, source mesh, kernel) pair for P0 sources.

    ``kernel`` is "H" (the T kernel, 6 coefficients) or "G" (U, 3);
    ``partition``: an explicit ``(admissible, dense)`` pair of block lists of
    element index arrays (the reference's ``BlockPartition``), else it is
    built from the cluster trees. ``matvec(coeffs, x)`` applies the view of
    the material ``coeffs`` (``basis.t_coeffs`` / ``u_coeffs``), built on
    first use and cached (at most COMPRESSED_VIEW_CACHE views).

    Statistics follow the reference's names: ``n_lowrank`` admissible and
    ``n_dense`` dense blocks of the partition; per material view
    ``n_capped`` (admissible blocks exact at the rank cap), ``n_retry``
    (first certificate failed), ``n_fallback`` (exact after the retry) and
    ``max_verified_err``, recorded as the worst over the views built.
    """

    def __init__(self, field_mesh, source_mesh, kernel: str, eps_arr,
                 tol: float = defaults.BLOCK_COMPRESSION_TOL,
                 min_leaf: int = defaults.CLUSTER_MIN_LEAF,
                 eta: float = defaults.ADMISSIBILITY_ETA,
                 max_admissible: int = defaults.MAX_ADMISSIBLE_BLOCK,
                 min_aca: int = defaults.ACA_MIN_BLOCK,
                 tree_cache: dict | None = None,
                 arrays: kb.MeshArrays | None = None,
                 partition=None,
                 seed: int = defaults.ACA_SEED,
                 near_factor: float = defaults.COMPRESSED_NEAR_RADIUS_FACTOR,
                 scratch_bytes: int = defaults.COMPRESSED_SCRATCH_BYTES,
                 recompress_max: int = defaults.ACA_RECOMPRESS_MAX):
        """``recompress_max``: factors of 2 .. recompress_max columns (at most
        64) are recompressed (the SVD of U V^T truncated at tol / 2, as
        aca.py:422-438 does) and kept when their certificate holds; 0 keeps
        the cross approximation's own factors."""
        self.n_basis = kernel_n_basis(kernel)          # raises on a traction kernel
        if kernel not in (KERNEL_T, KERNEL_U):
            raise ValueError(f"unknown kernel {kernel!r}")
        if not tol > 0.0:
            raise ValueError(f"tol must be positive, got {tol}")
        self.kernel = kernel
        self.tol = float(tol)
        self.seed = int(seed)
        self.near_factor = float(near_factor)
        self.scratch_bytes = int(scratch_bytes)
        self.recompress_max = int(recompress_max)
        arrays = arrays if arrays is not None else kb.MeshArrays()
        x_field = arrays.field_points(field_mesh)
        tri_verts, normals = arrays.source_arrays(source_mesh)
        self.n_field = int(x_field.shape[0])
        self.n_source = int(tri_verts.shape[0])
        self.shape = (3 * self.n_field, 3 * self.n_source)
        eps = kb.as_eps_array(eps_arr, self.n_source)
        t0 = time.perf_counter()
        if partition is None:
            tree_cache = {} if tree_cache is None else tree_cache

            def _tree(mesh):
                key = id(mesh)
                if key not in tree_cache:
                    root = cluster_tree(arrays.field_points(mesh), min_leaf)
                    tree_cache[key] = (root, tree_order(root))
                return tree_cache[key]

            (tf, of), (ts, os_) = _tree(field_mesh), _tree(source_mesh)
            adm_n, dense_n = partition_nodes(tf, ts, eta=eta, max_admissible=max_admissible, min_aca=min_aca)
            adm = [(a.indices, b.indices) for a, b in adm_n]
            dense = [(a.indices, b.indices) for a, b in dense_n]
            self.field_order, self.src_order = of, os_

            def ranges(pairs):
                return tuple(np.array(v, dtype=np.int32).reshape(-1) for v in (
                    [a.start for a, _ in pairs], [a.n for a, _ in pairs],
                    [b.start for _, b in pairs], [b.n for _, b in pairs]))

            self._adm_ranges, self._dense_ranges = ranges(adm_n), ranges(dense_n)
        else:
            adm = [(np.asarray(r, np.int64), np.asarray(c, np.int64)) for r, c in partition[0]]
            dense = [(np.asarray(r, np.int64), np.asarray(c, np.int64)) for r, c in partition[1]]
            blocks = adm + dense
            self.field_order = laminar_order(self.n_field, [r for r, _ in blocks])
            self.src_order = laminar_order(self.n_source, [c for _, c in blocks])
            pos_f = np.empty(self.n_field, np.int64)
            pos_f[self.field_order] = np.arange(self.n_field)
            pos_s = np.empty(self.n_source, np.int64)
            pos_s[self.src_order] = np.arange(self.n_source)
            self._adm_ranges = block_ranges(adm, pos_f, pos_s)
            self._dense_ranges = block_ranges(dense, pos_f, pos_s)
        covered = sum(r.size * c.size for r, c in adm) + sum(r.size * c.size for r, c in dense)
        if covered != self.n_field * self.n_source:
            raise ValueError(f"the partition covers {covered} element pairs of {self.n_field * self.n_source}")
        self.admissible, self.dense = adm, dense
        self.n_lowrank = len(adm)
        self.n_dense = len(dense)
        self.partition_s = time.perf_counter() - t0

        self._x = as_cuda(x_field[self.field_order])
        self._tv = as_cuda(tri_verts[self.src_order].reshape(self.n_source, 9))
        self._nrm = as_cuda(normals[self.src_order])
        self._eps = as_cuda(eps[self.src_order])
        self._field_order = as_cuda(self.field_order, torch.int64)
        self._src_order = as_cuda(self.src_order, torch.int64)
        self._views: OrderedDict[bytes, _View] = OrderedDict()
        self.n_capped = 0
        self.n_retry = 0
        self.n_fallback = 0
        self.n_view_fallback = 0
        self.max_verified_err = 0.0

    # -- views -----------------------------------------------------------
    def _coeffs(self, coeffs) -> np.ndarray:
        c = np.asarray(coeffs, dtype=float).ravel()
        if c.size != self.n_basis:
            raise ValueError(f"kernel {self.kernel!r} takes {self.n_basis} coefficients, got {c.size}")
        return c

    def _geometry(self, c: np.ndarray, keep: list) -> nat.PairGeometry:
        g = nat.PairGeometry()
        g.kernel = 0 if self.kernel == KERNEL_T else 1
        g.x_field, g.n_field = ptr(self._x), self.n_field
        g.tri_verts, g.normals, g.eps, g.n_src = ptr(self._tv), ptr(self._nrm), ptr(self._eps), self.n_source
        for k in range(6):
            g.coeffs[k] = float(c[k]) if k < c.size else 0.0
        g.near_factor = self.near_factor
        prep = torch.empty(max(1, int(nat.lib().mbem_pair_prep_bytes(self.n_field, self.n_source))),
                           dtype=torch.uint8, device=self._x.device)
        keep.append(prep)
        g.prep = ptr(prep)
        nat.call("mbem_pair_prepare", ctypes.byref(g), stream_handle())
        return g

    def _compress(self, g, v: _View):
        """Cross approximation of every admissible block, in batches whose
        scratch fits ``scratch_bytes``, then the recompression of its factors;
        returns per block (status, rank, err), the compacted factors with
        their offsets, and the count of blocks recompressed."""
        r0, nr, c0, nc = self._adm_ranges
        n = r0.size
        status = np.zeros(n, np.int32)
        rank = np.zeros(n, np.int32)
        err = np.zeros(n, np.float32)
        if n == 0:
            return status, rank, err, None, None, np.zeros(0, np.int64), np.zeros(0, np.int64), 0
        cap = rank_caps(nr, nc)
        ldu, ldv = _pad4(3 * nr), _pad4(3 * nc)
        cap_floats = 3 * cap.astype(np.int64) * (ldu + ldv)
        budget = max(1, self.scratch_bytes // 4)
        dev = self._x.device
        st = stream_handle()
        Us, Vs = [], []
        u_fin = np.zeros(n, np.int64)
        v_fin = np.zeros(n, np.int64)
        u_base = v_base = 0
        n_rc = 0
        lo = 0
        while lo < n:
            hi = lo + 1
            tot = cap_floats[lo]
            while hi < n and tot + cap_floats[hi] <= budget:
                tot += cap_floats[hi]
                hi += 1
            sl = slice(lo, hi)
            ucap = 3 * cap[sl].astype(np.int64) * ldu[sl]
            vcap = 3 * cap[sl].astype(np.int64) * ldv[sl]
            U = torch.empty(int(ucap.sum()), dtype=torch.float32, device=dev)
            V = torch.empty(int(vcap.sum()), dtype=torch.float32, device=dev)
            tmp = _View()
            b = nat.AcaBatch()
            b.n_blocks = hi - lo
            b.r0, b.nr, b.c0, b.nc = _i32(tmp, r0[sl]), _i32(tmp, nr[sl]), _i32(tmp, c0[sl]), _i32(tmp, nc[sl])
            b.max_pivots = _i32(tmp, cap[sl])
            b.u_off, b.v_off = _i64(tmp, _exclusive(ucap)), _i64(tmp, _exclusive(vcap))
            b.U, b.V = ptr(U), ptr(V)
            rk = torch.zeros(hi - lo, dtype=torch.int32, device=dev)
            stt = torch.zeros(hi - lo, dtype=torch.int32, device=dev)
            er = torch.zeros(hi - lo, dtype=torch.float32, device=dev)
            b.rank, b.status, b.err = ptr(rk), ptr(stt), ptr(er)
            b.tol = self.tol
            b.seed = self.seed
            b.first_index = lo
            b.max_nr, b.max_nc = int(nr[sl].max()), int(nc[sl].max())
            b.max_pivots_all = int(cap[sl].max())
            nat.call("mbem_aca_compress", ctypes.byref(g), ctypes.byref(b), st)
            rank[sl], status[sl], err[sl] = rk.cpu().numpy(), stt.cpu().numpy(), er.cpu().numpy()
            rb = rank[sl].astype(np.int64)
            # recompression of the converged factors (their K x K core), kept when
            # its certificate holds; the rest keep the cross approximation's
            kmax = min(self.recompress_max, nat.RC_KMAX)
            elig = np.flatnonzero(((status[sl] & 3) == nat.ACA_LOWRANK) & (rb >= 2) & (rb <= kmax)) \
                if kmax >= 2 else np.zeros(0, np.int64)
            rc_rank = np.zeros(hi - lo, np.int32)
            Ur = Vr = None
            if elig.size:
                ucap_r = rb[elig] * ldu[sl][elig]
                vcap_r = rb[elig] * ldv[sl][elig]
                Ur = torch.empty(max(4, int(ucap_r.sum())), dtype=torch.float32, device=dev)
                Vr = torch.empty(max(4, int(vcap_r.sum())), dtype=torch.float32, device=dev)
                ro = torch.zeros(elig.size, dtype=torch.int32, device=dev)
                re_ = torch.zeros(elig.size, dtype=torch.float32, device=dev)
                r = nat.AcaRecompression()
                r.n_blocks = int(elig.size)
                r.r0, r.nr = _i32(tmp, r0[sl][elig]), _i32(tmp, nr[sl][elig])
                r.c0, r.nc = _i32(tmp, c0[sl][elig]), _i32(tmp, nc[sl][elig])
                r.rank = _i32(tmp, rb[elig])
                r.u_off, r.v_off = _i64(tmp, _exclusive(ucap)[elig]), _i64(tmp, _exclusive(vcap)[elig])
                r.U, r.V = ptr(U), ptr(V)
                r.ur_off, r.vr_off = _i64(tmp, _exclusive(ucap_r)), _i64(tmp, _exclusive(vcap_r))
                r.Ur, r.Vr = ptr(Ur), ptr(Vr)
                r.rank_out, r.err_out = ptr(ro), ptr(re_)
                r.index = _i64(tmp, lo + elig)
                r.tol = self.tol
                r.seed = self.seed
                r.max_rank = int(rb[elig].max())
                nat.call("mbem_aca_recompress", ctypes.byref(g), ctypes.byref(r), st)
                ok = ro.cpu().numpy()
                got = ok > 0
                rc_rank[elig[got]] = ok[got]
                err[lo + elig[got]] = re_.cpu().numpy()[got]
                rank[lo + elig[got]] = ok[got]
                rc_src_u, rc_src_v = np.zeros(hi - lo, np.int64), np.zeros(hi - lo, np.int64)
                rc_src_u[elig], rc_src_v[elig] = _exclusive(ucap_r), _exclusive(vcap_r)
            usz = rank[sl].astype(np.int64) * ldu[sl]
            vsz = rank[sl].astype(np.int64) * ldv[sl]
            Uc = torch.empty(max(4, int(usz.sum())), dtype=torch.float32, device=dev)
            Vc = torch.empty(max(4, int(vsz.sum())), dtype=torch.float32, device=dev)
            ud, vd = _exclusive(usz), _exclusive(vsz)
            raw_rank = np.where(rc_rank > 0, 0, rank[sl]).astype(np.int32)
            dst_u, dst_v = _i64(tmp, ud), _i64(tmp, vd)
            nat.call("mbem_aca_compact", hi - lo, b.nr, b.nc, _i32(tmp, raw_rank), b.u_off, b.v_off, ptr(U), ptr(V),
                     dst_u, dst_v, ptr(Uc), ptr(Vc), st)
            if Ur is not None and (rc_rank > 0).any():
                nat.call("mbem_aca_compact", hi - lo, b.nr, b.nc, _i32(tmp, rc_rank), _i64(tmp, rc_src_u),
                         _i64(tmp, rc_src_v), ptr(Ur), ptr(Vr), dst_u, dst_v, ptr(Uc), ptr(Vc), st)
            n_rc += int((rc_rank > 0).sum())
            torch.cuda.current_stream().synchronize()
            u_fin[sl] = u_base + ud
            v_fin[sl] = v_base + vd
            u_base += Uc.numel()
            v_base += Vc.numel()
            Us.append(Uc)
            Vs.append(Vc)
            del U, V, Ur, Vr, tmp
            lo = hi
        U = torch.cat(Us) if len(Us) > 1 else Us[0]
        V = torch.cat(Vs) if len(Vs) > 1 else Vs[0]
        return status, rank, err, U, V, u_fin, v_fin, n_rc

    def _build_view(self, c: np.ndarray) -> _View:
        v = _View()
        sync = torch.cuda.synchronize
        t0 = time.perf_counter()
        g = self._geometry(c, v.keep)
        t1 = time.perf_counter()
        status, rank, err, U, V, u_off, v_off, n_rc = self._compress(g, v)
        sync()
        t2 = time.perf_counter()
        low = (status & 3) == nat.ACA_LOWRANK
        r0, nr, c0, nc = self._adm_ranges
        dr0, dnr, dc0, dnc = self._dense_ranges
        ex = ~low
        # exact admissible blocks first, then the partition's dense blocks (hop.py:466-468)
        d_r0 = np.concatenate([r0[ex], dr0]).astype(np.int32)
        d_nr = np.concatenate([nr[ex], dnr]).astype(np.int32)
        d_c0 = np.concatenate([c0[ex], dc0]).astype(np.int32)
        d_nc = np.concatenate([nc[ex], dnc]).astype(np.int32)
        dsz = 3 * d_nc.astype(np.int64) * _pad4(3 * d_nr)      # D^T: 3 nc rows of pad4(3 nr)
        d_off = _exclusive(dsz)
        total = int(dsz.sum())
        free, _ = torch.cuda.mem_get_info()
        if 4 * total > free:
            raise MemoryError(f"dense blocks need {4 * total / 1e9:.1f} GB, {free / 1e9:.1f} GB free")
        D = torch.empty(max(4, total), dtype=torch.float32, device=self._x.device)
        v.keep.append(D)
        col_ptr = np.concatenate([[0], np.cumsum(d_nc.astype(np.int64))]).astype(np.int64)
        s = v.struct
        s.d_r0, s.d_nr = _i32(v, d_r0, "d_r0"), _i32(v, d_nr, "d_nr")
        s.d_c0, s.d_nc = _i32(v, d_c0, "d_c0"), _i32(v, d_nc, "d_nc")
        s.d_off = _i64(v, d_off, "d_off")
        v.arrays["D"] = D
        nat.call("mbem_pair_dense_blocks", ctypes.byref(g), int(d_r0.size), s.d_r0, s.d_nr, s.d_c0, s.d_nc, s.d_off,
                 _i64(v, col_ptr), ptr(D), stream_handle())
        sync()
        t3 = time.perf_counter()
        lr_rank = rank[low]
        s.n_field, s.n_src = self.n_field, self.n_source
        s.field_order, s.src_order = ptr(self._field_order), ptr(self._src_order)
        s.n_lr = int(low.sum())
        s.lr_r0, s.lr_nr = _i32(v, r0[low], "lr_r0"), _i32(v, nr[low], "lr_nr")
        s.lr_c0, s.lr_nc = _i32(v, c0[low], "lr_c0"), _i32(v, nc[low], "lr_nc")
        s.lr_rank = _i32(v, lr_rank, "lr_rank")
        s.lr_u, s.lr_v = _i64(v, u_off[low], "lr_u"), _i64(v, v_off[low], "lr_v")
        s.lr_w = _i64(v, _exclusive(lr_rank), "lr_w")
        s.n_w = int(lr_rank.sum())
        if U is not None:
            v.keep += [U, V]
            v.arrays["U"], v.arrays["V"] = U, V
            s.U, s.V = ptr(U), ptr(V)
        s.n_dense = int(d_r0.size)
        s.D = ptr(D)
        all_r0 = np.concatenate([r0[low], d_r0])
        all_nr = np.concatenate([nr[low], d_nr])
        sr0, snr, sptr, sitems = row_strips(self.n_field, all_r0, all_nr)
        s.n_strips = int(sr0.size)
        s.strip_r0, s.strip_nr = _i32(v, sr0, "strip_r0"), _i32(v, snr, "strip_nr")
        s.strip_ptr, s.strip_items = _i64(v, sptr, "strip_ptr"), _i32(v, sitems, "strip_items")
        s.max_strip = int(snr.max()) if snr.size else 0
        item_rows = np.concatenate([lr_rank.astype(np.int64), 3 * d_nc.astype(np.int64)])
        uptr, uitem, uk0 = strip_units(sptr, sitems, item_rows)
        s.unit_ptr, s.unit_item, s.unit_k0 = _i64(v, uptr, "unit_ptr"), _i32(v, uitem, "unit_item"), \
            _i32(v, uk0, "unit_k0")
        # projection units: four factor rows of one low-rank block each
        npu = (lr_rank.astype(np.int64) + 3) // 4
        s.n_proj = int(npu.sum())
        pblk = np.repeat(np.arange(lr_rank.size), npu)
        pk0 = (np.arange(s.n_proj) - np.repeat(np.cumsum(npu) - npu, npu)) * 4
        s.proj_block, s.proj_k0 = _i32(v, pblk, "proj_block"), _i32(v, pk0, "proj_k0")
        s.max_lr_nc = int(nc[low].max()) if s.n_lr else 0
        v.work_bytes = int(nat.lib().mbem_compressed_matvec_workspace_size(ctypes.byref(s)))
        v.work = torch.empty(max(16, v.work_bytes), dtype=torch.uint8, device=self._x.device)
        t4 = time.perf_counter()
        lr_bytes = 4 * int((lr_rank.astype(np.int64) * (_pad4(3 * nr[low]) + _pad4(3 * nc[low]))).sum())
        v.nbytes = lr_bytes + 4 * int(D.numel()) + sum(int(t.numel() * t.element_size()) for t in v.keep[1:]
                                                        if t.dtype in (torch.int32, torch.int64))
        v.stats = {
            "n_capped": int(((status & 3) == nat.ACA_CAPPED).sum()),
            "n_retry": int(((status & nat.ACA_RETRIED) != 0).sum()),
            "n_fallback": int(((status & 3) == nat.ACA_FAILED).sum()),
            "n_recompressed": n_rc,
            "max_verified_err": float(err[low].max()) if low.any() else 0.0,
            "ranks": lr_rank.copy(),
            "status": status & 7,
            "err": err.copy(),
            "lowrank_bytes": lr_bytes,
            "dense_bytes": 4 * total,
            "n_strips": int(sr0.size),
            "build_s": {"prepare": t1 - t0, "aca": t2 - t1, "dense": t3 - t2, "layout": t4 - t3},
        }
        self.n_capped = max(self.n_capped, v.stats["n_capped"])
        self.n_retry = max(self.n_retry, v.stats["n_retry"])
        self.n_fallback = max(self.n_fallback, v.stats["n_fallback"])
        self.n_view_fallback = max(self.n_view_fallback, v.stats["n_capped"] + v.stats["n_fallback"])
        self.max_verified_err = max(self.max_verified_err, v.stats["max_verified_err"])
        return v

    def _view(self, coeffs) -> _View:
        c = self._coeffs(coeffs)
        key = c.tobytes()
        view = self._views.get(key)
        if view is None:
            view = self._build_view(c)
            self._views[key] = view
            while len(self._views) > defaults.COMPRESSED_VIEW_CACHE:
                self._views.popitem(last=False)
        else:
            self._views.move_to_end(key)
        return view

    def warm_views(self, coeffs_list) -> None:
        for c in coeffs_list:
            self._view(c)

    def view_stats(self, coeffs) -> dict:
        """Ranks, statuses, certified errors, bytes and build times of a view."""
        return self._view(coeffs).stats

    # -- operations ---------------------------------------------------------
    def matvec(self, coeffs, x):
        """The material view applied to ``x`` (3 n_source,): numpy in, numpy
        out; a torch tensor stays on the device."""
        view = self._view(coeffs)
        torch_in = is_torch(x)
        xd = as_cuda(x).reshape(-1)
        if xd.numel() != self.shape[1]:
            raise ValueError(f"x has {xd.numel()} entries, operator {self.shape}")
        y = torch.empty(self.shape[0], dtype=torch.float64, device=xd.device)
        self.apply_device(view, xd, y)
        return out_like(y, torch_in)

    def apply_device(self, view: _View, x: torch.Tensor, y: torch.Tensor) -> None:
        """y = A x for device FP64 vectors on the current stream (no checks)."""
        nat.call("mbem_compressed_matvec", ctypes.byref(view.struct), ptr(x), ptr(y), ptr(view.work),
                 view.work_bytes, stream_handle())

    def view_host(self, coeffs) -> dict:
        """A view's flat layout copied to the host: numpy arrays and sizes by
        the field names of ``mbem_compressed_view`` (for a CPU product of the
        same factors)."""
        view = self._view(coeffs)
        s = view.struct
        out = {k: t.cpu().numpy() for k, t in view.arrays.items()}
        out.update(n_field=self.n_field, n_src=self.n_source, n_lr=s.n_lr, n_w=s.n_w, n_dense=s.n_dense,
                   n_strips=s.n_strips, field_order=self.field_order.astype(np.int64),
                   src_order=self.src_order.astype(np.int64))
        for k in ("U", "V"):
            out.setdefault(k, np.zeros(4, np.float32))
        return out

    def to_dense(self, coeffs) -> np.ndarray:
        view = self._view(coeffs)
        out = torch.zeros(self.shape, dtype=torch.float64, device=self._x.device)
        nat.call("mbem_compressed_to_dense", ctypes.byref(view.struct), ptr(out), self.shape[1], stream_handle())
        return out.cpu().numpy()

    # -- stats ----------------------------------------------------------------
    def nbytes(self) -> int:
        """Device bytes of every cached view (factors, dense blocks, indices)."""
        return int(sum(v.nbytes for v in self._views.values()))

    def dense_equivalent_bytes(self) -> int:
        """Bytes of ONE dense FP64 material matrix."""
        return self.shape[0] * self.shape[1] * 8

    def view_nbytes(self, coeffs) -> int:
        return self._view(coeffs).nbytes

    def summary(self) -> str:
        ranks = [v.stats["ranks"] for v in self._views.values()]
        avg = float(np.mean(np.concatenate(ranks))) if ranks and sum(r.size for r in ranks) else 0.0
        return (f"PairCompressed {self.shape} [{len(self._views)} material view(s)]: {self.n_lowrank} admissible "
                f"blocks ({self.n_capped} dense at the rank cap, {self.n_retry} retried and {self.n_fallback} "
                f"exact after the retry; max certified err {self.max_verified_err:.1e}, avg rank {avg:.1f}), "
                f"{self.n_dense} dense leaf, {self.nbytes() / 1e6:.1f} MB held vs "
                f"{self.dense_equivalent_bytes() / 1e6:.1f} MB dense")
