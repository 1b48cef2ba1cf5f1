"""Host side of the compressed pair operator (``mbem_gb300.la.compressed``):
the cluster tree and partition against the reference's own
(``la/cluster.py`` build_cluster_tree / build_partition, written into
``tests/golden/compressed_small.npz`` by ``tests/golden/make_golden.py``),
the tree order that makes every block contiguous, the row strips of the flat
product, the rank caps, and the C port of the flat product."""

import numpy as np
import pytest

from conftest import golden_blocks


def _centroids(vertices, triangles):
    return np.asarray(vertices, float)[np.asarray(triangles)].mean(axis=1)


def _same_blocks(mine, ref):
    assert len(mine) == len(ref)
    for (r1, c1), (r2, c2) in zip(mine, ref):
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2)


def test_self_partition_matches_the_reference(compressed_small):
    """The 24x24-per-face cube's self pair: 1240 admissible and 4128 dense
    blocks, the same element sets in the same order."""
    from mbem_gb300.la import compressed as cm
    g = compressed_small
    tree = cm.cluster_tree(_centroids(g["self24_vertices"], g["self24_triangles"]))
    adm, dense = cm.partition_blocks(tree, tree)
    _same_blocks(adm, golden_blocks(g, "self24_adm"))
    _same_blocks(dense, golden_blocks(g, "self24_dense"))


@pytest.mark.parametrize("kernel", ["H", "G"])
def test_pair_partition_matches_the_reference(compressed_small, kernel):
    """Field: the cube's centroids, source: the centre fault."""
    from mbem_gb300.la import compressed as cm
    g = compressed_small
    tf = cm.cluster_tree(_centroids(g["cube_vertices"], g["cube_triangles"]))
    ts = cm.cluster_tree(_centroids(g["fault_vertices"], g["fault_triangles"]))
    adm, dense = cm.partition_blocks(tf, ts)
    _same_blocks(adm, golden_blocks(g, f"{kernel}_adm"))
    _same_blocks(dense, golden_blocks(g, f"{kernel}_dense"))
    assert len(adm) == int(g[f"{kernel}_n_lowrank"]) and len(dense) == int(g[f"{kernel}_n_dense"])


def _cube_tree(n_face=24):
    from mbem_gb300 import mesh
    from mbem_gb300.la import compressed as cm
    c = mesh.cube(n_face)
    tree = cm.cluster_tree(c.centroids())
    return c, tree, cm.tree_order(tree)


def test_tree_order_makes_every_block_contiguous():
    from mbem_gb300.la import compressed as cm
    c, tree, order = _cube_tree()
    assert np.array_equal(np.sort(order), np.arange(c.n_triangles))
    pos = np.empty_like(order)
    pos[order] = np.arange(order.size)
    adm, dense = cm.partition_nodes(tree, tree)
    for a, b in adm + dense:
        for node in (a, b):
            p = pos[node.indices]
            assert p.min() == node.start and p.max() == node.start + node.n - 1
    # the same order, recovered from the index sets alone
    blocks = [(a.indices, b.indices) for a, b in adm + dense]
    o2 = cm.laminar_order(c.n_triangles, [r for r, _ in blocks])
    pos2 = np.empty_like(o2)
    pos2[o2] = np.arange(o2.size)
    r0, nr, c0, nc = cm.block_ranges(blocks, pos2, pos2)
    assert int((nr.astype(np.int64) * nc).sum()) == c.n_triangles ** 2


def test_laminar_order_refuses_crossing_sets():
    from mbem_gb300.la import compressed as cm
    with pytest.raises(ValueError, match="laminar"):
        cm.laminar_order(6, [np.array([0, 1, 2]), np.array([2, 3])])
    with pytest.raises(ValueError, match="range"):
        cm.laminar_order(3, [np.array([0, 5])])
    o = cm.laminar_order(7, [np.array([5, 1]), np.array([1, 3, 5]), np.array([0, 2, 4, 6])])
    pos = np.empty_like(o)
    pos[o] = np.arange(7)
    for s in ([5, 1], [1, 3, 5], [0, 2, 4, 6]):
        p = np.sort(pos[s])
        assert p[-1] - p[0] + 1 == len(s)


def test_row_strips_cover_each_block_row_once():
    from mbem_gb300.la import compressed as cm
    rng = np.random.default_rng(3)
    n = 500
    bounds = np.unique(np.concatenate([[0, n], rng.integers(1, n, 40)]))
    # blocks: unions of consecutive intervals
    r0, nr = [], []
    for _ in range(60):
        i, j = np.sort(rng.choice(bounds.size, 2, replace=False))
        r0.append(bounds[i])
        nr.append(bounds[j] - bounds[i])
    r0, nr = np.array(r0), np.array(nr)
    s0, sn, sptr, items = cm.row_strips(n, r0, nr)
    assert s0[0] == 0 and (s0 + sn)[-1] == n and np.array_equal(s0[1:], (s0 + sn)[:-1])
    cover = np.zeros((r0.size, n), int)
    for s in range(s0.size):
        ids = items[sptr[s]:sptr[s + 1]]
        assert np.all(np.diff(ids) > 0)          # block order within a strip
        for b in ids:
            cover[b, s0[s]:s0[s] + sn[s]] += 1
    for b in range(r0.size):
        want = np.zeros(n, int)
        want[r0[b]:r0[b] + nr[b]] = 1
        assert np.array_equal(cover[b], want)


def test_strip_units_cover_every_factor_row_once():
    from mbem_gb300.la import compressed as cm
    rng = np.random.default_rng(8)
    sptr = np.array([0, 3, 3, 7, 8])                  # an empty strip in the middle
    items = rng.integers(0, 6, 8).astype(np.int32)
    rows = np.array([5, 32, 33, 64, 0, 100])          # factor rows of each block id
    uptr, uitem, uk0 = cm.strip_units(sptr, items, rows, unit=32)
    assert uptr[0] == 0 and uptr[-1] == uitem.size
    for s in range(sptr.size - 1):
        got = list(zip(uitem[uptr[s]:uptr[s + 1]], uk0[uptr[s]:uptr[s + 1]]))
        want = [(b, k) for b in items[sptr[s]:sptr[s + 1]] for k in range(0, max(rows[b], 1), 32)]
        assert got == want


def test_rank_caps_follow_the_reference_rule():
    from mbem_gb300.la import compressed as cm
    nr = np.array([64, 100, 1024, 20, 5, 300])
    nc = np.array([64, 1024, 1024, 20, 300, 5])
    # min(max(8, int(min(nr, nc) / 3)), nr, nc)
    assert list(cm.rank_caps(nr, nc)) == [21, 33, 341, 8, 5, 5]


def test_flat_product_port_on_a_handmade_view(oracle):
    """The C port of the flat product against numpy on random factors: two
    low-rank blocks, two dense blocks, a permuted element order."""
    from mbem_gb300.la import compressed as cm
    rng = np.random.default_rng(5)
    nf, ns = 7, 6
    fo, so = rng.permutation(nf), rng.permutation(ns)
    lr = [(0, 4, 0, 3, 2), (4, 3, 3, 3, 4)]            # r0, nr, c0, nc, rank (tree positions)
    dn = [(0, 4, 3, 3), (4, 3, 0, 3)]
    A = np.zeros((3 * nf, 3 * ns))
    U, V, lr_u, lr_v = [], [], [], []
    for r0, nr, c0, nc, k in lr:
        ldu, ldv = int(cm._pad4(3 * nr)), int(cm._pad4(3 * nc))
        u = rng.normal(size=(k, ldu)).astype(np.float32)
        v = rng.normal(size=(k, ldv)).astype(np.float32)
        u[:, 3 * nr:] = 0
        v[:, 3 * nc:] = 0
        lr_u.append(sum(x.size for x in U))
        lr_v.append(sum(x.size for x in V))
        U.append(u.ravel())
        V.append(v.ravel())
        blk = u[:, :3 * nr].astype(float).T @ v[:, :3 * nc].astype(float)
        rows = (3 * fo[r0:r0 + nr, None] + np.arange(3)).ravel()
        cols = (3 * so[c0:c0 + nc, None] + np.arange(3)).ravel()
        A[np.ix_(rows, cols)] += blk
    D, d_off = [], []
    for r0, nr, c0, nc in dn:
        ld = int(cm._pad4(3 * nr))
        d = rng.normal(size=(3 * nc, ld)).astype(np.float32)      # stored transposed
        d[:, 3 * nr:] = 0
        d_off.append(sum(x.size for x in D))
        D.append(d.ravel())
        rows = (3 * fo[r0:r0 + nr, None] + np.arange(3)).ravel()
        cols = (3 * so[c0:c0 + nc, None] + np.arange(3)).ravel()
        A[np.ix_(rows, cols)] += d[:, :3 * nr].astype(float).T
    all_r0 = np.array([b[0] for b in lr] + [b[0] for b in dn])
    all_nr = np.array([b[1] for b in lr] + [b[1] for b in dn])
    sr0, snr, sptr, sit = cm.row_strips(nf, all_r0, all_nr)
    ranks = np.array([b[4] for b in lr], np.int32)
    view = dict(n_field=nf, n_src=ns, field_order=fo.astype(np.int64), src_order=so.astype(np.int64),
                n_lr=2, lr_r0=np.array([b[0] for b in lr], np.int32), lr_nr=np.array([b[1] for b in lr], np.int32),
                lr_c0=np.array([b[2] for b in lr], np.int32), lr_nc=np.array([b[3] for b in lr], np.int32),
                lr_rank=ranks, lr_u=np.array(lr_u, np.int64), lr_v=np.array(lr_v, np.int64),
                lr_w=cm._exclusive(ranks), U=np.concatenate(U), V=np.concatenate(V), n_w=int(ranks.sum()),
                d_r0=np.array([b[0] for b in dn], np.int32), d_nr=np.array([b[1] for b in dn], np.int32),
                d_nc=np.array([b[3] for b in dn], np.int32),
                d_c0=np.array([b[2] for b in dn], np.int32), d_off=np.array(d_off, np.int64), D=np.concatenate(D),
                n_strips=sr0.size, strip_r0=sr0, strip_nr=snr, strip_ptr=sptr, strip_items=sit)
    x = rng.normal(size=3 * ns)
    y = oracle.flat_matvec(view, x)
    assert np.abs(y - A @ x).max() < 1e-12 * np.abs(A).sum(axis=1).max() * np.abs(x).max() * 10
