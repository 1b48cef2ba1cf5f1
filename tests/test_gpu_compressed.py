"""The GPU compressed pair operator (``mbem_gb300.la.compressed``) against
the reference's ``PairCompressed`` (``la/hop.py``) on its own partition and
material (``tests/golden/compressed_small.npz``: the 12x12-per-face cube's
centroids as field points, the 16x16 centre fault as sources, both kernels),
against the FP64 dense operator block by block, against the C port of the
flat product on the same factors, and on its edge cases.

Tolerances. Every admissible block is certified to ACA_CERTIFY_FACTOR x tol
(3e-4) on sampled rows and columns, so a product differs from the exact one,
and from the reference's (whose blocks carry the same kind of error), by a
small multiple of 1e-4 at most; the whole-block errors asserted here are the
same bound with a factor of 3 for what the sample does not see. Dense blocks
hold FP32 entries of the far quadrature or the FP64 closed form (<= 1e-6)."""

import numpy as np
import pytest
import torch

from conftest import golden_blocks

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _mesh(v, t):
    from mbem_gb300.mesh import TriMesh
    return TriMesh(np.asarray(v, float), np.asarray(t, np.int64))


def _dofs(e):
    e = np.asarray(e)
    return (3 * e[:, None] + np.arange(3)).ravel()


def _exact(kernel, field_mesh, source_mesh, eps, coeffs):
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.kernels import tri_nodal as tn
    a = kb.MeshArrays()
    x = a.field_points(field_mesh)
    tv, nrm = a.source_arrays(source_mesh)
    e = np.full(tv.shape[0], float(eps))
    if kernel == "H":
        return tn.t_matrix_direct(x, tv, nrm, e, *coeffs)
    return tn.u_matrix_direct(x, tv, e, *coeffs)


def _block_errors(pc, coeffs, A):
    D = pc.to_dense(coeffs)
    st = pc.view_stats(coeffs)
    low = (st["status"] & 3) == 0
    lr, ex = [], []
    for (rows, cols), is_low in zip(pc.admissible, low):
        ri, ci = _dofs(rows), _dofs(cols)
        B = A[np.ix_(ri, ci)]
        (lr if is_low else ex).append(np.linalg.norm(D[np.ix_(ri, ci)] - B) / np.linalg.norm(B))
    for rows, cols in pc.dense:
        ri, ci = _dofs(rows), _dofs(cols)
        B = A[np.ix_(ri, ci)]
        ex.append(np.linalg.norm(D[np.ix_(ri, ci)] - B) / max(np.linalg.norm(B), 1e-300))
    return np.array(lr), np.array(ex), D


@pytest.fixture(scope="module")
def golden_pair(compressed_small):
    g = compressed_small
    return g, _mesh(g["cube_vertices"], g["cube_triangles"]), _mesh(g["fault_vertices"], g["fault_triangles"])


@pytest.mark.parametrize("kernel", ["H", "G"])
def test_matches_the_reference_operator(golden_pair, kernel):
    from mbem_gb300.la.compressed import PairCompressed
    g, cube, fault = golden_pair
    part = (golden_blocks(g, f"{kernel}_adm"), golden_blocks(g, f"{kernel}_dense"))
    c = g[f"{kernel}_coeffs"]
    pc = PairCompressed(cube, fault, kernel, float(g["eps"]), partition=part)
    assert pc.n_lowrank == int(g[f"{kernel}_n_lowrank"]) and pc.n_dense == int(g[f"{kernel}_n_dense"])
    x = g["x"]
    y = pc.matvec(c, x)
    y_ref = g[f"{kernel}_y"]
    A = _exact(kernel, cube, fault, g["eps"], c)
    ye = A @ x
    err_ref = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
    err_exact = np.linalg.norm(y - ye) / np.linalg.norm(ye)
    err_ref_exact = np.linalg.norm(y_ref - ye) / np.linalg.norm(ye)
    print(f"{kernel}: |y - y_ref| {err_ref:.2e}, |y - y_exact| {err_exact:.2e}, reference's own "
          f"{err_ref_exact:.2e}; {pc.summary()}")
    assert err_ref < TOL and err_exact < TOL
    assert pc.max_verified_err <= 3 * TOL
    # recompressed, the factors' ranks are the reference's to within a quarter
    ranks = pc.view_stats(c)["ranks"]
    print(f"{kernel}: mean rank {ranks.mean():.1f} against the reference's {g[f'{kernel}_ranks'].mean():.1f}")
    assert ranks.mean() <= 1.25 * g[f"{kernel}_ranks"].mean()
    lr, ex, _ = _block_errors(pc, c, A)
    assert lr.size > 0 and lr.max() < 3 * 3 * TOL
    assert ex.max() < 1e-6


@pytest.mark.parametrize("kernel", ["H", "G"])
def test_self_pair_blocks_against_the_dense_operator(kernel):
    """The 16x16-per-face cube's self pair with the operator's own partition:
    admissible blocks at several tree levels, near pairs in the FP64 closed
    form, and a bitwise-repeatable product."""
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(16)
    eps = (4.0 / 16) / 2
    c = kb.t_coeffs(1.0, 1.0) if kernel == "H" else kb.u_coeffs(1.0, 1.0)
    pc = PairCompressed(cube, cube, kernel, eps)
    assert pc.n_lowrank > 0
    x = np.random.default_rng(2).normal(size=3 * cube.n_triangles)
    y = pc.matvec(c, x)
    assert np.array_equal(y, pc.matvec(c, x))
    A = _exact(kernel, cube, cube, eps, c)
    ye = A @ x
    assert np.linalg.norm(y - ye) / np.linalg.norm(ye) < TOL
    lr, ex, D = _block_errors(pc, c, A)
    assert lr.max() < 3 * 3 * TOL and np.median(lr) < TOL
    assert ex.max() < 1e-6
    # the product is the dense matrix it stands for
    assert np.linalg.norm(D @ x - y) / np.linalg.norm(y) < 1e-6


def test_product_matches_the_c_port_on_the_same_factors(oracle):
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(16)
    c = kb.t_coeffs(1.0, 0.5)
    pc = PairCompressed(cube, cube, "H", 0.125)
    x = np.random.default_rng(4).normal(size=3 * cube.n_triangles)
    y = pc.matvec(c, x)
    y_port = oracle.flat_matvec(pc.view_host(c), x)
    assert np.linalg.norm(y - y_port) / np.linalg.norm(y_port) < 1e-6


def test_recompression_keeps_the_operator():
    """With and without the recompression of the cross approximation's
    factors: the same operator to the tolerance, fewer factor columns."""
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(16)
    c = kb.t_coeffs(1.0, 1.0)
    raw = PairCompressed(cube, cube, "H", 0.125, recompress_max=0)
    rec = PairCompressed(cube, cube, "H", 0.125)
    x = np.random.default_rng(9).normal(size=3 * cube.n_triangles)
    ye = _exact("H", cube, cube, 0.125, c) @ x
    for pc in (raw, rec):
        y = pc.matvec(c, x)
        assert np.linalg.norm(y - ye) / np.linalg.norm(ye) < TOL
    sr, sw = rec.view_stats(c), raw.view_stats(c)
    assert sr["n_recompressed"] > 0 and sw["n_recompressed"] == 0
    assert sr["ranks"].sum() < sw["ranks"].sum()
    assert sr["max_verified_err"] <= 3 * TOL


def test_tight_tolerance_leaves_blocks_exact():
    """At tol = 1e-8 the FP32 cross approximation cannot certify a block (or
    reaches the rank cap): every admissible block is applied exactly and the
    product is the dense operator's to FP32 storage."""
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(16)
    c = kb.u_coeffs(1.0, 1.0)
    pc = PairCompressed(cube, cube, "G", 0.125, tol=1e-8)
    x = np.random.default_rng(6).normal(size=3 * cube.n_triangles)
    y = pc.matvec(c, x)
    st = pc.view_stats(c)
    assert pc.n_capped + pc.n_fallback == pc.n_lowrank
    assert st["ranks"].size == 0 and st["lowrank_bytes"] == 0
    ye = _exact("G", cube, cube, 0.125, c) @ x
    assert np.linalg.norm(y - ye) / np.linalg.norm(ye) < 1e-6


def test_loose_tolerance_stays_within_it():
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(16)
    c = kb.t_coeffs(1.0, 1.0)
    tol = 1e-2
    pc = PairCompressed(cube, cube, "H", 0.125, tol=tol)
    pc4 = PairCompressed(cube, cube, "H", 0.125)
    x = np.random.default_rng(7).normal(size=3 * cube.n_triangles)
    y = pc.matvec(c, x)
    ye = _exact("H", cube, cube, 0.125, c) @ x
    assert np.linalg.norm(y - ye) / np.linalg.norm(ye) < tol
    assert pc.max_verified_err <= 3 * tol
    assert pc.view_stats(c)["ranks"].mean() < pc4.view_stats(c)["ranks"].mean()


def test_device_vectors_and_view_cache():
    from mbem_gb300 import defaults, mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(8)
    pc = PairCompressed(cube, cube, "G", 0.25)
    x = torch.randn(3 * cube.n_triangles, dtype=torch.float64, device="cuda")
    y = pc.matvec(kb.u_coeffs(1.0, 1.0), x)
    assert isinstance(y, torch.Tensor) and y.is_cuda
    y_host = pc.matvec(kb.u_coeffs(1.0, 1.0), x.cpu().numpy())
    assert np.array_equal(y.cpu().numpy(), y_host)
    for k in range(defaults.COMPRESSED_VIEW_CACHE + 2):
        pc.matvec(kb.u_coeffs(1.0 + k, 1.0), x)
    assert len(pc._views) == defaults.COMPRESSED_VIEW_CACHE
    assert pc.nbytes() > 0 and "admissible blocks" in pc.summary()


def test_bad_inputs_are_refused():
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la import compressed as cm
    cube = mesh.cube(8)
    with pytest.raises(ValueError):
        cm.PairCompressed(cube, cube, "Ht", 0.25)
    pc = cm.PairCompressed(cube, cube, "H", 0.25)
    with pytest.raises(ValueError, match="coefficients"):
        pc.matvec(kb.u_coeffs(1.0, 1.0), np.zeros(3 * cube.n_triangles))
    with pytest.raises(ValueError, match="entries"):
        pc.matvec(kb.t_coeffs(1.0, 1.0), np.zeros(5))
    adm, dense = pc.admissible, pc.dense
    with pytest.raises(ValueError, match="covers"):
        cm.PairCompressed(cube, cube, "H", 0.25, partition=(adm, dense[:-1]))
    with pytest.raises(ValueError, match="eps"):
        cm.PairCompressed(cube, cube, "H", -1.0)
