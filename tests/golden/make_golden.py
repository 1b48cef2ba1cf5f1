"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a container that holds the reference sources (read-only) at
``/root/reference``; the GPU tests never run this script, they only read the
``.npz`` files it writes. numba is absent here, so a test-only stand-in
(``_numba_stub``: identity ``njit``, ``prange = range``) is put first on
``sys.path``; the reference's kernels then run as plain Python with the same
arithmetic.

    python tests/golden/make_golden.py p0_pairs cube_small c1_rows

Every fixture stores its inputs next to the reference's outputs, so the
tests feed the identical arrays to the CUDA path and to the C oracle.
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/src"
sys.dont_write_bytecode = True
sys.path[:0] = [os.path.join(HERE, "_numba_stub"), REF_SRC]


def _ref():
    import mbem.kernels.tri_kernels as tk
    import mbem.kernels.basis as kb
    return tk, kb


# ---------------------------------------------------------------------------
# P0 pair kernels on scattered geometry with edge cases
# ---------------------------------------------------------------------------

def pair_geometry(seed: int = 1234):
    """Scattered sources and observers, with the cases the reference guards:
    a degenerate (collinear) triangle, a needle, a tiny and a large
    triangle, reversed source normals, observers on a vertex, on an edge, at
    a centroid, coplanar outside, on an edge's extension, far away and just
    above a centroid."""
    rng = np.random.default_rng(seed)
    tv = rng.normal(size=(16, 3, 3))
    needle = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, 2e-3, 0.0]]) + 0.3
    tiny = rng.normal(size=(3, 3)) * 1e-3 + np.array([0.2, -0.1, 0.4])
    large = rng.normal(size=(3, 3)) * 10.0
    degen = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [2.0, 2.0, 2.0]])
    tv = np.concatenate([tv, needle[None], tiny[None], large[None], degen[None]])
    Ns = tv.shape[0]
    cr = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
    nrm = np.linalg.norm(cr, axis=1)
    normals = np.where(nrm[:, None] > 0, cr / np.where(nrm > 0, nrm, 1.0)[:, None],
                       np.array([0.0, 0.0, 1.0]))
    normals[[2, 7, 11]] *= -1.0                      # reversed normals
    eps = rng.uniform(0.05, 0.3, Ns)
    x = rng.normal(size=(24, 3)) * 1.5
    special = [
        tv[0, 0],                                    # on a vertex
        0.5 * (tv[1, 0] + tv[1, 1]),                 # on an edge
        tv[2].mean(axis=0),                          # at a centroid
        tv[3, 0] + 2.0 * (tv[3, 1] - tv[3, 0]) + 1.5 * (tv[3, 2] - tv[3, 0]),  # coplanar outside
        tv[4, 0] + 3.0 * (tv[4, 1] - tv[4, 0]),      # on an edge's line, outside
        np.array([50.0, -30.0, 20.0]),               # far
        tv[5].mean(axis=0) + 1e-9 * normals[5],      # just above a centroid
    ]
    x = np.concatenate([x, np.array(special)])
    density = rng.normal(size=(Ns, 3))
    density[6] = 0.0
    density[9] = 0.0
    density[10, 1] = 0.0
    return (np.ascontiguousarray(x), np.ascontiguousarray(tv),
            np.ascontiguousarray(normals), np.ascontiguousarray(eps),
            np.ascontiguousarray(density))


MATERIALS = np.array([[1.0, 1.0], [1.3, 1.95]])      # nu = 0.25 and nu = 0.30


def make_p0_pairs(path):
    tk, kb = _ref()
    x, tv, n, eps, dens = pair_geometry()
    out = dict(x_field=x, tri_verts=tv, normals=n, eps=eps, density=dens,
               materials=MATERIALS)
    t0 = time.time()
    out["t_basis"] = tk.t_basis_matrices(x, tv, n, eps)
    out["u_basis"] = tk.u_basis_matrices(x, tv, eps)
    for m, (mu, lam) in enumerate(MATERIALS):
        c = kb.t_coeffs(mu, lam)
        g = kb.u_coeffs(mu, lam)
        out[f"t_coeffs_{m}"] = c
        out[f"u_coeffs_{m}"] = g
        out[f"t_matrix_{m}"] = tk.t_matrix_direct(x, tv, n, eps, *c)
        out[f"u_matrix_{m}"] = tk.u_matrix_direct(x, tv, eps, *g)
        out[f"t_disp_{m}"] = tk.t_disp_contract(x, tv, n, eps, dens, *c)
        out[f"u_disp_{m}"] = tk.u_disp_contract(x, tv, eps, dens, *g)
        out[f"dd_stress_{m}"] = tk.dd_stress_contract(x, tv, n, eps, dens, mu, lam)
        out[f"kelvin_stress_{m}"] = tk.kelvin_stress_contract(x, tv, eps, dens, mu, lam)
        out[f"eigenstress_{m}"] = tk.eigenstress_contract(x, tv, n, eps, dens, mu, lam)
    print(f"p0_pairs: {time.time() - t0:.1f} s")
    np.savez_compressed(path, **out)


# ---------------------------------------------------------------------------
# Whole dense systems: cube + fault through the reference's own backend
# ---------------------------------------------------------------------------

def reference_cube_model(n_face: int, n_fault: int, mu: float, lam: float,
                         side: float = 4.0):
    """The traction-free cube with an embedded vertical fault, built with the
    reference's own mesh generators and model API."""
    import local_box_mesh as lbm
    from mollified_bem import ElasticMaterial
    from mbem.model import BCType, Patch, Region, RegionModel

    a = side / 2.0
    faces = [
        lbm.make_rectangular_patch((-a, a), (-a, a), a, n_face, n_face, normal_up=True),
        lbm.make_rectangular_patch((-a, a), (-a, a), -a, n_face, n_face, normal_up=False),
        lbm.make_vertical_panel("x", a, (-a, a), (-a, a), n_face, n_face, +1),
        lbm.make_vertical_panel("x", -a, (-a, a), (-a, a), n_face, n_face, -1),
        lbm.make_vertical_panel("y", a, (-a, a), (-a, a), n_face, n_face, +1),
        lbm.make_vertical_panel("y", -a, (-a, a), (-a, a), n_face, n_face, -1),
    ]
    cube = lbm._concatenate_meshes(faces)
    fmesh, _, _ = lbm.make_vertical_fault_xy(1.0, (-1.0, 0.0), n_fault, n_fault,
                                             strike_azimuth_deg=90.0)
    fmesh.vertices = fmesh.vertices + np.array([0.0, 0.0, 0.5])
    mat = ElasticMaterial(mu=mu, lam=lam)
    cube_p = Patch("cube", cube, BCType.FREE_TRACTION)
    fault_p = Patch("fault", fmesh, BCType.FAULT, value=np.array([1.0, 0.0, 0.0]))
    region = Region("body", mat, [cube_p], np.zeros(3), faults=[fault_p])
    return RegionModel([region]), cube, fmesh


def _system_fixture(n_face, n_fault, mu, lam, mode, points, rows=None,
                    fgmres_rtols=()):
    from mbem.backends.dense import AssembledDense, translation_basis
    from mbem.evaluate import evaluate_stress
    from mbem.model.equations import generate_system

    model, cube, fmesh = reference_cube_model(n_face, n_fault, mu, lam)
    eps = (4.0 / n_face) / 2.0
    t0 = time.time()
    system = generate_system(model)
    asm = AssembledDense(system, eps, mode, jump="calibrated", deflate=True)
    t1 = time.time()
    sol = asm.solve()
    t2 = time.time()
    out = dict(cube_vertices=cube.vertices, cube_triangles=cube.triangles,
               fault_vertices=fmesh.vertices, fault_triangles=fmesh.triangles,
               mu=mu, lam=lam, eps=eps, n_face=n_face, n_fault=n_fault,
               b=asm.b, x=sol["u:cube"].ravel(), cond=asm.report.cond_estimate,
               calib=next(iter(asm.calib.values())), assembly_s=t1 - t0,
               lu_s=t2 - t1)
    if rows is None:
        out["A"] = asm.A
    else:
        out["A_rows"] = np.ascontiguousarray(asm.A[rows])
        out["rows"] = np.asarray(rows, np.int64)
    # deflated FGMRES, the pairing the GPU backend uses
    if fgmres_rtols:
        from mbem.la.solver import fgmres
        Z = translation_basis(asm.layout)

        def proj(v):
            return v - Z @ (Z.T @ v)

        its = []
        for rtol in fgmres_rtols:
            xg, rep = fgmres(lambda v: proj(asm.A @ proj(v)), proj(asm.b),
                             rtol=rtol, restart=50, maxiter=600)
            its.append([rtol, rep.iterations, rep.true_relres,
                        float(np.linalg.norm(proj(xg) - out["x"]) / np.linalg.norm(out["x"]))])
        out["fgmres"] = np.array(its)
    t3 = time.time()
    sig, eig = evaluate_stress(model, "body", sol, points, eps,
                               subtract_anelastic=True, parts=True)
    out.update(points=points, stress=sig, stress_eigen=eig, readout_s=time.time() - t3)
    print(f"system n={n_face}: assembly {t1 - t0:.1f} s, LU {t2 - t1:.1f} s, "
          f"readout {time.time() - t3:.1f} s")
    return out


def make_cube_small(path):
    rng = np.random.default_rng(7)
    pts = rng.uniform(-1.5, 1.5, size=(10, 3))
    pts = np.concatenate([pts, [[0.1, 0.05, 0.2], [0.0, 0.0, 0.0], [0.45, -0.02, -0.3]]])
    out = _system_fixture(3, 2, 1.0, 1.0, "direct", pts)
    out2 = _system_fixture(2, 2, 1.3, 1.95, "direct", pts[:6])
    out.update({f"nu30_{k}": v for k, v in out2.items()})
    np.savez_compressed(path, **out)


def make_c1_rows(path):
    """Config-1 cube (12x12 per face, fault 8x8, eps = h/2): sampled rows of
    A, the full b, the deflated LU solution, FGMRES(50) iteration counts and a
    readout subset of the 64x64 grid on y = 0.1."""
    g = (np.arange(64) + 0.5) / 64.0 * 4.0 - 2.0
    X, Zc = np.meshgrid(g, g, indexing="xy")
    grid = np.column_stack([X.ravel(), np.full(X.size, 0.1), Zc.ravel()])
    pick = np.random.default_rng(11).choice(grid.shape[0], 16, replace=False)
    rng = np.random.default_rng(3)
    rows = np.unique(np.concatenate([[0, 1, 2, 2591, 2592, 5181, 5182, 5183],
                                     rng.choice(5184, 16, replace=False)]))
    out = _system_fixture(12, 8, 1.0, 1.0, "legacy", grid[pick], rows=rows,
                          fgmres_rtols=(1e-8, 1e-10))
    out["grid_index"] = pick
    np.savez_compressed(path, **out)


def make_nodal_pairs(path):
    """The order-generic public drivers (tri_nodal.py:1257-1404) at orders 1
    and 2, and the traction rows at orders 0, 1 and 2, on the scattered
    geometry (the collinear triangle dropped: nodal orders refuse it) plus
    observers far enough for both Gauss rules (D > 10 L and D > 40 L)."""
    import mbem.kernels.tri_nodal as tn
    _, kb = _ref()
    x, tv, n, eps, _ = pair_geometry()
    tv, n, eps = tv[:-1], n[:-1], eps[:-1]
    rng = np.random.default_rng(77)
    far = rng.normal(size=(6, 3))
    far = far / np.linalg.norm(far, axis=1)[:, None] * np.array([25.0, 30.0, 45.0, 80.0, 120.0, 200.0])[:, None]
    x = np.ascontiguousarray(np.concatenate([x, far]))
    nf = rng.normal(size=x.shape)
    nf = np.ascontiguousarray(nf / np.linalg.norm(nf, axis=1)[:, None])
    out = dict(x_field=x, n_field=nf, tri_verts=tv, normals=n, eps=eps, materials=MATERIALS)
    t0 = time.time()
    for order in (1, 2):
        K = tn.n_nodes(order)
        dens = rng.normal(size=(K * tv.shape[0], 3))
        dens[3 * K:4 * K] = 0.0
        out[f"density_{order}"] = dens
        mu, lam = MATERIALS[0]
        c = kb.t_coeffs(mu, lam)
        g = kb.u_coeffs(mu, lam)
        out[f"t_matrix_{order}"] = tn.t_matrix_direct(x, tv, n, eps, *c, order)
        out[f"u_matrix_{order}"] = tn.u_matrix_direct(x, tv, eps, *g, order)
        out[f"t_disp_{order}"] = tn.t_disp_contract(x, tv, n, eps, dens, *c, order)
        out[f"u_disp_{order}"] = tn.u_disp_contract(x, tv, eps, dens, *g, order)
        for m, (mu, lam) in enumerate(MATERIALS):
            out[f"dd_stress_{order}_{m}"] = tn.dd_stress_contract(x, tv, n, eps, dens, mu, lam, order)
            out[f"kelvin_stress_{order}_{m}"] = tn.kelvin_stress_contract(x, tv, eps, dens, mu, lam, order)
            out[f"eigenstress_{order}_{m}"] = tn.eigenstress_contract(x, tv, n, eps, dens, mu, lam, order)
        print(f"nodal order {order}: {time.time() - t0:.1f} s", flush=True)
    for order in (0, 1, 2):
        ids = kb.identity_ids(order, tv.shape[0])
        for which in ("slip", "force", "eigen", "total"):
            mu, lam = MATERIALS[1 if which == "slip" else 0]
            out[f"traction_{order}_{which}"] = tn.traction_matrix(x, nf, tv, n, eps, ids, ids.size, mu, lam,
                                                                  order, which)
        print(f"traction order {order}: {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(path, **out)


def make_traction_small(path):
    """A FAULT_TRACTION fault (solved slip under a uniform shear-traction
    drop, order 0) in a 2x2-per-face cube: the reference's whole system with
    traction rows, the fault-row frame and the constraint rows, and its LU
    solution."""
    import local_box_mesh as lbm
    from mollified_bem import ElasticMaterial
    from mbem.backends.dense import AssembledDense
    from mbem.model import BCType, Patch, Region, RegionModel
    from mbem.model.equations import generate_system

    model_ref, cube, fmesh = reference_cube_model(2, 2, 1.0, 1.0)
    mat = ElasticMaterial(mu=1.0, lam=1.0)
    drop = np.array([-1e-3, 0.0, 0.0])
    cube_p = Patch("cube", cube, BCType.FREE_TRACTION)
    fault_p = Patch("fault", fmesh, BCType.FAULT_TRACTION, value=drop)
    model = RegionModel([Region("body", mat, [cube_p], np.zeros(3), faults=[fault_p])])
    eps = (4.0 / 2) / 2.0
    t0 = time.time()
    asm = AssembledDense(generate_system(model), eps, "direct", jump="calibrated", deflate=True)
    sol = asm.solve()
    print(f"traction_small: {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(path, cube_vertices=cube.vertices, cube_triangles=cube.triangles,
                        fault_vertices=fmesh.vertices, fault_triangles=fmesh.triangles, eps=eps,
                        drop=drop, A=asm.A, b=asm.b, x_u=sol["u:cube"], x_b=sol["b:fault"])


def make_condense_small(path):
    """``AssembledDense.condense()`` of the reference on an anchored body: a
    3x3-per-face cube with prescribed (zero) displacement and a 3x3
    FAULT_TRACTION fault under a shear drop. Two cases: strike and dip
    enforced with the fault elements at |x| > 0.3 locked ("tangential"), and
    all three components enforced with no lock ("opening"). Stored per case:
    S, L, X, x0, the free nodes, the frame rows, the coordinate range and the
    LAPACK condition estimate of the eliminated block."""
    import local_box_mesh as lbm  # noqa: F401  (the reference's generators, through reference_cube_model)
    from mollified_bem import ElasticMaterial
    from mbem.backends.dense import AssembledDense
    from mbem.model import BCType, Patch, Region, RegionModel
    from mbem.model.equations import generate_system

    _, cube, fmesh = reference_cube_model(3, 3, 1.0, 1.0)
    mat = ElasticMaterial(mu=1.0, lam=1.0)
    eps = (4.0 / 3) / 2.0
    cent = fmesh.vertices[fmesh.triangles].mean(axis=1)
    locked = np.abs(cent[:, 0]) > 0.3
    out = dict(cube_vertices=cube.vertices, cube_triangles=cube.triangles, fault_vertices=fmesh.vertices,
               fault_triangles=fmesh.triangles, eps=eps, locked=locked)
    cases = {"tangential": dict(value=np.array([-1e-3, 0.0, 0.0]), allow_opening=False, locked=locked),
             "opening": dict(value=np.array([-1e-3, 2e-4, 0.0]), allow_opening=True, locked=None)}
    for tag, kw in cases.items():
        t0 = time.time()
        cube_p = Patch("cube", cube, BCType.PRESCRIBED_DISPLACEMENT, value=np.zeros(3))
        fault_p = Patch("fault", fmesh, BCType.FAULT_TRACTION, **kw)
        model = RegionModel([Region("body", mat, [cube_p], np.zeros(3), faults=[fault_p])])
        asm = AssembledDense(generate_system(model), eps, "direct", jump="calibrated", deflate=False)
        c = asm.condense()
        (fc,) = c.faults
        out.update({f"{tag}_S": c.S, f"{tag}_L": c.L, f"{tag}_X": c.X, f"{tag}_x0": c.x0,
                    f"{tag}_free": fc.free, f"{tag}_frame": fc.frame, f"{tag}_range": np.array([fc.start, fc.stop]),
                    f"{tag}_cond": c.cond_estimate, f"{tag}_value": kw["value"],
                    f"{tag}_x": asm.solve()["b:fault"]})
        print(f"condense_small {tag}: {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(path, **out)


def make_compressed_small(path):
    """The reference's compressed pair operator (``la/hop.py``
    ``PairCompressed``, default tolerance and partition rules) for the pair
    (field: the 12x12-per-face cube's centroids, source: the 16x16 centre
    fault, eps = h_fault / 2), both kernels: its partition (admissible and
    dense blocks as element index lists), its statistics, and its material
    view (mu = lam = 1) applied to a seeded random vector. Also the
    partition alone (no kernel work) of the 24x24-per-face cube's self pair,
    whose tree has admissible blocks at several levels."""
    from mbem.la.cluster import build_cluster_tree, build_partition
    from mbem.la.hop import PairCompressed
    import mbem.kernels.basis as kb

    def flat(blocks):
        rows = np.concatenate([r for r, _ in blocks]) if blocks else np.zeros(0, np.int64)
        cols = np.concatenate([c_ for _, c_ in blocks]) if blocks else np.zeros(0, np.int64)
        rp = np.concatenate([[0], np.cumsum([len(r) for r, _ in blocks])])
        cp = np.concatenate([[0], np.cumsum([len(c_) for _, c_ in blocks])])
        return rows, cols, rp, cp

    out = {}
    _, cube24, _ = reference_cube_model(24, 8, 1.0, 1.0)
    tree = build_cluster_tree(kb.MeshArrays().field_points(cube24))
    part = build_partition(tree, tree)
    for key, blocks in (("self24_adm", part.admissible), ("self24_dense", part.dense)):
        r, c_, rp, cp = flat(blocks)
        out.update({f"{key}_rows": r, f"{key}_cols": c_, f"{key}_rptr": rp, f"{key}_cptr": cp})
    out["self24_vertices"] = cube24.vertices
    out["self24_triangles"] = cube24.triangles
    print(f"compressed_small: cube-24 self partition {len(part.admissible)} admissible, "
          f"{len(part.dense)} dense", flush=True)

    _, cube, fault = reference_cube_model(12, 16, 1.0, 1.0)
    eps = (1.0 / 16) / 2.0
    x = np.random.default_rng(12).normal(size=3 * fault.n_triangles)
    out.update(cube_vertices=cube.vertices, cube_triangles=cube.triangles, fault_vertices=fault.vertices,
               fault_triangles=fault.triangles, eps=eps, x=x)
    for kernel, coeffs in (("H", kb.t_coeffs(1.0, 1.0)), ("G", kb.u_coeffs(1.0, 1.0))):
        t0 = time.time()
        pc = PairCompressed(cube, fault, kernel, np.full(fault.n_triangles, eps), n_workers=1)
        y = pc.matvec(coeffs, x)
        p = pc._part
        ar, ac, arp, acp = flat(p.admissible)
        dr, dc, drp, dcp = flat(p.dense)
        print(f"compressed_small {kernel}: {time.time() - t0:.1f} s; {pc.summary()}", flush=True)
        view = pc._view(coeffs)
        out.update({f"{kernel}_coeffs": coeffs, f"{kernel}_y": y, f"{kernel}_adm_rows": ar,
                    f"{kernel}_adm_cols": ac, f"{kernel}_adm_rptr": arp, f"{kernel}_adm_cptr": acp,
                    f"{kernel}_dense_rows": dr, f"{kernel}_dense_cols": dc, f"{kernel}_dense_rptr": drp,
                    f"{kernel}_dense_cptr": dcp, f"{kernel}_n_lowrank": pc.n_lowrank,
                    f"{kernel}_n_dense": pc.n_dense, f"{kernel}_n_capped": pc.n_capped,
                    f"{kernel}_n_retry": pc.n_retry, f"{kernel}_n_fallback": pc.n_fallback,
                    f"{kernel}_max_verified_err": pc.max_verified_err, f"{kernel}_tol": pc.tol,
                    f"{kernel}_ranks": np.asarray(view.ranks), f"{kernel}_nbytes": view.nbytes()})
    np.savez_compressed(path, **out)


def make_volume_small(path):
    """The volume sampler on the small cube + fault system (3 x 3 per face,
    fault 2 x 2, eps = h/2): a padded grid with points outside the body, its
    region codes, clearances and sampled fields; a section grid; and, on
    scattered points (some on a face, some just off one), the closure sums
    of point_in_region, the exact distances to both meshes and on_patch."""
    from mbem import volume
    from mbem.backends.dense import AssembledDense
    from mbem.geometry import distance_to_mesh
    from mbem.model.equations import generate_system

    t0 = time.time()
    model, cube, fmesh = reference_cube_model(3, 2, 1.0, 1.0)
    eps = (4.0 / 3) / 2.0
    asm = AssembledDense(generate_system(model), eps, "direct", jump="calibrated", deflate=True)
    sol = asm.solve()
    region = model.regions[0]
    grid = volume.make_grid(model, 1.0, pad=1.0)
    section = volume.section_grid(model, "y", 0.1, 0.5)
    code = volume.classify(model, grid)
    c_h, c_eps, c_fault = volume.clearance(model, grid, eps)
    fields = volume.sample(model, sol, eps, grid, code, eigenstress=True)
    half = {k: 0.5 * fields[k] for k in volume.PRIMARY}
    diff = volume.difference(fields, half, code > 0)
    vti = volume.as_vti_arrays(grid, fields, code, c_h, c_eps, c_fault)
    rng = np.random.default_rng(11)
    sc = rng.uniform(-3.0, 3.0, size=(48, 3))
    near = np.array([[2.0 - 1e-3, 0.3, 0.2], [2.0 + 1e-3, 0.3, 0.2], [0.1, -2.0 + 1e-6, 0.4],
                     [0.2, 0.3, 1.999999], [1.9, 1.95, -1.97], [0.0, 1e-3, 0.0], [0.3, -0.05, 0.45]])
    on_face = np.array([[2.0, 0.3, 0.1], [-0.7, -2.0, 1.2], [0.5, 0.25, 2.0], [2.0, 2.0, 0.4]])
    sc_pts = np.concatenate([sc, near])
    inside, total = model.point_in_region(region, sc_pts, closure=True)
    all_pts = np.concatenate([sc_pts, on_face])
    d_cube, i_cube = distance_to_mesh(all_pts, cube)
    d_fault, i_fault = distance_to_mesh(all_pts, fmesh)
    onp = volume.on_patch(all_pts, region.patches[0])
    out = dict(cube_vertices=cube.vertices, cube_triangles=cube.triangles,
               fault_vertices=fmesh.vertices, fault_triangles=fmesh.triangles, eps=eps,
               x=sol["u:cube"], grid_points=grid.points, grid_origin=np.array(grid.origin),
               grid_dims=np.array(grid.dims), section_points=section.points,
               section_origin=np.array(section.origin), section_dims=np.array(section.dims),
               code=code, c_h=c_h, c_eps=c_eps, c_fault=c_fault,
               sc_points=sc_pts, sc_inside=inside, sc_total=total, all_points=all_pts,
               d_cube=d_cube, i_cube=i_cube, d_fault=d_fault, i_fault=i_fault, on_patch=onp,
               vti_keys=np.array(sorted(vti)), vti_sigma_xy=vti["sigma_xy"], vti_u=vti["u"])
    out.update({f"f_{k}": v for k, v in fields.items()})
    out.update({f"d_{k}": v for k, v in diff.items()})
    np.savez_compressed(path, **out)
    print(f"volume_small: {time.time() - t0:.1f} s", flush=True)


def make_volume_regions(path):
    """Region codes and clearances of the reference's volume module on a
    two-region model: a traction-free host cube of side 4 (3 x 3 per face)
    with an inclusion cube of side 2 (2 x 2 per face) whose surface is an
    INTERFACE patch of both regions. Points: a padded grid, points ON the
    interface (faces, an edge, a corner), 1e-6 either side of it, and on the
    outer surface; with each region's closure sums."""
    import local_box_mesh as lbm
    from mollified_bem import ElasticMaterial
    from mbem import volume
    from mbem.model import BCType, Patch, Region, RegionModel

    def box(a, n):
        return lbm._concatenate_meshes([
            lbm.make_rectangular_patch((-a, a), (-a, a), a, n, n, normal_up=True),
            lbm.make_rectangular_patch((-a, a), (-a, a), -a, n, n, normal_up=False),
            lbm.make_vertical_panel("x", a, (-a, a), (-a, a), n, n, +1),
            lbm.make_vertical_panel("x", -a, (-a, a), (-a, a), n, n, -1),
            lbm.make_vertical_panel("y", a, (-a, a), (-a, a), n, n, +1),
            lbm.make_vertical_panel("y", -a, (-a, a), (-a, a), n, n, -1)])

    t0 = time.time()
    outer, inner = box(2.0, 3), box(1.0, 2)
    host_p = Patch("outer", outer, BCType.FREE_TRACTION)
    iface = Patch("iface", inner, BCType.INTERFACE)
    host = Region("host", ElasticMaterial(mu=1.0, lam=1.0), [host_p, iface], np.array([1.5, 1.5, 1.5]))
    incl = Region("incl", ElasticMaterial(mu=2.0, lam=3.0), [iface], np.zeros(3))
    model = RegionModel([host, incl])
    grid = volume.make_grid(model, 0.5, pad=0.5)
    extra = np.array([[1.0, 0.3, 0.2], [0.5, -1.0, 0.7], [0.2, 0.1, 1.0], [-1.0, -1.0, 0.3], [1.0, 1.0, 1.0],
                      [1.0 - 1e-6, 0.3, 0.2], [1.0 + 1e-6, 0.3, 0.2], [0.2, 0.1, -1.0 + 1e-6],
                      [0.2, 0.1, -1.0 - 1e-6], [2.0, 0.4, -0.3], [-0.6, 2.0, 1.1], [0.0, 0.0, 0.0]])
    pts = np.concatenate([grid.points, extra])
    g2 = volume.Grid(origin=grid.origin, spacing=grid.spacing, dims=(pts.shape[0], 1, 1), points=pts)
    code = volume.classify(model, g2)
    c_h, c_eps, c_fault = volume.clearance(model, g2, 0.1)
    totals = np.stack([model.point_in_region(r, pts, closure=True)[1] for r in model.regions])
    sig = np.array([model.orientation(host, host_p), model.orientation(host, iface), model.orientation(incl, iface)])
    np.savez_compressed(path, outer_vertices=outer.vertices, outer_triangles=outer.triangles,
                        inner_vertices=inner.vertices, inner_triangles=inner.triangles, points=pts,
                        n_grid=grid.points.shape[0], code=code, c_h=c_h, c_eps=c_eps, c_fault=c_fault,
                        totals=totals, orientation=sig)
    print(f"volume_regions: {time.time() - t0:.1f} s", flush=True)


CASES = {"p0_pairs": make_p0_pairs, "cube_small": make_cube_small,
         "c1_rows": make_c1_rows, "nodal_pairs": make_nodal_pairs,
         "traction_small": make_traction_small, "condense_small": make_condense_small,
         "compressed_small": make_compressed_small,
         "volume_small": make_volume_small,
         "volume_regions": make_volume_regions}

if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for name in names:
        CASES[name](os.path.join(HERE, f"{name}.npz"))
