"""One launch (or a few) of a hot kernel on a small case, for profilers
(test tooling, not part of the package): ``python tests/kernel_cases.py <case>``.

tcgemm    the block solver's GEMM: (20,736 x 62,208 BF16) x (62,208 x 256)
traction  FAULT_TRACTION assembly, cube 16 x 16, fault 12 x 12, dip 60,
          with its block-Jacobi build (traction rows, bj_build_kernel)
dfgemm    the block residual of the mixed operator, cube 24, 64 RHS
nodal     the P2 DD-minus-eigen readout of a 16 x 16 fault at 20,000 points
mixedmv   the FP32 double-float operator product, cube 24 (20,736 unknowns)
bf16mv    the BF16 inner product of the mixed solve, cube 24
mm        the persistent multi-mesh product: 8 cubes, grids drawn in [8, 20]
mm16      its BF16 inner operator (mm_matvec16_kernel) on the same 8 cubes
readout   the mixed P2 stress readout: fault 32 x 32, 100,000 observers
asm64     the FP64 P0 assembly of cube 12 (p0_matrix_kernel) and the FP64 P1
          assembly of cube 8 (nodal_matrix_kernel)
asm32     the mixed P0 assembly of cube 24 (far_assemble_kernel)
lu        the FP32 GPU LU of an 8,192 x 8,192 matrix (lu_panel_kernel, the
          tensor-core trailing update) and one refined solve
learned   FAULT_TRACTION cube 16 x 16, fault 12 x 12: the learned two-level
          preconditioner's setup and its FGMRES solve
volume    the volume sampler's geometry on cube 24 (6,912 triangles): region
          codes and clearances of a 40^3 grid (solid_angle_kernel,
          mesh_distance_kernel)
vsample   the mixed readout of the same 40^3 grid after a mixed solve of cube 24
          + fault 16: readout_far_kernel<EIG> (stress and eigenstress) and
          disp_readout_kernel, each over the cube and the fault
learned48 the learned two-level preconditioner's setup on the mixed operator of
          cube 48 + fault 32 (the headline's), twice after one assembly: the
          chunks, block-Jacobi inverses, features, A Phi gather and the coarse
          inverse (cluster_*, bj_build_kernel, knn_kernel, nn_*, gjnp_*)
learned24 the same on cube 24 + fault 16
compressed  the compressed pair operator of the cube 64 self pair, T kernel
          (49,152 elements): its build (aca_kernel, pair_dense_kernel) and eight
          products (cm_gather_kernel, cm_project_kernel, cm_strip_kernel)
"""

from __future__ import annotations

import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def run(which: str) -> None:
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model, fault_traction_model
    from mbem_gb300.model import generate_system
    if which == "tcgemm":
        from mbem_gb300.la.multirhs import gemm_bf16_t
        n, k = 20736, 256
        A = torch.randn((n, 3 * n), device="cuda").to(torch.bfloat16)
        X = torch.randn((k, 3 * n), device="cuda").to(torch.bfloat16)
        W = torch.empty((k, n), device="cuda")
        for _ in range(3):
            gemm_bf16_t(A, X, 3 * n, W)
    elif which == "traction":
        model, eps = fault_traction_model(16, 12, 60.0)
        asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
        asm.block_jacobi()
    elif which == "dfgemm":
        from mbem_gb300.la.multirhs import BlockSolver
        model, eps = cube_fault_model(24, 16)
        asm = DenseBackend(jump="calibrated", deflate=True, precision="mixed").assemble(generate_system(model),
                                                                                         eps)
        bs = BlockSolver(asm)
        B = torch.randn((64, bs.n), dtype=torch.float64, device="cuda")
        for _ in range(2):
            bs.residual(B, B)
    elif which == "nodal":
        from mbem_gb300 import mesh as M
        from mbem_gb300.kernels import tri_nodal as tn
        fault = M.centre_fault(16)
        tv = fault.tri_verts()
        nrm, _ = fault.normals_and_areas()
        rng = np.random.default_rng(0)
        x = rng.uniform(-1, 1, size=(20000, 3))
        d = rng.normal(size=(6 * tv.shape[0], 3))
        e = np.full(tv.shape[0], 0.01)
        for _ in range(2):
            tn.elastic_stress_contract(x, tv, nrm, e, d, 1.0, 1.0, order=2)
    elif which in ("mixedmv", "bf16mv"):
        from mbem_gb300.la.mixed import Bf16Inner
        model, eps = cube_fault_model(24, 16)
        asm = DenseBackend(jump="calibrated", deflate=True, precision="mixed",
                           precond="bf16_inner").assemble(generate_system(model), eps)
        x = torch.randn(asm.op.n, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        inner = Bf16Inner(asm.op, 1, asm.u_ranges())
        for _ in range(3):
            (asm.op.matvec if which == "mixedmv" else inner.matvec)(x, out=y)
    elif which in ("mm", "mm16"):
        from mbem_gb300.la.multimesh import MeshBatch, random_cube_batch
        be = DenseBackend(jump="calibrated", deflate=True, precision="mixed",
                          precond="bf16_inner" if which == "mm16" else None)
        systems = [be.assemble(generate_system(m), e)
                   for m, e in (cube_fault_model(nf, nq) for nf, nq in random_cube_batch(8, 8, 20, 3))]
        mb = MeshBatch(systems)
        if which == "mm":
            x = torch.randn(mb.n_total, dtype=torch.float64, device="cuda")
            for _ in range(3):
                mb.matvec(x)
        else:
            mb.solve_mixed(rtol=1e-8)
    elif which == "readout":
        from mbem_gb300 import mesh as M
        from mbem_gb300.kernels import tri_nodal as tn
        fault = M.centre_fault(32)
        tv = fault.tri_verts()
        nrm, _ = fault.normals_and_areas()
        rng = np.random.default_rng(0)
        x = rng.uniform(-1, 1, size=(100000, 3))
        d = rng.normal(size=(6 * tv.shape[0], 3))
        e = np.full(tv.shape[0], 0.004)
        for _ in range(2):
            tn.elastic_stress_readout(x, tv, nrm, e, d, 1.0, 1.0, order=2)
    elif which == "asm64":
        for nf, nq, order in ((12, 8, 0), (8, 6, 1)):
            model, eps = cube_fault_model(nf, nq, cube_order=order)
            DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    elif which == "asm32":
        model, eps = cube_fault_model(24, 16)
        DenseBackend(jump="calibrated", deflate=True, precision="mixed").assemble(generate_system(model), eps)
    elif which == "learned":
        from mbem_gb300.la.learned import LearnedPreconditioner
        from mbem_gb300.la.train_learned import load_default
        model, eps = fault_traction_model(16, 12, 90.0)
        asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-8).assemble(generate_system(model), eps)
        pc = LearnedPreconditioner(asm, load_default())
        asm.solve_device(precond=pc)
    elif which == "lu":
        from mbem_gb300.la.lu import Factor
        n = 8192
        g = torch.Generator(device="cpu").manual_seed(0)
        A = (torch.randn(n, n, generator=g, dtype=torch.float64)
             + n ** 0.5 * torch.eye(n, dtype=torch.float64)).cuda()
        Factor(A).solve(torch.ones(n, dtype=torch.float64, device="cuda"))
    elif which == "volume":
        from mbem_gb300 import volume as V
        model, eps = cube_fault_model(24, 16)
        grid = V.make_grid(model, 4.0 / 40)
        V.classify(model, grid)
        V.clearance(model, grid, eps)
    elif which == "vsample":
        from mbem_gb300 import volume as V
        model, eps = cube_fault_model(24, 16)
        sol = DenseBackend(jump="calibrated", deflate=True, rtol=1e-8, precision="mixed",
                           precond="bf16_inner").assemble(generate_system(model), eps).solve()
        grid = V.make_grid(model, 4.0 / 40)
        V.sample(model, sol, eps, grid, V.classify(model, grid), precision="mixed")
    elif which in ("learned48", "learned24"):
        from mbem_gb300.la.learned import LearnedPreconditioner
        from mbem_gb300.la.precond import MAX_NODES, BlockJacobi
        from mbem_gb300.la.train_learned import load_default
        model, eps = cube_fault_model(48, 32) if which == "learned48" else cube_fault_model(24, 16)
        asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-8, precision="mixed",
                           precond="bf16_learned").assemble(generate_system(model), eps)
        params = load_default()
        for _ in range(2):
            groups = [(s_.offset, asm.device_patch_arrays(s_.patch)["coll"].view(-1, 3)) for s_ in asm.layout.slots]
            bj = BlockJacobi.from_device_points(asm.layout.n_unknowns, groups, MAX_NODES).build_mixed(asm.op)
            LearnedPreconditioner(asm, params, bj=bj)
    elif which == "compressed":
        from mbem_gb300 import mesh
        from mbem_gb300.kernels import basis as kb
        from mbem_gb300.la.compressed import PairCompressed
        c = mesh.cube(64)
        pc = PairCompressed(c, c, "H", (4.0 / 64) / 2)
        view = pc._view(kb.t_coeffs(1.0, 1.0))
        x = torch.randn(3 * c.n_triangles, dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(8):
            pc.apply_device(view, x, y)
    else:
        raise SystemExit(f"unknown case {which!r}")
    torch.cuda.synchronize()


if __name__ == "__main__":
    run(sys.argv[1])
