"""Many meshes in one solve (persistent batched matvec, lockstep deflated
GMRES with device-side Givens, one CUDA graph per restart cycle) against
the single-system mixed-precision operator and FGMRES.

Tolerances: the batched product equals each mesh's mixed matvec to 1e-13
(same double-float sums, FP64 near blocks); solutions agree with the
single-system solves to 1e-9 relative; every mesh's true residual is below
rtol.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [(4, 2), (7, 4), (5, 3), (6, 4), (3, 2)]


@pytest.fixture(scope="module")
def batch(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.la.multimesh import MeshBatch
    from mbem_gb300.model import generate_system
    be = DenseBackend(jump="calibrated", deflate=True, rtol=1e-10, precision="mixed")
    systems = []
    for nf, nq in SHAPES:
        model, eps = cube_fault_model(nf, nq, 1.0, 1.0)
        systems.append(be.assemble(generate_system(model), eps))
    return systems, MeshBatch(systems, restart=50)


def _deflated_relres(asm, x):
    r = asm.b - asm.op.matvec(x)
    ur = asm.u_ranges()
    def proj(v):
        v = v.clone()
        for o, n in ur:
            seg = v[o:o + n].view(-1, 3)
            seg -= seg.mean(dim=0)
        return v
    return float(proj(r).norm() / proj(asm.b).norm())


def test_batched_matvec_equals_per_mesh(batch):
    systems, mb = batch
    xs = [torch.randn(a.op.n, dtype=torch.float64, device="cuda") for a in systems]
    Y = mb.matvec(mb.gather(xs))
    for a, x, y in zip(systems, xs, mb.scatter(Y)):
        ref = a.op.matvec(x)
        assert float((y - ref).abs().max() / ref.abs().max()) < 1e-13
    # the padding stays zero
    mask = torch.ones(mb.n_total, dtype=torch.bool, device="cuda")
    for o, n in zip(mb.offsets, mb.sizes):
        mask[o:o + n] = False
    assert float(Y[mask].abs().max()) == 0.0


@pytest.mark.parametrize("graph", [True, False])
def test_batched_solve_matches_single_solves(batch, graph):
    systems, mb = batch
    X, rep = mb.solve(rtol=1e-10, graph=graph)
    assert rep.all_converged
    for a, x, its in zip(systems, mb.scatter(X), rep.iterations):
        x1 = a.solve_device(rtol=1e-10)
        assert float((x - x1).norm() / x1.norm()) < 1e-9
        assert abs(its - a.report.iterations) <= 2
        assert _deflated_relres(a, x) < 1e-10


def test_batched_restart_cycles_and_zero_rhs(batch):
    systems, mb = batch
    B = mb.gather([a.b for a in systems])
    o, n = mb.offsets[2], mb.sizes[2]
    B[o:o + n] = 0.0                        # one mesh has nothing to solve
    X, rep = mb.solve(B, rtol=1e-9, max_cycles=60)
    assert rep.all_converged and rep.cycles >= 1
    assert float(X[o:o + n].abs().max()) == 0.0
    mb2 = type(mb)(systems, restart=6)      # several restart cycles per mesh
    X2, rep2 = mb2.solve(rtol=1e-9, max_cycles=60)
    assert rep2.all_converged and rep2.cycles > 1
    for a, x in zip(systems, mb2.scatter(X2)):
        assert _deflated_relres(a, x) < 1e-9


def test_mixed_batch_solve(gpu):
    """The mixed batch solve (BF16 inner solves inside refinement on the
    accurate operators): every mesh's true residual of the accurate operator
    below rtol, solutions within 1e-9 of the single-system solves."""
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.la.multimesh import MeshBatch
    from mbem_gb300.model import generate_system
    be = DenseBackend(jump="calibrated", deflate=True, rtol=1e-10, precision="mixed", precond="bf16_inner")
    systems = [be.assemble(generate_system(m), e) for m, e in (cube_fault_model(nf, nq) for nf, nq in SHAPES)]
    mb = MeshBatch(systems)
    assert mb.has_bf16
    for graph in (True, False):
        X, rep = mb.solve_mixed(rtol=1e-10, graph=graph)
        assert rep.all_converged and max(rep.relres) < 1e-10 and rep.cycles >= 1
        for a, x in zip(systems, mb.scatter(X)):
            x1 = a.solve_device(rtol=1e-11, precond="none")
            assert float((x - x1).norm() / x1.norm()) < 1e-9
            assert _deflated_relres(a, x) < 1e-10
