"""Cluster block-Jacobi preconditioner (la/preconditioner.py:421-470) on the
GPU: chunk inverses against numpy's FP64 inverses of the same diagonal
chunks, the mixed-operator build against the dense build, and preconditioned
FGMRES against the plain solve.

Tolerance: the inverses are FP32 (a flexible preconditioner needs no more):
apply() agrees with the FP64 block solve to 1e-4 relative; solutions with
and without the preconditioner agree to the solver tolerance.
"""

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _cube(n_face=4, n_fault=2, **kw):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, n_fault)
    return DenseBackend(jump="calibrated", deflate=True, rtol=1e-12, **kw).assemble(generate_system(model), eps)


def _block_solve(bj, A, r):
    z = np.zeros_like(r)
    for dofs, D in bj.dense_blocks_host(A):
        z[dofs] = np.linalg.solve(D, r[dofs])
    return z


@pytest.mark.parametrize("max_nodes", [75, 16, 5])
def test_block_jacobi_dense_matches_block_solves(gpu, max_nodes):
    from mbem_gb300.la.precond import BlockJacobi
    asm = _cube(6, 2)
    bj = BlockJacobi.for_layout(asm.layout, max_nodes).build_dense(asm.A)
    assert bj.chunk_sizes.max() <= 3 * max_nodes and bj.chunk_sizes.sum() == asm.A.shape[0]
    r = torch.from_numpy(np.random.default_rng(3).normal(size=asm.A.shape[0])).cuda()
    z = bj.apply(r).cpu().numpy()
    want = _block_solve(bj, asm.A.cpu().numpy(), r.cpu().numpy())
    assert rel_err(z, want) < 1e-4


def test_block_jacobi_mixed_build_matches_its_operator(gpu):
    from mbem_gb300.la.precond import BlockJacobi
    asm = _cube(8, 4, precision="mixed")
    bj = BlockJacobi.for_layout(asm.layout).build_mixed(asm.op)
    A = asm.op.dense64().cpu().numpy()
    r = np.random.default_rng(4).normal(size=A.shape[0])
    z = bj.apply(torch.from_numpy(r).cuda()).cpu().numpy()
    assert rel_err(z, _block_solve(bj, A, r)) < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_preconditioned_solve_matches_plain(gpu, precision):
    asm = _cube(8, 4, precision=precision)
    x0 = asm.solve_device(precond="none").clone()
    plain = asm.report
    x1 = asm.solve_device(precond="block_jacobi")
    pre = asm.report
    assert plain.converged and pre.converged
    assert pre.true_relres < 1e-12
    assert rel_err(x1.cpu().numpy(), x0.cpu().numpy()) < 1e-10


def test_block_jacobi_fault_traction_system(gpu, traction_small):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import BCType, generate_system
    g = traction_small
    model, eps = cube_fault_model(2, 2, fault_kind=BCType.FAULT_TRACTION, fault_value=g["drop"])
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12,
                       precond="block_jacobi").assemble(generate_system(model), eps)
    sol = asm.solve()
    assert asm.report.converged
    assert rel_err(sol["b:fault"], g["x_b"]) < 1e-10


def test_singular_chunk_is_reported(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300.la.precond import BlockJacobi
    pts = np.array([[0.0, 0, 0], [1.0, 0, 0], [5.0, 0, 0], [6.0, 0, 0]])
    bj = BlockJacobi(12, [(0, pts)], max_nodes=2)
    A = torch.eye(12, dtype=torch.float64, device="cuda")
    A[6:, 6:] = 0.0                            # the second chunk is singular
    with pytest.raises(nat.MbemError):
        bj.build_dense(A)
    z = bj.apply(torch.arange(12, dtype=torch.float64, device="cuda")).cpu().numpy()
    assert np.array_equal(z, np.arange(12.0))  # identity on both chunks
