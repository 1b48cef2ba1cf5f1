"""The GPU dense LU (FP32 factors with partial pivoting, FP64 refinement)
against FP64 references: P A = L U to FP32 rounding (1e-5 of |A|), solutions
refined to 1e-10 of the FP64 direct solve, a zero column reported as
singular, and the bordered (deflated) dense-backend solve equal to FGMRES's
solution (1e-9)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lu_check(n, seed=0):
    from mbem_gb300.la.lu import Factor
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(n, n, generator=g, dtype=torch.float64).cuda()
    f = Factor(A)
    LU = f.LU.double()
    L = torch.tril(LU, -1) + torch.eye(n, dtype=torch.float64, device="cuda")
    U = torch.triu(LU)
    PA = A[f.perm.long()]
    err = float((PA - L @ U).abs().max() / A.abs().max())
    assert err < 1e-5 * max(1.0, n / 256), err
    # partial pivoting: every multiplier at most 1 in magnitude
    assert float(torch.tril(LU, -1).abs().max()) <= 1.0 + 1e-6
    b = torch.randn(n, generator=g, dtype=torch.float64).cuda()
    x = f.solve(b)
    ref = torch.linalg.solve(A, b)
    assert float((x - ref).norm() / ref.norm()) < 1e-10
    return f


@pytest.mark.parametrize("n", [1, 50, 64, 200, 1000, 2049])
def test_factor_and_refined_solve(gpu, n):
    f = _lu_check(n)
    assert f.info == 0 and f.report["passes"] >= 1


def test_pivots_follow_lapack_order_on_a_permutation(gpu):
    """A permuted identity: the pivots undo the permutation exactly."""
    from mbem_gb300.la.lu import Factor
    n = 300
    p = np.random.default_rng(3).permutation(n)
    A = torch.zeros(n, n, dtype=torch.float64)
    A[torch.arange(n), torch.from_numpy(p)] = 2.0
    f = Factor(A.cuda())
    assert torch.equal(f.LU.cpu().diag(), torch.full((n,), 2.0))
    assert sorted(f.perm.cpu().tolist()) == list(range(n))


def test_singular_matrix_is_refused(gpu):
    from mbem_gb300.la.lu import Factor
    A = torch.randn(130, 130, dtype=torch.float64)
    A[:, 77] = 0.0
    with pytest.raises(np.linalg.LinAlgError):
        Factor(A.cuda())


@pytest.mark.parametrize("n, col", [(130, 77), (300, 0), (300, 299)])
def test_all_nan_column_is_a_zero_pivot(gpu, n, col):
    """A column whose remaining entries are all NaN has no pivot candidate
    (|NaN| compares false): the C ABI reports it in info as a zero pivot,
    keeps every pivot index inside the matrix and swaps nothing."""
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    A = torch.randn(n, n, dtype=torch.float32, device="cuda")
    A[:, col] = float("nan")
    piv = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    size = int(nat.lib().mbem_lu_workspace_size(n, sms))
    work = torch.empty(size, dtype=torch.uint8, device="cuda")
    nat.call("mbem_lu_factor_f32", ptr(A), A.stride(0), n, ptr(piv), ptr(work), size, ptr(info), stream_handle())
    torch.cuda.synchronize()
    assert int(info.item()) == col + 1
    p = piv.cpu().numpy()
    assert p[col] == col
    assert np.all(p >= np.arange(n)) and np.all(p < n)
    # the factorisation through the Python front end refuses it
    from mbem_gb300.la.lu import Factor
    B = torch.randn(n, n, dtype=torch.float32, device="cuda")
    B[:, col] = float("nan")
    with pytest.raises(np.linalg.LinAlgError):
        Factor(None, lambda x: x, lu32=B)


def test_dense_backend_lu_solve(gpu, cube_small):
    """DenseBackend(lu="gpu"): the bordered deflated system factored on the
    GPU, the same solution as the reference (the golden) and FGMRES."""
    from conftest import rel_err
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    g = cube_small
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    asm = DenseBackend(jump="calibrated", deflate=True, lu="gpu").assemble(generate_system(model), eps)
    sol = asm.solve()
    assert rel_err(sol["u:cube"].ravel(), g["x"]) < 1e-9
    assert asm.report.converged and asm.report.true_relres < 1e-10


@pytest.mark.parametrize("n,k", [(300, 7), (1000, 64), (2049, 130)])
def test_multi_rhs_solve(gpu, n, k):
    """Many right-hand sides at once (tensor-core block updates): the
    unrefined solve within FP32 accuracy of the FP64 solve, the refined one
    to 1e-10."""
    from mbem_gb300.la.lu import Factor, _many, solve_many
    g = torch.Generator(device="cpu").manual_seed(n + k)
    # eigenvalues in a disc of radius sqrt(n) about 3 sqrt(n): well conditioned
    A = (torch.randn(n, n, generator=g, dtype=torch.float64) + 3 * n ** 0.5 * torch.eye(n, dtype=torch.float64)).cuda()
    B = torch.randn(n, k, generator=g, dtype=torch.float64).cuda()
    f = Factor(A)
    ref = torch.linalg.solve(A, B)
    X0 = _many(f, B)
    assert float((X0 - ref).norm() / ref.norm()) < 1e-5
    X = solve_many(f, B)
    assert float((X - ref).norm() / ref.norm()) < 1e-10
    # one column through the single-column path agrees
    x1 = f.solve(B[:, 3].contiguous())
    assert float((x1 - ref[:, 3]).norm() / ref[:, 3].norm()) < 1e-10
