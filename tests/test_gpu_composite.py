"""The mixed solve with the learned two-level preconditioner inside its BF16
inner solve (``precond="bf16_learned"``) and its pieces:

- ``mbem_dense_inverse_f32`` (blocked Gauss-Jordan, without row
  interchanges where that passes its check, else with partial pivoting):
  M M^-1 = I to FP32 accuracy (5e-4 scaled by the condition), pivoting on a
  permutation, a leading dimension beyond n, a singular matrix refused;
- ``mbem_nn_setup_mixed``: A Phi of the BF16 inner operator (A16 far field
  plus FP64 near blocks) equal to the same product in FP64 torch to 2e-5 of
  its largest entry, and the coarse inverse times A_c (+ the translation
  shift) equal to I to 1e-3;
- the composite solve: converged to the 1e-8 true residual of the mixed
  operator, within 1e-7 of the plain mixed solve's solution, in fewer inner
  steps.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inverse(M, ld=None):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    n = M.shape[0]
    ld = n if ld is None else ld
    buf = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    buf[:, :n] = M
    need = int(nat.lib().mbem_dense_inverse_f32_workspace_size(n))
    work = torch.empty(need, dtype=torch.uint8, device="cuda")
    nat.call("mbem_dense_inverse_f32", ptr(buf), n, ld, ptr(work), need, stream_handle())
    return buf[:, :n]


@pytest.mark.parametrize("n, ld", [(1, 1), (5, 8), (16, 16), (17, 20), (100, 100), (1000, 1004), (3072, 3072), (3200, 3204)])
def test_dense_inverse_f32(gpu, n, ld):
    g = torch.Generator(device="cpu").manual_seed(n)
    A = (torch.randn(n, n, generator=g, dtype=torch.float64) + 2.0 * np.sqrt(n) * torch.eye(n, dtype=torch.float64))
    A = A[torch.randperm(n, generator=g)]                  # the pivots must find the large entries
    inv = _inverse(A.float().cuda(), ld).double().cpu()
    err = float((A @ inv - torch.eye(n, dtype=torch.float64)).abs().max())
    cond = float(torch.linalg.cond(A))
    assert err < 5e-4 * max(1.0, cond / 10.0), (err, cond)


def _inverse_counts():
    import ctypes
    from mbem_gb300 import _native as nat
    a, b = ctypes.c_int64(0), ctypes.c_int64(0)
    nat.lib().mbem_dense_inverse_f32_stats(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


@pytest.mark.parametrize("n, ld", [(1024, 1024), (1500, 1504), (3072, 3072)])
def test_dense_inverse_f32_without_interchanges(gpu, n, ld):
    """A matrix with dominant diagonal blocks (as the coarse Galerkin matrix
    has) is inverted without row interchanges, to the same FP32 accuracy;
    a row-permuted one fails that attempt's check and is inverted with
    pivoting."""
    g = torch.Generator(device="cpu").manual_seed(n + 7)
    A = torch.randn(n, n, generator=g, dtype=torch.float64) / np.sqrt(n) + torch.eye(n, dtype=torch.float64)
    _inverse_counts()
    inv = _inverse(A.float().cuda(), ld).double().cpu()
    assert _inverse_counts() == (1, 0)
    err = float((A @ inv - torch.eye(n, dtype=torch.float64)).abs().max())
    assert err < 5e-4 * max(1.0, float(torch.linalg.cond(A)) / 10.0), err
    P = A[torch.randperm(n, generator=g)]
    inv = _inverse(P.float().cuda(), ld).double().cpu()
    assert _inverse_counts() == (0, 1)
    err = float((P @ inv - torch.eye(n, dtype=torch.float64)).abs().max())
    assert err < 5e-4 * max(1.0, float(torch.linalg.cond(P)) / 10.0), err


def test_dense_inverse_f32_refuses_singular(gpu):
    from mbem_gb300 import _native as nat
    A = torch.randn(50, 50, dtype=torch.float32)
    A[:, 17] = 0.0
    with pytest.raises(nat.MbemError) as info:
        _inverse(A.cuda())
    assert info.value.code == nat.ERR_NUMERIC


def _inner_dense(asm):
    """The BF16 inner operator (A16 far field + FP64 near blocks) as an FP64 matrix."""
    op = asm.op
    n = op.n
    A = op.A16[:, :n].float().double()
    for nb in op.near:
        rp = nb.rowptr.cpu().numpy()
        f = torch.from_numpy(np.repeat(np.arange(nb.n_field), np.diff(rp))).to(A.device)
        for i in range(3):
            for j in range(3):
                A[nb.row0 + 3 * f + i, nb.col0 + 3 * nb.cols + j] += nb.vals[:, 3 * i + j]
    return A


@pytest.fixture(scope="module")
def cube12(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(12, 8)
    system = generate_system(model)
    mk = lambda pc: DenseBackend(jump="calibrated", deflate=True, rtol=1e-8, precision="mixed",  # noqa: E731
                                 precond=pc).assemble(system, eps)
    return mk


def test_mixed_coarse_operator_and_inverse(cube12):
    from mbem_gb300.la.learned import LearnedPreconditioner
    from mbem_gb300.la.train_learned import load_default
    asm = cube12("bf16_inner")
    lp = LearnedPreconditioner(asm, load_default())
    n, nc = lp.bj.n, 6 * lp.bj.n_chunks
    # Phi (n x nc) from the basis rows and the chunk of every unknown
    chunk_of = torch.empty(n, dtype=torch.int64, device="cuda")
    for c, nodes in enumerate(lp.bj.chunk_nodes()):
        d = torch.from_numpy((3 * nodes[:, None] + np.arange(3)).ravel()).cuda()
        chunk_of[d] = c
    Phi = torch.zeros((n, nc), dtype=torch.float64, device="cuda")
    rows = torch.arange(n, device="cuda")
    for k in range(6):
        Phi[rows, 6 * chunk_of + k] = lp.basis[:, k].double()
    APhi = _inner_dense(asm) @ Phi
    got = lp.APhi32[:, :nc].double()
    assert float((got - APhi).abs().max()) < 2e-5 * float(APhi.abs().max())
    # A_c^-1 (A_c + U U^T) = I, with U = Phi^T Z for the translations Z
    from mbem_gb300.backends.dense import translation_basis
    Z = torch.from_numpy(translation_basis(asm.layout)).cuda()
    U = Phi.T @ Z
    Ac = Phi.T @ got + U @ U.T
    E = lp.Ac_inv32[:, :nc].double() @ Ac - torch.eye(nc, dtype=torch.float64, device="cuda")
    assert float(E.abs().max()) < 1e-3


def test_composite_solve_matches_plain_mixed_solve(cube12):
    from mbem_gb300.la.mixed import inner_stats
    plain = cube12("bf16_inner")
    inner_stats()
    x0 = plain.solve_device()
    steps0, _, _ = inner_stats()
    assert plain.report.converged and plain.report.true_relres < 1e-8
    comp = cube12("bf16_learned")
    x1 = comp.solve_device()
    steps1, applies1, _ = inner_stats()
    assert comp.report.converged and comp.report.true_relres < 1e-8
    assert float((x1 - x0).norm() / x0.norm()) < 1e-7
    print(f"cube 12 inner steps: plain {steps0}, learned two-level {steps1} ({applies1} inner solves)")
    assert steps1 < steps0


def test_device_features_equal_host_features(gpu):
    """``node_features_device`` (mbem_knn neighbourhoods) equals the host
    ``node_features`` on a cube whose vertices are jittered (no distance ties
    among the neighbours), with the device-made chunks of the mixed operator."""
    from mbem_gb300 import mesh as M
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.la.learned import node_features, node_features_device
    from mbem_gb300.model import BCType, Patch, Region, RegionModel, generate_system
    cube = M.cube(8)
    jitter = np.random.default_rng(8).normal(scale=0.01, size=cube.vertices.shape)
    cube.vertices = cube.vertices + jitter
    fault = M.centre_fault(4)
    model = RegionModel([Region("body", M.ElasticMaterial(1.0, 1.0), [Patch("cube", cube, BCType.FREE_TRACTION)],
                                np.zeros(3), faults=[Patch("fault", fault, BCType.FAULT,
                                                           value=np.array([1.0, 0.0, 0.0]))])])
    asm = DenseBackend(jump="calibrated", deflate=True, precision="mixed",
                       precond="bf16_inner").assemble(generate_system(model), 0.25)
    bj = asm.block_jacobi()
    dev = node_features_device(asm, bj).cpu().numpy()
    host = node_features(asm.layout, bj.chunk_nodes())
    assert np.abs(dev - host).max() < 1e-5 * max(1.0, np.abs(host).max())
