"""Deflated FGMRES on the device against dense direct solves."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_fgmres_solves_well_conditioned_system(gpu):
    from mbem_gb300.la.solver import fgmres_dense
    rng = np.random.default_rng(0)
    n = 301                                  # odd: exercises the scalar tails
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 3.0 * np.eye(n)
    b = rng.normal(size=n)
    x, rep = fgmres_dense(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda(), rtol=1e-12, restart=20)
    assert rep.converged and rep.true_relres < 1e-12
    assert np.abs(x.cpu().numpy() - np.linalg.solve(A, b)).max() < 1e-10
    assert rep.restarts >= 0 and len(rep.residual_history) == rep.iterations


def test_fgmres_zero_rhs_and_stagnation(gpu):
    from mbem_gb300.la.solver import fgmres_dense
    n = 64
    A = torch.eye(n, dtype=torch.float64, device="cuda")
    x, rep = fgmres_dense(A, torch.zeros(n, dtype=torch.float64, device="cuda"))
    assert rep.converged and rep.iterations == 0 and float(x.abs().max()) == 0.0
    # a singular operator with b outside its range: reported, not raised
    S = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    S[: n // 2, : n // 2] = torch.eye(n // 2, dtype=torch.float64, device="cuda")
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x, rep = fgmres_dense(S, b, rtol=1e-10, restart=10, maxiter=60, stagnation_window=15)
    assert not rep.converged
    assert rep.true_relres > 0.5


def test_projection_removes_translations(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    n = 3 * 50 + 7
    v = torch.randn(n, dtype=torch.float64, device="cuda")
    out = torch.empty_like(v)
    rng = np.array([0, 150], dtype=np.int64)
    work = torch.empty(384, dtype=torch.float64, device="cuda")
    nat.call("mbem_project_translation", ptr(v), ptr(out), n, rng.ctypes.data, 1, ptr(work), stream_handle())
    # in place gives the same result
    v2 = v.clone()
    nat.call("mbem_project_translation", ptr(v2), ptr(v2), n, rng.ctypes.data, 1, ptr(work), stream_handle())
    assert torch.equal(v2, out)
    o = out.cpu().numpy()
    vv = v.cpu().numpy()
    for k in range(3):
        assert abs(o[k:150:3].mean()) < 1e-14
        assert np.allclose(o[k:150:3], vv[k:150:3] - vv[k:150:3].mean(), atol=1e-14)
    assert np.array_equal(o[150:], vv[150:])


def test_dgemv_and_rowsum(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    rng = np.random.default_rng(1)
    A = rng.normal(size=(37, 3 * 41))
    x = rng.normal(size=3 * 41)
    Ad = torch.from_numpy(A).cuda()
    y = torch.zeros(37, dtype=torch.float64, device="cuda")
    nat.call("mbem_dgemv", ptr(Ad), Ad.stride(0), 37, 3 * 41, ptr(torch.from_numpy(x).cuda()), 2.0, 0.0,
             ptr(y), stream_handle())
    assert np.abs(y.cpu().numpy() - 2.0 * A @ x).max() < 1e-12
    rs = torch.empty((37, 3), dtype=torch.float64, device="cuda")
    nat.call("mbem_block_rowsum3", ptr(Ad), Ad.stride(0), 37, 41, 1.0, 0, ptr(rs), stream_handle())
    assert np.abs(rs.cpu().numpy() - A.reshape(37, 41, 3).sum(axis=1)).max() < 1e-12
