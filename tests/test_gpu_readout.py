"""The mixed-precision nodal stress readout (FP32 quadrature far field, FP64
nodal near pairs) against the FP64 nodal readout of the same density
(``elastic_stress_contract``, pinned to the reference by test_gpu_nodal).

Tolerance: every observer's stress within 2e-5 of the largest stress of the
set (FP32 quadrature of the far pairs: ~1e-6 observed is the design target).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(order, n_fault=8, n_obs=3000, seed=0):
    from mbem_gb300 import mesh as M
    fault = M.centre_fault(n_fault)
    tv = fault.tri_verts()
    nrm, _ = fault.normals_and_areas()
    edge = np.linalg.norm(tv[:, [1, 2, 0]] - tv, axis=2).mean()
    eps = np.full(tv.shape[0], 0.07 * edge)
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(n_obs, 3))
    k = n_obs // 10
    x[:k, 1] = rng.uniform(-2 * eps[0], 2 * eps[0], size=k)      # near the fault plane y = 0
    x[:k, 0] = rng.uniform(-0.5, 0.5, size=k)
    x[:k, 2] = rng.uniform(-0.5, 0.5, size=k)
    K = (order + 1) * (order + 2) // 2
    d = rng.normal(size=(K * tv.shape[0], 3))
    return x, tv, nrm, eps, d


@pytest.mark.parametrize("order", [0, 1, 2])
def test_mixed_readout_matches_fp64(gpu, order):
    from mbem_gb300.kernels import tri_nodal as tn
    x, tv, n, e, d = _case(order)
    mu, lam = 1.3, 1.95
    ref = tn.elastic_stress_contract(x, tv, n, e, d, mu, lam, order=order)
    got = tn.elastic_stress_readout(x, tv, n, e, d, mu, lam, order=order)
    scale = np.abs(ref).max()
    err = np.abs(got - ref).reshape(len(x), -1).max(axis=1) / scale
    assert err.max() < 2e-5, (err.max(), np.argmax(err))
    # the near pairs took the FP64 path: the observers on the plane agree to rounding
    assert err[:len(x) // 10].max() < 2e-5


def test_mixed_readout_accumulates_and_scales(gpu):
    from mbem_gb300.kernels import tri_nodal as tn
    x, tv, n, e, d = _case(2, n_fault=4, n_obs=500, seed=3)
    base = tn.elastic_stress_readout(x, tv, n, e, d, 1.0, 1.0, order=2)
    out = torch.ones((len(x), 3, 3), dtype=torch.float64, device="cuda")
    tn.elastic_stress_readout(x, tv, n, e, d, 1.0, 1.0, order=2, out=out, alpha=-2.0, accumulate=True)
    assert np.allclose(out.cpu().numpy(), 1.0 - 2.0 * base, rtol=1e-12, atol=1e-12 * np.abs(base).max())


def test_evaluate_stress_mixed_matches_fp64(gpu, cube_small):
    """evaluate_stress(precision="mixed") on the small cube's solution."""
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.evaluate import evaluate_stress
    from mbem_gb300.model import generate_system
    g = cube_small
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12).assemble(generate_system(model), eps)
    sol = asm.solve()
    ref = evaluate_stress(model, "body", sol, g["points"], eps, warn_near=False)
    got = evaluate_stress(model, "body", sol, g["points"], eps, warn_near=False, precision="mixed")
    assert np.abs(got - ref).max() < 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("order", [0, 2])
def test_mixed_readout_eigenstress_part_matches_fp64(gpu, order):
    """eig_out: the eigenstress of the same pairs from the same pass, against
    the FP64 eigenstress contraction (tolerance relative to its largest
    value, which sits on the fault plane)."""
    from mbem_gb300.kernels import tri_nodal as tn
    x, tv, n, e, d = _case(order, n_obs=2000, seed=5)
    mu, lam = 1.3, 1.95
    ref_e = tn.eigenstress_contract(x, tv, n, e, d, mu, lam, order=order)
    ref_s = tn.elastic_stress_readout(x, tv, n, e, d, mu, lam, order=order)
    eig = torch.zeros((len(x), 3, 3), dtype=torch.float64, device="cuda")
    got_s = tn.elastic_stress_readout(x, tv, n, e, d, mu, lam, order=order, eig_out=eig)
    assert np.abs(eig.cpu().numpy() - ref_e).max() < 2e-5 * np.abs(ref_e).max()
    # the elastic part agrees with the launch without eig_out to FP32 rounding
    assert np.abs(got_s - ref_s).max() < 1e-6 * np.abs(ref_s).max()
    acc = torch.ones_like(eig)
    tn.elastic_stress_readout(x, tv, n, e, d, mu, lam, order=order, eig_out=acc, alpha=-2.0, accumulate=True)
    assert np.allclose(acc.cpu().numpy(), 1.0 - 2.0 * eig.cpu().numpy(), rtol=1e-12,
                       atol=1e-12 * np.abs(ref_e).max())


def test_evaluate_stress_mixed_parts_match_fp64(gpu, cube_small):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.evaluate import evaluate_stress
    from mbem_gb300.model import generate_system
    g = cube_small
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=1e-12).assemble(generate_system(model), eps)
    sol = asm.solve()
    rs, re = evaluate_stress(model, "body", sol, g["points"], eps, warn_near=False, parts=True)
    gs, ge = evaluate_stress(model, "body", sol, g["points"], eps, warn_near=False, parts=True, precision="mixed")
    assert np.abs(gs - rs).max() < 2e-5 * np.abs(rs).max()
    assert np.abs(ge - re).max() < 2e-5 * np.abs(re).max()
    assert np.abs(ge - g["stress_eigen"]).max() < 2e-5 * np.abs(g["stress_eigen"]).max()
