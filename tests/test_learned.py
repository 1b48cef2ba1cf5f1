"""The learned preconditioner: the CPU oracle's backpropagation against
finite differences, the CUDA forward/backward/Adam kernels against the
oracle, and what the trained network gains over block-Jacobi alone.

Tolerances: the oracle's gradient matches central differences to 1e-6
relative (FP64); the GPU kernels run in FP32 and match the oracle to 2e-4
relative (the loss and every parameter gradient).
"""

import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import learned_oracle as lo


def _instance(seed=0, n=23, k=5, S=6):
    rng = np.random.default_rng(seed)
    feat = rng.normal(size=(n * k, lo.F)).astype(np.float32)
    nbr = np.stack([np.concatenate([[i], rng.choice(np.delete(np.arange(n), i), k - 1, replace=False)])
                    for i in range(n)]).astype(np.int32)
    params = (rng.normal(size=lo.N_PARAMS) * 0.3).astype(np.float32)
    rho = rng.normal(size=(S, 3 * n)).astype(np.float32)
    e = rng.normal(size=(S, 3 * n)).astype(np.float32)
    return feat, nbr, params, rho, e


def test_oracle_gradient_matches_finite_differences():
    feat, nbr, params, rho, e = _instance()
    p = params.astype(float)
    _, g = lo.loss_and_grad(feat, p, nbr, rho.astype(float), e.astype(float))
    rng = np.random.default_rng(1)
    for idx in rng.choice(lo.N_PARAMS, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (lo.loss_and_grad(feat, pp, nbr, rho, e)[0] - lo.loss_and_grad(feat, pm, nbr, rho, e)[0]) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])) + 1e-8


@pytest.mark.gpu
def test_gpu_network_kernels_match_oracle(gpu):
    from mbem_gb300.la.learned import Trainer, edge_blocks
    feat, nbr, params, rho, e = _instance(seed=2)
    dev = "cuda"
    w_gpu = edge_blocks(torch.from_numpy(feat).to(dev), torch.from_numpy(params).to(dev)).cpu().numpy()
    w_ref, _, _ = lo.forward(feat, params)
    assert rel_err(w_gpu, w_ref) < 2e-4
    tr = Trainer(params=params)
    loss = tr.batch_grad(torch.from_numpy(feat).to(dev), torch.from_numpy(nbr).to(dev),
                         torch.from_numpy(rho).to(dev), torch.from_numpy(e).to(dev))
    loss_ref, g_ref = lo.loss_and_grad(feat, params, nbr, rho.astype(float), e.astype(float))
    assert abs(float(loss.item()) - loss_ref) < 2e-4 * loss_ref
    assert rel_err(tr.grad.cpu().numpy(), g_ref) < 2e-4
    # one Adam step (bias-corrected, step 1): p - lr * g / (|g| + eps)
    tr.step(torch.from_numpy(feat).to(dev), torch.from_numpy(nbr).to(dev), torch.from_numpy(rho).to(dev),
            torch.from_numpy(e).to(dev))
    want = params - tr.lr * g_ref / (np.abs(g_ref) + 1e-8)
    assert rel_err(tr.params.cpu().numpy(), want) < 1e-3


@pytest.mark.gpu
def test_learned_apply_is_block_jacobi_plus_correction(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import fault_traction_model
    from mbem_gb300.la.learned import LearnedPreconditioner, init_params
    from mbem_gb300.model import generate_system
    model, eps = fault_traction_model(4, 2, dip_deg=60)
    asm = DenseBackend(jump="calibrated", deflate=True).assemble(generate_system(model), eps)
    p = init_params(3)
    lp0 = LearnedPreconditioner(asm, p)                      # zero output layer: block-Jacobi itself
    r = torch.from_numpy(np.random.default_rng(0).normal(size=asm.b.shape[0])).cuda()
    assert torch.equal(lp0.apply(r), asm.block_jacobi().apply(r))
    p[-9 - 9 * lo.H:] = np.random.default_rng(1).normal(size=9 + 9 * lo.H) * 0.05
    lp = LearnedPreconditioner(asm, p)
    rho = asm.block_jacobi().apply(r).cpu().numpy()
    w, _, _ = lo.forward(lp.graph.feat, p)
    want = lo.apply(lp.graph.nbr, w, rho[None, :])[0]
    assert rel_err(lp.apply(r).cpu().numpy(), want) < 1e-5


@pytest.mark.gpu
def test_trained_network_beats_block_jacobi(gpu):
    """Train on two small meshes (dips 45 and 80 degrees), then solve a
    held-out mesh and dip: the learned preconditioner takes fewer FGMRES
    iterations than block-Jacobi alone, and the solutions agree."""
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import fault_traction_model
    from mbem_gb300.la.learned import LearnedPreconditioner, node_graph, train, training_pairs
    from mbem_gb300.model import generate_system
    backend = DenseBackend(jump="calibrated", deflate=True, rtol=1e-10, maxiter=500)
    data = []
    for n_face, n_fault, dip in [(6, 4, 45.0), (8, 6, 80.0)]:
        model, eps = fault_traction_model(n_face, n_fault, dip)
        asm = backend.assemble(generate_system(model), eps)
        rho, e = training_pairs(asm, 768, seed=n_face)
        data.append((node_graph(asm.layout), rho, e))
    params, tr = train(data, steps=600, batch=64, lr=3e-3, log_every=100)
    assert tr.history[-1][1] < 0.8 * tr.history[0][1]
    model, eps = fault_traction_model(10, 8, 62.0)
    asm = backend.assemble(generate_system(model), eps)
    x_bj = asm.solve_device(precond="block_jacobi").clone()
    its_bj = asm.report.iterations
    x_nn = asm.solve_device(precond=LearnedPreconditioner(asm, params))
    its_nn = asm.report.iterations
    assert asm.report.converged
    assert rel_err(x_nn.cpu().numpy(), x_bj.cpu().numpy()) < 1e-8
    assert its_nn < its_bj, (its_nn, its_bj, tr.history)
