"""Every tile configuration of the tunable kernels computes the same
product (tolerance: 1e-13 relative for the double-float FP32 and multi-mesh
products, whose summation order changes with the chunk width; 1e-5 for the
BF16 inner product's FP32 sums and the split-K GEMM), and the tuner leaves
the fastest one selected."""

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mixed_system(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(9, 6, 1.0, 1.0)
    return DenseBackend(jump="calibrated", deflate=True, precision="mixed",
                        precond="bf16_inner").assemble(generate_system(model), eps)


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_all_matvec_configurations_agree(mixed_system):
    from mbem_gb300 import autotune as at
    from mbem_gb300.la.mixed import Bf16Inner
    asm = mixed_system
    x = torch.randn(asm.op.n, dtype=torch.float64, device="cuda")
    inner = Bf16Inner(asm.op, 1, asm.u_ranges())
    try:
        at.select("mixed_matvec", 0)
        at.select("bf16_matvec", 0)
        ref32, ref16 = asm.op.matvec(x), inner.matvec(x)
        for c in range(at.count("mixed_matvec")):
            at.select("mixed_matvec", c)
            assert _rel(asm.op.matvec(x), ref32) < 1e-13, at.describe("mixed_matvec", c)
        for c in range(at.count("bf16_matvec")):
            at.select("bf16_matvec", c)
            assert _rel(inner.matvec(x), ref16) < 1e-5, at.describe("bf16_matvec", c)
    finally:
        at.select("mixed_matvec", 0)
        at.select("bf16_matvec", 0)


def test_tuner_on_a_mixed_operator(mixed_system):
    from mbem_gb300 import autotune as at
    try:
        out = at.tune_mixed_operator(mixed_system, at.Autotuner(cache_path="", reps=3, warmup=1))
        for fam, res in out.items():
            assert res["best"] == at.current(fam)
            assert len(res["times_ms"]) == at.count(fam) and min(res["times_ms"]) > 0
        mixed_system.solve_device()
        assert mixed_system.report.converged
    finally:
        for fam in at.FAMILIES:
            at.select(fam, 0)


def test_multi_mesh_and_gemm_configurations_agree(gpu):
    from mbem_gb300 import autotune as at
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.la.multimesh import MeshBatch
    from mbem_gb300.la.multirhs import gemm_bf16_t
    from mbem_gb300.model import generate_system
    be = DenseBackend(jump="calibrated", deflate=True, precision="mixed")
    systems = [be.assemble(generate_system(m), e) for m, e in (cube_fault_model(5, 3), cube_fault_model(8, 4))]
    mb = MeshBatch(systems)
    X = torch.randn(mb.n_total, dtype=torch.float64, device="cuda")
    try:
        ref = mb.matvec(X)
        for c in range(at.count("mm_matvec")):
            at.select("mm_matvec", c)
            assert _rel(mb.matvec(X), ref) < 1e-13, at.describe("mm_matvec", c)
        at.tune_mesh_batch(mb, at.Autotuner(cache_path="", reps=2, warmup=1))
        Xs, rep = mb.solve(rtol=1e-9)
        assert rep.all_converged
        # the tensor-core GEMM under every K split
        M, K, k = 512, 4096, 64
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        Xt = torch.randn(k, K, device="cuda").to(torch.bfloat16)
        at.select("gemm_split", 0)
        Y0 = gemm_bf16_t(A, Xt, K, torch.empty((k, M), dtype=torch.float32, device="cuda"))
        for c in range(at.count("gemm_split")):
            at.select("gemm_split", c)
            Y = gemm_bf16_t(A, Xt, K, torch.empty((k, M), dtype=torch.float32, device="cuda"))
            assert _rel(Y, Y0) < 1e-5, at.describe("gemm_split", c)
    finally:
        for fam in at.FAMILIES:
            at.select(fam, 0)
