"""The dense backend's diagnostics (src/mbem/backends/dense.py:124-244,
555-562): the assembly-time warnings on small crafted models, and the 1-norm
condition estimate from the GPU LU factors against numpy's exact
``cond(A, 1)`` (within a factor of 3, the estimator's usual bound) and the
reference's own LAPACK estimate of the small cube's bordered system."""

import warnings

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _outcrop_model(kind):
    """A 6x6-per-face cube whose fault (4x4, side 1) has its top edge 0.05
    below the top face: the face's collocation points next to the fault lie
    within one fault-eps of it, and the fault's top nodes within one cube-eps
    of the face."""
    from mbem_gb300 import mesh as M
    from mbem_gb300.model import BCType, Patch, Region, RegionModel
    fault = M.centre_fault(4)
    fault.vertices = fault.vertices + np.array([0.0, 0.0, 1.45])
    cube_p = Patch("cube", M.cube(6), BCType.FREE_TRACTION)
    value = np.array([1.0, 0.0, 0.0]) if kind is BCType.FAULT else np.array([-1e-3, 0.0, 0.0])
    fault_p = Patch("fault", fault, kind, value=value)
    return RegionModel([Region("body", M.ElasticMaterial(1.0, 1.0), [cube_p], np.zeros(3), faults=[fault_p])])


def _warnings_of(fn):
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        fn()
    return [str(w.message) for w in rec]


def test_collocation_near_fault_warns(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.model import BCType, generate_system
    system = generate_system(_outcrop_model(BCType.FAULT))
    msgs = _warnings_of(lambda: DenseBackend(jump="calibrated", deflate=True).assemble(system, 4.0 / 6 / 2))
    near = [m for m in msgs if "boundary collocation point(s)" in m]
    assert len(near) == 1 and "cube/fault" in near[0]
    assert not any("FAULT_TRACTION node" in m for m in msgs)


def test_fault_rows_near_boundary_warn(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.model import BCType, generate_system
    system = generate_system(_outcrop_model(BCType.FAULT_TRACTION))
    msgs = _warnings_of(lambda: DenseBackend(jump="calibrated", deflate=True).assemble(system, 4.0 / 6 / 2))
    rows = [m for m in msgs if "FAULT_TRACTION node(s)" in m]
    assert len(rows) == 1 and "fault/cube" in rows[0]


def test_half_jump_eps_warns_and_well_placed_models_do_not(gpu):
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(4, 2)
    system = generate_system(model)
    # eps = the grid spacing: eps / (mean edge) = 1 / 1.138 > 0.5
    msgs = _warnings_of(lambda: DenseBackend(jump="half").assemble(system, 2 * eps))
    assert any("jump='half' with eps/h" in m and "limit 0.5" in m for m in msgs)
    # the configs' own models: nothing to warn about
    msgs = _warnings_of(lambda: DenseBackend(jump="calibrated", deflate=True).assemble(system, eps))
    assert msgs == []


@pytest.mark.parametrize("n, grade", [(300, 2.0), (1000, 3.0), (777, 4.5)])
def test_condition_estimate_within_three_of_exact(gpu, n, grade):
    """Random orthogonal U, V and singular values graded over `grade`
    decades: the estimate lies within a factor 3 of cond_1 (a lower bound of
    the FP32 factors' own condition, which FP32 rounding moves by up to
    ~cond x 1e-7 x sqrt(n) relative)."""
    from mbem_gb300.la.lu import Factor
    rng = np.random.default_rng(n)
    U, _ = np.linalg.qr(rng.normal(size=(n, n)))
    V, _ = np.linalg.qr(rng.normal(size=(n, n)))
    A = (U * np.logspace(0, -grade, n)) @ V.T
    exact = np.linalg.cond(A, 1)
    est = Factor(torch.from_numpy(A).cuda()).cond()
    print(f"n {n}: cond_1 {exact:.3e}, estimate {est:.3e}")
    assert exact / 3.0 <= est <= exact * 1.3


def test_condition_estimate_of_a_diagonal_and_the_warning(gpu):
    """A diagonal matrix is factored exactly: the estimate is its exact
    1-norm condition number; above 1e10 the backend's warning fires."""
    from mbem_gb300.backends.dense import warn_condition
    from mbem_gb300.la.lu import Factor
    d = np.ones(200)
    d[57] = 1e-11
    f = Factor(torch.from_numpy(np.diag(d)).cuda())
    assert f.cond() == pytest.approx(1e11, rel=1e-6)
    with pytest.warns(UserWarning, match="condition estimate 1.00e\\+11 exceeds 1e\\+10"):
        warn_condition(f.cond())


def test_lu_solve_reports_the_condition_estimate(gpu, cube_small):
    """DenseBackend(lu="gpu") on the small cube: the bordered deflated
    system's estimate, against the reference's LAPACK gecon estimate of the
    same system (tests/golden/cube_small.npz) and numpy's exact cond_1."""
    from mbem_gb300.backends.dense import DenseBackend, translation_basis
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    g = cube_small
    model, eps = cube_fault_model(int(g["n_face"]), int(g["n_fault"]), float(g["mu"]), float(g["lam"]))
    asm = DenseBackend(jump="calibrated", deflate=True, lu="gpu").assemble(generate_system(model), eps)
    asm.solve_device()
    est = asm.report.cond_estimate
    A = asm.A.cpu().numpy()
    Z = translation_basis(asm.layout)
    n = A.shape[0]
    K = np.zeros((n + 3, n + 3))
    K[:n, :n], K[:n, n:], K[n:, :n] = A, Z, Z.T
    exact = np.linalg.cond(K, 1)
    print(f"small cube: cond_1 {exact:.3e}, estimate {est:.3e}, reference gecon {float(g['cond']):.3e}")
    assert exact / 3.0 <= est <= exact * 1.01
    assert float(g["cond"]) / 3.0 <= est <= 3.0 * float(g["cond"])
