"""The oracle's FGMRES (a restatement of the reference's ``la/solver.py``
fgmres) on the cube-12 workload's system assembled by the C oracle: it takes
the reference's own iteration counts to 1e-8 and 1e-10 and reaches the same
true residuals and solutions (``tests/golden/c1_rows.npz``, written by the
reference). This pins the CPU baseline's complete solve."""

import numpy as np
import pytest

from conftest import rel_err


@pytest.fixture(scope="module")
def c1_system(oracle):
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    from oracle.cpu_system import assemble
    model, eps = cube_fault_model(12, 8)
    system = generate_system(model)
    A, b, _ = assemble(oracle, system, eps)
    ur = [(s.offset, s.size) for s in system.layout.slots if s.kind == "u"]
    return A, b, ur


def test_port_fgmres_takes_the_reference_iterations(oracle, c1_system, c1_rows):
    from oracle.fgmres_oracle import deflated_fgmres
    A, b, ur = c1_system
    assert rel_err(b, c1_rows["b"]) < 1e-12
    for rtol, its_ref, true_ref, x_diff_ref in c1_rows["fgmres"]:
        x, rep = deflated_fgmres(lambda v: oracle.dgemv(A, v), b, ur, rtol=rtol, restart=50)
        assert rep["converged"]
        assert rep["iterations"] == int(its_ref)
        assert abs(rep["true_relres"] - true_ref) < 1e-4 * true_ref
        diff = np.linalg.norm(x - c1_rows["x"]) / np.linalg.norm(c1_rows["x"])
        assert abs(diff - x_diff_ref) < 1e-3 * x_diff_ref


def test_port_fgmres_stops_on_stagnation():
    """A singular system whose residual cannot fall: the stagnation window
    ends the solve, which reports it."""
    from oracle.fgmres_oracle import fgmres
    A = np.diag([1.0, 2.0, 0.0])
    b = np.array([1.0, 1.0, 1.0])
    x, rep = fgmres(lambda v: A @ v, b, rtol=1e-12, restart=2, maxiter=60, stagnation_window=10)
    assert rep["stagnated"] and not rep["converged"]
    assert rep["iterations"] < 60
