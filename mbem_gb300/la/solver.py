"""Flexible GMRES on the GPU with the reference's reporting
(``src/mbem/la/solver.py:31-68`` SolveReport, :115-245 fgmres).

The iteration runs in the CUDA library (``mbem_fgmres_dense``): FP64 matvec,
classical Gram-Schmidt applied twice, Givens rotations on the host over the
(restart+1) Hessenberg scalars, stagnation stop, and the true-residual
verdict. Deflation (``backends/hmat.py:678-690``): P A P y = P b with
P = I - Z Z^T over the u-slots; the returned x is P y.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import ptr, stream_handle


@dataclass
class SolveReport:
    converged: bool
    iterations: int
    true_relres: float
    arnoldi_relres: float
    stagnated: bool = False
    restarts: int = 0
    residual_history: list = field(default_factory=list)
    precond_summary: dict | None = None
    recycle_dim: int = 0
    setup_matvecs: int = 0
    matvecs: int = 0                 # operator applications
    matvec_ms: float = 0.0           # their device time (when timed)

    def __str__(self):
        status = "converged" if self.converged else ("STAGNATED" if self.stagnated else "NOT CONVERGED")
        return f"FGMRES {status}: {self.iterations} iters, true relres {self.true_relres:.3e}"


_DEFAULTS = dict(rtol=defaults.GMRES_RTOL, restart=defaults.GMRES_RESTART, maxiter=defaults.GMRES_MAXITER,
                 stagnation_window=defaults.GMRES_STAGNATION_WINDOW,
                 stagnation_factor=defaults.GMRES_STAGNATION_FACTOR, u_ranges=(), workspace=None,
                 time_matvec=False, precond=None)


def fgmres_mixed(op, b: torch.Tensor, x0: torch.Tensor | None = None, **kw):
    """FGMRES on a ``la.mixed.MixedOperator`` (same contract as fgmres_dense)."""
    return _fgmres(None, op, b, x0, **{**_DEFAULTS, **kw})


def fgmres_dense(A: torch.Tensor, b: torch.Tensor, x0: torch.Tensor | None = None, **kw):
    """Solve A x = b for a dense FP64 CUDA matrix. Keywords: rtol, restart,
    maxiter, stagnation_window, stagnation_factor, ``u_ranges`` = [(offset,
    size), ...] of the u-slots to deflate (empty: no deflation), workspace,
    time_matvec (CUDA-event time of every operator application), precond
    (a right preconditioner: ``la.precond.BlockJacobi`` or
    ``la.learned.LearnedPreconditioner``; the iteration is then flexible,
    x = x0 + Z y with z_j = M^-1 v_j). Returns (x, SolveReport)."""
    if A.dtype != torch.float64 or not A.is_cuda or A.shape[0] != b.shape[0] or A.stride(1) != 1:
        raise ValueError("A must be a float64 CUDA matrix (n, n) with unit column stride")
    return _fgmres(A, None, b, x0, **{**_DEFAULTS, **kw})


def _precond_args(precond):
    """(kind, state pointer, keep-alive) for the C params."""
    if precond is None:
        return 0, None, None
    kind = getattr(precond, "PRECOND_KIND", None)
    if kind not in (1, 2, 3):
        raise TypeError(f"unsupported preconditioner {type(precond).__name__}")
    if not getattr(precond, "built", True):
        raise RuntimeError("preconditioner used before it was built")
    st = precond.struct()
    return kind, ctypes.cast(ctypes.byref(st), ctypes.c_void_p), st


def _fgmres(A, mop, b, x0, rtol, restart, maxiter, stagnation_window, stagnation_factor, u_ranges,
            workspace, time_matvec, precond):
    n = b.shape[0]
    dev = (A if A is not None else mop.A32).device
    b = b.to(dtype=torch.float64, device=dev).contiguous()
    x = (torch.zeros(n, dtype=torch.float64, device=dev) if x0 is None
         else x0.to(dtype=torch.float64, device=dev).clone().contiguous())
    restart = int(min(restart, maxiter))
    need = nat.lib().mbem_fgmres_workspace_size(n, restart)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    rng = np.ascontiguousarray(np.asarray(u_ranges, dtype=np.int64).reshape(-1))
    prm = nat.FgmresParams(restart=restart, maxiter=int(maxiter), rtol=float(rtol),
                           stagnation_window=int(stagnation_window),
                           stagnation_factor=float(stagnation_factor),
                           n_u_ranges=len(rng) // 2,
                           u_ranges=rng.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) if rng.size else None,
                           precond=0, precond_state=None, time_matvec=int(bool(time_matvec)),
                           x_is_zero=int(x0 is None))
    kind, state, _keep = _precond_args(precond)
    prm.precond = kind
    prm.precond_state = state
    hist = np.zeros(max(int(maxiter), 1))
    rep = nat.FgmresReport()
    rep.history = hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    if A is not None:
        nat.call("mbem_fgmres_dense", ptr(A), A.stride(0), n, ptr(b), ptr(x), ctypes.byref(prm),
                 ptr(workspace), need, ctypes.byref(rep), stream_handle())
    else:
        op = mop.struct()
        nat.call("mbem_fgmres_mixed", ctypes.byref(op), ptr(b), ptr(x), ctypes.byref(prm),
                 ptr(workspace), need, ctypes.byref(rep), stream_handle())
    report = SolveReport(converged=bool(rep.converged), iterations=int(rep.iterations),
                         true_relres=float(rep.true_relres), arnoldi_relres=float(rep.arnoldi_relres),
                         stagnated=bool(rep.stagnated), restarts=int(rep.restarts),
                         residual_history=hist[:rep.iterations].tolist(), matvecs=int(rep.matvecs),
                         matvec_ms=float(rep.matvec_ms))
    return x, report
