"""A dense operator factored once on the GPU: LU with partial pivoting in
FP32, every solve refined in FP64 (the reference's ``la/lu.py`` ``Factor``
with ``how="gpu"``: src/mbem/la/lu.py:110-258).

``Factor(A)`` factors a float64 CUDA matrix (kept: the refinement reads it)
in single precision with the library's blocked GPU LU
(``mbem_lu_factor_f32``); ``solve(B)`` returns ``A^-1 B`` in double by the
reference's refinement: solve from the single factors, the residual in
double, correct, stopped on the SIZE OF THE CORRECTION (what is left after a
correction ``d`` that contracted at ``rho`` is ``rho / (1 - rho) |d|``,
lu.py:22-31). Where the corrections do not contract the matrix is not
single-precision material and ``solve`` raises (the reference falls back to
LAPACK in double on the host; this path has no host fallback).
"""

from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import ptr, stream_handle


class SingleFactorError(RuntimeError):
    """The refinement from single-precision factors did not contract."""


class Factor:
    """``A`` (n, n) float64 CUDA, factored in FP32 on the device.
    ``matvec(x) -> A x`` in FP64 overrides the product the refinement uses
    (for an operator held in another form, e.g. a bordered one)."""

    def __init__(self, A: torch.Tensor, matvec=None, lu32: torch.Tensor | None = None):
        if A is not None and (A.dtype != torch.float64 or not A.is_cuda or A.dim() != 2
                              or A.shape[0] != A.shape[1]):
            raise ValueError("Factor: a square float64 CUDA matrix")
        if A is not None and not torch.isfinite(A).all():
            raise ValueError("factor: the matrix must not contain infs or NaNs")
        self._A = A
        self._matvec = matvec
        if lu32 is None:
            lu32 = A.to(torch.float32).contiguous()
        self.n = n = int(lu32.shape[0])
        self.report = {"how": "gpu"}
        dev = lu32.device
        t0 = time.perf_counter()
        # the 1-norm of the factored matrix, for the condition estimate,
        # taken before the factors overwrite it
        self.anorm = column_abs_max(lu32)
        self._cond = None
        self.LU = lu32
        self.piv = torch.empty(n, dtype=torch.int32, device=dev)
        info = torch.zeros(1, dtype=torch.int32, device=dev)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        size = int(nat.lib().mbem_lu_workspace_size(n, sms))
        work = torch.empty(size, dtype=torch.uint8, device=dev)
        nat.call("mbem_lu_factor_f32", ptr(self.LU), self.LU.stride(0), n, ptr(self.piv), ptr(work), size,
                 ptr(info), stream_handle())
        self.info = int(info.item())
        # the pivots as one permutation: position i holds original row perm[i]
        piv = self.piv.cpu().numpy()
        perm = np.arange(n, dtype=np.int64)
        for k, p in enumerate(piv):
            if p != k:
                perm[k], perm[p] = perm[p], perm[k]
        self.perm = torch.from_numpy(perm.astype(np.int32)).to(dev)
        self._xf = torch.empty(n, dtype=torch.float32, device=dev)
        torch.cuda.synchronize(dev)
        self.report["factor_s"] = time.perf_counter() - t0
        if self.info:
            raise np.linalg.LinAlgError(f"factor: the matrix is singular (zero pivot at column {self.info - 1})")

    @property
    def nbytes(self) -> int:
        return 4 * self.n ** 2

    def _single(self, b: torch.Tensor) -> torch.Tensor:
        """A^-1 b from the single factors, as double (one column)."""
        x = torch.empty_like(b)
        nat.call("mbem_lu_solve_f32", ptr(self.LU), self.LU.stride(0), self.n, ptr(self.perm), ptr(b), ptr(x),
                 ptr(self._xf), stream_handle())
        return x

    def _single_t(self, b: torch.Tensor) -> torch.Tensor:
        """A^-T b from the single factors, as double (one column)."""
        x = torch.empty_like(b)
        nat.call("mbem_lu_solve_t_f32", ptr(self.LU), self.LU.stride(0), self.n, ptr(self.perm), ptr(b), ptr(x),
                 ptr(self._xf), stream_handle())
        return x

    def cond(self) -> float:
        """1-norm condition estimate |A|_1 est(|A^-1|_1) (lu.py:241-258: the
        reference's gecon / onenormest), from the single factors by
        ``onenorm_inverse_estimate``; computed once."""
        if self._cond is None:
            est = onenorm_inverse_estimate(self._single, self._single_t, self.n, self.LU.device)
            c = self.anorm * est
            self._cond = c if np.isfinite(c) else float("inf")
        return self._cond

    def _apply(self, x: torch.Tensor) -> torch.Tensor:
        if self._matvec is not None:
            return self._matvec(x)
        y = torch.empty_like(x)
        nat.call("mbem_dgemv", ptr(self._A), self._A.stride(0), self.n, self.n, ptr(x), 1.0, 0.0, ptr(y),
                 stream_handle())
        return y

    def solve(self, B: torch.Tensor) -> torch.Tensor:
        """A^-1 B for B (n,) or (n, k) float64 CUDA, refined in double."""
        B = B.to(torch.float64)
        cols = B.reshape(self.n, -1)
        out = torch.empty_like(cols)
        passes, worst_left, worst_size = 0, 0.0, 0.0
        for j in range(cols.shape[1]):
            b = cols[:, j].contiguous()
            x = self._single(b)
            xn = float(x.norm())
            if xn == 0.0:
                out[:, j] = x
                continue
            tol, before = defaults.LU_REFINE_TOL, None
            done, rate, size, left, k = False, 0.0, 0.0, 0.0, 0
            while not done and k < defaults.LU_REFINE_PASSES:
                d = self._single((b - self._apply(x)).contiguous())
                x += d
                k += 1
                now = float(d.norm()) / float(x.norm())
                rate = now if before is None else (now / before if before > 0.0 else 0.0)
                size, before = now, now
                left = rate / (1.0 - rate) * size if rate < 1.0 else float("inf")
                done = left <= tol or size <= tol
                if rate > defaults.LU_REFINE_RATE:
                    break
            if not done:
                raise SingleFactorError(
                    f"dense LU in single precision: the refinement did not contract (rate {rate:.1e}, "
                    f"{left:.1e} left after {k} corrections); the matrix is too ill-conditioned for "
                    f"single-precision factors")
            passes = max(passes, k)
            if left >= worst_left:
                worst_left, worst_size = left, size
            out[:, j] = x
        self.report["passes"] = max(passes, self.report.get("passes", 0))
        self.report["correction"], self.report["left"] = worst_size, worst_left
        return out.reshape(B.shape)


def column_abs_max(M: torch.Tensor, rows_per_pass: int = 4096) -> float:
    """|M|_1 = the largest column sum of magnitudes, in row blocks (no copy of M)."""
    acc = torch.zeros(M.shape[1], dtype=torch.float64, device=M.device)
    for r0 in range(0, M.shape[0], rows_per_pass):
        acc += M[r0:r0 + rows_per_pass].abs().sum(dim=0, dtype=torch.float64)
    return float(acc.max()) if acc.numel() else 0.0


def onenorm_inverse_estimate(solve, solve_t, n: int, dev, max_iter: int = 5) -> float:
    """Estimate of |A^-1|_1 from products with A^-1 and A^-T (``solve``,
    ``solve_t``: float64 CUDA vector -> vector): Hager's ascent over the
    vertices of the unit 1-norm ball with Higham's safeguards (Higham,
    "FORTRAN codes for estimating the one-norm of a real or complex matrix",
    ACM TOMS 14, 1988, Algorithm 4.1): start from the uniform vector, follow
    the largest entry of A^-T sign(A^-1 x) to a unit vector, stop when the
    sign pattern repeats, the estimate stops growing or the index repeats,
    and take the larger of that and the alternating test vector's
    2 |A^-1 b|_1 / (3 n). A lower bound of |A^-1|_1, usually within a factor
    of 3 of it."""
    x = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev)
    y = solve(x)
    est = float(y.abs().sum())
    if n == 1:
        return est

    def signs(v):
        return torch.where(v >= 0, 1.0, -1.0).to(torch.float64)
    xi = signs(y)
    z = solve_t(xi)
    j = int(z.abs().argmax())
    for _ in range(1, max_iter):
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        x[j] = 1.0
        y = solve(x)
        prev = est
        est = float(y.abs().sum())
        xi_new = signs(y)
        if bool(torch.equal(xi_new, xi)) or est <= prev:
            est = max(est, prev)
            break
        xi = xi_new
        z = solve_t(xi)
        j_prev, j = j, int(z.abs().argmax())
        if float(z[j_prev].abs()) >= float(z[j].abs()):
            break
    i = torch.arange(n, dtype=torch.float64, device=dev)
    b = (1.0 + i / (n - 1)) * torch.where(i % 2 == 0, 1.0, -1.0).to(torch.float64)
    alt = 2.0 * float(solve(b).abs().sum()) / (3.0 * n)
    return max(est, alt)


def _many(f: "Factor", B: torch.Tensor) -> torch.Tensor:
    """A^-1 B (n, k) from the single factors, as double."""
    n, k = B.shape
    X = torch.empty_like(B)
    size = int(nat.lib().mbem_lu_solve_many_workspace_size(n, k))
    work = torch.empty(size, dtype=torch.uint8, device=B.device)
    nat.call("mbem_lu_solve_many_f32", ptr(f.LU), f.LU.stride(0), n, ptr(f.perm), ptr(B), B.stride(0), k, ptr(X),
             X.stride(0), ptr(work), size, stream_handle())
    return X


def solve_many(f: "Factor", B: torch.Tensor, matmat=None) -> torch.Tensor:
    """A^-1 B for B (n, k) float64 CUDA: the blocked multi-column solve from
    the single factors, refined in double by the reference's rule on the
    worst column (``matmat(X) -> A X`` in FP64; default: the kept matrix)."""
    B = B.to(torch.float64).contiguous()
    if matmat is None:
        if f._A is None:
            raise ValueError("solve_many needs the FP64 matrix or a matmat")

        def matmat(X):
            Y = torch.empty_like(X)
            nat.call("mbem_dgemm_multi", ptr(f._A), f._A.stride(0), f.n, f.n, ptr(X), X.shape[1], ptr(Y),
                     stream_handle())
            return Y
    X = _many(f, B)
    live = X.norm(dim=0) > 0.0
    if not bool(live.any()):
        return X
    tol, before = defaults.LU_REFINE_TOL, None
    done, rate, size, left, k = False, 0.0, 0.0, 0.0, 0
    while not done and k < defaults.LU_REFINE_PASSES:
        D = _many(f, (B - matmat(X)).contiguous())
        X += D
        k += 1
        now = D[:, live].norm(dim=0) / X[:, live].norm(dim=0)
        if before is None:
            rate = float(now.max())
        else:
            rate = float(torch.where(before > 0, now / before, torch.zeros_like(now)).max())
        size, before = float(now.max()), now
        left = rate / (1.0 - rate) * size if rate < 1.0 else float("inf")
        done = left <= tol or size <= tol
        if rate > defaults.LU_REFINE_RATE:
            break
    if not done:
        raise SingleFactorError(
            f"dense LU in single precision: the refinement did not contract (rate {rate:.1e}, {left:.1e} left "
            f"after {k} corrections)")
    f.report["passes"] = max(k, f.report.get("passes", 0))
    f.report["correction"], f.report["left"] = size, left
    return X


def factor(A: torch.Tensor, matvec=None) -> Factor:
    return Factor(A, matvec)


def phase_stats(timing: bool = False) -> dict:
    """Device ms of the factorisations' phases since the last call; switches
    the phase timing of later factorisations on or off."""
    arr = (ctypes.c_double * 3)()
    nat.lib().mbem_lu_stats(int(timing), arr)
    return dict(zip(("panels", "block_rows", "update"), list(arr)))
