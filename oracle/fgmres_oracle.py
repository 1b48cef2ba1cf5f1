"""Restarted right-preconditioned FGMRES in numpy (TEST INFRASTRUCTURE, not the
product).

Restates the reference's ``fgmres`` (``src/mbem/la/solver.py:115-245``):
restart cycles from the true residual, modified Gram-Schmidt, Givens
rotations updated column by column, the stagnation window, and the final
true-residual verdict. With ``u_ranges`` it solves the deflated system
P A P y = P b, x = P y, where P removes the mean of every u-slot's x, y and z
components (the translation deflation of ``src/mbem/backends/hmat.py:678-690``
over ``dense.py:190-208``'s orthonormal basis).

Only ``tests/`` and the CPU legs of ``bench.py`` use it: the CPU baseline's
solve and a check that the port reaches the reference's own iteration counts
on the cube-12 system.
"""

from __future__ import annotations

import numpy as np


def projector(u_ranges):
    """v -> P v: every u-slot's three components made zero-mean."""
    rng = [(int(o), int(s)) for o, s in u_ranges]

    def apply(v):
        out = np.array(v, dtype=np.float64, copy=True)
        for off, size in rng:
            seg = out[off:off + size].reshape(-1, 3)
            seg -= seg.mean(axis=0)
        return out
    return apply


def fgmres(matvec, b, rtol=1e-8, restart=50, maxiter=1000, stagnation_window=200, stagnation_factor=1.001,
           precond=None):
    """Solve A x = b with ``matvec(v) -> A v``; ``precond(v) -> M v`` a right
    preconditioner (identity when None). Returns (x, report dict with
    iterations, true_relres, arnoldi_relres, restarts, converged, stagnated,
    matvecs)."""
    b = np.asarray(b, dtype=np.float64)
    n = b.shape[0]
    apply_m = precond if precond is not None else (lambda v: v)
    bnorm = float(np.linalg.norm(b))
    rep = {"iterations": 0, "true_relres": 0.0, "arnoldi_relres": 0.0, "restarts": 0, "converged": True,
           "stagnated": False, "matvecs": 0}
    x = np.zeros(n)
    if bnorm == 0.0:
        return x, rep
    its = 0
    cycles = 0
    best, best_at = np.inf, 0
    stagnated = False
    history = []
    matvecs = 0
    while its < maxiter and not stagnated:
        r = b - matvec(x)
        matvecs += 1
        beta = float(np.linalg.norm(r))
        if beta / bnorm < rtol:
            break
        m = min(restart, maxiter - its)
        V = np.zeros((m + 1, n))
        Z = np.zeros((m, n))
        H = np.zeros((m + 1, m))
        c = np.zeros(m)
        s = np.zeros(m)
        g = np.zeros(m + 1)
        V[0] = r / beta
        g[0] = beta
        done = 0
        for j in range(m):
            Z[j] = apply_m(V[j])
            w = matvec(Z[j])
            matvecs += 1
            for i in range(j + 1):              # modified Gram-Schmidt
                H[i, j] = float(V[i] @ w)
                w = w - H[i, j] * V[i]
            H[j + 1, j] = float(np.linalg.norm(w))
            if H[j + 1, j] > 1e-300:
                V[j + 1] = w / H[j + 1, j]
            for i in range(j):                  # earlier rotations on the new column
                hi, hk = H[i, j], H[i + 1, j]
                H[i, j] = c[i] * hi + s[i] * hk
                H[i + 1, j] = -s[i] * hi + c[i] * hk
            d = float(np.hypot(H[j, j], H[j + 1, j]))
            if d == 0.0:
                done = j + 1
                break
            a = abs(H[j, j])
            c[j] = a / d if a > 0.0 else 0.0
            s[j] = (np.sign(H[j, j]) * H[j + 1, j] / d) if a > 0.0 else 1.0
            H[j, j] = c[j] * H[j, j] + s[j] * H[j + 1, j]
            H[j + 1, j] = 0.0
            g[j + 1] = -s[j] * g[j]
            g[j] = c[j] * g[j]
            its += 1
            done = j + 1
            res = abs(g[j + 1]) / bnorm
            history.append(res)
            if res < best / stagnation_factor:
                best, best_at = res, its
            elif its - best_at >= stagnation_window:
                stagnated = True
                break
            if res < rtol or its >= maxiter:
                break
        if done > 0:
            y = np.zeros(done)
            for i in range(done - 1, -1, -1):   # back substitution on the rotated H
                y[i] = (g[i] - H[i, i + 1:done] @ y[i + 1:done]) / H[i, i]
            x = x + Z[:done].T @ y
        cycles += 1
        if stagnated:
            break
    true = float(np.linalg.norm(b - matvec(x)) / bnorm)
    matvecs += 1
    rep.update(iterations=its, true_relres=true, arnoldi_relres=history[-1] if history else true,
               restarts=cycles - 1, converged=true < rtol, stagnated=stagnated and not true < rtol,
               matvecs=matvecs)
    return x, rep


def deflated_fgmres(matvec, b, u_ranges, **kw):
    """FGMRES on P A P y = P b; returns (x = P y, report)."""
    P = projector(u_ranges)
    y, rep = fgmres(lambda v: P(matvec(P(v))), P(b), **kw)
    return P(y), rep
