"""Many right-hand sides: the tensor-core product Y = A X (``mbem_gemm_bf16``)
that replaces one matvec per right-hand side by one GEMM per iteration.

The reference solves many right-hand sides by one LU factorisation and its
triangular solves (src/mbem/la/lu.py:110-258, the refinement product at
:210); here the operator stays in HBM once as BF16 and every product over
the whole block of right-hand sides reads it once.
"""

from __future__ import annotations

import torch

from .. import _native as nat
from .._device import ptr, stream_handle

MAX_RHS = 256


def gemm_bf16(A: torch.Tensor, Xt: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Y (M, n) FP32 = A (M, K) @ Xt (n, K)^T for BF16 CUDA tensors with
    unit column stride; n <= 256 (larger blocks: call per 256 columns)."""
    if A.dtype != torch.bfloat16 or Xt.dtype != torch.bfloat16 or not A.is_cuda:
        raise ValueError("A and Xt must be bfloat16 CUDA tensors")
    if A.stride(1) != 1 or Xt.stride(1) != 1 or A.shape[1] != Xt.shape[1]:
        raise ValueError("A (M, K) and Xt (n, K) need unit column strides and one K")
    M, K = A.shape
    n = Xt.shape[0]
    if not 1 <= n <= MAX_RHS:
        raise ValueError(f"1..{MAX_RHS} right-hand sides per product (got {n})")
    Y = out if out is not None else torch.empty((M, n), dtype=torch.float32, device=A.device)
    nat.call("mbem_gemm_bf16", ptr(A), A.stride(0), ptr(Xt), Xt.stride(0), M, K, n, ptr(Y), Y.stride(0),
             stream_handle())
    return Y


def gemm_check():
    """Synchronises and raises if a tensor-core pipeline wait gave up."""
    nat.call("mbem_gemm_bf16_check", stream_handle())


_split_work = {}


def gemm_bf16_t(A: torch.Tensor, Xt: torch.Tensor, K: int, out: torch.Tensor, split: bool = True) -> torch.Tensor:
    """out (n, M) FP32 = (A[:, :K] @ Xt[:, :K]^T)^T, out's rows at out.stride(0);
    with ``split`` K is divided over the SMs when the row tiles alone
    would leave them unevenly loaded."""
    M = A.shape[0]
    n = Xt.shape[0]
    if not split:
        nat.call("mbem_gemm_bf16_t", ptr(A), A.stride(0), ptr(Xt), Xt.stride(0), M, K, n, ptr(out),
                 out.stride(0), stream_handle())
        return out
    need = nat.lib().mbem_gemm_bf16_workspace_size(M, n)
    key = (A.device.index, need)
    work = _split_work.get(key)
    if work is None:
        work = torch.empty(need // 4, dtype=torch.float32, device=A.device)
        _split_work.clear()
        _split_work[key] = work
    nat.call("mbem_gemm_bf16_t_split", ptr(A), A.stride(0), ptr(Xt), Xt.stride(0), M, K, n, ptr(out),
             out.stride(0), ptr(work), need, stream_handle())
    return out


# ---------------------------------------------------------------------------
# a block of right-hand sides: batched GMRES on the BF16 tensor-core
# operator inside FP64-accurate iterative refinement
# ---------------------------------------------------------------------------
import ctypes  # noqa: E402
from dataclasses import dataclass, field  # noqa: E402

import numpy as np  # noqa: E402


@dataclass
class BlockReport:
    converged: bool
    outer: int                        # refinement steps
    inner_iterations: list = field(default_factory=list)   # batched GMRES iterations per step
    true_relres: np.ndarray = None    # per right-hand side |b - A x| / |b|
    gemm_ms: float = 0.0              # tensor-core GEMM time
    residual_ms: float = 0.0          # FP64-accurate residuals
    inner_ms: float = 0.0             # batched GMRES (GEMM included)

    def __str__(self):
        worst = float(np.max(self.true_relres)) if self.true_relres is not None else float("nan")
        return (f"block solve {'converged' if self.converged else 'NOT CONVERGED'}: {self.outer} refinement steps, "
                f"inner {self.inner_iterations}, worst relres {worst:.3e}")


def _pad8(n: int) -> int:
    return (n + 7) // 8 * 8


class BlockSolver:
    """Solves A X = B for up to 256 right-hand sides at once.

    The refinement loop computes the residual R = P (B - A X) with the
    accurate operator (the mixed operator's FP32 far field with double-float
    accumulation and its FP64 near blocks, or the FP64 dense matrix), and
    corrects X by batched GMRES on the BF16 copy of the operator, whose
    every step is one tensor-core GEMM over the whole block. P removes the
    rigid translations of the u-slots of a deflated system."""

    def __init__(self, asm, inner_restart: int = 30, inner_rtol: float = 3e-5, terms: int = 3):
        """``terms``: 1 = the operator in BF16 (relative error ~2^-9 per
        product: about five refinement steps to 1e-8); 3 = A and the Krylov
        vectors each split into BF16 high and low parts, A_hi V_hi + A_hi
        V_lo + A_lo V_hi in one GEMM over a three-fold K (error ~2^-16: two
        refinement steps)."""
        if terms not in (1, 3):
            raise ValueError("terms must be 1 or 3")
        self.terms = terms
        self.asm = asm
        self.op = asm.op
        self.A = asm.A
        if self.op is None and self.A is None:
            raise ValueError("the assembled system holds no operator")
        dev = (self.A if self.A is not None else self.op.A32).device
        self.device = dev
        self.n = n = int(asm.b.shape[0])
        self.ldp = _pad8(n)
        # A16 = [A_hi | A_hi | A_lo] (terms 3) or A_hi, each block ldp wide
        self.A16 = torch.zeros((n, terms * self.ldp), dtype=torch.bfloat16, device=dev)
        hi = self.A16[:, :self.ldp]
        lo = self.A16[:, 2 * self.ldp:] if terms == 3 else None
        st = stream_handle()
        ld16 = self.A16.stride(0)
        if self.op is not None:
            s = self.op.struct()
            nat.call("mbem_mixed_to_bf16x2", ctypes.byref(s), ptr(hi), ptr(lo) if lo is not None else None, ld16, st)
        elif lo is not None:
            nat.call("mbem_to_bf16x2", ptr(self.A), 1, self.A.stride(0), n, n, ptr(hi), ptr(lo), ld16, st)
        else:
            nat.call("mbem_to_bf16", ptr(self.A), 1, self.A.stride(0), n, n, ptr(hi), ld16, st)
        if terms == 3:
            self.A16[:, self.ldp:self.ldp + n] = hi[:, :n]
        rng = np.ascontiguousarray(np.asarray(asm.u_ranges(), dtype=np.int64).reshape(-1))
        self._ranges = rng
        self.inner_restart = inner_restart
        self.inner_rtol = inner_rtol

    # -- pieces ---------------------------------------------------------
    def project(self, X: torch.Tensor):
        if self._ranges.size == 0:
            return X
        is64 = 1 if X.dtype == torch.float64 else 0
        nat.call("mbem_batch_project", ptr(X), is64, X.shape[0], X.shape[1],
                 self._ranges.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(self._ranges) // 2,
                 stream_handle())
        return X

    def residual(self, B: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
        """P (B - A X) for (k, n) FP64 blocks with the accurate operator."""
        k = B.shape[0]
        R = torch.empty_like(B)
        if self.op is not None:
            need = nat.lib().mbem_batch_residual_workspace_size(k, self.n)
            work = torch.empty(need // 8, dtype=torch.float64, device=self.device)
            s = self.op.struct()
            nat.call("mbem_batch_residual_mixed", ctypes.byref(s), ptr(B), ptr(X), k, ptr(R), ptr(work), need,
                     stream_handle())
        else:
            Y = torch.empty((self.n, k), dtype=torch.float64, device=self.device)
            Xc = X.T.contiguous()
            nat.call("mbem_dgemm_multi", ptr(self.A), self.A.stride(0), self.n, self.n, ptr(Xc), k, ptr(Y),
                     stream_handle())
            R = B - Y.T
        return self.project(R)

    def inner_gmres(self, R: torch.Tensor, m: int, rtol: float):
        """D (k, n) FP64 with |R - A16 D| small for every row, by batched
        GMRES(m) on the BF16 operator; returns (D, iterations, gemm_ms)."""
        k, n = R.shape
        dev = self.device
        st = stream_handle()
        V = torch.empty((m + 1, k, n), dtype=torch.float32, device=dev)
        Vbf = torch.zeros((k, self.terms * self.ldp), dtype=torch.bfloat16, device=dev)
        ld = self.ldp
        terms = self.terms
        W = torch.empty((k, n), dtype=torch.float32, device=dev)
        norms = torch.empty(k, dtype=torch.float64, device=dev)
        Hd = torch.empty((m + 1, k), dtype=torch.float64, device=dev)
        H2d = torch.empty((m + 1, k), dtype=torch.float64, device=dev)

        def normalize(src, is64, j):
            # V[j] = src / |src|; the GEMM operand [V_hi | V_lo | V_hi] (or V_hi)
            nat.call("mbem_batch_normalize", ptr(src), is64, k, n, ptr(norms), ptr(V[j]), None, st)
            vh = V[j].to(torch.bfloat16)
            Vbf[:, :n] = vh
            if terms == 3:
                Vbf[:, ld:ld + n] = (V[j] - vh.float()).to(torch.bfloat16)
                Vbf[:, 2 * ld:2 * ld + n] = vh
            return norms.cpu().numpy().copy()

        beta = normalize(R, 1, 0)
        live = beta > 0
        H = np.zeros((m + 1, m, k))
        cs = np.zeros((m, k))
        sn = np.zeros((m, k))
        g = np.zeros((m + 1, k))
        g[0] = beta
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        gemm_ms = 0.0
        jdone = 0
        for j in range(m):
            ev0.record()
            gemm_bf16_t(self.A16, Vbf, terms * ld, W)
            ev1.record()
            self.project(W)
            nat.call("mbem_batch_dots", ptr(V), j + 1, ptr(W), k, n, ptr(Hd), st)
            nat.call("mbem_batch_axpy", ptr(W), ptr(V), j + 1, ptr(Hd), -1.0, k, n, st)
            nat.call("mbem_batch_dots", ptr(V), j + 1, ptr(W), k, n, ptr(H2d), st)
            nat.call("mbem_batch_axpy", ptr(W), ptr(V), j + 1, ptr(H2d), -1.0, k, n, st)
            hn = normalize(W, 0, j + 1)
            h = (Hd[:j + 1] + H2d[:j + 1]).cpu().numpy()
            gemm_ms += ev0.elapsed_time(ev1)
            col = np.vstack([h, hn[None, :]])            # (j + 2, k)
            for i in range(j):                           # accumulated rotations
                a, b = col[i].copy(), col[i + 1].copy()
                col[i] = cs[i] * a + sn[i] * b
                col[i + 1] = -sn[i] * a + cs[i] * b
            den = np.hypot(col[j], col[j + 1])
            ok = den > 0
            cs[j] = np.where(ok, np.abs(col[j]) / np.where(ok, den, 1.0), 1.0)
            sgn = np.where(col[j] >= 0, 1.0, -1.0)
            sn[j] = np.where(ok, sgn * col[j + 1] / np.where(ok, den, 1.0), 0.0)
            col[j] = cs[j] * col[j] + sn[j] * col[j + 1]
            col[j + 1] = 0.0
            H[:j + 2, j] = col
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            jdone = j + 1
            rel = np.where(live, np.abs(g[j + 1]) / np.where(live, beta, 1.0), 0.0)
            if np.all(rel < rtol):
                break
        # back substitution per right-hand side
        Y = np.zeros((jdone, k))
        for i in range(jdone - 1, -1, -1):
            s = g[i] - (H[i, i + 1:jdone].T * Y[i + 1:jdone].T).sum(axis=1) if i + 1 < jdone else g[i].copy()
            d = H[i, i]
            Y[i] = np.where(d != 0, s / np.where(d != 0, d, 1.0), 0.0)
        D = torch.zeros((k, n), dtype=torch.float64, device=dev)
        Yd = torch.from_numpy(np.ascontiguousarray(Y)).to(dev)
        nat.call("mbem_batch_update", ptr(D), ptr(V), jdone, ptr(Yd), k, n, st)
        return D, jdone, gemm_ms

    # -- the solve ------------------------------------------------------
    def solve(self, B: torch.Tensor, rtol: float = 1e-8, max_outer: int = 12):
        """X (k, n) FP64 for B (k, n) FP64 on the device, and a BlockReport."""
        B = self.project(B.to(dtype=torch.float64, device=self.device).contiguous().clone())
        k = B.shape[0]
        if not 1 <= k <= MAX_RHS:
            raise ValueError(f"1..{MAX_RHS} right-hand sides per block (got {k})")
        bnorm = torch.linalg.vector_norm(B, dim=1).cpu().numpy()
        X = torch.zeros_like(B)
        rep = BlockReport(converged=False, outer=0)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        rep.residual_ms = 0.0
        rep.inner_ms = 0.0
        for outer in range(max_outer + 1):
            ev[0].record()
            R = B.clone() if outer == 0 else self.residual(B, X)     # X = 0: R = P B
            ev[1].record()
            ev[1].synchronize()
            rep.residual_ms += ev[0].elapsed_time(ev[1])
            rel = torch.linalg.vector_norm(R, dim=1).cpu().numpy() / np.where(bnorm > 0, bnorm, 1.0)
            rep.true_relres = rel
            if np.all(rel < rtol) or outer == max_outer:
                rep.converged = bool(np.all(rel < rtol))
                break
            ev[0].record()
            D, its, ms = self.inner_gmres(R, self.inner_restart, self.inner_rtol)
            ev[1].record()
            ev[1].synchronize()
            rep.inner_ms += ev[0].elapsed_time(ev[1])
            rep.inner_iterations.append(its)
            rep.gemm_ms += ms
            X += D
            self.project(X)
            rep.outer = outer + 1
        gemm_check()
        return X, rep


def slip_rhs(asm, fault, slips) -> torch.Tensor:
    """B (k, n) FP64: the right-hand sides of k slip patterns (k, n_dofs, 3)
    on a prescribed-slip fault, every other datum of the system zero. Each
    RHS term of the fault (equations.py:296-309: scale -sigma times the T
    block) is assembled once in FP64 and applied to all patterns at once."""
    from ..kernels import KERNEL_T
    from ..kernels import basis as kb
    from ..kernels import tri_nodal as tn
    slips = np.asarray(slips, float)
    k = slips.shape[0]
    dev = asm.b.device
    B = torch.zeros((k, asm.b.shape[0]), dtype=torch.float64, device=dev)
    S = torch.from_numpy(np.ascontiguousarray(slips.reshape(k, -1).T)).to(dev)     # (3 n_src, k)
    held = asm._arrays
    if held is None:
        asm._arrays = asm._arrays_in if asm._arrays_in is not None else {}
    for rt in asm.system.rhs_terms:
        if rt.source_patch is not fault:
            continue
        if rt.kernel != KERNEL_T:
            raise NotImplementedError("slip right-hand sides through the T kernel only")
        mat = asm.materials[rt.region.name]
        f = asm._patch_arrays(rt.field_patch)
        s = asm._patch_arrays(rt.source_patch)
        c = kb.t_coeffs(mat.mu, mat.lam)
        T = tn.t_matrix_direct(f["coll"], s["tv"], s["normals"], s["eps"], *c, order=rt.source_patch.order)
        Y = torch.empty((T.shape[0], k), dtype=torch.float64, device=dev)
        nat.call("mbem_dgemm_multi", ptr(T), T.stride(0), T.shape[0], T.shape[1], ptr(S), k, ptr(Y),
                 stream_handle())
        B[:, rt.row.offset:rt.row.stop] += rt.scale * Y.T
    asm._arrays = held
    return B
