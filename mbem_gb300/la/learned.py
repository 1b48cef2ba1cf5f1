"""Learned right preconditioner for FGMRES: cluster block-Jacobi with a
learned coarse space.

Each block-Jacobi chunk c (``la.precond``) gets six coarse vectors: its
three translations and three learned vectors, whose 3x3 block on node i of
the chunk (unknowns 3i..3i+2 of a u-, t- or b-slot) is phi_i = MLP(g_i);
on node i the basis block is [I | phi_i]. g_i is the node's geometry: its place in
the chunk (offset from the chunk centroid over the chunk radius), its
normal, its slot kind, the shape of its neighbourhood (the mean offset of
its nearest same-slot nodes, which points away from a patch edge), its size
against the chunk's. The translations alone are a Nicolaides coarse space;
the learned vectors add what they miss. The preconditioner is

    y = A_c^-1 Phi^T r,   z = Phi y + BJ (r - (A Phi) y),   A_c = Phi^T A Phi,

set up once per mesh (``mbem_nn_setup_dense``) and applied by
``mbem_nn_apply`` (no pass over A).

Training (all on the GPU, the library's own kernels): pairs (r, e = A^-1 r)
from direct dense solves of smaller meshes (the bordered deflated system of
src/mbem/backends/dense.py:384-388, LU-factored once); the coarse space
should hold what block-Jacobi misses, eps = e - BJ r, so the loss is the
chunk-wise least-squares projection error of eps onto the coarse space;
Adam. Residuals come from smooth random fields, images A s of smooth
fields, and white noise.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .. import _native as nat
from .._device import ptr, stream_handle

NEIGHBOURS = 12


# ---------------------------------------------------------------------------
# node geometry and features (host)
# ---------------------------------------------------------------------------
def layout_nodes(layout):
    """Per global node (unknowns 3i..3i+2): position, normal, size (sqrt of
    the element area), kind (1 for a solved-slip b node), slot index."""
    n = layout.n_unknowns // 3
    pos = np.zeros((n, 3))
    nrm = np.zeros((n, 3))
    h = np.ones(n)
    kind = np.zeros(n)
    slot = np.zeros(n, np.int64)
    for si, s in enumerate(layout.slots):
        p = s.patch
        i0 = s.offset // 3
        m = s.size // 3
        pos[i0:i0 + m] = p.collocation_points()
        nrm[i0:i0 + m] = p.collocation_normals()
        _, areas = p.mesh.normals_and_areas()
        K = m // p.mesh.n_triangles
        h[i0:i0 + m] = np.repeat(np.sqrt(np.asarray(areas, float)), K)
        kind[i0:i0 + m] = 1.0 if s.kind == "b" else 0.0
        slot[i0:i0 + m] = si
    return pos, nrm, h, kind, slot


def knn(pos: np.ndarray, k: int) -> np.ndarray:
    """(n, k) nearest nodes by distance, the node itself first."""
    n = pos.shape[0]
    k = min(k, n)
    try:
        from scipy.spatial import cKDTree
        _, idx = cKDTree(pos).query(pos, k=k)
        idx = np.asarray(idx, np.int64).reshape(n, k)
    except ImportError:            # small meshes without scipy
        d2 = ((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1)
        idx = np.argsort(d2, axis=1, kind="stable")[:, :k]
    for i in np.flatnonzero(idx[:, 0] != np.arange(n)):    # coincident nodes: self first
        idx[i] = [i] + [j for j in idx[i] if j != i][:k - 1]
    return idx


def node_features(layout, chunks) -> np.ndarray:
    """(n, MBEM_NN_FEAT) float32 node features; chunks: node-index arrays."""
    pos, nrm, h, kind, slot = layout_nodes(layout)
    n = pos.shape[0]
    cof = np.empty(n, np.int64)
    cen = np.zeros((len(chunks), 3))
    rad = np.zeros(len(chunks))
    for c, nodes in enumerate(chunks):
        cof[nodes] = c
        cen[c] = pos[nodes].mean(axis=0)
        rad[c] = np.linalg.norm(pos[nodes] - cen[c], axis=1).max() + 1e-12 * max(1.0, h[nodes].max())
    nb = knn(pos, NEIGHBOURS)
    same = slot[nb] == slot[:, None]
    off = ((pos[nb] - pos[:, None, :]) * same[..., None]).sum(1) / np.maximum(same.sum(1), 1)[:, None] / h[:, None]
    rel = (pos - cen[cof]) / rad[cof][:, None]
    f = np.zeros((n, nat.NN_FEAT), np.float32)
    f[:, 0:3] = rel
    f[:, 3] = np.linalg.norm(rel, axis=1)
    f[:, 4:7] = nrm
    f[:, 7] = kind
    f[:, 8:11] = off
    f[:, 11] = np.linalg.norm(off, axis=1)
    f[:, 12] = np.sum(nrm * rel, axis=1)
    f[:, 13] = np.log(h / rad[cof])
    f[:, 14] = 1.0
    f[:, 15] = same.mean(axis=1)
    return f


def device_nodes(asm):
    """``layout_nodes`` from the assembly's device mesh arrays: (pos, nrm, h,
    kind, slot) CUDA tensors, one row per node."""
    pos, nrm, h, kind, slot = [], [], [], [], []
    for si, s_ in enumerate(asm.layout.slots):
        a = asm.device_patch_arrays(s_.patch)
        m = s_.size // 3
        K = m // s_.patch.mesh.n_triangles
        tv = a["tv"].view(-1, 3, 3)
        area = 0.5 * torch.linalg.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0]).norm(dim=1)
        pos.append(a["coll"].view(-1, 3))
        nrm.append(a["coll_n"].view(-1, 3))
        h.append(torch.repeat_interleave(area.sqrt(), K))
        kind.append(torch.full((m,), 1.0 if s_.kind == "b" else 0.0, dtype=torch.float64, device=tv.device))
        slot.append(torch.full((m,), si, dtype=torch.int64, device=tv.device))
    return torch.cat(pos), torch.cat(nrm), torch.cat(h), torch.cat(kind), torch.cat(slot)


def node_features_device(asm, bj) -> torch.Tensor:
    """``node_features`` on the device (the same sixteen features; the
    neighbourhoods from ``mbem_knn``, ties to the lower index)."""
    pos, nrm, h, kind, slot = device_nodes(asm)
    dev = pos.device
    n = pos.shape[0]
    cof = bj.chunk_of_node()
    C = bj.n_chunks
    cnt = torch.zeros(C, dtype=torch.float64, device=dev).index_add_(0, cof, torch.ones(n, dtype=torch.float64,
                                                                                        device=dev))
    cen = torch.zeros((C, 3), dtype=torch.float64, device=dev).index_add_(0, cof, pos) / cnt[:, None]
    dist = (pos - cen[cof]).norm(dim=1)
    rad = torch.zeros(C, dtype=torch.float64, device=dev).scatter_reduce_(0, cof, dist, "amax")
    hmax = torch.zeros(C, dtype=torch.float64, device=dev).scatter_reduce_(0, cof, h, "amax")
    rad = rad + 1e-12 * torch.clamp(hmax, min=1.0)
    k = min(NEIGHBOURS, n)
    centred = (pos - pos.mean(dim=0)).float().contiguous()
    nb = torch.empty((n, k), dtype=torch.int64, device=dev)
    nat.call("mbem_knn", ptr(centred), n, k, ptr(nb), stream_handle())
    same = slot[nb] == slot[:, None]
    cnt_same = same.sum(dim=1).clamp(min=1).to(torch.float64)
    off = ((pos[nb] - pos[:, None, :]) * same[..., None]).sum(dim=1) / cnt_same[:, None] / h[:, None]
    rel = (pos - cen[cof]) / rad[cof][:, None]
    f = torch.zeros((n, nat.NN_FEAT), dtype=torch.float64, device=dev)
    f[:, 0:3] = rel
    f[:, 3] = rel.norm(dim=1)
    f[:, 4:7] = nrm
    f[:, 7] = kind
    f[:, 8:11] = off
    f[:, 11] = off.norm(dim=1)
    f[:, 12] = (nrm * rel).sum(dim=1)
    f[:, 13] = torch.log(h / rad[cof])
    f[:, 14] = 1.0
    f[:, 15] = same.to(torch.float64).mean(dim=1)
    return f.float().contiguous()


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------
def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-uniform hidden layers, small random output weights (the
    learned vectors must not vanish, or the projection has no gradient),
    zero output bias."""
    rng = np.random.default_rng(seed)
    F, H = nat.NN_FEAT, nat.NN_HIDDEN

    def glorot(o, i):
        a = math.sqrt(6.0 / (i + o))
        return rng.uniform(-a, a, size=(o, i))

    parts = [glorot(H, F), np.zeros(H), glorot(H, H), np.zeros(H), rng.normal(0.0, 0.1, size=(9, H)), np.zeros(9)]
    p = np.concatenate([x.ravel() for x in parts]).astype(np.float32)
    assert p.size == nat.NN_PARAMS
    return p


def mlp_forward(feat: torch.Tensor, params: torch.Tensor, act: torch.Tensor | None = None) -> torch.Tensor:
    """(n_items, 9) FP32 network outputs for features (n_items, F) on the device."""
    E = feat.shape[0]
    out = torch.empty((E, 9), dtype=torch.float32, device=feat.device)
    nat.call("mbem_nn_forward", ptr(feat), E, ptr(params), ptr(act) if act is not None else None, ptr(out),
             stream_handle())
    return out


# ---------------------------------------------------------------------------
# the preconditioner (inference)
# ---------------------------------------------------------------------------
class LearnedGeometry:
    """The mesh-only half of the learned preconditioner's setup, on the
    stream current when it is made: the network's input features, its
    coarse vectors phi, the chunk bases and, for a deflated system, the
    translation shift. ``bj``: the block-Jacobi chunks (their inverses may
    come later)."""

    def __init__(self, asm, bj, params, setup: str = "fp32"):
        dev = bj.device
        n = bj.n
        nc = 6 * bj.n_chunks
        self.params = torch.as_tensor(np.asarray(params, np.float32)).to(dev)
        if setup == "fp32":
            self.feat = node_features_device(asm, bj)
        else:
            self.feat = torch.from_numpy(node_features(asm.layout, bj.chunk_nodes())).to(dev)
        self.phi = mlp_forward(self.feat, self.params)
        self.basis = torch.empty((n, 6), dtype=torch.float32, device=dev)
        rng = np.ascontiguousarray(np.asarray(asm.u_ranges(), dtype=np.int64).reshape(-1))
        self.shift = torch.zeros((nc, 3), dtype=torch.float64, device=dev) if rng.size else None
        nat.call("mbem_nn_basis", ctypes.byref(bj.struct()), ptr(self.phi),
                 rng.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) if rng.size else None, len(rng) // 2,
                 ptr(self.basis), ptr(self.shift) if self.shift is not None else None, stream_handle())

    def tensors(self) -> list:
        return [t for t in (self.params, self.feat, self.phi, self.basis, self.shift) if t is not None]


class LearnedPreconditioner:
    """Block-Jacobi with the learned coarse space for one assembled FP64
    system. ``params``: the trained network (FP32, MBEM_NN_PARAMS)."""

    PRECOND_KIND = 2

    def __init__(self, asm, params, bj=None, setup: str = "fp32", geometry: LearnedGeometry | None = None):
        """``setup``: "fp32" (the default: device node features, A Phi with
        FP32 products, FP32 coarse inverse) or "fp64" (host features, FP64 A
        Phi and Gauss-Jordan; a dense FP64 system only). ``geometry``: the
        mesh-only half made beforehand (``LearnedGeometry`` of the same
        chunks and parameters), else made here."""
        if setup not in ("fp32", "fp64"):
            raise ValueError(f"setup must be 'fp32' or 'fp64' (got {setup!r})")
        mixed = asm.A is None
        if mixed and setup == "fp64":
            raise ValueError("the mixed operator's setup is FP32")
        if mixed and getattr(asm, "op", None) is None:
            raise NotImplementedError("the learned preconditioner needs a dense FP64 system or a mixed operator")
        self.bj = bj if bj is not None else asm.block_jacobi()
        dev = self.bj.device
        n = self.bj.n
        nc = 6 * self.bj.n_chunks
        import time
        t0 = time.perf_counter()
        geo = geometry if geometry is not None else LearnedGeometry(asm, self.bj, params, setup)
        self.params, self.feat, self.phi, self.basis = geo.params, geo.feat, geo.phi, geo.basis
        shift = geo.shift
        t1 = time.perf_counter()
        self.work = torch.empty(nat.lib().mbem_nn_apply_workspace_size(n, nc) // 8 + 1, dtype=torch.float64,
                                device=dev)
        self._bj_struct = self.bj.struct()
        st = stream_handle()
        if setup == "fp32":
            self._setup32(asm, n, nc, shift, dev, st, t0)
            return
        self.APhi = torch.empty((n, nc), dtype=torch.float64, device=dev)
        self.Ac_inv = torch.empty((nc, nc), dtype=torch.float64, device=dev)
        self._struct = nat.NnPrecond(n=n, n_coarse=nc, bj=ctypes.pointer(self._bj_struct), basis=ptr(self.basis),
                                     APhi=ptr(self.APhi), Ac_inv=ptr(self.Ac_inv), work=ptr(self.work))
        A = asm.A
        t2 = time.perf_counter()
        nat.call("mbem_nn_coarse_operator_dense", ptr(A), A.stride(0), ctypes.byref(self._struct),
                 ptr(shift) if shift is not None else None, 0 if shift is None else shift.shape[1], st)
        t3 = time.perf_counter()
        need = nat.lib().mbem_dense_inverse_workspace_size(nc)
        inv_work = torch.empty(need, dtype=torch.uint8, device=dev)
        nat.call("mbem_dense_inverse", ptr(self.Ac_inv), nc, ptr(inv_work), need, st)
        self.built = True
        t4 = time.perf_counter()
        # host times (the kernels run behind them; the inverse synchronises)
        self.setup_s = {"features_host": t1 - t0, "basis_device": t2 - t1, "coarse_operator_device": t3 - t2,
                        "coarse_inverse_device": t4 - t3}

    def _setup32(self, asm, n, nc, shift, dev, st, t0):
        """The FP32 setup: A Phi from the mixed operator's BF16 inner operator
        (mbem_nn_setup_mixed) or from the dense FP64 matrix
        (mbem_nn_setup_dense32), A_c and its FP32 inverse."""
        import time
        inner = asm.bf16_inner() if asm.A is None else None
        t1 = time.perf_counter()
        ld32 = (nc + 3) // 4 * 4
        self.APhi = self.Ac_inv = None
        self.APhi32 = torch.empty((n, ld32), dtype=torch.float32, device=dev)
        self.Ac_inv32 = torch.empty((nc, ld32), dtype=torch.float32, device=dev)
        self._struct = nat.NnPrecond(n=n, n_coarse=nc, bj=ctypes.pointer(self._bj_struct), basis=ptr(self.basis),
                                     APhi=None, Ac_inv=None, work=ptr(self.work), APhi32=ptr(self.APhi32),
                                     Ac_inv32=ptr(self.Ac_inv32), ld32=ld32)
        need = int(nat.lib().mbem_dense_inverse_f32_workspace_size(nc))
        inv_work = torch.empty(need, dtype=torch.uint8, device=dev)
        t2 = time.perf_counter()
        sh = (ptr(shift) if shift is not None else None, 0 if shift is None else shift.shape[1])
        if inner is not None:
            saved = inner.precond
            inner.precond = None
            ist = inner.struct()
            inner.precond = saved
            nat.call("mbem_nn_setup_mixed", ctypes.byref(ist), ctypes.byref(self._struct), *sh, ptr(inv_work), need,
                     st)
        else:
            A = asm.A
            nat.call("mbem_nn_setup_dense32", ptr(A), A.stride(0), ctypes.byref(self._struct), *sh, ptr(inv_work),
                     need, st)
        self.built = True
        t3 = time.perf_counter()
        # host times: the inverse synchronises, so the last holds the device work queued before it
        self.setup_s = {"features_device": t1 - t0, "basis_device": t2 - t1, "coarse_operator_and_inverse": t3 - t2}

    def struct(self):
        return self._struct

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        r = r.to(dtype=torch.float64, device=self.work.device).contiguous()
        z = torch.empty_like(r)
        nat.call("mbem_nn_apply", ctypes.byref(self._struct), ptr(r), ptr(z), stream_handle())
        return z


# ---------------------------------------------------------------------------
# training data and training
# ---------------------------------------------------------------------------
def smooth_fields(pos: np.ndarray, n_samples: int, rng, n_modes: int = 24) -> np.ndarray:
    """(S, 3 n) random smooth fields: sums of random plane waves over the
    node positions, wavelength 0.3 .. 3 box units, per component."""
    n = pos.shape[0]
    out = np.empty((n_samples, n, 3))
    for s in range(n_samples):
        ell = 10.0 ** rng.uniform(math.log10(0.3), math.log10(3.0))
        kv = rng.normal(size=(n_modes, 3, 3)) / ell
        ph = rng.uniform(0, 2 * math.pi, size=(n_modes, 3))
        amp = rng.normal(size=(n_modes, 3)) / math.sqrt(n_modes)
        arg = np.einsum("nd,mcd->nmc", pos, kv) + ph[None]
        out[s] = np.einsum("nmc,mc->nc", np.cos(arg), amp)
    return out.reshape(n_samples, 3 * n)


def training_errors(asm, n_samples: int, seed: int = 0, chunk: int = 512) -> torch.Tensor:
    """(S, N) FP32 block-Jacobi errors eps = A^-1 r - BJ r on the device for
    one assembled FP64 system (A^-1: the deflated solution, the bordered
    system factored by the project's GPU LU and solved with FP64
    refinement)."""
    from ..backends.dense import translation_basis
    A = asm.A
    N = A.shape[0]
    dev = A.device
    rng = np.random.default_rng(seed)
    pos = layout_nodes(asm.layout)[0]
    Z = torch.from_numpy(translation_basis(asm.layout)).to(dev)
    nz = Z.shape[1]
    B = torch.zeros((N + nz, N + nz), dtype=torch.float64, device=dev)
    B[:N, :N] = A
    if nz:
        B[:N, N:] = Z
        B[N:, :N] = Z.T
    from .lu import Factor, solve_many
    fac = Factor(B)                          # the project's GPU LU (FP32 factors, FP64 refinement)
    bj = asm.block_jacobi()
    eps = torch.empty((n_samples, N), dtype=torch.float32, device=dev)
    for s0 in range(0, n_samples, chunk):
        S = min(chunk, n_samples - s0)
        n1, n2 = int(0.4 * S), int(0.3 * S)
        R = torch.empty((S, N), dtype=torch.float64, device=dev)
        R[:n1] = torch.from_numpy(smooth_fields(pos, n1, rng)).to(dev)
        R[n1:n1 + n2] = torch.from_numpy(smooth_fields(pos, n2, rng)).to(dev) @ A.T
        R[n1 + n2:] = torch.from_numpy(rng.normal(size=(S - n1 - n2, N))).to(dev)
        if nz:
            R = R - (R @ Z) @ Z.T                # the residuals of the deflated system
        rhs = torch.zeros((N + nz, S), dtype=torch.float64, device=dev)
        rhs[:N] = R.T
        E = solve_many(fac, rhs)[:N].T.contiguous()
        for q in range(S):
            E[q] -= bj.apply(R[q])
        eps[s0:s0 + S] = E.float()
    return eps


class TrainingMesh:
    """One training system: its block-Jacobi chunks, node features and
    block-Jacobi errors, on the device."""

    def __init__(self, asm, n_samples: int, seed: int = 0):
        self.bj = asm.block_jacobi()
        self.feat = torch.from_numpy(node_features(asm.layout, self.bj.chunk_nodes())).to(self.bj.device)
        self.eps = training_errors(asm, n_samples, seed)
        self.chunks = self.bj.chunk_nodes()


class Trainer:
    """Adam on the network's parameters with the library's training kernels."""

    def __init__(self, params=None, lr: float = 2e-3, seed: int = 0, device="cuda"):
        self.device = torch.device(device)
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        self.params = torch.from_numpy(p.copy()).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.lr = lr
        self.step_count = 0
        self.loss_dev = torch.zeros(1, dtype=torch.float64, device=self.device)
        self.history = []

    def batch_grad(self, feat: torch.Tensor, bj, eps: torch.Tensor) -> torch.Tensor:
        """Loss (device scalar) of one batch of block-Jacobi errors (S, N);
        leaves dloss/dparams in self.grad."""
        S = eps.shape[0]
        n_items = feat.shape[0]
        act = torch.empty((n_items, 2 * nat.NN_HIDDEN), dtype=torch.float32, device=self.device)
        phi = mlp_forward(feat, self.params, act)
        inv_e2 = (1.0 / (eps.double() ** 2).sum(1)).float().contiguous()
        dphi = torch.empty_like(phi)
        partial = torch.empty(bj.n_chunks, dtype=torch.float64, device=self.device)
        st = stream_handle()
        nat.call("mbem_nn_coarse_loss_grad", ctypes.byref(bj.struct()), ptr(phi), ptr(eps), ptr(inv_e2), S,
                 ptr(dphi), ptr(partial), ptr(self.loss_dev), st)
        need = nat.lib().mbem_nn_backward_workspace_size(n_items)
        work = torch.empty(need, dtype=torch.uint8, device=self.device)
        nat.call("mbem_nn_backward", ptr(feat), n_items, ptr(self.params), ptr(act), ptr(dphi), ptr(self.grad),
                 ptr(work), need, st)
        return self.loss_dev

    def step(self, feat, bj, eps):
        loss = self.batch_grad(feat, bj, eps)
        self.step_count += 1
        nat.call("mbem_nn_adam", ptr(self.params), ptr(self.grad), ptr(self.m), ptr(self.v), self.params.numel(),
                 self.lr, 0.9, 0.999, 1e-8, self.step_count, stream_handle())
        return loss


def train(meshes, steps: int = 600, batch: int = 64, lr: float = 2e-3, seed: int = 0, log_every: int = 0):
    """Trains on a list of ``TrainingMesh`` (batches drawn round-robin over
    the meshes); returns (params np.float32, Trainer)."""
    tr = Trainer(lr=lr, seed=seed)
    rng = np.random.default_rng(seed + 1)
    for it in range(steps):
        m = meshes[it % len(meshes)]
        idx = torch.from_numpy(rng.choice(m.eps.shape[0], size=min(batch, m.eps.shape[0]),
                                          replace=False)).to(tr.device)
        loss = tr.step(m.feat, m.bj, m.eps.index_select(0, idx).contiguous())
        if log_every and (it % log_every == 0 or it == steps - 1):
            tr.history.append((it, float(loss.item())))
    return tr.params.cpu().numpy(), tr


def coarse_loss(params, mesh: TrainingMesh) -> float:
    """The projection loss of a parameter set on all of a mesh's errors."""
    tr = Trainer(params=params, device=mesh.bj.device)
    return float(tr.batch_grad(mesh.feat, mesh.bj, mesh.eps).item())
