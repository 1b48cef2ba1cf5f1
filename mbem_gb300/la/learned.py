"""Learned right preconditioner for FGMRES: a mesh-local network that
corrects the cluster block-Jacobi step.

    rho = BJ r,    z_i = rho_i + sum_{j in knn(i)} W_ij rho_j,    W_ij = MLP(g_ij)

Node i owns unknowns 3i..3i+2 (a collocation node of a u-, t- or b-slot);
knn(i) are its k nearest nodes over every slot, itself first; g_ij is the
pair's geometry in units of node i's element size (relative position and
distance, both normals, the slot kinds, the size ratio). The network sees
no residual, so W is computed once per mesh (``mbem_nn_forward``) and an
apply is one block-Jacobi apply plus one 3x3-block product over the k-NN
graph (``mbem_nn_apply``). With the last layer at zero the preconditioner is
block-Jacobi itself, which is where training starts.

Training (all on the GPU, the library's own kernels): pairs (r, e = A^-1 r)
from direct dense solves of smaller meshes (the bordered deflated system of
src/mbem/backends/dense.py:384-388, LU-factored once), residuals drawn from
smooth random fields, images A s of smooth fields and white noise;
loss (1/S) sum_s |z_s - e_s|^2 / |e_s|^2; Adam.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from .. import _native as nat
from .._device import ptr, stream_handle
from ..model.core import BCType

K_DEFAULT = 16


# ---------------------------------------------------------------------------
# mesh graph and features (host)
# ---------------------------------------------------------------------------
@dataclass
class NodeGraph:
    pos: np.ndarray       # (n, 3)
    nrm: np.ndarray       # (n, 3)
    h: np.ndarray         # (n,) element size (sqrt of the element area)
    kind: np.ndarray      # (n,) 1 for a solved-slip (b) node, else 0
    nbr: np.ndarray       # (n, k) int32, self first
    feat: np.ndarray      # (n k, F) float32


def layout_nodes(layout):
    """Per global node (unknowns 3i..3i+2): position, normal, size, kind."""
    n = layout.n_unknowns // 3
    pos = np.zeros((n, 3))
    nrm = np.zeros((n, 3))
    h = np.ones(n)
    kind = np.zeros(n)
    for s in layout.slots:
        p = s.patch
        i0 = s.offset // 3
        m = s.size // 3
        pos[i0:i0 + m] = p.collocation_points()
        nrm[i0:i0 + m] = p.collocation_normals()
        _, areas = p.mesh.normals_and_areas()
        K = m // p.mesh.n_triangles
        h[i0:i0 + m] = np.repeat(np.sqrt(np.asarray(areas, float)), K)
        kind[i0:i0 + m] = 1.0 if s.kind == "b" else 0.0
    return pos, nrm, h, kind


def knn(pos: np.ndarray, k: int) -> np.ndarray:
    """(n, k) nearest nodes by distance, each row starting with the node itself."""
    n = pos.shape[0]
    k = min(k, n)
    try:
        from scipy.spatial import cKDTree
        _, idx = cKDTree(pos).query(pos, k=k)
        idx = np.asarray(idx, np.int64).reshape(n, k)
    except ImportError:            # small meshes without scipy
        d2 = ((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1)
        idx = np.argsort(d2, axis=1, kind="stable")[:, :k]
    rows = np.arange(n)
    for i in np.flatnonzero(idx[:, 0] != rows):       # coincident nodes: put self first
        r = [i] + [j for j in idx[i] if j != i][:k - 1]
        idx[i] = r
    return idx.astype(np.int32)


def edge_features(pos, nrm, h, kind, nbr) -> np.ndarray:
    n, k = nbr.shape
    i = np.repeat(np.arange(n), k)
    j = nbr.reshape(-1).astype(np.int64)
    hi = h[i][:, None]
    d = (pos[j] - pos[i]) / hi
    f = np.zeros((n * k, nat.NN_FEAT), np.float32)
    f[:, 0:3] = d
    f[:, 3] = np.linalg.norm(d, axis=1)
    f[:, 4:7] = nrm[i]
    f[:, 7:10] = nrm[j]
    f[:, 10] = np.sum(nrm[i] * nrm[j], axis=1)
    f[:, 11] = kind[i]
    f[:, 12] = kind[j]
    f[:, 13] = np.log(h[j] / h[i])
    f[:, 14] = (i == j)
    f[:, 15] = np.sum(nrm[i] * d, axis=1)
    return f


def node_graph(layout, k: int = K_DEFAULT) -> NodeGraph:
    pos, nrm, h, kind = layout_nodes(layout)
    nbr = knn(pos, k)
    return NodeGraph(pos, nrm, h, kind, nbr, edge_features(pos, nrm, h, kind, nbr))


# ---------------------------------------------------------------------------
# the network's parameters
# ---------------------------------------------------------------------------
def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-uniform hidden layers, zero output layer (the identity
    correction: the preconditioner starts as block-Jacobi)."""
    rng = np.random.default_rng(seed)
    F, H = nat.NN_FEAT, nat.NN_HIDDEN

    def glorot(o, i):
        a = math.sqrt(6.0 / (i + o))
        return rng.uniform(-a, a, size=(o, i))

    parts = [glorot(H, F), np.zeros(H), glorot(H, H), np.zeros(H), np.zeros((9, H)), np.zeros(9)]
    p = np.concatenate([x.ravel() for x in parts]).astype(np.float32)
    assert p.size == nat.NN_PARAMS
    return p


def edge_blocks(feat: torch.Tensor, params: torch.Tensor, act: torch.Tensor | None = None) -> torch.Tensor:
    """W (E, 9) FP32 from features (E, F) on the device."""
    E = feat.shape[0]
    w = torch.empty((E, 9), dtype=torch.float32, device=feat.device)
    nat.call("mbem_nn_forward", ptr(feat), E, ptr(params), ptr(act) if act is not None else None, ptr(w),
             stream_handle())
    return w


# ---------------------------------------------------------------------------
# the preconditioner (inference)
# ---------------------------------------------------------------------------
class LearnedPreconditioner:
    """M^-1 r = (I + W) BJ r for one assembled system. ``params``: the
    trained network (np or torch FP32, MBEM_NN_PARAMS)."""

    PRECOND_KIND = 2

    def __init__(self, asm, params, k: int = K_DEFAULT, bj=None):
        self.graph = node_graph(asm.layout, k)
        self.bj = bj if bj is not None else asm.block_jacobi()
        dev = self.bj.device
        self.params = torch.as_tensor(np.asarray(params, np.float32)).to(dev)
        self.nbr = torch.from_numpy(self.graph.nbr).to(dev)
        self.feat = torch.from_numpy(self.graph.feat).to(dev)
        self.w = edge_blocks(self.feat, self.params)
        n_nodes, kk = self.graph.nbr.shape
        self.work = torch.empty(3 * n_nodes, dtype=torch.float64, device=dev)
        self._bj_struct = self.bj.struct()
        self._struct = nat.NnPrecond(n_nodes=n_nodes, k=kk, nbr=ptr(self.nbr), w=ptr(self.w),
                                     bj=ctypes.pointer(self._bj_struct), work=ptr(self.work))
        self.built = True

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
def _smooth_fields(pos: np.ndarray, n_samples: int, rng, n_modes: int = 24) -> np.ndarray:
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


def training_pairs(asm, n_samples: int, seed: int = 0, chunk: int = 512):
    """(rho (S, N) FP32, e (S, N) FP32) on the device for one assembled FP64
    system: e = the deflated solution of A e = r (bordered LU), rho = BJ r."""
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
    LU, piv = torch.linalg.lu_factor(B)
    del B
    bj = asm.block_jacobi()
    rho = torch.empty((n_samples, N), dtype=torch.float32, device=dev)
    e = torch.empty((n_samples, N), dtype=torch.float32, device=dev)
    for s0 in range(0, n_samples, chunk):
        S = min(chunk, n_samples - s0)
        n1 = int(0.4 * S)
        n2 = int(0.3 * S)
        R = np.empty((S, N))
        R[:n1] = _smooth_fields(pos, n1, rng)
        sm = torch.from_numpy(_smooth_fields(pos, n2, rng)).to(dev)
        R[n1:n1 + n2] = (sm @ A.T).cpu().numpy()
        R[n1 + n2:] = rng.normal(size=(S - n1 - n2, N))
        Rt = torch.from_numpy(R).to(dev)
        if nz:
            Rt = Rt - (Rt @ Z) @ Z.T            # the residuals of the deflated system
        rhs = torch.zeros((N + nz, S), dtype=torch.float64, device=dev)
        rhs[:N] = Rt.T
        E = torch.linalg.lu_solve(LU, piv, rhs)[:N].T
        e[s0:s0 + S] = E.float()
        for q in range(S):
            rho[s0 + q] = bj.apply(Rt[q]).float()
    return rho, e


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

    def batch_grad(self, feat, nbr, rho, e):
        """loss (device scalar) and self.grad for one batch (rho, e: (S, N))."""
        S, N = rho.shape
        n_nodes, k = nbr.shape
        E = feat.shape[0]
        act = torch.empty((E, 2 * nat.NN_HIDDEN), dtype=torch.float32, device=self.device)
        w = edge_blocks(feat, self.params, act)
        z = torch.empty_like(rho)
        st = stream_handle()
        nat.call("mbem_nn_apply_batch", ptr(nbr), n_nodes, k, ptr(w), ptr(rho), S, ptr(z), st)
        inv_e2 = (1.0 / (e.double() ** 2).sum(1)).float().contiguous()
        dz = torch.empty_like(rho)
        partial = torch.empty(nat.lib().mbem_nn_loss_partial_count(S, N), dtype=torch.float64, device=self.device)
        nat.call("mbem_nn_loss_grad", ptr(z), ptr(e), ptr(inv_e2), S, N, ptr(dz), ptr(partial), ptr(self.loss_dev),
                 st)
        G = torch.empty((E, 9), dtype=torch.float32, device=self.device)
        nat.call("mbem_nn_edge_grad", ptr(nbr), n_nodes, k, ptr(dz), ptr(rho), S, ptr(G), st)
        need = nat.lib().mbem_nn_backward_workspace_size(E)
        work = torch.empty(need, dtype=torch.uint8, device=self.device)
        nat.call("mbem_nn_backward", ptr(feat), E, ptr(self.params), ptr(act), ptr(G), ptr(self.grad), ptr(work),
                 need, st)
        return self.loss_dev

    def step(self, feat, nbr, rho, e):
        loss = self.batch_grad(feat, nbr, rho, e)
        self.step_count += 1
        nat.call("mbem_nn_adam", ptr(self.params), ptr(self.grad), ptr(self.m), ptr(self.v), self.params.numel(),
                 self.lr, 0.9, 0.999, 1e-8, self.step_count, stream_handle())
        return loss


def train(datasets, steps: int = 400, batch: int = 64, lr: float = 2e-3, seed: int = 0, log_every: int = 0):
    """Trains on [(graph, rho, e), ...] (one per training mesh, batches drawn
    round-robin over the meshes); returns (params np.float32, Trainer)."""
    tr = Trainer(lr=lr, seed=seed)
    rng = np.random.default_rng(seed + 1)
    dev = tr.device
    prepared = [(torch.from_numpy(g.feat).to(dev), torch.from_numpy(g.nbr).to(dev), rho, e)
                for g, rho, e in datasets]
    for it in range(steps):
        feat, nbr, rho, e = prepared[it % len(prepared)]
        idx = torch.from_numpy(rng.choice(rho.shape[0], size=min(batch, rho.shape[0]), replace=False)).to(dev)
        loss = tr.step(feat, nbr, rho.index_select(0, idx).contiguous(), e.index_select(0, idx).contiguous())
        if log_every and (it % log_every == 0 or it == steps - 1):
            tr.history.append((it, float(loss.item())))
    return tr.params.cpu().numpy(), tr


def validation_loss(params, graph, rho, e) -> float:
    """Mean relative squared error of (I + W) rho against e."""
    tr = Trainer(params=params)
    feat = torch.from_numpy(graph.feat).to(tr.device)
    nbr = torch.from_numpy(graph.nbr).to(tr.device)
    return float(tr.batch_grad(feat, nbr, rho, e).item())
