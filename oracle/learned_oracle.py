"""CPU oracle (FP64 numpy) of the learned preconditioner: the network's
forward pass and the gradient of the training loss by explicit
backpropagation (no autograd), the coarse-space loss, and the preconditioner
apply.

Test infrastructure only: the GPU kernels in mbem_gb300/csrc/nn.cu are
checked against these functions. The learned preconditioner has no
counterpart in the reference (it replaces the block-Jacobi rung of
src/mbem/la/preconditioner.py:421-470), so the oracle restates its
definition:

    phi_i = MLP(g_i)  (3x3 per node),  MLP: F -> H (tanh) -> H (tanh) -> 9
    B_i = [I | phi_i] (3x6),  Phi[3i + a, 6c(i) + k] = B_i[a, k]
    loss = (1/S) sum_s sum_c |eps_sc - Phi_c y_sc|^2 / |eps_s|^2,
           y_sc = (G_c + 1e-8 trace(G_c)/6 I)^-1 Phi_c^T eps_sc,  G_c = Phi_c^T Phi_c
    z = Phi y + BJ (r - A Phi y),  y = (Phi^T A Phi)^-1 Phi^T r

Parameter layout (flat): W1 (H, F), b1 (H), W2 (H, H), b2 (H), W3 (9, H), b3 (9).
"""

from __future__ import annotations

import numpy as np

F, H = 16, 32
N_PARAMS = H * F + H + H * H + H + 9 * H + 9


def unpack(params: np.ndarray):
    p = np.asarray(params, float)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + 9 * H].reshape(9, H); o += 9 * H
    b3 = p[o:o + 9]; o += 9
    assert o == N_PARAMS
    return W1, b1, W2, b2, W3, b3


def forward(feat: np.ndarray, params: np.ndarray):
    """(w (E, 9), h1 (E, H), h2 (E, H))."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    g = np.asarray(feat, float)
    h1 = np.tanh(g @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3.T + b3, h1, h2


def _basis(phi_nodes):
    """(3m, 6) chunk basis [I | phi_i] stacked over the chunk's nodes."""
    m = phi_nodes.shape[0]
    B = np.concatenate([np.broadcast_to(np.eye(3), (m, 3, 3)), phi_nodes], axis=2)
    return B.reshape(3 * m, 6)


def coarse_loss_grad(chunks, phi, eps):
    """(loss, dloss/dphi (n, 9)) of the chunk-wise projection loss; chunks:
    list of node-index arrays, phi (n, 3, 3), eps (S, 3 n)."""
    phi = np.asarray(phi, float).reshape(-1, 3, 3)
    n = phi.shape[0]
    S = eps.shape[0]
    E = np.asarray(eps, float).reshape(S, n, 3)
    inv = 1.0 / np.sum(E.reshape(S, -1) ** 2, axis=1)
    loss = 0.0
    grad = np.zeros((n, 3, 3))
    for nodes in chunks:
        Pm = _basis(phi[nodes])                           # (3m, 6)
        ec = E[:, nodes, :].reshape(S, -1)                # (S, 3m)
        G = Pm.T @ Pm
        G = G + 1e-8 * np.trace(G) / 6.0 * np.eye(6)
        y = np.linalg.solve(G, (ec @ Pm).T).T             # (S, 6)
        res = ec - y @ Pm.T
        loss += float(np.sum(np.sum(res * res, axis=1) * inv) / S)
        g = -(2.0 / S) * np.einsum("s,sp,sk->pk", inv, res, y[:, 3:])    # (3m, 3)
        grad[nodes] += g.reshape(-1, 3, 3)
    return loss, grad.reshape(n, 9)


def loss_and_grad(feat, params, chunks, eps):
    """(loss, dloss/dparams) of the coarse-space loss through the MLP."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    out, h1, h2 = forward(feat, params)
    loss, d3 = coarse_loss_grad(chunks, out, eps)
    d2 = (d3 @ W3) * (1.0 - h2 * h2)
    d1 = (d2 @ W2) * (1.0 - h1 * h1)
    grads = [d1.T @ np.asarray(feat, float), d1.sum(0), d2.T @ h1, d2.sum(0), d3.T @ h2, d3.sum(0)]
    return loss, np.concatenate([g.ravel() for g in grads])


def two_level_apply(A, chunks, phi, bj_solve, r, Z=None):
    """z = Phi y + BJ (r - A Phi y), y = (Phi^T (A + Z Z^T) Phi)^-1 Phi^T r
    (dense); Z: the null space of a calibrated A (A Z = 0), or None."""
    phi = np.asarray(phi, float).reshape(-1, 3, 3)
    n3 = A.shape[0]
    Phi = np.zeros((n3, 6 * len(chunks)))
    for c, nodes in enumerate(chunks):
        for a in range(3):
            Phi[3 * nodes + a, 6 * c + a] = 1.0
            Phi[3 * nodes + a, 6 * c + 3:6 * c + 6] = phi[nodes, a, :]
    AP = A @ Phi
    Ac = Phi.T @ AP
    if Z is not None:
        Ac = Ac + (Phi.T @ Z) @ (Z.T @ Phi)
    y = np.linalg.solve(Ac, Phi.T @ r)
    return Phi @ y + bj_solve(r - AP @ y)
