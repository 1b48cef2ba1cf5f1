"""CPU oracle (FP64 numpy) of the learned preconditioner's network: forward
pass, batched apply, loss and the gradient of the loss with respect to the
parameters, by explicit backpropagation (no autograd).

Test infrastructure only: the GPU kernels in mbem_gb300/csrc/nn.cu are
checked against these functions. The network has no counterpart in the
reference (it is the learned replacement of the block-Jacobi rung of
src/mbem/la/preconditioner.py:421-470), so the oracle restates the
network's definition:

    W_e = MLP(g_e),  MLP: F -> H (tanh) -> H (tanh) -> 9
    z_s,i = rho_s,i + sum_q W_(i,q) rho_s,nbr(i,q)
    loss = (1/S) sum_s |z_s - e_s|^2 / |e_s|^2

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


def apply(nbr: np.ndarray, w: np.ndarray, rho: np.ndarray) -> np.ndarray:
    """z (S, 3 n) = rho + W rho for rho (S, 3 n)."""
    n, k = nbr.shape
    S = rho.shape[0]
    r = rho.reshape(S, n, 3)
    Wb = w.reshape(n, k, 3, 3)
    z = r + np.einsum("iqab,sqib->sia", Wb, r[:, nbr, :].transpose(0, 2, 1, 3))
    return z.reshape(S, 3 * n)


def loss_and_grad(feat, params, nbr, rho, e):
    """(loss, dloss/dparams) for one batch."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    w, h1, h2 = forward(feat, params)
    S = rho.shape[0]
    n, k = nbr.shape
    z = apply(nbr, w, rho)
    inv_e2 = 1.0 / np.sum(e * e, axis=1)
    d = z - e
    loss = float(np.sum(d * d * inv_e2[:, None]) / S)
    dz = (2.0 / S) * d * inv_e2[:, None]
    dzr = dz.reshape(S, n, 3)
    rr = rho.reshape(S, n, 3)
    # G_(i,q)[a, b] = sum_s dz[s, i, a] rho[s, nbr(i, q), b]
    G = np.einsum("sia,sqib->iqab", dzr, rr[:, nbr, :].transpose(0, 2, 1, 3)).reshape(n * k, 9)
    d3 = G
    d2 = (d3 @ W3) * (1.0 - h2 * h2)
    d1 = (d2 @ W2) * (1.0 - h1 * h1)
    grads = [d1.T @ np.asarray(feat, float), d1.sum(0), d2.T @ h1, d2.sum(0), d3.T @ h2, d3.sum(0)]
    return loss, np.concatenate([g.ravel() for g in grads])
