"""CPU assembly of a BlockSystem with the C oracle (TEST INFRASTRUCTURE, not
the product).

Walks the terms that ``mbem_gb300.model.generate_system`` emits exactly as
the reference's AssembledDense._build does (``src/mbem/backends/dense.py:480-528``):
blocks, the calibrated diagonal from the blocks' row sums, the RHS products.
Used by ``tests/`` to check the host-side model logic on a machine without a
GPU and as the oracle system at sizes the reference cannot hold, and by the
CPU legs of ``bench.py`` for the port's own complete solve.
"""

from __future__ import annotations

import numpy as np

from mbem_gb300.kernels import KERNEL_T, KERNEL_U
from mbem_gb300.kernels import basis as kb
from mbem_gb300.model.equations import calibrated_diagonal, term_diagonal


def _block(orc, q, p, kernel, mat, eps):
    x = q.collocation_points()
    tv = p.tri_verts()
    n, _ = p.mesh.normals_and_areas()
    e = kb.resolve_patch_eps(eps, p)
    if p.order != 0:
        raise NotImplementedError("the C oracle is P0")
    if kernel == KERNEL_T:
        return orc.matrix("t", x, tv, n, e, kb.t_coeffs(mat.mu, mat.lam))
    if kernel == KERNEL_U:
        return orc.matrix("u", x, tv, None, e, kb.u_coeffs(mat.mu, mat.lam))
    raise NotImplementedError(kernel)


def assemble(orc, system, eps, jump="calibrated"):
    lay = system.layout
    n = lay.n_unknowns
    cache = {}

    def block(q, p, kernel, region):
        key = (id(q), id(p), kernel)
        if key not in cache:
            cache[key] = _block(orc, q, p, kernel, region.material, eps)
        return cache[key]

    calib = None
    if jump == "calibrated":
        calib = calibrated_diagonal(
            system, lambda r, q, p: block(q, p, KERNEL_T, r).reshape(q.n_nodes, 3, p.n_nodes, 3).sum(axis=2))
    A = np.zeros((n, n))
    for t in system.terms:
        A[t.row.offset:t.row.stop, t.col.offset:t.col.stop] += t.scale * block(
            t.field_patch, t.source_patch, t.kernel, t.region)
        D = term_diagonal(t, calib)
        if D is not None:
            shape = t.field_patch.collocation_shape()
            K = shape.shape[0]
            for c in range(D.shape[0]):
                s, kc = divmod(c, K)
                for k in range(K):
                    r0, c0 = t.row.offset + 3 * c, t.col.offset + 3 * (K * s + k)
                    A[r0:r0 + 3, c0:c0 + 3] += shape[kc, k] * D[c]
    b = np.zeros(n)
    for rt in system.rhs_terms:
        b[rt.row.offset:rt.row.stop] += rt.scale * (block(rt.field_patch, rt.source_patch, rt.kernel,
                                                          rt.region) @ rt.vector)
    return A, b, calib


def deflated_solve(A, b, layout):
    """The reference's bordered solve [[A, Z], [Z^T, 0]] (dense.py:538-566)."""
    from mbem_gb300.backends.dense import translation_basis
    Z = translation_basis(layout)
    n = A.shape[0]
    K = np.zeros((n + 3, n + 3))
    K[:n, :n] = A
    K[:n, n:] = Z
    K[n:, :n] = Z.T
    return np.linalg.solve(K, np.concatenate([b, np.zeros(3)]))[:n]
