"""The mixed operator's far-field quadrature rules against the FP64 closed
form of the oracle (oracle/p0_oracle.c, the reference's T block): a numpy
restatement of the far T block (the formula of csrc/far_quad.cuh far_block,
in FP64 arithmetic) with the rule tables of far_quad.cuh make_rules. Radon's
7-point rule, which the far field uses from D/L = 5 on, is exact to degree 5
and within 1e-7 of the closed form there; at D/L = 7.07, where the collapsed
3 x 3 rule took over before, it is the more accurate of the two."""

import numpy as np
import pytest

from mbem_gb300.kernels import basis as kb

oracle = pytest.importorskip("oracle.oracle")


def _collapsed(n):
    g, gw = np.polynomial.legendre.leggauss(n)
    pts = []
    for i in range(n):
        for j in range(n):
            gi, gj = 0.5 * (g[i] + 1.0), 0.5 * (g[j] + 1.0)
            pts.append((gi, gj * (1.0 - gi), 0.25 * gw[i] * gw[j] * (1.0 - gi)))
    return np.array(pts)


def _radon():
    s15 = np.sqrt(15.0)
    p1, q1, w1 = (6 - s15) / 21, (9 + 2 * s15) / 21, (155 - s15) / 2400
    p2, q2, w2 = (6 + s15) / 21, (9 - 2 * s15) / 21, (155 + s15) / 2400
    return np.array([(1 / 3, 1 / 3, 9 / 80), (p1, p1, w1), (p1, q1, w1), (q1, p1, w1),
                     (p2, p2, w2), (p2, q2, w2), (q2, p2, w2)])


def _far_t_block(x, tv, n, eps, c, rule):
    """far_block<true>'s sums and epilogue for one pair (FP64)."""
    e1, e2 = tv[1] - tv[0], tv[2] - tv[0]
    area2 = np.linalg.norm(np.cross(e1, e2))
    y = tv[0] + rule[:, :1] * e1 + rule[:, 1:2] * e2
    d = x - y
    r2 = (d * d).sum(1)
    iR = 1.0 / np.sqrt(r2 + eps * eps)
    w3 = rule[:, 2] * iR ** 3
    w5 = w3 * iR ** 2
    V3, V5 = (w3[:, None] * d).sum(0), (w5[:, None] * d).sum(0)
    t = ((w5 * r2)[:, None] * d).sum(0)
    W = np.einsum("q,qi,qj->ij", w5 * (d @ n), d, d)
    ca, cb = c[0] + 4 * c[1] + 2 * c[4], c[3] + c[4]
    ce3, ce6 = c[2] * eps ** 2, c[5] * eps ** 2
    gam = cb * (n @ V3) + ce6 * (n @ V5)
    alpha = ca * V3 - 3 * c[1] * t + ce3 * V5
    beta = cb * V3 + ce6 * V5
    return area2 * (np.outer(alpha, n) + np.outer(n, beta) - 6 * c[4] * W + gam * np.eye(3))


def test_radon_rule_is_exact_to_degree_five():
    from math import factorial
    r = _radon()
    assert abs(r[:, 2].sum() - 0.5) < 1e-15
    for deg in range(6):
        for a in range(deg + 1):
            exact = factorial(a) * factorial(deg - a) / factorial(deg + 2)
            assert abs((r[:, 2] * r[:, 0] ** a * r[:, 1] ** (deg - a)).sum() - exact) < 1e-15


# beyond D/L ~ 15 the bound is the closed form's own FP64 cancellation (~1e-10)
@pytest.mark.parametrize("ratio, bound", [(5.0, 1.0e-7), (7.07, 2.0e-8), (10.0, 3.0e-9), (20.0, 1.0e-9),
                                          (40.0, 1.0e-9)])
def test_radon_far_block_against_the_closed_form(ratio, bound):
    h = 4.0 / 48
    tv = np.array([[0.0, 0.0, 0.0], [h, 0.0, 0.0], [0.0, h, 0.0]])
    n = np.array([0.0, 0.0, 1.0])
    eps = h / 2
    L = np.sqrt(2.0) * h
    c = kb.t_coeffs(1.0, 1.0)
    rng = np.random.default_rng(int(ratio * 100))
    dirs = rng.normal(size=(64, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    x = np.array([h / 3, h / 3, 0.0]) + ratio * L * dirs
    ref = oracle.matrix("t", x, tv[None], n[None], np.array([eps]), c)
    worst_radon = worst_c3 = 0.0
    for f in range(x.shape[0]):
        blk = ref[3 * f:3 * f + 3, :]
        scale = np.linalg.norm(blk)
        worst_radon = max(worst_radon, np.linalg.norm(_far_t_block(x[f], tv, n, eps, c, _radon()) - blk) / scale)
        worst_c3 = max(worst_c3, np.linalg.norm(_far_t_block(x[f], tv, n, eps, c, _collapsed(3)) - blk) / scale)
    assert worst_radon < bound, worst_radon
    if ratio == 7.07:
        assert worst_radon < 0.2 * worst_c3, (worst_radon, worst_c3)
