"""The arithmetic counter on the oracle (no GPU): the van Oosterom solid
angle counts exactly what its formula holds (9 differences, three norms,
a cross and three dot products, the denominator: 62 FLOPs, 3 sqrt and an
atan2), and the pair kinds of the cube workload keep their counts."""

import numpy as np
import pytest

from mbem_gb300 import mesh as M
from oracle import flop_count as fc


@pytest.fixture(scope="module")
def cube4():
    cube = M.cube(4)
    nrm, _ = cube.normals_and_areas()
    return cube.centroids(), cube.tri_verts(), nrm, 0.5


def test_solid_angle_count_is_exact(cube4):
    x, tv, n, eps = cube4
    w = fc.pair_work("solid_angle", x, tv, n, eps)
    assert w["pairs"] == x.shape[0] * tv.shape[0]
    assert (w["add"], w["mul"], w["div"], w["special"]) == (29.0, 33.0, 0.0, 4.0)


def test_pair_counts_are_in_their_bands(cube4):
    """Bands around the counts on the cube-12 workload (cube_table): the
    closed forms' branch mix moves them only a little between meshes."""
    x, tv, n, eps = cube4
    bands = {"t": (2800, 3200), "u": (650, 720), "dd_stress": (20000, 22000), "kelvin_stress": (2800, 3200),
             "eigenstress": (2450, 2650)}
    for kind, (lo, hi) in bands.items():
        w = fc.pair_work(kind, x, tv, n, eps)
        assert lo <= w["flops"] <= hi, (kind, w)
        assert w["special"] > 0 and w["div"] > 0
