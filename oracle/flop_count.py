"""Algorithmic work per (observer, source) pair, counted on the oracle
(TEST INFRASTRUCTURE, not the product).

``flop_count.cpp`` compiles ``p0_oracle.c`` with a counting ``double`` and
walks pairs through its pair functions; this module builds it and reports,
per pair, the FLOPs (adds + multiplies, an FMA being two) with divides and
special functions (sqrt, log, atan2) beside them, averaged over the pairs of
a workload (pairs on one face take the closed form's coplanar shortcuts, so
the average depends on the mix).

    python oracle/flop_count.py        # the table for the cube-12 workload
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "flop_count.cpp")
LIB = os.path.join(HERE, "_build", "libflop_count.so")
KINDS = {"t": 0, "u": 1, "dd_stress": 2, "kelvin_stress": 3, "eigenstress": 4, "solid_angle": 5}

_lib = None


def build() -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", SRC, "-o", LIB], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        newest = max(os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "p0_oracle.c")))
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
            build()
        h = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int64
        h.flop_count.argtypes = [ctypes.c_int, P, I, P, P, P, I, P]
        h.flop_count.restype = ctypes.c_longlong
        _lib = h
    return _lib


def pair_work(kind: str, x_field, tri_verts, normals, eps) -> dict:
    """Counts per pair, averaged over every (observer, source) pair."""
    x = np.ascontiguousarray(x_field, dtype=np.float64)
    tv = np.ascontiguousarray(tri_verts, dtype=np.float64)
    n = np.ascontiguousarray(normals, dtype=np.float64)
    e = np.ascontiguousarray(np.broadcast_to(eps, (tv.shape[0],)), dtype=np.float64)
    counts = np.zeros(4, dtype=np.int64)
    pairs = lib().flop_count(KINDS[kind], x.ctypes.data, x.shape[0], tv.ctypes.data, n.ctypes.data, e.ctypes.data,
                             tv.shape[0], counts.ctypes.data)
    add, mul, div, special = (float(c) / max(pairs, 1) for c in counts)
    return {"pairs": int(pairs), "flops": add + mul, "add": add, "mul": mul, "div": div, "special": special}


def cube_table(n_face: int = 12, stride: int = 4) -> dict:
    """Every kind on the cube workload: every cube source against every
    ``stride``-th collocation point (centroids), eps = half the grid spacing."""
    sys.path.insert(0, os.path.dirname(HERE))
    from mbem_gb300 import mesh as M
    cube = M.cube(n_face)
    tv = cube.tri_verts()
    nrm, _ = cube.normals_and_areas()
    x = cube.centroids()[::stride]
    eps = (4.0 / n_face) / 2.0
    return {k: pair_work(k, x, tv, nrm, eps) for k in KINDS}


if __name__ == "__main__":
    for k, v in cube_table().items():
        print(f"{k:14s} pairs {v['pairs']:8d}  flops {v['flops']:8.1f}  (add {v['add']:.1f}, mul {v['mul']:.1f})  "
              f"div {v['div']:.1f}  special {v['special']:.1f}")
