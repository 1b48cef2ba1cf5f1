"""ctypes front end of the C oracle (TEST INFRASTRUCTURE, not the product).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
use this module, to check the CUDA path or as the timed CPU baseline. It restates the
reference's P0 kernels (``src/mbem/kernels/tri_kernels.py``) in plain C with
OpenMP (``p0_oracle.c``); ``tests/test_oracle.py`` pins it to golden vectors
that the reference itself produced (``tests/golden/``).

Build: ``python oracle/build.py`` (gcc -O2 -fopenmp -ffp-contract=off, so
x86_64 and aarch64 round alike).
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "p0_oracle.c")
LIB = os.path.join(HERE, "_build", "libp0_oracle.so")

_lib = None


def build() -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
            build()
        h = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int64
        h.oracle_matrix.argtypes = [ctypes.c_int, P, I, P, P, P, I, P, I, I, P]
        h.oracle_contract.argtypes = [ctypes.c_int, P, I, P, P, P, I, P, P, I, I, P]
        h.oracle_dgemv.argtypes = [P, I, I, P, I, I, P]
        h.oracle_flat_matvec.argtypes = [I, I, P, P, I, P, P, P, P, P, P, P, P, P, P, I, P, P, P, P, P, P, I, P,
                                         P, P, P, P, P]
        h.oracle_flat_matvec.restype = None
        h.oracle_set_threads.argtypes = [ctypes.c_int]
        h.oracle_set_threads.restype = ctypes.c_int
        _lib = h
    return _lib


def set_threads(n: int) -> int:
    """Set the OpenMP thread count (n <= 0 keeps it); returns the count in use."""
    return lib().oracle_set_threads(int(n))


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _geom(x_field, tri_verts, normals, eps):
    x = _c(x_field).reshape(-1, 3)
    tv = _c(tri_verts).reshape(-1, 3, 3)
    n = _c(normals).reshape(-1, 3) if normals is not None else np.zeros((tv.shape[0], 3))
    e = _c(eps).reshape(-1)
    return x, tv, n, e


def matrix(kind: str, x_field, tri_verts, normals, eps, coeffs=None, src_range=None):
    """kind: "t" / "u" direct matrices (coeffs 6 / 3), "t_basis" / "u_basis"
    stacks. ``src_range`` = (s0, s1) computes only those source columns
    (the others stay zero) for bounded CPU timing."""
    k = {"t": 0, "u": 1, "t_basis": 2, "u_basis": 3}[kind]
    x, tv, n, e = _geom(x_field, tri_verts, normals, eps)
    Nf, Ns = x.shape[0], tv.shape[0]
    nb = {0: 1, 1: 1, 2: 6, 3: 3}[k]
    out = np.zeros((nb, 3 * Nf, 3 * Ns)) if nb > 1 else np.zeros((3 * Nf, 3 * Ns))
    c = _c(coeffs if coeffs is not None else np.zeros(6))
    s0, s1 = src_range if src_range is not None else (0, Ns)
    lib().oracle_matrix(k, _p(x), Nf, _p(tv), _p(n), _p(e), Ns, _p(c), int(s0), int(s1), _p(out))
    return out


def contract(kind: str, x_field, tri_verts, normals, eps, density, coeffs=None, mu=None, lam=None,
             field_range=None):
    """kind: "t_disp", "u_disp" (coeffs), "dd", "kelvin", "eigen" (mu, lam).
    ``field_range`` = (f0, f1) evaluates only those observers."""
    k = {"t_disp": 0, "u_disp": 1, "dd": 2, "kelvin": 3, "eigen": 4}[kind]
    x, tv, n, e = _geom(x_field, tri_verts, normals, eps)
    d = _c(density).reshape(-1, 3)
    Nf, Ns = x.shape[0], tv.shape[0]
    out = np.zeros((Nf, 3)) if k <= 1 else np.zeros((Nf, 3, 3))
    c = _c(coeffs) if k <= 1 else _c([mu, lam])
    f0, f1 = field_range if field_range is not None else (0, Nf)
    lib().oracle_contract(k, _p(x), Nf, _p(tv), _p(n), _p(e), Ns, _p(d), _p(c), int(f0), int(f1),
                          _p(out))
    return out


def dgemv(A, x, row_range=None):
    A = _c(A)
    x = _c(x)
    y = np.zeros(A.shape[0])
    r0, r1 = row_range if row_range is not None else (0, A.shape[0])
    lib().oracle_dgemv(_p(A), A.shape[0], A.shape[1], _p(x), int(r0), int(r1), _p(y))
    return y


def flat_matvec(view: dict, x) -> np.ndarray:
    """y = A x for a compressed pair's flat view held on the host: ``view``
    maps the field names of the C view (``mbem_compressed_view``) to numpy
    arrays (``PairCompressed.view_host``)."""
    v = view
    x = _c(x)
    y = np.zeros(3 * int(v["n_field"]))
    lib().oracle_flat_matvec(
        int(v["n_field"]), int(v["n_src"]), _p(v["field_order"]), _p(v["src_order"]), int(v["n_lr"]),
        _p(v["lr_r0"]), _p(v["lr_nr"]), _p(v["lr_c0"]), _p(v["lr_nc"]), _p(v["lr_rank"]), _p(v["lr_u"]),
        _p(v["lr_v"]), _p(v["lr_w"]), _p(v["U"]), _p(v["V"]), int(v["n_w"]), _p(v["d_r0"]), _p(v["d_nr"]),
        _p(v["d_nc"]),
        _p(v["d_c0"]), _p(v["d_off"]), _p(v["D"]), int(v["n_strips"]), _p(v["strip_r0"]), _p(v["strip_nr"]),
        _p(v["strip_ptr"]), _p(v["strip_items"]), _p(x), _p(y))
    return y
