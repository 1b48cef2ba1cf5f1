"""Public kernel drivers with the reference's signatures, on the GPU.

Mirrors ``src/mbem/kernels/tri_nodal.py:1257-1404`` (the order-generic public
drivers; order 0 is the P0 pair code of ``tri_kernels.py``). Every driver
runs hand-written sm_103a CUDA through the C ABI (``include/mbem_gb300.h``)
in FP64; there is no CPU path. Inputs are numpy arrays (the reference's
types: results come back as numpy) or torch tensors (results stay on the
device). Column layout, node order and basis slots are the reference's:
column ``3 (K s + k) + j``, densities ``(K N_s, 3)``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _native as nat
from .. import defaults
from .._device import as_cuda, is_torch, out_like, ptr, stream_handle


def n_nodes(order: int) -> int:
    """Lagrange nodes per triangle, 1 / 3 / 6 for order 0 / 1 / 2
    (tri_nodal.py:50-54)."""
    if order not in (0, 1, 2):
        raise ValueError(f"order must be 0, 1 or 2 (got {order!r})")
    return (order + 1) * (order + 2) // 2


def _check_shape(tri_verts: np.ndarray) -> None:
    """Refuse needles for a nodal density (tri_nodal.py:1239-1254)."""
    tv = np.asarray(tri_verts.detach().cpu() if isinstance(tri_verts, torch.Tensor) else tri_verts,
                    float)
    if tv.shape[0] == 0:
        return
    e = np.stack([tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 1], tv[:, 0] - tv[:, 2]])
    L = np.linalg.norm(e, axis=2).max(axis=0)
    area2 = np.linalg.norm(np.cross(e[0], -e[2]), axis=1)
    ratio = area2 / np.where(L > 0.0, L * L, 1.0)
    bad = ratio < defaults.NODAL_MIN_HEIGHT_OVER_L
    if bad.any():
        raise ValueError(
            f"{int(bad.sum())} source triangle(s) have height / L < "
            f"{defaults.NODAL_MIN_HEIGHT_OVER_L:g} (min {ratio.min():.2e}): "
            "a nodal (order >= 1) density is not accurate on needles")


def _geom(x_field, tri_verts, eps_arr, normals=None):
    x = as_cuda(x_field).reshape(-1, 3)
    tv = as_cuda(tri_verts).reshape(-1, 3, 3)
    e = as_cuda(eps_arr).reshape(-1)
    if e.shape[0] != tv.shape[0]:
        raise ValueError(f"eps array shape ({e.shape[0]},) != ({tv.shape[0]},)")
    n = None if normals is None else as_cuda(normals).reshape(-1, 3)
    return x, tv, e, n


def _coeffs(*c):
    return nat.dbl_array(c)


def t_matrix_direct(x_field, tri_verts, normals, eps_arr, c1, c2, c3, c4, c5, c6, order=0,
                    out=None, alpha=1.0, accumulate=False):
    """T-kernel matrix (3 N_f, 3 K N_s) with t_coeffs applied in-loop.

    ``out`` (torch, optional) receives the block: ``out = alpha M`` or, with
    ``accumulate``, ``out += alpha M``; it may be a strided row block of a
    larger matrix (unit column stride)."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    res = _out_matrix(out, 3 * x.shape[0], 3 * K * tv.shape[0])
    nat.call("mbem_t_matrix_direct", ptr(x), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0],
             _coeffs(c1, c2, c3, c4, c5, c6), order, float(alpha), int(bool(accumulate)), ptr(res),
             res.stride(0), stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts))


def u_matrix_direct(x_field, tri_verts, eps_arr, g1, g2, g3, order=0, out=None, alpha=1.0,
                    accumulate=False):
    """U-kernel matrix (3 N_f, 3 K N_s) with u_coeffs applied in-loop."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, _ = _geom(x_field, tri_verts, eps_arr)
    res = _out_matrix(out, 3 * x.shape[0], 3 * K * tv.shape[0])
    nat.call("mbem_u_matrix_direct", ptr(x), x.shape[0], ptr(tv), ptr(e), tv.shape[0],
             _coeffs(g1, g2, g3), order, float(alpha), int(bool(accumulate)), ptr(res),
             res.stride(0), stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts))


def _out_matrix(out, rows, cols):
    if out is None:
        return torch.empty((rows, cols), dtype=torch.float64, device=torch.device("cuda"))
    if not isinstance(out, torch.Tensor) or out.dtype != torch.float64 or not out.is_cuda:
        raise ValueError("out must be a float64 CUDA tensor")
    if tuple(out.shape) != (rows, cols) or out.stride(1) != 1:
        raise ValueError(f"out must be ({rows}, {cols}) with unit column stride, got "
                         f"{tuple(out.shape)} strides {out.stride()}")
    return out


def t_basis_matrices(x_field, tri_verts, normals, eps_arr, order=0):
    """T-kernel basis stack (6, 3 N_f, 3 K N_s)."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    res = torch.empty((6, 3 * x.shape[0], 3 * K * tv.shape[0]), dtype=torch.float64, device=x.device)
    nat.call("mbem_t_basis_matrices", ptr(x), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0], order,
             ptr(res), stream_handle())
    return out_like(res, is_torch(x_field, tri_verts))


def u_basis_matrices(x_field, tri_verts, eps_arr, order=0):
    """U-kernel basis stack (3, 3 N_f, 3 K N_s)."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, _ = _geom(x_field, tri_verts, eps_arr)
    res = torch.empty((3, 3 * x.shape[0], 3 * K * tv.shape[0]), dtype=torch.float64, device=x.device)
    nat.call("mbem_u_basis_matrices", ptr(x), x.shape[0], ptr(tv), ptr(e), tv.shape[0], order,
             ptr(res), stream_handle())
    return out_like(res, is_torch(x_field, tri_verts))


def _density(density, n_rows):
    d = as_cuda(density).reshape(-1, 3)
    if d.shape[0] != n_rows:
        raise ValueError(f"density has {d.shape[0]} rows, expected {n_rows}")
    return d


def t_disp_contract(x_field, tri_verts, normals, eps_arr, density, c1, c2, c3, c4, c5, c6, order=0,
                    out=None, alpha=1.0, accumulate=False):
    """Displacement (N_f, 3) of a nodal SLIP density (K N_s, 3)."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    d = _density(density, K * tv.shape[0])
    res = out if out is not None else torch.empty((x.shape[0], 3), dtype=torch.float64, device=x.device)
    nat.call("mbem_t_disp_contract", ptr(x), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0], ptr(d),
             _coeffs(c1, c2, c3, c4, c5, c6), order, float(alpha), int(bool(accumulate)), ptr(res),
             stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts, density))


def t_disp_readout(x_field, tri_verts, normals, eps_arr, density, c1, c2, c3, c4, c5, c6, order=0,
                   out=None, alpha=1.0, accumulate=False, near_factor=defaults.MIXED_NEAR_RADIUS_FACTOR):
    """As ``t_disp_contract`` at order 0, in mixed precision: far pairs by the
    FP32 quadrature of the mixed operator, near pairs (centroid distance below
    ``near_factor`` max(eps, h)) by the FP64 closed form; within ~1e-6 of the
    FP64 contraction."""
    if order != 0:
        raise NotImplementedError("the mixed displacement readout is for P0 densities (order 0)")
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    d = _density(density, tv.shape[0])
    res = out if out is not None else torch.empty((x.shape[0], 3), dtype=torch.float64, device=x.device)
    nat.call("mbem_t_disp_readout", ptr(x), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0], ptr(d),
             _coeffs(c1, c2, c3, c4, c5, c6), float(near_factor), float(alpha), int(bool(accumulate)), ptr(res),
             stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts, density))


def u_disp_contract(x_field, tri_verts, eps_arr, density, g1, g2, g3, order=0, out=None, alpha=1.0,
                    accumulate=False):
    """Displacement (N_f, 3) of a nodal FORCE density (K N_s, 3)."""
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, _ = _geom(x_field, tri_verts, eps_arr)
    d = _density(density, K * tv.shape[0])
    res = out if out is not None else torch.empty((x.shape[0], 3), dtype=torch.float64, device=x.device)
    nat.call("mbem_u_disp_contract", ptr(x), x.shape[0], ptr(tv), ptr(e), tv.shape[0], ptr(d),
             _coeffs(g1, g2, g3), order, float(alpha), int(bool(accumulate)), ptr(res), stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts, density))


def _stress(kind, x_field, tri_verts, normals, eps_arr, density, mu, lam, order, out, alpha,
            accumulate):
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    d = _density(density, K * tv.shape[0])
    res = out if out is not None else torch.empty((x.shape[0], 3, 3), dtype=torch.float64,
                                                  device=x.device)
    nat.call("mbem_stress_contract", kind, ptr(x), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0],
             ptr(d), float(mu), float(lam), order, float(alpha), int(bool(accumulate)), ptr(res),
             stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts, density))


def dd_stress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam, order=0, out=None,
                       alpha=1.0, accumulate=False):
    """TOTAL stress (N_f, 3, 3) of a nodal SLIP density (eigenstress
    included). Material as (mu, lam)."""
    return _stress(nat.STRESS_DD, x_field, tri_verts, normals, eps_arr, density, mu, lam, order, out,
                   alpha, accumulate)


def kelvin_stress_contract(x_field, tri_verts, eps_arr, density, mu, lam, order=0, out=None, alpha=1.0,
                           accumulate=False):
    """Stress (N_f, 3, 3) of a nodal FORCE density. Material as (mu, lam)."""
    return _stress(nat.STRESS_KELVIN, x_field, tri_verts, None, eps_arr, density, mu, lam, order, out,
                   alpha, accumulate)


def eigenstress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam, order=0, out=None,
                         alpha=1.0, accumulate=False):
    """Exact eigenstress +C:eps* (N_f, 3, 3) of a nodal SLIP density, summed
    over every source element."""
    return _stress(nat.STRESS_EIGEN, x_field, tri_verts, normals, eps_arr, density, mu, lam, order,
                   out, alpha, accumulate)


def elastic_stress_contract(x_field, tri_verts, normals, eps_arr, density, mu, lam, order=0, out=None,
                            alpha=1.0, accumulate=False):
    """``dd_stress_contract - eigenstress_contract`` in one pass (the
    subtract-anelastic double layer of evaluate.py:383-407, up to its sign)."""
    return _stress(nat.STRESS_ELASTIC, x_field, tri_verts, normals, eps_arr, density, mu, lam, order,
                   out, alpha, accumulate)


_TRACTION_KINDS = {"slip": 0, "force": 1, "eigen": 2, "total": 3}


def traction_matrix(x_field, n_field, tri_verts, normals, eps_arr, ids, n_cols, mu, lam, order,
                    which="slip", out=None, alpha=1.0):
    """Traction rows (3 N_f, 3 n_cols) of a nodal density, columns scattered
    by ``ids`` (N_s, K) (tri_nodal.py:1370-1404)."""
    if which not in _TRACTION_KINDS:
        raise KeyError(which)
    K = n_nodes(order)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    nf = as_cuda(n_field).reshape(-1, 3)
    ids_np = np.ascontiguousarray(np.asarray(ids.cpu() if isinstance(ids, torch.Tensor) else ids,
                                             dtype=np.int64))
    if ids_np.shape != (tv.shape[0], K):
        raise ValueError(f"ids shape {ids_np.shape} != ({tv.shape[0]}, {K})")
    if ids_np.size and (ids_np.min() < 0 or ids_np.max() >= n_cols):
        raise ValueError(f"ids must index 0 .. n_cols - 1 = {int(n_cols) - 1}")
    if order:
        _check_shape(tri_verts)
    if which == "force":
        n = torch.zeros_like(tv[:, 0, :])
    ids_d = as_cuda(ids_np, dtype=torch.int64)
    res = _out_matrix(out, 3 * x.shape[0], 3 * int(n_cols)) if out is not None else torch.zeros(
        (3 * x.shape[0], 3 * int(n_cols)), dtype=torch.float64, device=x.device)
    nat.call("mbem_traction_matrix", ptr(x), ptr(nf), x.shape[0], ptr(tv), ptr(n), ptr(e), tv.shape[0],
             ptr(ids_d), int(n_cols), float(mu), float(lam), order, _TRACTION_KINDS[which],
             float(alpha), ptr(res), res.stride(0), stream_handle())
    return res if out is not None else out_like(res, is_torch(x_field, tri_verts))


def elastic_stress_readout(x_field, tri_verts, normals, eps_arr, density, mu, lam, order=0, near_factor=3.0,
                           out=None, alpha=1.0, accumulate=False, eig_out=None):
    """The elastic stress (DD minus eigen) of a nodal slip density at many
    points, mixed precision (FP32 quadrature far field, FP64 near pairs):
    ``elastic_stress_contract``'s result to ~1e-6. The observers are ordered
    along a Morton curve for the launch (neighbouring threads then take the
    same quadrature rule), the result in the caller's order. ``eig_out`` (a
    CUDA (N, 3, 3) tensor) receives alpha times the eigenstress of the same
    pairs, (+)= as ``out`` (``eigenstress_contract``'s result to ~1e-6)."""
    import torch
    K = n_nodes(order)
    if order:
        _check_shape(tri_verts)
    x, tv, e, n = _geom(x_field, tri_verts, eps_arr, normals)
    d = _density(density, K * tv.shape[0])
    N = x.shape[0]
    dev = x.device
    # Morton order of the observers
    lo = x.min(dim=0).values
    span = torch.clamp(x.max(dim=0).values - lo, min=1e-300)
    q = ((x - lo) / span * 1023.0).round().to(torch.int64).clamp(0, 1023)

    def spread(v):
        v = (v | (v << 16)) & 0x030000FF
        v = (v | (v << 8)) & 0x0300F00F
        v = (v | (v << 4)) & 0x030C30C3
        return (v | (v << 2)) & 0x09249249
    code = spread(q[:, 0]) | (spread(q[:, 1]) << 1) | (spread(q[:, 2]) << 2)
    perm = torch.argsort(code)
    xs = x.index_select(0, perm).contiguous()
    ns = tv.shape[0]
    rec = torch.empty(nat.lib().mbem_readout_record_bytes(ns) // 4, dtype=torch.float32, device=dev)
    counts = torch.empty(max(N, 1), dtype=torch.int64, device=dev)
    rowptr = torch.empty(N + 1, dtype=torch.int64, device=dev)
    n_near = ctypes.c_int64(0)
    st = stream_handle()
    nat.call("mbem_readout_prepare", ptr(xs), N, ptr(tv), ptr(n), ptr(e), ns, ptr(d), order, float(near_factor),
             ptr(rec), ptr(counts), ptr(rowptr), ctypes.byref(n_near), st)
    m = max(int(n_near.value), 1)
    pair_obs = torch.empty(m, dtype=torch.int64, device=dev)
    pair_src = torch.empty(m, dtype=torch.int32, device=dev)
    pair_out = torch.empty((m, 9), dtype=torch.float64, device=dev)
    res = torch.empty((N, 3, 3), dtype=torch.float64, device=dev)
    eig = None
    if eig_out is not None:
        if not (isinstance(eig_out, torch.Tensor) and eig_out.is_cuda and eig_out.shape == (N, 3, 3)):
            raise TypeError("eig_out must be a CUDA (N, 3, 3) tensor")
        pair_eig = torch.empty((m, 9), dtype=torch.float64, device=dev)
        eig = torch.empty((N, 3, 3), dtype=torch.float64, device=dev)
        nat.call("mbem_readout_evaluate_parts", ptr(xs), N, ptr(tv), ptr(n), ptr(e), ns, ptr(d), float(mu),
                 float(lam), order, ptr(rec), ptr(rowptr), int(n_near.value), ptr(pair_obs), ptr(pair_src),
                 ptr(pair_out), ptr(pair_eig), 1.0, 0, ptr(res), ptr(eig), st)
        full_e = torch.empty_like(eig)
        full_e[perm] = eig
        if accumulate:
            eig_out += alpha * full_e
        else:
            eig_out.copy_(alpha * full_e)
    else:
        nat.call("mbem_readout_evaluate", ptr(xs), N, ptr(tv), ptr(n), ptr(e), ns, ptr(d), float(mu), float(lam),
                 order, ptr(rec), ptr(rowptr), int(n_near.value), ptr(pair_obs), ptr(pair_src), ptr(pair_out), 1.0,
                 0, ptr(res), st)
    full = torch.empty_like(res)
    full[perm] = res
    if out is not None:
        o = out if isinstance(out, torch.Tensor) else None
        if o is None:
            raise TypeError("out must be a CUDA tensor")
        if accumulate:
            o += alpha * full
        else:
            o.copy_(alpha * full)
        return o
    full = alpha * full if alpha != 1.0 else full
    return out_like(full, is_torch(x_field, tri_verts, density))
