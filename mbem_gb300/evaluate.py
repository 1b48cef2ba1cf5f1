"""Representation-formula readout on the GPU (``src/mbem/evaluate.py``).

``evaluate_stress(model, region, solution, points, eps,
subtract_anelastic=True)`` (evaluate.py:598-695):

    sigma = sum_p [ -sigma_p (S_H - E) u_p + sigma_p S_G t_p ]
            - sum_f sigma_f (S_H - E) slip_f

Each double layer (boundary u_p or fault slip) is ONE fused CUDA pass that
evaluates the DD stress and the exact finite-triangle eigenstress from the
same moment tables (they share I7), where the reference runs the DD kernel
and then a KD-tree near list of the eigenstress (evaluate.py:298-326). The
fused pass sums the eigenstress over every element; beyond the reference's
near radius 20 (eps + h) the terms it omits are below 1e-12 of the on-fault
value, so the two agree to that level.
"""

from __future__ import annotations

import warnings

import numpy as np
import torch

from . import defaults
from ._device import as_cuda, is_torch, out_like
from .kernels import basis as kb
from .kernels import tri_nodal as tn
from .model.core import BCType, Region, RegionModel


def _region(model: RegionModel, region) -> Region:
    if isinstance(region, Region):
        return region
    for r in model.regions:
        if r.name == region:
            return r
    raise KeyError(f"no region named {region!r} (regions: {[r.name for r in model.regions]})")


def _density(model: RegionModel, patch, kind: str, solution: dict) -> np.ndarray:
    if kind == "slip":
        if patch.bc is BCType.FAULT_TRACTION:
            return patch.expand(np.asarray(solution[f"b:{patch.name}"]))
        return patch.density()
    fixed = {"u": BCType.PRESCRIBED_DISPLACEMENT, "t": BCType.FREE_TRACTION}
    if kind not in fixed:
        raise ValueError(f"unknown density kind {kind!r}")
    if patch.bc is fixed[kind]:
        return model.value_of(patch)
    return np.asarray(solution[f"{kind}:{patch.name}"])


def _src(patch, eps):
    normals, _ = patch.mesh.normals_and_areas()
    return (as_cuda(patch.tri_verts()), as_cuda(normals), as_cuda(kb.resolve_patch_eps(eps, patch)))


def _warn_near_boundary(points: np.ndarray, region: Region) -> None:
    """Points within NEAR_BOUNDARY_H_RATIO local h of a boundary patch
    (distance to the nearest centroid as the estimate)."""
    for p in region.patches:
        cen = p.mesh.centroids()
        h = kb.element_sizes(p.mesh)
        if points.shape[0] == 0:
            return
        d2 = ((points[:, None, :] - cen[None, :, :]) ** 2).sum(-1) if points.shape[0] * cen.shape[0] < 4e7 \
            else None
        if d2 is None:
            return
        idx = d2.argmin(axis=1)
        ratio = np.sqrt(d2[np.arange(points.shape[0]), idx]) / h[idx]
        close = ratio < defaults.NEAR_BOUNDARY_H_RATIO
        if close.any():
            warnings.warn(f"{int(close.sum())} of {close.size} observation point(s) lie within "
                          f"{defaults.NEAR_BOUNDARY_H_RATIO}*local-h of boundary patch {p.name}")


def evaluate_stress(model: RegionModel, region, solution: dict, points, eps,
                    subtract_anelastic: bool = True, warn_near: bool = True, parts: bool = False,
                    near=None, precision: str = "fp64"):
    """Stress (N, 3, 3) at ``points`` of ``region``; with ``parts`` also the
    summed eigenstress. ``near`` (continuous near-field recovery) is not part
    of the GPU path. ``precision="mixed"``: the double layers' elastic stress
    by FP32 quadrature for the far pairs and FP64 for the near ones (within
    ~1e-6 of the FP64 readout; subtract_anelastic only)."""
    if near is not None:
        raise NotImplementedError("near-field recovery (near=) is not on the GPU readout path")
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed' (got {precision!r})")
    if precision == "mixed" and not subtract_anelastic:
        raise NotImplementedError("the mixed readout evaluates the elastic stress (subtract_anelastic=True)")
    region = _region(model, region)
    torch_in = is_torch(points)
    pts = as_cuda(points).reshape(-1, 3)
    if warn_near and not torch_in:
        _warn_near_boundary(np.asarray(points, float).reshape(-1, 3), region)
    sig = torch.zeros((pts.shape[0], 3, 3), dtype=torch.float64, device=pts.device)
    eig = torch.zeros_like(sig) if parts else None
    mat = region.material
    mu, lam = mat.mu, mat.lam

    def double_layer(patch, jump, sigma):
        tv, nrm, e = _src(patch, eps)
        d = as_cuda(np.asarray(jump, float).reshape(-1, 3))
        if subtract_anelastic and precision == "mixed":
            # the eigenstress (parts) from the same quadrature and near pairs:
            # eig += sigma E, sig -= sigma (S_H - E)
            if parts:
                e_tmp = torch.zeros_like(eig)
                tn.elastic_stress_readout(pts, tv, nrm, e, d, mu, lam, patch.order, out=sig, alpha=-sigma,
                                          accumulate=True, eig_out=e_tmp)
                eig.sub_(e_tmp)
            else:
                tn.elastic_stress_readout(pts, tv, nrm, e, d, mu, lam, patch.order, out=sig, alpha=-sigma,
                                          accumulate=True)
            return
        elif subtract_anelastic:
            tn.elastic_stress_contract(pts, tv, nrm, e, d, mu, lam, patch.order, out=sig,
                                       alpha=-sigma, accumulate=True)
        else:
            tn.dd_stress_contract(pts, tv, nrm, e, d, mu, lam, patch.order, out=sig, alpha=-sigma,
                                  accumulate=True)
        if parts:
            tn.eigenstress_contract(pts, tv, nrm, e, d, mu, lam, patch.order, out=eig, alpha=sigma,
                                    accumulate=True)

    for p in region.patches:
        sigma = float(model.orientation(region, p))
        u_p = _density(model, p, "u", solution)
        if np.any(u_p):
            double_layer(p, u_p, sigma)
        t_p = _density(model, p, "t", solution)
        if np.any(t_p):
            tv, _, e = _src(p, eps)
            tn.kelvin_stress_contract(pts, tv, e, as_cuda(np.asarray(t_p, float).reshape(-1, 3)), mu, lam,
                                      p.order, out=sig, alpha=sigma, accumulate=True)
    for f in region.faults:
        sigma = float(model.orientation(region, f))
        slip = _density(model, f, "slip", solution)
        if np.any(slip):
            double_layer(f, slip, sigma)
    if parts:
        return out_like(sig, torch_in), out_like(eig, torch_in)
    return out_like(sig, torch_in)


def evaluate_displacement(model: RegionModel, region, solution: dict, points, eps, warn_near=True,
                          near=None, precision: str = "fp64"):
    """Displacement (N, 3) at interior ``points`` (evaluate.py:194-250).
    ``precision="mixed"``: the P0 double layers (boundary u and fault slip)
    by FP32 quadrature for the far pairs and the FP64 closed form for the
    near ones (within ~1e-6 of the FP64 readout); single layers and P1/P2
    double layers stay FP64."""
    if near is not None:
        raise NotImplementedError("near-field recovery (near=) is not on the GPU readout path")
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed' (got {precision!r})")
    region = _region(model, region)
    torch_in = is_torch(points)
    pts = as_cuda(points).reshape(-1, 3)
    u = torch.zeros((pts.shape[0], 3), dtype=torch.float64, device=pts.device)
    mat = region.material
    c = kb.t_coeffs(mat.mu, mat.lam)
    g = kb.u_coeffs(mat.mu, mat.lam)
    def double_layer(patch, tv, nrm, e, jump, sigma):
        d = as_cuda(np.asarray(jump, float).reshape(-1, 3))
        if precision == "mixed" and patch.order == 0:
            tn.t_disp_readout(pts, tv, nrm, e, d, *c, 0, out=u, alpha=-sigma, accumulate=True)
        else:
            tn.t_disp_contract(pts, tv, nrm, e, d, *c, patch.order, out=u, alpha=-sigma, accumulate=True)

    for p in region.patches:
        sigma = float(model.orientation(region, p))
        tv, nrm, e = _src(p, eps)
        u_p = _density(model, p, "u", solution)
        if np.any(u_p):
            double_layer(p, tv, nrm, e, u_p, sigma)
        t_p = _density(model, p, "t", solution)
        if np.any(t_p):
            tn.u_disp_contract(pts, tv, e, as_cuda(np.asarray(t_p, float).reshape(-1, 3)), *g, p.order,
                               out=u, alpha=sigma, accumulate=True)
    for f in region.faults:
        sigma = float(model.orientation(region, f))
        slip = _density(model, f, "slip", solution)
        if np.any(slip):
            tv, nrm, e = _src(f, eps)
            double_layer(f, tv, nrm, e, slip, sigma)
    return out_like(u, torch_in)
