"""What the dense backend warns about while it assembles
(``src/mbem/backends/dense.py:124-244``): settings and geometry that the
method does not correct and that a user should know of.

- ``jump="half"`` with eps/h above ``HALF_JUMP_MAX_EPS_OVER_H`` on any patch:
  that pairing does not converge under mesh refinement.
- A boundary collocation point within ``COLLOCATION_FAULT_CLEARANCE_EPS``
  fault-eps of a fault element of its region (a fault outcrop): the row reads
  the fault's mollified blob, not the one-sided field its condition means.
- The mirror case: a FAULT_TRACTION node that close to a boundary patch.

The distances are exact point-to-triangle distances from the GPU kernel
(``geometry.distance_to_mesh``), measured in units of the eps of the nearest
element. Nothing is changed in the system; each case is one warning.
"""

from __future__ import annotations

import warnings

import numpy as np

from .. import defaults
from ..kernels import basis as kb


def _eps_or_none(spec, patch):
    """The patch's per-element eps, or None when the spec is unusable (the
    assembly reports that itself)."""
    try:
        return kb.resolve_patch_eps(spec, patch)
    except ValueError:
        return None


def warn_half_jump_eps(system, eps, jump: str) -> None:
    if jump != "half":
        return
    ratios = []
    for region in system.model.regions:
        for patch in (*region.patches, *region.faults):
            e = _eps_or_none(eps, patch)
            if e is not None:
                ratios.append((float(np.max(e / kb.element_sizes(patch.mesh))), patch.name))
    if not ratios:
        return
    worst, name = max(ratios)
    if worst > defaults.HALF_JUMP_MAX_EPS_OVER_H:
        warnings.warn(f"jump='half' with eps/h = {worst:.2f} on patch '{name}' (limit "
                      f"{defaults.HALF_JUMP_MAX_EPS_OVER_H}): this combination was measured NON-convergent under "
                      f"h-refinement; use jump='calibrated' or a smaller eps")


def _clearance(points: np.ndarray, mesh, eps_of_element: np.ndarray):
    """(number of points closer than the clearance limit, smallest d / eps;
    inf when none is). A point farther from the mesh's bounding box than the
    limit times the largest eps cannot count, so only the others go to the
    exact distance."""
    from ..geometry import distance_to_mesh
    if points.shape[0] == 0 or mesh.n_triangles == 0:
        return 0, np.inf
    limit = defaults.COLLOCATION_FAULT_CLEARANCE_EPS
    v = np.asarray(mesh.vertices, float)[np.unique(np.asarray(mesh.triangles))]
    lo, hi = v.min(axis=0), v.max(axis=0)
    gap = np.maximum(np.maximum(lo - points, points - hi), 0.0)
    near = np.sqrt((gap * gap).sum(axis=1)) <= limit * float(np.max(eps_of_element))
    if not near.any():
        return 0, np.inf
    d, idx = distance_to_mesh(points[near], mesh)
    ratio = np.asarray(d) / eps_of_element[np.asarray(idx)]
    count = int(np.count_nonzero(ratio < limit))
    return count, (float(ratio.min()) if count else np.inf)


def _report(found, what: str, where: str, tail: str) -> None:
    if not found:
        return
    count = sum(c for c, _, _ in found)
    worst = min(r for _, r, _ in found)
    names = ", ".join(n for _, _, n in found)
    warnings.warn(f"{count} {what} lie within {defaults.COLLOCATION_FAULT_CLEARANCE_EPS:g} {where} ({names}; "
                  f"min d/eps = {worst:.2f}): {tail}")


def warn_collocation_near_fault(system, eps) -> None:
    found = []
    for region in system.model.regions:
        for fault in region.faults:
            e = _eps_or_none(eps, fault)
            if e is None:
                continue
            for patch in region.patches:
                count, worst = _clearance(patch.collocation_points(), fault.mesh, e)
                if count:
                    found.append((count, worst, f"{patch.name}/{fault.name}"))
    _report(found, "boundary collocation point(s)", "fault-eps of a fault element",
            "the fault's mollified field there is the blob average across the slip surface, not the one-sided "
            "value the boundary condition means (fault outcrop); the row is not corrected")


def warn_fault_rows_near_boundary(system, eps) -> None:
    found = []
    for region, fault in system.traction_faults():
        if getattr(fault, "slip", None) is not None:
            continue                      # an interface's rows read no kernel
        pts = fault.collocation_points()
        for patch in region.patches:
            e = _eps_or_none(eps, patch)
            if e is None:
                continue
            count, worst = _clearance(pts, patch.mesh, e)
            if count:
                found.append((count, worst, f"{fault.name}/{patch.name}"))
    _report(found, "FAULT_TRACTION node(s)", "boundary-eps of a boundary patch",
            "those traction rows see the patch's blob average (an outcrop); the row is not corrected")


def warn_assembly(system, eps, jump: str) -> None:
    """The three assembly-time warnings, in the reference's order (dense.py:376-378)."""
    warn_half_jump_eps(system, eps, jump)
    warn_collocation_near_fault(system, eps)
    warn_fault_rows_near_boundary(system, eps)
