"""Sample a solved model on a 3-D grid (``src/mbem/volume.py``).

The representation formula evaluated at grid points in the interior: the
grid (half a cell inside the bounding box, so no plane of samples lies on a
face, volume.py:139-165), the region of every point (the Gauss closure sum,
``RegionModel.point_in_region``, then the points ON a patch given to the
first region that owns it, volume.py:199-252), the clearance arrays that say
how far each point sits from a boundary patch and from a fault
(volume.py:255-301), and the chunked readout (volume.py:370-444): the
displacement, the elastic stress, the strain from Hooke inverted, and the
eigenstress from the same pass, with the derived scalars a render is
coloured by.

Every per-point computation runs on the GPU: the solid-angle and distance
kernels of ``csrc/geometry.cu`` and the readout kernels behind
``evaluate_displacement`` / ``evaluate_stress``. The outputs are numpy
arrays (NaN outside every region), as the reference's. Continuous
near-field recovery (``near=``, ``recover.NearField``) and ``stand_off``,
which exists only for it, are not part of this path.
"""

from __future__ import annotations

import dataclasses
import time

import numpy as np
import torch

from . import defaults
from ._device import as_cuda
from .evaluate import evaluate_displacement, evaluate_stress
from .geometry import MeshGeometry
from .kernels import basis as kb
from .model.core import _ON_PATCH_TOL

# tensor components written out, in the order a viewer labels them
SYM6 = (("xx", 0, 0), ("yy", 1, 1), ("zz", 2, 2), ("xy", 0, 1), ("yz", 1, 2), ("xz", 0, 2))
PRIMARY = ("u", "sigma", "strain", "eigenstress")
SCALARS = ("u_mag", "von_mises", "mean_stress", "max_shear", "dilatation")


@dataclasses.dataclass(frozen=True)
class Grid:
    """A regular grid, x fastest (volume.py:105-119)."""
    origin: tuple
    spacing: tuple
    dims: tuple                      # (nx, ny, nz) point counts
    points: np.ndarray               # (N, 3), C order over (nz, ny, nx)

    @property
    def shape(self) -> tuple:
        nx, ny, nz = self.dims
        return (nz, ny, nx)

    def fold(self, a: np.ndarray) -> np.ndarray:
        """``(N, ...)`` -> ``(nz, ny, nx, ...)``."""
        return a.reshape(self.shape + a.shape[1:])


def model_bounds(model) -> tuple:
    """``(lo, hi)``: the bounding box of every boundary patch's vertices
    (volume.py:122-136)."""
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    for r in model.regions:
        for p in r.patches:
            v = np.asarray(p.mesh.vertices, float)
            lo = np.minimum(lo, v.min(axis=0))
            hi = np.maximum(hi, v.max(axis=0))
    return lo, hi


def _axis(lo: float, hi: float, spacing: float) -> np.ndarray:
    o = lo + 0.5 * spacing
    return o + spacing * np.arange(int(np.floor((hi - o) / spacing)) + 1)


def _grid(axes: list, spacing: float) -> Grid:
    Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return Grid(origin=tuple(float(a[0]) for a in axes), spacing=(spacing,) * 3,
                dims=tuple(len(a) for a in axes), points=np.column_stack([X.ravel(), Y.ravel(), Z.ravel()]))


def make_grid(model, spacing: float, pad: float = 0.0) -> Grid:
    """A grid over the model's box grown by ``pad``, offset half a cell from
    its low corner on every axis (volume.py:139-165): with a pad of whole
    cells and no offset a plane of samples would lie on each face, where the
    closure sum is 2 pi and the side is decided by rounding."""
    lo, hi = model_bounds(model)
    lo, hi = lo - pad, hi + pad
    return _grid([_axis(lo[d], hi[d], spacing) for d in range(3)], spacing)


def section_grid(model, axis: str, at: float, spacing: float) -> Grid:
    """One plane of points, ``axis`` held at ``at`` strictly inside the box,
    the other two laid out as ``make_grid`` does (volume.py:168-196)."""
    if axis not in ("x", "y", "z"):
        raise ValueError(f"a section is across x, y or z, not {axis!r}")
    k = "xyz".index(axis)
    lo, hi = model_bounds(model)
    if not lo[k] < at < hi[k]:
        raise ValueError(f"the section {axis} = {at} is outside the model, which spans {lo[k]:g} to {hi[k]:g} there")
    axes = [np.array([float(at)]) if d == k else _axis(lo[d], hi[d], spacing) for d in range(3)]
    return _grid(axes, spacing)


def _points(points) -> torch.Tensor:
    return as_cuda(points).reshape(-1, 3)


def on_patch(points, patch) -> np.ndarray:
    """``(N,) bool``: the points within _ON_PATCH_TOL of the nearest
    element's size of ``patch`` (volume.py:199-227), from the exact distance
    to the mesh."""
    pts = _points(points)
    d, idx = MeshGeometry(patch.mesh).distance(pts)
    tol = torch.from_numpy(_ON_PATCH_TOL * kb.element_sizes(patch.mesh)).to(pts.device)
    return (d < tol[idx]).cpu().numpy()


def classify(model, grid: Grid) -> np.ndarray:
    """``(N,) int8``: 0 outside every region, else the 1-based index of the
    region holding the point (volume.py:230-252). A point ON a patch goes to
    the first region that owns the patch."""
    pts = _points(grid.points)
    code = torch.zeros(pts.shape[0], dtype=torch.int8, device=pts.device)
    for i, r in enumerate(model.regions, start=1):
        hit = model.point_in_region(r, pts) & (code == 0)
        code[hit] = i
    settled = torch.zeros(pts.shape[0], dtype=torch.bool, device=pts.device)
    for i, r in enumerate(model.regions, start=1):
        for p in r.patches:
            d, idx = MeshGeometry(p.mesh).distance(pts)
            tol = torch.from_numpy(_ON_PATCH_TOL * kb.element_sizes(p.mesh)).to(pts.device)
            on = (d < tol[idx]) & ~settled
            code[on] = i
            settled |= on
    return code.cpu().numpy()


def clearance(model, grid: Grid, eps) -> tuple:
    """``(clearance_h, clearance_eps, fault_eps)``, each ``(N,)``
    (volume.py:255-301): over the boundary patches, the distance in units of
    the nearest element's size and of its eps; over the faults, the distance
    in units of the nearest fault element's eps."""
    pts = _points(grid.points)
    n = pts.shape[0]
    inf = torch.full((n,), float("inf"), dtype=torch.float64, device=pts.device)
    c_h, c_eps, c_fault = inf.clone(), inf.clone(), inf.clone()

    def eps_of(patch):
        e = np.broadcast_to(np.atleast_1d(kb.resolve_patch_eps(eps, patch)), (patch.mesh.n_triangles,))
        return torch.from_numpy(np.array(e, dtype=float)).to(pts.device)

    for r in model.regions:
        for p in r.patches:
            d, idx = MeshGeometry(p.mesh).distance(pts)
            h = torch.from_numpy(kb.element_sizes(p.mesh)).to(pts.device)
            c_h = torch.minimum(c_h, d / h[idx])
            c_eps = torch.minimum(c_eps, d / eps_of(p)[idx])
        for f in r.faults:
            d, idx = MeshGeometry(f.mesh).distance(pts)
            c_fault = torch.minimum(c_fault, d / eps_of(f)[idx])
    return c_h.cpu().numpy(), c_eps.cpu().numpy(), c_fault.cpu().numpy()


def _strain(sig: torch.Tensor, mu: float, lam: float) -> torch.Tensor:
    """Hooke inverted from (mu, lam): tr(sigma) = (2 mu + 3 lam) tr(e),
    e = (sigma - lam tr(e) I) / (2 mu) (volume.py:304-314)."""
    tr_e = sig.diagonal(dim1=-2, dim2=-1).sum(-1) / (2.0 * mu + 3.0 * lam)
    e = sig.clone()
    for k in range(3):
        e[:, k, k] -= lam * tr_e
    return e / (2.0 * mu)


def eigvalsh3(a: torch.Tensor, sweeps: int = 6) -> torch.Tensor:
    """Ascending eigenvalues of symmetric (N, 3, 3) matrices, elementwise on
    the device with no solver library: cyclic Jacobi rotations (Golub and
    Van Loan, Matrix Computations, sec. 8.5), each zeroing one off-diagonal
    entry with t = sign(theta) / (|theta| + hypot(theta, 1)),
    theta = (a_qq - a_pp) / (2 a_pq). Backward stable, so every eigenvalue
    is within a few eps of ||A|| of the exact one, near-equal pairs
    included; convergence is quadratic and six sweeps reach rounding."""
    m = 0.5 * (a + a.transpose(1, 2))
    d = [m[:, 0, 0].clone(), m[:, 1, 1].clone(), m[:, 2, 2].clone()]
    off = {(0, 1): m[:, 0, 1].clone(), (0, 2): m[:, 0, 2].clone(), (1, 2): m[:, 1, 2].clone()}

    def get(i, j):
        return off[(min(i, j), max(i, j))]

    for _ in range(sweeps):
        for p, q in ((0, 1), (0, 2), (1, 2)):
            r = 3 - p - q
            apq = off[(p, q)]
            nz = apq != 0
            safe = torch.where(nz, apq, torch.ones_like(apq))
            theta = (d[q] - d[p]) / (2.0 * safe)
            t = torch.sign(theta) / (theta.abs() + torch.hypot(theta, torch.ones_like(theta)))
            t = torch.where(nz, torch.where(theta == 0, torch.ones_like(t), t), torch.zeros_like(t))
            c = 1.0 / torch.sqrt(t * t + 1.0)
            s_ = t * c
            d[p] = d[p] - t * apq
            d[q] = d[q] + t * apq
            arp, arq = get(r, p), get(r, q)
            off[(min(r, p), max(r, p))] = c * arp - s_ * arq
            off[(min(r, q), max(r, q))] = s_ * arp + c * arq
            off[(p, q)] = torch.zeros_like(apq)
    return torch.sort(torch.stack(d, dim=1), dim=1).values


def _derived(u: torch.Tensor, sig: torch.Tensor, e: torch.Tensor) -> dict:
    """The scalars a volume render is coloured by (volume.py:317-328)."""
    tr = sig.diagonal(dim1=-2, dim2=-1).sum(-1)
    eye = torch.eye(3, dtype=sig.dtype, device=sig.device)
    dev = sig - (tr / 3.0)[:, None, None] * eye
    w = eigvalsh3(sig)                           # ascending
    return {
        "u_mag": torch.linalg.norm(u, dim=1),
        "von_mises": torch.sqrt(1.5 * (dev * dev).sum(dim=(1, 2))),
        "mean_stress": tr / 3.0,
        "max_shear": 0.5 * (w[:, 2] - w[:, 0]),
        "dilatation": e.diagonal(dim1=-2, dim2=-1).sum(-1),
    }


def _with_scalars(out: dict, inside: torch.Tensor) -> dict:
    n = inside.shape[0]
    dev = inside.device
    scalars = {k: torch.full((n,), float("nan"), dtype=torch.float64, device=dev) for k in SCALARS}
    sel = torch.nonzero(inside).flatten()
    if sel.numel():
        d = _derived(out["u"][sel], out["sigma"][sel], out["strain"][sel])
        for k, v in d.items():
            scalars[k][sel] = v
    out.update(scalars)
    return out


def sample(model, solution: dict, eps, grid: Grid, code: np.ndarray, chunk: int | None = None,
           eigenstress: bool = True, progress=None, near=None, precision: str = "fp64") -> dict:
    """Evaluate one solved state on ``grid`` (volume.py:370-444): ``u``,
    ``sigma`` (elastic), ``strain``, ``eigenstress`` (with ``eigenstress``)
    and the derived scalars, each ``(N, ...)``, NaN where ``code`` is 0.
    Each point is read with its own region's material and patch set.
    ``precision="mixed"`` takes the elastic stress and the P0 displacement
    from the FP32-far / FP64-near readouts."""
    if near is not None:
        raise NotImplementedError("near-field recovery (near=) is not on the GPU readout path")
    chunk = chunk or defaults.VOLUME_CHUNK_DEVICE
    pts_all = _points(grid.points)
    dev = pts_all.device
    n = pts_all.shape[0]
    code = np.asarray(code)
    if code.shape != (n,):
        raise ValueError(f"code must hold one region code a grid point ({n}), got shape {code.shape}")
    code_t = torch.as_tensor(code, device=dev)
    nan = float("nan")
    out = {"u": torch.full((n, 3), nan, dtype=torch.float64, device=dev),
           "sigma": torch.full((n, 3, 3), nan, dtype=torch.float64, device=dev),
           "strain": torch.full((n, 3, 3), nan, dtype=torch.float64, device=dev)}
    if eigenstress:
        out["eigenstress"] = torch.full((n, 3, 3), nan, dtype=torch.float64, device=dev)
    for i, r in enumerate(model.regions, start=1):
        where = torch.nonzero(code_t == i).flatten()
        if where.numel() == 0:
            continue
        mu, lam = r.material.mu, r.material.lam
        for s in range(0, where.numel(), chunk):
            sel = where[s:s + chunk]
            pts = pts_all[sel].contiguous()
            out["u"][sel] = evaluate_displacement(model, r, solution, pts, eps, warn_near=False,
                                                  precision=precision)
            got = evaluate_stress(model, r, solution, pts, eps, subtract_anelastic=True, warn_near=False,
                                  parts=eigenstress, precision=precision)
            sig = got[0] if eigenstress else got
            out["sigma"][sel] = sig
            out["strain"][sel] = _strain(sig, mu, lam)
            if eigenstress:
                out["eigenstress"][sel] = got[1]
            if progress is not None:
                progress(r.name, min(s + chunk, where.numel()), where.numel())
    _with_scalars(out, code_t > 0)
    return {k: v.cpu().numpy() for k, v in out.items()}


def difference(fa: dict, fb: dict, inside: np.ndarray) -> dict:
    """``fa - fb`` where both are defined, with the scalars recomputed from
    the differenced tensors (volume.py:447-471)."""
    ins = torch.from_numpy(np.asarray(inside, bool))
    out = {}
    for k in PRIMARY:
        if k in fa and k in fb:
            d = torch.from_numpy(np.asarray(fa[k], float) - np.asarray(fb[k], float))
            d[~ins] = float("nan")
            out[k] = d
    _with_scalars(out, ins)
    return {k: v.numpy() for k, v in out.items()}


def as_vti_arrays(grid: Grid, fields: dict, code: np.ndarray, c_h: np.ndarray, c_eps: np.ndarray,
                  c_fault: np.ndarray | None = None) -> dict:
    """name -> ``(nz, ny, nx, ...)``, tensors split into their six
    independent components (volume.py:474-497)."""
    arrays = {}
    for name, a in fields.items():
        if a.ndim == 3:
            for comp, i, j in SYM6:
                arrays[f"{name}_{comp}"] = grid.fold(a[:, i, j])
        else:
            arrays[name] = grid.fold(a)
    arrays["region"] = grid.fold(np.asarray(code).astype(float))
    arrays["clearance_h"] = grid.fold(c_h)
    arrays["clearance_eps"] = grid.fold(c_eps)
    if c_fault is not None:
        arrays["fault_eps"] = grid.fold(c_fault)
    return arrays


def timed(label: str, fn, log=None):
    """Run ``fn``; return ``(value, seconds)``, optionally logged."""
    t0 = time.perf_counter()
    v = fn()
    dt = time.perf_counter() - t0
    if log is not None:
        log(f"  {label:22s} {dt:8.2f} s")
    return v, dt
