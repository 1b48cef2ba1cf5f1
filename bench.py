"""Time-to-solve benchmark of the dense mollified-BEM hot path on one GB300.

One step = one complete solve of the workload: assemble the collocation
operator of the calibrated dense backend (CUDA pair kernels, straight into
HBM), the calibration row sums and free-term diagonal, the fault right-hand
side, then deflated FGMRES(50) on the device to a true relative residual of
1e-8. The headline (``--precision mixed``, default) is the mixed-precision
operator (FP32 quadrature far field, FP64 closed-form near field; its
residual evaluated in double-float), solved by flexible FGMRES whose
preconditioner is a GMRES solve on the far field rounded to BF16 (written by
the same assembly pass); the plain FP64 path on the same
workload is timed beside it (``fp64_path``) for the mixed/FP64 ratio the
metric names. ``value`` is seconds per solve with the mesh arrays already
resident in HBM; ``e2e`` is the same through the public API from host numpy
arrays (model -> assemble -> solve -> numpy solution), host<->device copies
inside.

Workloads (mesh: traction-free cube of side 4, n x n squares per face, two
triangles each; vertical fault 1 x 1 at the centre, uniform slip (1,0,0);
mu = 1, lam = 1; eps = half the cube grid spacing):
  cube48: n = 48, fault 32 x 32 -> 27,648 + 2,048 elements, 82,944 unknowns
          (A = 55 GB FP64, larger than L2: no flush needed)
  cube12: n = 12, fault 8 x 8 -> 5,184 unknowns (quick check)

``--impl reference`` times the CPU restatement of the reference's path
(oracle/: the C kernels with OpenMP on all host cores and the numpy FGMRES)
on the host: a complete solve of the cube-12 workload, then one window of
the workload's own operator assembled and applied per step (the step time
is that window's); the value is the time to solve the workload estimated
from them (PortBaseline).

Multi-GPU: the path does not shard across GPUs here (replicas only): under
torchrun every rank solves its own replica; value is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "cube48": dict(n_face=48, n_fault=32),
    "cube24": dict(n_face=24, n_fault=16),
    "cube12": dict(n_face=12, n_fault=8),
}
RTOL = 1e-8
RESTART = 50
METRIC = ("time-to-solve at 1e-8 rel. residual (true residual of the solved operator, evaluated in FP64; "
          "assembly included)")


def _dist():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1 and not torch.distributed.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        torch.distributed.init_process_group(backend)
    return rank, ws


def _barrier(ws):
    import torch
    if ws > 1:
        torch.distributed.barrier()


def _max_over_ranks(v, ws):
    import torch
    if ws == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def fp64_peak_tflops():
    """DFMA throughput of this GPU (own probe kernel, CUDA events)."""
    import torch
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    for _ in range(2):
        nat.call("mbem_fp64_fma_probe", ptr(out), iters, blocks, threads, stream_handle())
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    nat.call("mbem_fp64_fma_probe", ptr(out), iters, blocks, threads, stream_handle())
    e.record()
    e.synchronize()
    sec = s.elapsed_time(e) / 1e3
    return 16.0 * iters * blocks * threads / sec / 1e12


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def _timed_steps(step, steps, ws):
    """Runs ``steps`` steps between barriers + syncs; returns (device s per
    step as max over ranks, wall s per step, per-step results)."""
    import torch
    torch.cuda.synchronize()
    _barrier(ws)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    start.record()
    out = [step() for _ in range(steps)]
    end.record()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / steps
    dev = _max_over_ranks(start.elapsed_time(end) / 1e3 / steps, ws)
    return dev, wall, out


def run_ours(args, rank, ws):
    import torch
    from mbem_gb300 import _native as nat
    from mbem_gb300 import defaults
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cfg = WORKLOADS[args.workload]
    model, eps = cube_fault_model(cfg["n_face"], cfg["n_fault"])
    system = generate_system(model)
    n = system.layout.n_unknowns
    arrays = {}     # device-resident mesh arrays, filled by the first assembly

    def make_step(precision, timer=None, precond=None):
        backend = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART,
                               precision=precision, precond=precond or _precond_for(precision, args.precond))

        def step():
            asm = backend.assemble(system, eps, arrays=arrays, timer=timer)
            x = asm.solve_device(time_matvec=True)
            rep = asm.report
            nnz = sum(nl.nnz for nl in asm.op.near) if asm.op is not None else 0
            asm.A = None
            asm.op = None
            return rep, nnz, x
        return step

    # the tile shapes of the operator products, chosen by the autotuner on
    # this workload before the warm-up (a one-time setup, like a compile)
    tuned = None
    if args.precision == "mixed" and not args.skip_tune:
        from mbem_gb300 import autotune
        tb = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART, precision="mixed",
                          precond="bf16_inner")
        t0 = time.perf_counter()
        tasm = tb.assemble(system, eps, arrays=arrays)
        tuned = autotune.tune_mixed_operator(tasm, autotune.Autotuner(cache_path=""))
        del tasm
        tuned["s"] = time.perf_counter() - t0
        torch.cuda.empty_cache()

    # headline: the mixed-precision path
    timer = []
    step = make_step(args.precision, timer)
    for _ in range(args.warmup):
        step()
    timer.clear()
    from mbem_gb300.la.mixed import inner_stats
    inner_stats(timing=True)
    launches0 = nat.lib().mbem_launch_count()
    with ClockSampler(local) as clk:
        dev_s, wall, res = _timed_steps(step, args.steps, ws)
    launches = nat.lib().mbem_launch_count() - launches0
    inner_steps, inner_solves, inner_ms = inner_stats(timing=False)
    rep, nnz, x_last = res[-1]
    del res

    # the plain FP64 path on the same workload, for the ratio the metric names
    fp64 = None
    if args.precision != "fp64" and not args.skip_fp64:
        timer64 = []
        step64 = make_step("fp64", timer64)
        step64()
        timer64.clear()
        dev64, wall64, res64 = _timed_steps(step64, max(1, args.fp64_steps), ws)
        asm64 = [s.elapsed_time(e) for (k, nf, ns, s, e) in timer64 if k == "H"]
        fp64 = {"ms_per_step": dev64 * 1e3, "iterations": res64[-1][0].iterations,
                "true_relres": res64[-1][0].true_relres, "steps": max(1, args.fp64_steps),
                "assembly_ms_per_step": float(np.sum(asm64)) / max(1, args.fp64_steps),
                "speedup_mixed_vs_fp64": dev64 / dev_s}

    # the other mixed variant (with / without the learned two-level
    # preconditioner inside the BF16 inner solve), timed the same way
    other = None
    if args.precision == "mixed" and not args.skip_variant:
        alt = "bf16_inner" if args.precond == "bf16_learned" else "bf16_learned"
        stepv = make_step("mixed", precond=alt)
        stepv()
        inner_stats(timing=False)
        devv, wallv, resv = _timed_steps(stepv, max(1, args.fp64_steps), ws)
        sv, av, _ = inner_stats(timing=False)
        other = {"precond": alt, "what": ("the mixed solve with the learned two-level preconditioner (block-Jacobi "
                                          "+ learned coarse space, set up in every step) inside the BF16 inner "
                                          "solve" if alt == "bf16_learned" else "the mixed solve without it"),
                 "ms_per_step": devv * 1e3, "outer_iterations": resv[-1][0].iterations,
                 "inner_steps_per_step": sv / max(1, args.fp64_steps), "true_relres": resv[-1][0].true_relres,
                 "headline_speedup_over_it": devv / dev_s,
                 "max_rel_diff_vs_headline_solution": float((resv[-1][2] - x_last).norm() / x_last.norm())}
        del resv
    # the headline solution against the reference's FP64 system
    accuracy = None
    if args.precision == "mixed" and not args.skip_fp64:
        accuracy = headline_accuracy(model, system, eps, x_last, arrays)
    del x_last

    # end to end through the public API from host arrays
    e2e = None
    if not args.skip_e2e:
        from mbem_gb300 import mesh as M
        from mbem_gb300.model import BCType, Patch, Region, RegionModel
        host_cube = M.cube(cfg["n_face"])
        host_fault = M.centre_fault(cfg["n_fault"])
        backend = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART,
                               precision=args.precision, precond=_precond_for(args.precision, args.precond))

        def e2e_step():
            cube_p = Patch("cube", host_cube, BCType.FREE_TRACTION)
            fault_p = Patch("fault", host_fault, BCType.FAULT, value=np.array([1.0, 0.0, 0.0]))
            m = RegionModel([Region("body", M.ElasticMaterial(1.0, 1.0), [cube_p], np.zeros(3),
                                    faults=[fault_p])])
            asm = backend.assemble(generate_system(m), eps)
            sol = asm.solve()
            asm.A = None
            asm.op = None
            return sol

        e2e_step()
        torch.cuda.synchronize()
        _barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = _max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, ws)
        n_c, n_f = host_cube.n_triangles, host_fault.n_triangles
        h2d = 8 * (n_c * (9 + 3 + 1 + 3 + 3) + n_f * (9 + 3 + 1) + 3 * n_f + 9 * n_c)
        e2e = {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 8 * n}

    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    mv_ms = rep.matvec_ms / max(1, rep.matvecs)
    if args.precision == "mixed":
        # the mixed matvec: the FP32 far field once, the near blocks (72 B +
        # an 8 B index each), x read, y written
        mv_bytes = 4.0 * n * n + 80.0 * nnz + 16.0 * n
        kernel = "mixed matvec (split_vec + sgemv_df_tma_kernel + near_matvec_kernel)"
    else:
        mv_bytes = 8.0 * n * n + 16.0 * n
        kernel = "dgemv_vec_kernel"
    achieved = mv_bytes / (mv_ms / 1e3) / 1e9
    peak_source = ("MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks.get("hbm_gbs")
                   else "fallback 6.8 TB/s (of fallback)")
    roofline = {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak,
                "traffic": TRAFFIC_OVER_ALGORITHMIC * mv_bytes if args.precision == "mixed" else None,
                "bytes_per_launch": mv_bytes, "launch_ms": mv_ms, "launches_per_step": rep.matvecs,
                "peak_source": peak_source}
    roofline_outer = None
    if args.precision == "mixed" and inner_steps > 0:
        # the inner BF16 product dominates the solve: the BF16 far field once
        # (2 B an entry), the FP64 near blocks, x (FP32) read, y written
        b16 = 2.0 * n * n + 80.0 * nnz + 12.0 * n
        ms16 = inner_ms / inner_steps
        a16 = b16 / (ms16 / 1e3) / 1e9
        roofline_outer = roofline
        roofline = {"kernel": "BF16 inner matvec (d2f + sgemv_bf16_tma_kernel + near_matvec_kernel)",
                    "bound": "hbm", "achieved": a16, "peak": hbm_peak, "unit": "GB/s", "frac": a16 / hbm_peak,
                    "traffic": TRAFFIC_OVER_ALGORITHMIC * b16, "bytes_per_launch": b16, "launch_ms": ms16,
                    "launches_per_step": inner_steps / args.steps, "peak_source": peak_source}
    asm_ms = [s.elapsed_time(e) for (k, nf, ns, s, e) in timer]
    line = {
        "metric": METRIC,
        "value": dev_s,
        "unit": "s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("mixed: fp32 far field / bf16 inner solve / fp64 near field, residual and refinement"
                  if args.precision == "mixed" else "f64"),
        "data": "synthetic (seeded mesh generators; no dataset)",
        "config": {"workload": args.workload, "n_face": cfg["n_face"], "n_fault": cfg["n_fault"],
                   "unknowns": n, "precision": args.precision,
                   "solver": f"deflated FGMRES({RESTART})" + (
                       f", BF16 inner GMRES (<= {defaults.MIXED_INNER_ITERATIONS} steps to "
                       f"{defaults.MIXED_INNER_RTOL:g}) as flexible preconditioner" + (
                           ", right-preconditioned by the learned two-level preconditioner (block-Jacobi + "
                           "learned coarse space, set up in the step)" if args.precond == "bf16_learned" else "")
                       if args.precision == "mixed" else ""),
                   "rtol": RTOL, "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "inputs larger than L2 (A = %.1f GB FP32 far field)" % (4.0 * n * n / 1e9)
                   if args.precision == "mixed" else
                   "inputs larger than L2 (A = %.1f GB FP64)" % (8.0 * n * n / 1e9)},
        "iterations": rep.iterations,
        "inner_steps_per_step": inner_steps / args.steps,
        "true_relres": rep.true_relres,
        "wall_s_per_step": wall,
        "matvec_ms_per_step": rep.matvec_ms,
        "assembly_kernels_ms_per_step": float(np.sum(asm_ms)) / args.steps,
        "fp64_path": fp64,
        "accuracy_vs_fp64_system": accuracy,
        "mixed_variant": other,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": roofline,
        "roofline_outer_matvec": roofline_outer,
        "autotune": tuned,
        "fp64_peak_tflops": fp64_peak_tflops(),
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if not args.skip_extra:
        line["workloads"] = extra_workloads(args, peaks)
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    return line


def _deflated_relres(b, Ax, u_ranges):
    """|P (b - A x)| / |P b| with P the translation deflation over the
    u-slots (the residual FGMRES reports)."""
    r = b - Ax
    pb = b.clone()
    for off, size in u_ranges:
        for v in (r, pb):
            seg = v[off:off + size].view(-1, 3)
            seg.sub_(seg.mean(dim=0))
    return float(r.norm() / pb.norm())


def headline_accuracy(model, system, eps, x_mixed, arrays, n_readout=32):
    """What the mixed headline's solution is worth against the reference's
    own FP64 system on the same workload: the FP64 closed-form operator (the
    reference's dense backend, every entry by the closed form) is assembled
    and solved by plain FGMRES to the same 1e-8; then
      - the FP64 operator's deflated relative residual at the mixed solution;
      - the relative difference of the two solutions (both the zero-mean
        translation representative);
      - the readout at an n_readout x n_readout grid on y = 0.1 (the cube-12
        workload's plane): displacement, eigenstress-subtracted stress and the
        traction on the plane (sigma . e_y) from the mixed solution through the
        mixed readout, against the FP64 solution through the FP64 readout;
        each as max |difference| / max |FP64 value|."""
    import torch
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import readout_grid
    from mbem_gb300.evaluate import evaluate_displacement, evaluate_stress
    be = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART)
    asm = be.assemble(system, eps, arrays=arrays)
    x64 = asm.solve_device()
    rep64 = asm.report
    A = asm.A
    n = A.shape[0]
    Ax = torch.empty(n, dtype=torch.float64, device=A.device)
    nat.call("mbem_dgemv", ptr(A), A.stride(0), n, n, ptr(x_mixed), 1.0, 0.0, ptr(Ax), stream_handle())
    relres = _deflated_relres(asm.b, Ax, asm.u_ranges())
    diff = float((x_mixed - x64).norm() / x64.norm())
    lay = asm.layout
    sol64 = {s.name: x64[s.offset:s.stop].reshape(-1, 3).cpu().numpy() for s in lay.slots}
    solm = {s.name: x_mixed[s.offset:s.stop].reshape(-1, 3).cpu().numpy() for s in lay.slots}
    asm.A = None
    del asm, A
    torch.cuda.empty_cache()
    pts = readout_grid(n_readout)
    reg = model.regions[0]
    u64 = evaluate_displacement(model, reg, sol64, pts, eps)
    um = evaluate_displacement(model, reg, solm, pts, eps, precision="mixed")
    s64 = evaluate_stress(model, reg, sol64, pts, eps, subtract_anelastic=True)
    sm = evaluate_stress(model, reg, solm, pts, eps, subtract_anelastic=True, precision="mixed")

    def rel(a, b):
        return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())
    return {"fp64_operator_relres_at_mixed_solution": relres,
            "max_rel_diff_mixed_vs_fp64_solution": diff,
            "fp64_solution": {"iterations": rep64.iterations, "true_relres": rep64.true_relres},
            "readout_points": int(pts.shape[0]),
            "readout_rel_err": {"displacement": rel(um, u64), "stress_minus_eigenstress": rel(sm, s64),
                                "traction_on_plane": rel(np.asarray(sm)[:, :, 1], np.asarray(s64)[:, :, 1])},
            "what": "mixed solution (mixed operator, mixed readout) against the FP64 closed-form system "
                    "solved to the same tolerance (FP64 readout)"}


def _precond_for(precision, choice="bf16_learned"):
    """The headline solve's preconditioner: for the mixed operator the BF16
    inner solve, with (``bf16_learned``) or without (``bf16_inner``) the
    learned two-level preconditioner inside it; none for FP64 (the
    reference's plain FGMRES)."""
    return choice if precision == "mixed" else None


def _sync_time(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def multi_rhs_workload(peaks, n_face=24, n_fault=16, n_rhs=256):
    """Many right-hand sides (cube 24 x 24 per face, fault 16 x 16, 256 slip
    patterns from a Gaussian random field): the mixed operator, its
    three-term BF16 copy and the block solver (batched GMRES on the tcgen05
    GEMM inside FP64-accurate refinement), against the plain FP64 path
    solving the 256 systems one by one (FGMRES on the FP64 matrix)."""
    import torch
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model, gaussian_slips
    from mbem_gb300.la.multirhs import BlockSolver, gemm_bf16_t, slip_rhs
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, n_fault)
    system = generate_system(model)
    fault = model.regions[0].faults[0]
    slips = gaussian_slips(fault, n_rhs)
    out = {"config": {"n_face": n_face, "n_fault": n_fault, "unknowns": system.layout.n_unknowns, "n_rhs": n_rhs,
                      "slips": "Gaussian random field, length 0.3, unit variance, seeds 0..%d" % (n_rhs - 1)}}
    mixed = DenseBackend(jump="calibrated", deflate=True, precision="mixed")
    # warm-up pass, then the timed one
    for timed in (False, True):
        asm, t_asm = _sync_time(lambda: mixed.assemble(system, eps))
        B, t_rhs = _sync_time(lambda: slip_rhs(asm, fault, slips))
        bs, t_bf = _sync_time(lambda: BlockSolver(asm))
        (X, rep), t_solve = _sync_time(lambda: bs.solve(B, rtol=RTOL))
        if timed:
            break
        # after the warm-up pass: the GEMM's K split, tuned on the solver's own operator
        from mbem_gb300 import autotune
        Vt = torch.randn((n_rhs, bs.A16.shape[1]), device="cuda").to(torch.bfloat16)
        Wt = torch.empty((n_rhs, bs.n), device="cuda")
        out["autotune"] = autotune.Autotuner(cache_path="").tune(
            "gemm_split", f"M={bs.n},K={bs.A16.shape[1]},k={n_rhs}",
            lambda: gemm_bf16_t(bs.A16, Vt, bs.A16.shape[1], Wt)).summary()
        del Vt, Wt, bs, asm
        torch.cuda.empty_cache()
    total = t_asm + t_rhs + t_bf + t_solve
    n = bs.n
    Vbf = torch.randn((n_rhs, bs.A16.shape[1]), device="cuda").to(torch.bfloat16)
    W = torch.empty((n_rhs, n), device="cuda")
    K = bs.A16.shape[1]
    for _ in range(3):
        gemm_bf16_t(bs.A16, Vbf, K, W)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        gemm_bf16_t(bs.A16, Vbf, K, W)
    e1.record()
    torch.cuda.synchronize()
    gemm_ms = e0.elapsed_time(e1) / 10
    flops = 2.0 * n * K * n_rhs
    bf16_peak = peaks.get("bf16_tflops") or 1900.0
    out["mixed_block"] = {"s": total, "assembly_s": t_asm, "rhs_s": t_rhs, "bf16_copy_s": t_bf, "solve_s": t_solve,
                          "refinement_steps": rep.outer, "inner_iterations": rep.inner_iterations,
                          "worst_true_relres": float(np.max(rep.true_relres)), "gemm_ms_in_solve": rep.gemm_ms,
                          "residual_ms_in_solve": rep.residual_ms}
    out["roofline_gemm"] = {"kernel": "tc_gemm_kernel (tcgen05.mma kind::f16, TMA, TMEM)", "bound": "tensor",
                            "achieved": flops / (gemm_ms / 1e3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                            "frac": flops / (gemm_ms / 1e3) / 1e12 / bf16_peak, "launch_ms": gemm_ms,
                            "flops_per_launch": flops, "hbm_gbs_of_A": 2.0 * n * K / (gemm_ms / 1e3) / 1e9,
                            "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if peaks.get("bf16_tflops")
                            else "fallback 1.9 PFLOP/s (of fallback)"}
    del bs, asm
    torch.cuda.empty_cache()
    # plain FP64: one FGMRES per right-hand side
    fp64 = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART)
    asm, t_asm = _sync_time(lambda: fp64.assemble(system, eps))
    B, t_rhs = _sync_time(lambda: slip_rhs(asm, fault, slips))
    its = []
    diff = 0.0

    def solve_all():
        nonlocal diff
        for r in range(n_rhs):
            asm.b = B[r].clone()
            x = asm.solve_device()
            its.append(asm.report.iterations)
            diff = max(diff, float(torch.linalg.vector_norm(x - X[r]) / torch.linalg.vector_norm(x)))
    _, t_solve = _sync_time(solve_all)
    t64 = t_asm + t_rhs + t_solve
    out["fp64_one_by_one"] = {"s": t64, "assembly_s": t_asm, "rhs_s": t_rhs, "solve_s": t_solve,
                              "mean_iterations": float(np.mean(its))}
    out["speedup_vs_fp64"] = t64 / total
    out["max_rel_diff_mixed_vs_fp64_solution"] = diff
    del asm
    torch.cuda.empty_cache()
    return out


def fault_traction_workload(n_face=32, n_fault=24, dip=90.0):
    """The FAULT_TRACTION cube (32 x 32 per face, fault 24 x 24, uniform
    shear drop 1e-3 mu): FGMRES with block-Jacobi, with the learned coarse
    space (shipped parameters, trained on 12- and 16-per-face meshes), and
    without a preconditioner, on the FP64 operator; then on the mixed
    operator, the BF16 inner solve with the learned preconditioner or
    block-Jacobi inside it."""
    import ctypes

    import torch
    from mbem_gb300 import _native as nat
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import fault_traction_model
    from mbem_gb300.la.learned import LearnedPreconditioner
    from mbem_gb300.la.train_learned import load_default
    from mbem_gb300.model import generate_system
    model, eps = fault_traction_model(n_face, n_fault, dip)
    system = generate_system(model)
    params = load_default()
    out = {"config": {"n_face": n_face, "n_fault": n_fault, "dip_deg": dip, "unknowns": system.layout.n_unknowns,
                      "rtol": RTOL}}
    backend = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART, maxiter=1000)
    backend.assemble(system, eps).release()       # warm-up: first-use costs of the kernels are not timed
    torch.cuda.empty_cache()
    asm, t_asm = _sync_time(lambda: backend.assemble(system, eps))
    out["assembly_s"] = t_asm
    for name in ("block_jacobi", "learned", "block_jacobi", "learned"):     # second pass timed
        asm._bj = None

        def setup():
            return "block_jacobi" if name == "block_jacobi" else LearnedPreconditioner(asm, params)

        def bj_build():
            asm.block_jacobi()
        _, t_bj = _sync_time(bj_build)
        pc, t_setup = _sync_time(setup)
        _, t_solve = _sync_time(lambda: asm.solve_device(precond=pc))
        if name == "learned":
            out["learned_setup_parts_s"] = pc.setup_s
        out[name] = {"setup_s": t_bj + t_setup, "solve_s": t_solve, "iterations": asm.report.iterations,
                     "true_relres": asm.report.true_relres, "converged": asm.report.converged,
                     "time_to_solve_s": t_asm + t_bj + t_setup + t_solve}
    _, t_plain = _sync_time(lambda: asm.solve_device(precond="none", maxiter=300))
    out["none"] = {"solve_s": t_plain, "iterations": asm.report.iterations, "true_relres": asm.report.true_relres,
                   "converged": asm.report.converged}
    out["learned_vs_block_jacobi_time"] = out["block_jacobi"]["time_to_solve_s"] / out["learned"]["time_to_solve_s"]
    x64 = asm.solve_device(precond=LearnedPreconditioner(asm, params))
    del asm
    torch.cuda.empty_cache()
    # the same system on the mixed operator (FP32 far field + BF16 copy, FP64
    # near blocks; the fault's traction rows assembled in FP64 and split):
    # the BF16 inner solve with the learned two-level preconditioner or with
    # block-Jacobi inside it, and block-Jacobi on the outer solve
    mixed = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART, maxiter=1000,
                         precision="mixed", precond="bf16_inner")
    for timed in (False, True):
        amx, t_asm = _sync_time(lambda: mixed.assemble(system, eps))
        res = {}
        for name in ("bf16_learned", "bf16_block_jacobi", "learned", "block_jacobi"):
            amx._bj = None
            amx._learned = None

            def setup():
                if name == "bf16_learned":
                    return amx.bf16_learned(params)
                if name == "bf16_block_jacobi":
                    inner = amx.bf16_inner()
                    inner.set_preconditioner(amx.block_jacobi())
                    return inner
                if name == "learned":
                    return LearnedPreconditioner(amx, params)
                return amx.block_jacobi()
            pc, t_setup = _sync_time(setup)
            steps, applies = ctypes.c_int64(0), ctypes.c_int64(0)
            nat.lib().mbem_inner_bf16_stats(0, ctypes.byref(steps), ctypes.byref(applies), None)
            x, t_solve = _sync_time(lambda: amx.solve_device(precond=pc))
            nat.lib().mbem_inner_bf16_stats(0, ctypes.byref(steps), ctypes.byref(applies), None)
            rep = amx.report
            res[name] = {"setup_s": t_setup, "solve_s": t_solve, "outer_iterations": rep.iterations,
                         "inner_steps": int(steps.value),
                         "true_relres": rep.true_relres, "converged": rep.converged,
                         "time_to_solve_s": t_asm + t_setup + t_solve,
                         "max_rel_diff_vs_fp64_solution": float((x - x64).norm() / x64.norm())}
        if timed:
            best = min(res, key=lambda k: res[k]["time_to_solve_s"])
            out["mixed"] = {"assembly_s": t_asm, **res,
                            "learned_vs_block_jacobi_time": min(res["bf16_block_jacobi"]["time_to_solve_s"],
                                                                res["block_jacobi"]["time_to_solve_s"])
                            / min(res["bf16_learned"]["time_to_solve_s"], res["learned"]["time_to_solve_s"]),
                            "fastest": best,
                            "speedup_vs_fp64_learned": out["learned"]["time_to_solve_s"]
                            / res[best]["time_to_solve_s"]}
        del amx
        torch.cuda.empty_cache()
    return out


def p2_readout_workload(n_fault=64, n_obs=1_000_000, n_check=2000):
    """Stress readout of a P2 fault (64 x 64, 8,192 triangles, 49,152 nodal
    slips from default_rng(5)) at 1 M points uniform in [-1, 1]^3, 10 % of
    them redrawn within 2 eps of the fault plane; eps = 0.07 x the smallest
    mean edge. Mixed precision (FP32 quadrature far pairs, FP64 near pairs)
    for all points; the FP64 nodal readout on n_check of them gives the error
    and, scaled by the point count, the FP64 time."""
    import torch
    from mbem_gb300 import mesh as M
    from mbem_gb300.kernels import tri_nodal as tn
    fault = M.centre_fault(n_fault)
    tv = fault.tri_verts()
    nrm, _ = fault.normals_and_areas()
    edge = np.linalg.norm(tv[:, [1, 2, 0]] - tv, axis=2).mean(axis=1)
    eps_val = 0.07 * float(edge.min())
    eps = np.full(tv.shape[0], eps_val)
    slip = np.random.default_rng(5).normal(size=(6 * tv.shape[0], 3))
    rng = np.random.default_rng(11)
    x = rng.uniform(-1.0, 1.0, size=(n_obs, 3))
    k = n_obs // 10
    x[:k, 1] = rng.uniform(-2 * eps_val, 2 * eps_val, size=k)
    dev = "cuda"
    xt, tvt, nt, et, st_ = (torch.from_numpy(a).to(dev) for a in (x, tv, nrm, eps, slip))
    for _ in range(2):      # warm-up, then timed
        res, t_mixed = _sync_time(lambda: tn.elastic_stress_readout(xt, tvt, nt, et, st_, 1.0, 1.0, order=2))
    idx = np.concatenate([np.arange(0, k, k // (n_check // 2)), np.arange(k, n_obs, (n_obs - k) // (n_check // 2))])
    ref, t64 = _sync_time(lambda: tn.elastic_stress_contract(xt[idx], tvt, nt, et, st_, 1.0, 1.0, order=2))
    got = res[idx]
    scale = float(ref.abs().max())
    dev_abs = (got - ref).abs().reshape(len(idx), -1).max(dim=1).values
    err = dev_abs / scale
    own = dev_abs / torch.clamp(ref.abs().reshape(len(idx), -1).max(dim=1).values, min=1e-12 * scale)
    return {"config": {"n_fault": n_fault, "triangles": int(tv.shape[0]), "nodal_slips": int(6 * tv.shape[0]),
                       "observers": n_obs, "eps": eps_val, "near_plane_fraction": 0.1},
            "mixed_s": t_mixed, "pairs_per_s": n_obs * tv.shape[0] / t_mixed,
            "fp64_s_for_check_points": t64, "fp64_s_extrapolated": t64 * n_obs / len(idx),
            "speedup_vs_fp64": t64 * n_obs / len(idx) / t_mixed,
            "check_points": int(len(idx)), "max_err_rel_to_max_stress": float(err.max()),
            "median_err_rel_to_max_stress": float(err.median()),
            "max_err_rel_to_own_stress": float(own.max()), "median_err_rel_to_own_stress": float(own.median())}


def multi_mesh_workload(peaks, n_mesh=64, lo=8, hi=32, seed=7):
    """64 cubes whose per-face grids are drawn uniformly in [8, 32] (fault
    grid two thirds of the face grid, uniform slip), each assembled as its
    own mixed-precision operator, solved together by one lockstep GMRES(50)
    whose every operator application is one persistent launch and whose
    every restart cycle is one CUDA graph; against the same operators solved
    one after another by the single-system FGMRES."""
    import torch
    from mbem_gb300 import _native as nat
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.la.multimesh import MeshBatch, random_cube_batch
    from mbem_gb300.model import generate_system

    shapes = random_cube_batch(n_mesh, lo, hi, seed)
    # every operator with its BF16 copy (the mixed batch solve's inner operator)
    be = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART, precision="mixed",
                      precond="bf16_inner")
    systems = []

    def assemble_all():
        systems.clear()
        for nf, nq in shapes:
            model, eps = cube_fault_model(nf, nq)
            systems.append(be.assemble(generate_system(model), eps))
    _, t_asm = _sync_time(assemble_all)
    n_total = sum(a.op.n for a in systems)
    mb = MeshBatch(systems, restart=RESTART)
    B = mb.gather([a.b for a in systems])
    from mbem_gb300 import autotune
    t0 = time.perf_counter()
    tuned = autotune.tune_mesh_batch(mb, autotune.Autotuner(cache_path=""))
    tuned["s"] = time.perf_counter() - t0
    mb.solve(B, rtol=RTOL)                      # warm-up: captures the cycle graph
    launches0 = nat.lib().mbem_launch_count()
    (X, rep), t_batch = _sync_time(lambda: mb.solve(B, rtol=RTOL))
    launches = nat.lib().mbem_launch_count() - launches0
    (Xn, repn), t_nograph = _sync_time(lambda: mb.solve(B, rtol=RTOL, graph=False))
    # the mixed batch solve: lockstep BF16 inner solves inside refinement
    mb.solve_mixed(B, rtol=RTOL)
    (Xm, repm), t_mixed = _sync_time(lambda: mb.solve_mixed(B, rtol=RTOL))
    # the batched operator alone: one persistent launch over every mesh
    Xr = torch.randn(mb.n_total, dtype=torch.float64, device="cuda")
    mb.matvec(Xr)
    reps = 5
    _, t_mv = _sync_time(lambda: [mb.matvec(Xr) for _ in range(reps)])
    mv_s = t_mv / reps
    mv_bytes = sum(4.0 * a.op.n * a.op.n for a in systems)
    # one system after another, same operators: the single-system FGMRES
    # (plain, the batched GMRES's algorithm) and the single-system mixed
    # solve (BF16 inner, the mixed batch solve's algorithm)
    single_its = []

    def one_by_one(precond):
        single_its.clear()
        out = []
        for a in systems:
            out.append(a.solve_device(rtol=RTOL, precond=precond))
            single_its.append(a.report.iterations)
        return out
    one_by_one("none")
    xs, t_single = _sync_time(lambda: one_by_one("none"))
    plain_its = list(single_its)
    diff = max(float((x - y).norm() / y.norm()) for x, y in zip(mb.scatter(X), xs))
    one_by_one("bf16_inner")
    xsm, t_single_mixed = _sync_time(lambda: one_by_one("bf16_inner"))
    diff_mixed = max(float((x - y).norm() / y.norm()) for x, y in zip(mb.scatter(Xm), xs))
    hbm = peaks.get("hbm_gbs") or 6800.0
    out = {"config": {"meshes": n_mesh, "per_face_grids": [s[0] for s in shapes], "unknowns_total": n_total,
                      "largest": max(a.op.n for a in systems), "smallest": min(a.op.n for a in systems),
                      "far_field_gb": mv_bytes / 1e9, "rtol": RTOL, "restart": RESTART},
           "assembly_s": t_asm,
           "autotune": tuned,
           "batched": {"s": t_batch, "cycles": rep.cycles, "converged": rep.all_converged,
                       "iterations_max": max(rep.iterations), "iterations_mean": float(np.mean(rep.iterations)),
                       "worst_relres": max(rep.relres), "gpu_launches": int(launches)},
           "batched_without_graph_s": t_nograph,
           "batched_mixed": {"s": t_mixed, "refinement_steps": repm.cycles, "converged": repm.all_converged,
                             "inner_steps_max": max(repm.iterations),
                             "inner_steps_mean": float(np.mean(repm.iterations)),
                             "worst_relres": max(repm.relres),
                             "max_rel_diff_vs_plain_single_solves": diff_mixed},
           "one_by_one_mixed": {"s": t_single_mixed},
           "speedup_batched_mixed_vs_one_by_one_mixed": t_single_mixed / t_mixed,
           "speedup_batched_mixed_vs_one_by_one_plain": t_single / t_mixed,
           "one_by_one_fgmres": {"s": t_single, "iterations_max": max(plain_its),
                                 "iterations_mean": float(np.mean(plain_its))},
           "speedup_batched_vs_one_by_one": t_single / t_batch,
           "max_rel_diff_batched_vs_single": diff,
           "roofline_batched_matvec": {"kernel": "mm_matvec_kernel (persistent, all meshes)", "bound": "hbm",
                                       "achieved": mv_bytes / mv_s / 1e9, "peak": hbm, "unit": "GB/s",
                                       "frac": mv_bytes / mv_s / 1e9 / hbm, "launch_ms": mv_s * 1e3,
                                       "bytes_per_launch": mv_bytes}}
    del mb, systems[:], X, Xn, Xm, xs, xsm
    torch.cuda.empty_cache()
    return out


def p1_variant_workload(n_face=24, n_fault=16):
    """The P1 variant of the 83k-unknown box: cube 24 x 24 per face at order 1
    (three nodes per triangle, 62,208 unknowns), fault 16 x 16 at P0; the
    mixed operator (nodal FP32 far quadrature, FP64 nodal near blocks) with
    the BF16 inner solve against the plain FP64 nodal path, both from mesh
    arrays to a 1e-8 true residual."""
    import torch
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, n_fault, cube_order=1)
    system = generate_system(model)
    out = {"config": {"n_face": n_face, "n_fault": n_fault, "cube_order": 1, "fault_order": 0,
                      "unknowns": system.layout.n_unknowns, "rtol": RTOL}}
    res = {}
    for name, kw in (("mixed", dict(precision="mixed", precond="bf16_inner")), ("fp64", dict())):
        be = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, restart=RESTART, **kw)
        arrays = {}
        for timed in (False, True):
            asm, t_asm = _sync_time(lambda: be.assemble(system, eps, arrays=arrays))
            x, t_solve = _sync_time(lambda: asm.solve_device())
            if not timed:
                del asm, x
                torch.cuda.empty_cache()
        rep = asm.report
        res[name] = x.clone()
        out[name] = {"s": t_asm + t_solve, "assembly_s": t_asm, "solve_s": t_solve, "iterations": rep.iterations,
                     "true_relres": rep.true_relres, "converged": rep.converged}
        del asm, x
        torch.cuda.empty_cache()
    out["speedup_mixed_vs_fp64"] = out["fp64"]["s"] / out["mixed"]["s"]
    out["max_rel_diff_mixed_vs_fp64_solution"] = float((res["mixed"] - res["fp64"]).norm() / res["fp64"].norm())
    return out


def dense_lu_workload(n_face=35):
    """The reference's dense-LU route (la/lu.py Factor, how="gpu": FP32 factors,
    FP64 refinement) at the size its published card number is quoted on:
    cube 35 x 35 per face, 44,100 unknowns (the reference: 44,085), the
    bordered deflated system factored on the GPU and solved to its
    refinement tolerance; FGMRES on the same FP64 operator beside it."""
    import torch
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.la.lu import phase_stats
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, max(2, round(2 * n_face / 3)))
    system = generate_system(model)
    be = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, lu="gpu")
    out = {}
    for timed in (False, True):
        asm, t_asm = _sync_time(lambda: be.assemble(system, eps))
        phase_stats(timing=timed)
        f, t_fac = _sync_time(lambda: asm.factor())
        phases = phase_stats(timing=False)
        x, t_sol = _sync_time(lambda: asm.solve_device())
        if not timed:
            del asm, f, x
            torch.cuda.empty_cache()
    n = int(asm.A.shape[0])
    rep = asm.report
    x_lu = x.clone()
    asm.lu = None
    xg, t_g = _sync_time(lambda: asm.solve_device(rtol=1e-10))
    out = {"config": {"n_face": n_face, "unknowns": n, "bordered": n + 3, "factors": "FP32 (panel FP32, trailing "
                      "update on the tensor cores as six BF16 piece products)", "refinement": "FP64"},
           "assembly_s": t_asm, "factor_s": t_fac, "factor_phases_ms": phases, "refined_solve_s": t_sol,
           "refinement_passes": int(f.report["passes"]), "left_after_refinement": float(f.report["left"]),
           "true_relres": rep.true_relres,
           "factor_tflops_equivalent": (2.0 / 3.0) * (n + 3) ** 3 / t_fac / 1e12,
           "published_card_reference_s": {"value": 2.0, "unknowns": 44085,
                                          "hardware": "RTX PRO 5000 48 GB, cupy FP32 factors + FP64 refinement"},
           "fgmres_same_operator": {"s": t_g, "iterations": asm.report.iterations},
           "max_rel_diff_lu_vs_fgmres": float((x_lu - xg).norm() / xg.norm())}
    del asm, f, x, xg
    torch.cuda.empty_cache()
    return out


def volume_workload(n_face=24, n_fault=16, n_grid=62, pad_cells=2, n_cpu=1024, cpu=True):
    """The volume sampler on the cube 24 x 24 per face with the 16 x 16
    fault, solved (mixed, 1e-8): a grid of (n_grid + 2 pad_cells)^3 points
    half a cell off every face (some outside the body); region codes
    (solid-angle closure over the 6,912 cube triangles plus the on-patch
    distance test), the clearances (distances to the cube and the fault),
    and the sampled displacement, elastic stress, strain, eigenstress and
    scalars, with the stress and displacement from the mixed and from the
    FP64 readouts. With ``cpu``, the CPU baseline of the classification
    (volume_cpu_baseline) beside it."""
    import torch
    from mbem_gb300 import volume as V
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.geometry import MeshGeometry
    from mbem_gb300.model import generate_system
    model, eps = cube_fault_model(n_face, n_fault)
    asm = DenseBackend(jump="calibrated", deflate=True, rtol=RTOL, precision="mixed",
                       precond="bf16_inner").assemble(generate_system(model), eps)
    sol = asm.solve()
    del asm
    torch.cuda.empty_cache()
    h = 4.0 / n_grid
    grid = V.make_grid(model, h, pad=pad_cells * h)
    n = grid.points.shape[0]
    cube = model.regions[0].patches[0]
    # warm-up on a small grid
    small = V.make_grid(model, 0.5)
    V.sample(model, sol, eps, small, V.classify(model, small), precision="mixed")
    code, t_cls = _sync_time(lambda: V.classify(model, grid))
    (c_h, c_eps, c_f), t_clr = _sync_time(lambda: V.clearance(model, grid, eps))
    f_mixed, t_mixed = _sync_time(lambda: V.sample(model, sol, eps, grid, code, precision="mixed"))
    f_fp64, t_fp64 = _sync_time(lambda: V.sample(model, sol, eps, grid, code))
    inside = code > 0
    diff = float(np.abs(f_mixed["sigma"][inside] - f_fp64["sigma"][inside]).max()
                 / np.abs(f_fp64["sigma"][inside]).max())
    diff_u = float(np.abs(f_mixed["u"][inside] - f_fp64["u"][inside]).max() / np.abs(f_fp64["u"][inside]).max())
    diff_e = float(np.abs(f_mixed["eigenstress"][inside] - f_fp64["eigenstress"][inside]).max()
                   / np.abs(f_fp64["eigenstress"][inside]).max())
    # the two geometry kernels alone (CUDA events on the launching stream)
    pts = torch.from_numpy(grid.points).cuda()
    geo = MeshGeometry(cube.mesh)
    pairs = n * geo.n_tri
    kt = {}
    for name, fn in (("solid_angle_kernel", lambda: geo.solid_angle(pts)),
                     ("mesh_distance_kernel", lambda: geo.distance(pts))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        kt[name] = {"ms": ms, "point_triangle_pairs_per_s": pairs / (ms * 1e-3)}
    out = {"config": {"n_face": n_face, "n_fault": n_fault, "grid": list(grid.dims), "points": n,
                       "points_inside": int(inside.sum()), "cube_triangles": geo.n_tri,
                       "fault_triangles": model.regions[0].faults[0].mesh.n_triangles},
            "classify_s": t_cls, "clearance_s": t_clr, "sample_mixed_s": t_mixed, "sample_fp64_s": t_fp64,
            "points_per_s_mixed": n / (t_cls + t_clr + t_mixed),
            "max_rel_diff_stress_mixed_vs_fp64": diff, "max_rel_diff_u_mixed_vs_fp64": diff_u,
            "max_rel_diff_eigenstress_mixed_vs_fp64": diff_e,
            "geometry_kernels": kt}
    if cpu:
        out["cpu_baseline"] = volume_cpu_baseline(grid.points, code, cube.tri_verts(), n_cpu)
    return out


def compressed_workload(peaks, n_face=128, reps=20, cpu=True, recompressed=True):
    """The compressed pair operator (la/hop.py PairCompressed) on the cube's
    self pair, T kernel, mu = lam = 1, eps = h/2: 128 x 128 per face is
    196,608 elements, 589,824 unknowns, whose dense FP64 matrix (2.8 TB) is
    ten times this GPU's HBM and whose mixed operator (FP32 far field + BF16
    copy, 2.1 TB) would not fit either. Times the partition (host), the
    material view's build (cross approximation of every admissible block,
    dense blocks), and the product: device time with CUDA events over
    back-to-back products (the working set, ~50 GB, is far above L2), and
    end to end from a pinned host vector to a host result. The CPU baseline
    is the C port of the reference's flat product (oracle/p0_oracle.c
    oracle_flat_matvec, OpenMP on every host core) on the same factors."""
    import torch
    from mbem_gb300 import mesh
    from mbem_gb300.kernels import basis as kb
    from mbem_gb300.la.compressed import PairCompressed
    cube = mesh.cube(n_face)
    n = cube.n_triangles
    eps = (4.0 / n_face) / 2
    c = kb.t_coeffs(1.0, 1.0)
    t0 = time.perf_counter()
    pc = PairCompressed(cube, cube, "H", eps)
    t_part = time.perf_counter() - t0
    t0 = time.perf_counter()
    view = pc._view(c)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    st = pc.view_stats(c)
    x = torch.randn(3 * n, dtype=torch.float64, device="cuda")
    y = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    for _ in range(3):
        pc.apply_device(view, x, y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        pc.apply_device(view, x, y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # end to end: pinned host x in, host y out, every product
    xh = torch.randn(3 * n, dtype=torch.float64).pin_memory()
    yh = torch.empty(3 * n, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        x.copy_(xh, non_blocking=True)
        pc.apply_device(view, x, y)
        yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / reps * 1e3
    factor_bytes = st["lowrank_bytes"] + st["dense_bytes"]
    vec_bytes = 8 * 3 * n * 2 + 4 * 3 * n * 2
    achieved = (factor_bytes + vec_bytes) / (ms / 1e3) / 1e9
    hbm = peaks.get("hbm_gbs") or 6800.0
    ranks = st["ranks"]
    out = {"config": {"workload": f"cube{n_face} self pair, T kernel", "elements": n, "unknowns": 3 * n,
                      "dense_fp64_bytes": 8 * (3 * n) ** 2, "tol": pc.tol,
                      "l2": f"working set {factor_bytes / 1e9:.1f} GB, far above L2"},
           "partition_s": t_part, "view_build_s": t_build, "view_build_breakdown_s": st["build_s"],
           "n_admissible": pc.n_lowrank, "n_dense": pc.n_dense, "n_capped": st["n_capped"],
           "n_retry": st["n_retry"], "n_fallback": st["n_fallback"], "max_verified_err": st["max_verified_err"],
           "n_recompressed": st["n_recompressed"],
           "rank_columns": {"mean": float(ranks.mean()) if ranks.size else 0.0,
                            "median": float(np.median(ranks)) if ranks.size else 0.0,
                            "max": int(ranks.max()) if ranks.size else 0},
           "lowrank_bytes": st["lowrank_bytes"], "dense_bytes": st["dense_bytes"], "held_bytes": pc.nbytes(),
           "matvec_ms": ms, "gpu_launches_per_matvec": 3,
           "kernels_per_matvec": ["cm_gather_kernel", "cm_project_kernel (reads V)",
                                  "cm_strip_kernel (reads U and the dense blocks)"],
           "e2e": {"value": e2e_ms, "unit": "ms per product", "h2d_bytes_per_step": 8 * 3 * n,
                   "d2h_bytes_per_step": 8 * 3 * n},
           "roofline": {"kernel": "compressed matvec (cm_gather + cm_project + cm_strip)", "bound": "hbm",
                        "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "bytes_per_launch": factor_bytes + vec_bytes, "launch_ms": ms,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks.get("hbm_gbs")
                        else "fallback 6.8 TB/s (of fallback)"}}
    if recompressed:
        # the same operator without the recompression of the cross
        # approximation's factors (larger factors, a shorter build)
        t0 = time.perf_counter()
        pr = PairCompressed(cube, cube, "H", eps, recompress_max=0)
        vr = pr._view(c)
        torch.cuda.synchronize()
        tb = time.perf_counter() - t0
        sr = pr.view_stats(c)
        for _ in range(3):
            pr.apply_device(vr, x, y)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            pr.apply_device(vr, x, y)
        e1.record()
        torch.cuda.synchronize()
        msr = e0.elapsed_time(e1) / reps
        rr = sr["ranks"]
        out["without_recompression"] = {
            "recompress_max": 0, "build_s": tb, "matvec_ms": msr,
            "rank_columns_mean": float(rr.mean()) if rr.size else 0.0,
            "lowrank_bytes": sr["lowrank_bytes"], "dense_bytes": sr["dense_bytes"],
            "n_capped": sr["n_capped"], "n_retry": sr["n_retry"], "n_fallback": sr["n_fallback"],
            "max_verified_err": sr["max_verified_err"],
            "achieved_gbs": (sr["lowrank_bytes"] + sr["dense_bytes"] + vec_bytes) / (msr / 1e3) / 1e9}
        del vr, pr
        torch.cuda.empty_cache()
    if cpu:
        from oracle import oracle as orc
        threads = orc.set_threads(os.cpu_count() or 1)
        host = pc.view_host(c)
        xv = x.cpu().numpy()
        y_gpu = pc.matvec(c, xv)
        orc.flat_matvec(host, xv)
        t0 = time.perf_counter()
        n_cpu = 3
        for _ in range(n_cpu):
            y_cpu = orc.flat_matvec(host, xv)
        cpu_ms = (time.perf_counter() - t0) / n_cpu * 1e3
        out["cpu_baseline"] = {"value": cpu_ms, "unit": "ms per product", "cores": threads, "kind": "port",
                               "sample": f"{n_cpu} complete products of the same factors (C port of "
                                         f"flatview.py _flat_matvec, FP32 storage, FP64 sums); host "
                                         f"{os.uname().machine}",
                               "max_rel_diff_vs_gpu": float(np.linalg.norm(y_cpu - y_gpu) / np.linalg.norm(y_cpu))}
        del host
    del view, pc
    torch.cuda.empty_cache()
    return out


def extra_workloads(args, peaks):
    out = {}
    for name, fn in (("volume_cube24_grid66", lambda: volume_workload(cpu=not args.skip_cpu)),
                     ("multi_rhs_cube24_256", lambda: multi_rhs_workload(peaks)),
                     ("multi_mesh_64_cubes", lambda: multi_mesh_workload(peaks)),
                     ("p1_variant_cube24", p1_variant_workload),
                     ("dense_lu_cube35", dense_lu_workload),
                     ("fault_traction_cube32_learned", fault_traction_workload),
                     ("fault_traction_cube32_dip60_learned", lambda: fault_traction_workload(dip=60.0)),
                     ("p2_readout_1m", p2_readout_workload),
                     ("compressed_cube128_self_H", lambda: compressed_workload(peaks, cpu=not args.skip_cpu))):
        if args.extra and name not in args.extra.split(","):
            continue
        try:
            out[name] = fn()
        except Exception as err:     # one workload failing must not hide the headline
            out[name] = {"error": f"{type(err).__name__}: {err}"}
    return out


# DRAM bytes over algorithmic bytes of the mixed matvec, from the ncu capture
# of sgemv_df_tma_kernel at 20,736 unknowns (profiles/): 1.720 GB read for a
# 1.720 GB FP32 matrix.
TRAFFIC_OVER_ALGORITHMIC = 1.0


# ---------------------------------------------------------------------------
# CPU legs (the oracle restatement of the reference's kernels)
# ---------------------------------------------------------------------------

class PortBaseline:
    """The CPU restatement of the reference's path (oracle/: the C kernels
    with OpenMP on all host cores, the numpy FGMRES of the reference's
    la/solver.py) timed on this host.

    A complete solve of the workload at 82,944 unknowns (55 GB of FP64
    operator, ~50 s on 16 cores) does not fit a bounded step, so the port
      - solves the cube-12 workload (5,184 unknowns) completely, once:
        assembly of the calibrated operator and the fault right-hand side,
        then deflated FGMRES(50) to 1e-8 with the true residual checked, which
        gives the port's own iteration count;
      - and in every step assembles one window of source columns of the
        workload's own operator (all field points) and applies that column
        block in an FP64 product: the measured pair rate and product rate on
        the real operator.
    The time to solve the workload is then (operator + right-hand-side pairs)
    / pair rate + (iterations + 3) products + the cube-12 solve's Krylov
    vector work scaled by the unknowns. The iteration count is the port's
    cube-12 count (20 to 1e-8); plain FGMRES on the cube-48 operator takes 27
    on the GPU, so the estimate under-counts the port's solve."""

    def __init__(self, workload: str, step_s: float = 2.5):
        from mbem_gb300.cases import cube_fault_model
        from mbem_gb300.kernels import basis as kb
        from oracle import oracle as orc
        self.orc = orc
        self.threads = orc.set_threads(os.cpu_count() or 1)
        cfg = WORKLOADS[workload]
        model, eps = cube_fault_model(cfg["n_face"], cfg["n_fault"])
        cube = model.regions[0].patches[0]
        fault = model.regions[0].faults[0]
        self.x = cube.collocation_points()
        self.tv = cube.tri_verts()
        self.nrm, _ = cube.mesh.normals_and_areas()
        self.e = np.full(self.tv.shape[0], eps)
        self.c = kb.t_coeffs(1.0, 1.0)
        self.Ns = self.tv.shape[0]
        self.n = 3 * self.Ns
        self.n_fault = fault.n_triangles
        self.pairs = self.x.shape[0] * (self.Ns + self.n_fault)
        self.step_s = step_s
        self.window = None
        self.solve12 = None
        self.samples = []

    def cube12_solve(self):
        """The port's complete solve of the cube-12 workload (timed)."""
        from mbem_gb300.cases import cube_fault_model
        from mbem_gb300.model import generate_system
        from oracle.cpu_system import assemble
        from oracle.fgmres_oracle import deflated_fgmres
        model, eps = cube_fault_model(12, 8)
        system = generate_system(model)
        ur = [(s.offset, s.size) for s in system.layout.slots if s.kind == "u"]
        t0 = time.perf_counter()
        A, b, _ = assemble(self.orc, system, eps)
        t1 = time.perf_counter()
        mv = []

        def matvec(v):
            ta = time.perf_counter()
            y = self.orc.dgemv(A, v)
            mv.append(time.perf_counter() - ta)
            return y
        _, rep = deflated_fgmres(matvec, b, ur, rtol=RTOL, restart=RESTART)
        t2 = time.perf_counter()
        n12 = A.shape[0]
        self.solve12 = {"unknowns": n12, "s": t2 - t0, "assembly_s": t1 - t0, "fgmres_s": t2 - t1,
                        "iterations": rep["iterations"], "matvecs": rep["matvecs"],
                        "true_relres": rep["true_relres"], "converged": bool(rep["converged"]),
                        "krylov_s": (t2 - t1) - float(np.sum(mv))}
        return self.solve12

    def sample(self, i: int):
        """Step i: assemble source window i of the workload's operator for
        every field point, then apply it once (FP64 product)."""
        if self.window is None:           # size the window so a step takes ~step_s
            s1 = 64
            t0 = time.perf_counter()
            self.orc.matrix("t", self.x, self.tv[:s1], self.nrm[:s1], self.e[:s1], self.c)
            dt = time.perf_counter() - t0
            self.window = int(min(self.Ns, max(64, s1 * 0.8 * self.step_s / max(dt, 1e-6))))
        w = self.window
        s0 = (i * w) % max(1, self.Ns - w + 1)
        s1 = s0 + w
        t0 = time.perf_counter()
        blk = self.orc.matrix("t", self.x, self.tv[s0:s1], self.nrm[s0:s1], self.e[s0:s1], self.c)
        t1 = time.perf_counter()
        xv = np.ones(3 * w)
        self.orc.dgemv(blk, xv)
        t2 = time.perf_counter()
        smp = {"columns": (s0, s1), "pairs": self.x.shape[0] * w, "assembly_s": t1 - t0, "product_s": t2 - t1,
               "s": t2 - t0}
        self.samples.append(smp)
        return smp

    def estimate(self):
        """Seconds to solve the workload, from the samples and the cube-12 solve."""
        pairs = sum(s["pairs"] for s in self.samples)
        rate = pairs / sum(s["assembly_s"] for s in self.samples)
        entries = sum(3 * s["pairs"] * 3 for s in self.samples)      # 9 entries a pair
        mv_rate = entries / sum(s["product_s"] for s in self.samples)
        its = self.solve12["iterations"]
        asm = self.pairs / rate
        mv = self.n * self.n / mv_rate
        krylov = self.solve12["krylov_s"] * self.n / self.solve12["unknowns"]
        total = asm + (its + 3) * mv + krylov
        return total, {"assembly_s": asm, "pair_rate_per_s": rate, "product_s": mv, "products": its + 3,
                       "krylov_s": krylov, "iterations": its,
                       "iterations_source": "the port's own FGMRES on the cube-12 workload (to 1e-8)"}

    def describe(self):
        w = self.window
        return (f"complete cube-12 solve (port assembly + port FGMRES, {self.solve12['iterations']} its, "
                f"{self.solve12['s']:.2f} s) + {len(self.samples)} windows of {w} of {self.Ns} source columns "
                f"x {self.x.shape[0]} field points of the workload's operator, each assembled and applied; "
                f"host {os.uname().machine}")


def cpu_baseline(args, n_samples: int = 4):
    """The GPU arm's cpu_baseline: the port's cube-12 solve and a few
    windows of the workload's operator (about 10 s of host work)."""
    pb = PortBaseline(args.workload)
    pb.cube12_solve()
    for i in range(n_samples):
        pb.sample(i)
    total, parts = pb.estimate()
    return {"value": total, "unit": "s", "cores": pb.threads, "kind": "port", "sample": pb.describe(),
            "estimate": parts, "measured_cube12_solve": pb.solve12}


def volume_cpu_baseline(points, code, tri_verts, n_cpu=1024):
    """The CPU baseline of the volume sampler's classification: the numpy
    restatement (one host core) on a bounded random sample of the grid,
    with its agreement with the GPU codes of the same points."""
    from oracle import geometry_oracle as go
    n = points.shape[0]
    sel = np.random.default_rng(0).choice(n, size=min(n_cpu, n), replace=False)
    t0 = time.perf_counter()
    cpu_code = go.classify([[(tri_verts, 1.0)]], points[sel])
    t_cpu = time.perf_counter() - t0
    return {"value": sel.size / t_cpu, "unit": "points/s", "cores": 1, "kind": "port",
            "sample": f"region codes of {sel.size} of {n} grid points (numpy, {t_cpu:.2f} s)",
            "agrees_with_gpu": bool(np.array_equal(cpu_code, code[sel]))}


def run_reference(args, rank, ws):
    """The reference arm: the port on the host cores (rank 0 only). Warm-up
    runs the cube-12 solve; every step is one window of the workload's
    operator, timed for real (ms_per_step); value is the estimated time to
    solve the workload (PortBaseline)."""
    if rank != 0:
        return None
    pb = PortBaseline(args.workload)
    pb.cube12_solve()
    for i in range(args.warmup):
        pb.sample(i)
    pb.samples.clear()
    t0 = time.perf_counter()
    for i in range(args.steps):
        pb.sample(args.warmup + i)
    step_s = (time.perf_counter() - t0) / max(1, args.steps)
    v, parts = pb.estimate()
    cfg = WORKLOADS[args.workload]
    return {"metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded mesh generators; no dataset)",
            "config": {"workload": args.workload, "n_face": cfg["n_face"], "n_fault": cfg["n_fault"],
                       "unknowns": pb.n, "precision": "fp64", "solver": f"deflated FGMRES({RESTART})",
                       "rtol": RTOL},
            "impl": "reference",
            "step": "one window of the workload's operator assembled and applied by the port (the value is "
                    "the estimated complete solve from these steps and the port's complete cube-12 solve)",
            "cpu_baseline": {"value": v, "unit": "s", "cores": pb.threads, "kind": "port", "sample": pb.describe(),
                             "estimate": parts, "measured_cube12_solve": pb.solve12},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cube48", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--skip-tune", action="store_true", help="keep the default tile shapes")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--precond", default="bf16_learned", choices=["bf16_learned", "bf16_inner"],
                    help="the mixed headline's preconditioner (the other is timed beside it)")
    ap.add_argument("--skip-variant", action="store_true", help="skip timing the other mixed preconditioner")
    ap.add_argument("--skip-extra", action="store_true",
                    help="skip the many-right-hand-side and FAULT_TRACTION workloads")
    ap.add_argument("--extra", default="", help="comma-separated names of the extra workloads to run (default: all)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, ws = _dist()
    if args.impl == "reference":
        line = run_reference(args, rank, ws)
    else:
        line = run_ours(args, rank, ws)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
