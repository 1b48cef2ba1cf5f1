"""Autotuner for the tile shapes of the streaming kernels.

Four kernel families have several compiled tile configurations (the C
library's ``mbem_tune_*`` entry points):

- ``mixed_matvec``: the FP32 double-float operator product (rows per CTA,
  columns per ring chunk, ring stages);
- ``bf16_matvec``: the BF16 inner product of the mixed solve (same knobs);
- ``mm_matvec``: the persistent multi-mesh product (chunk, stages);
- ``gemm_split``: the K split of the tensor-core GEMM (wave cost model or a
  fixed count).

``Autotuner.tune`` runs the caller's own workload once per configuration,
times it with CUDA events (median of ``reps`` after ``warmup`` runs), keeps
the fastest configuration selected for the process, and records every
timing in a JSON cache keyed by device, family and workload key, so a later
process on the same device and workload selects it without timing again.
"""

from __future__ import annotations

import json
import os
import statistics
from dataclasses import asdict, dataclass, field

import torch

from . import _native as nat

FAMILIES = {"mixed_matvec": nat.TUNE_MIXED_MATVEC, "bf16_matvec": nat.TUNE_BF16_MATVEC,
            "mm_matvec": nat.TUNE_MM_MATVEC, "gemm_split": nat.TUNE_GEMM_SPLIT}


def _fam(family: str) -> int:
    if family not in FAMILIES:
        raise ValueError(f"unknown kernel family {family!r} (one of {sorted(FAMILIES)})")
    return FAMILIES[family]


def count(family: str) -> int:
    return int(nat.lib().mbem_tune_count(_fam(family)))


def describe(family: str, config: int) -> str:
    buf = nat.ctypes.create_string_buffer(64)
    nat.call("mbem_tune_describe", _fam(family), int(config), buf, len(buf))
    return buf.value.decode()


def current(family: str) -> int:
    return int(nat.lib().mbem_tune_get(_fam(family)))


def select(family: str, config: int) -> None:
    nat.call("mbem_tune_set", _fam(family), int(config))


def cuda_time_ms(run, reps: int = 5, warmup: int = 2) -> float:
    """Median device time of ``run()`` in ms (CUDA events on the current stream)."""
    for _ in range(warmup):
        run()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for s, e in evs:
        s.record()
        run()
        e.record()
    torch.cuda.synchronize()
    return float(statistics.median(s.elapsed_time(e) for s, e in evs))


def default_cache_path() -> str:
    return os.environ.get("MBEM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mbem_gb300", "autotune.json"))


@dataclass
class TuneResult:
    family: str
    key: str
    best: int
    best_desc: str
    times_ms: list = field(default_factory=list)   # per configuration (None where not timed)
    cached: bool = False

    def summary(self) -> dict:
        d = asdict(self)
        d["configs"] = [describe(self.family, c) for c in range(len(self.times_ms))]
        return d


class Autotuner:
    """Times every tile configuration of a family on a workload and selects
    the fastest. ``cache_path=""`` keeps results in this process only;
    ``timer(run) -> ms`` replaces the CUDA-event timer (tests)."""

    def __init__(self, cache_path: str | None = None, reps: int = 5, warmup: int = 2, timer=None,
                 device: str | None = None):
        self.cache_path = default_cache_path() if cache_path is None else cache_path
        self.reps, self.warmup = reps, warmup
        self.timer = timer or (lambda run: cuda_time_ms(run, self.reps, self.warmup))
        self._device = device
        self._cache = self._load()

    @property
    def device(self) -> str:
        if self._device is None:
            props = torch.cuda.get_device_properties(torch.cuda.current_device())
            self._device = f"{props.name}|sm{props.major}{props.minor}|{props.multi_processor_count}"
        return self._device

    def _load(self) -> dict:
        if not self.cache_path or not os.path.exists(self.cache_path):
            return {}
        try:
            with open(self.cache_path) as f:
                data = json.load(f)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def _save(self) -> None:
        if not self.cache_path:
            return
        os.makedirs(os.path.dirname(os.path.abspath(self.cache_path)), exist_ok=True)
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self._cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def tune(self, family: str, key: str, run, force: bool = False) -> TuneResult:
        """Selects the fastest configuration of ``family`` for ``run()`` (a
        launch of that family's kernel on the caller's data)."""
        n = count(family)
        entry = f"{self.device}|{family}|{key}"
        hit = self._cache.get(entry)
        if hit is not None and not force and 0 <= int(hit.get("best", -1)) < n \
                and len(hit.get("times_ms", [])) == n:
            select(family, int(hit["best"]))
            return TuneResult(family, key, int(hit["best"]), describe(family, int(hit["best"])),
                              list(hit["times_ms"]), cached=True)
        times = []
        for c in range(n):
            select(family, c)
            times.append(float(self.timer(run)))
        best = min(range(n), key=lambda c: (times[c], c))
        select(family, best)
        self._cache[entry] = {"best": best, "times_ms": times}
        self._save()
        return TuneResult(family, key, best, describe(family, best), times)


def tune_mixed_operator(asm, tuner: Autotuner | None = None) -> dict:
    """Tunes the FP32 operator product (and the BF16 inner product when the
    system has the BF16 copy) of an assembled mixed-precision system."""
    from .la.mixed import Bf16Inner
    tuner = tuner or Autotuner()
    op = asm.op
    if op is None:
        raise ValueError("tune_mixed_operator needs a mixed-precision system")
    x = torch.randn(op.n, dtype=torch.float64, device=op.A32.device)
    y = torch.empty_like(x)
    out = {"mixed_matvec": tuner.tune("mixed_matvec", f"n={op.n}", lambda: op.matvec(x, out=y)).summary()}
    inner = getattr(asm, "_inner", None)
    if inner is None and op.A16 is not None:
        inner = Bf16Inner(op, 1, asm.u_ranges())
    if inner is not None:
        out["bf16_matvec"] = tuner.tune("bf16_matvec", f"n={op.n}", lambda: inner.matvec(x, out=y)).summary()
    return out


def tune_mesh_batch(batch, tuner: Autotuner | None = None) -> dict:
    """Tunes the persistent multi-mesh product on a ``la.multimesh.MeshBatch``."""
    tuner = tuner or Autotuner()
    x = torch.randn(batch.n_total, dtype=torch.float64, device=batch.device)
    key = f"meshes={batch.n_mesh},n={batch.n_total}"
    return {"mm_matvec": tuner.tune("mm_matvec", key, lambda: batch.matvec(x)).summary()}
