"""Deterministic unknown layout (``src/mbem/model/layout.py:33-108``).

Regions in model order; within a region, patches in declaration order
(skipping patches already emitted): FREE_TRACTION emits its u-slot,
PRESCRIBED_DISPLACEMENT its t-slot, INTERFACE u then t; then the b-slots of
the region's FAULT_TRACTION faults. A slot holds 3 n_dofs values; rows are
the patch's collocation points, so the system is square.
"""

from __future__ import annotations

from dataclasses import dataclass

from .core import BCType, Patch, Region, RegionModel


@dataclass(frozen=True)
class Slot:
    patch: Patch
    kind: str
    offset: int
    size: int

    @property
    def name(self) -> str:
        return f"{self.kind}:{self.patch.name}"

    @property
    def stop(self) -> int:
        return self.offset + self.size


class UnknownLayout:
    def __init__(self, model: RegionModel):
        self.model = model
        self.slots: list[Slot] = []
        self._by_key: dict = {}
        offset = 0
        emitted: set = set()
        kinds_of = {BCType.FREE_TRACTION: ("u",), BCType.PRESCRIBED_DISPLACEMENT: ("t",),
                    BCType.INTERFACE: ("u", "t")}
        for region in model.regions:
            for patch in region.patches:
                if id(patch) in emitted:
                    continue
                emitted.add(id(patch))
                for kind in kinds_of[patch.bc]:
                    offset = self._add(patch, kind, offset)
            for f in region.faults:
                if f.bc is not BCType.FAULT_TRACTION or id(f) in emitted:
                    continue
                emitted.add(id(f))
                offset = self._add(f, "b", offset)
        self.n_unknowns = offset

    def _add(self, patch, kind, offset) -> int:
        slot = Slot(patch, kind, offset, 3 * patch.n_dofs)
        self.slots.append(slot)
        self._by_key[(id(patch), kind)] = slot
        return offset + slot.size

    def has_kind(self, kind: str) -> bool:
        return any(s.kind == kind for s in self.slots)

    def slot(self, patch: Patch, kind: str) -> Slot:
        return self._by_key[(id(patch), kind)]

    def has_slot(self, patch: Patch, kind: str) -> bool:
        return (id(patch), kind) in self._by_key

    def row_slot(self, region: Region, patch: Patch) -> Slot:
        if patch.bc is BCType.FAULT_TRACTION:
            return self.slot(patch, "b")
        if patch.bc is BCType.FREE_TRACTION:
            return self.slot(patch, "u")
        if patch.bc is BCType.PRESCRIBED_DISPLACEMENT:
            return self.slot(patch, "t")
        if patch.bc is BCType.INTERFACE:
            first, second = self.model.interface_regions(patch)
            if region is first:
                return self.slot(patch, "u")
            if region is second:
                return self.slot(patch, "t")
            raise ValueError(f"region '{region.name}' is not incident to interface '{patch.name}'")
        raise ValueError(f"no collocation row for bc {patch.bc}")
