"""The C-ABI library builds, loads and exports every symbol the header
declares (no compute call: this runs without a GPU)."""

import os
import re

from mbem_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mbem_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mbem_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_what_the_binding_binds():
    assert header_symbols() == sorted(_native.exported_symbols())


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_native.LIB_PATH):
        from mbem_gb300 import build
        build.build()
    lib = _native.lib()
    for name in header_symbols():
        assert hasattr(lib, name), name
    assert lib.mbem_version() >= 1


def test_multi_mesh_layout_rules():
    """The batch layout check is host code: segments follow one another,
    each rounded up to MBEM_MM_SEGMENT; anything else is refused."""
    import ctypes
    lib = _native.lib()

    def meshes(sizes, offsets):
        arr = (_native.MmMesh * len(sizes))()
        for i, (n, o) in enumerate(zip(sizes, offsets)):
            # placeholder (never dereferenced) 16-byte aligned pointers
            arr[i] = _native.MmMesh(4096, (n + 3) // 4 * 4, n, o, 4096, 4096, 4096, 0, n, None, 0)
        return arr

    seg = _native.MM_SEGMENT
    sizes = [300, 2400, 9]
    offs = [0, seg, seg + 5 * seg]
    assert lib.mbem_mm_total(meshes(sizes, offs), 3) == seg + 5 * seg + seg
    assert lib.mbem_mm_workspace_size(meshes(sizes, offs), 3, 50) > 0
    assert lib.mbem_mm_total(meshes(sizes, [0, seg, 7 * seg]), 3) == -1          # a gap
    assert lib.mbem_mm_total(meshes([300, 2400], [0, 300]), 2) == -1             # not rounded up
    assert lib.mbem_mm_total(meshes([301], [0]), 1) == -1                        # not a multiple of 3
    assert lib.mbem_mm_workspace_size(meshes(sizes, offs), 3, _native.MM_MAX_RESTART + 1) == 0
    assert ctypes.sizeof(_native.MmMesh) == 88


def test_geometry_entry_points_check_their_arguments():
    """Host-side checks of the mesh-geometry entry points (no kernel runs:
    each call is refused, or has no points, before any launch)."""
    lib = _native.lib()
    assert lib.mbem_geom_record_bytes(10) == 10 * 32 * 4
    assert lib.mbem_geom_record_bytes(0) == 0
    fake = 4096                       # never dereferenced
    assert lib.mbem_mesh_distance(fake, fake, 0, fake, 5, 1.0, fake, fake, None) == _native.ERR_ARG
    assert lib.mbem_mesh_distance(fake + 4, fake, 3, fake, 5, 1.0, fake, fake, None) == _native.ERR_ARG
    assert lib.mbem_solid_angle_sum(fake, fake, 3, fake, 0, 1.0, 0, fake, None) == _native.OK
    assert lib.mbem_geom_prepare(None, 3, fake, None) == _native.ERR_ARG
