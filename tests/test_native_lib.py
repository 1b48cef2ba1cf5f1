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
