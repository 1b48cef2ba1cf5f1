"""Shared fixtures: the ``gpu`` marker, the golden fixtures, the oracle."""

from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 and the built mbem_gb300 library")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as g:
        return {k: g[k] for k in g.files}


@pytest.fixture(scope="session")
def p0_pairs():
    return load_golden("p0_pairs")


@pytest.fixture(scope="session")
def cube_small():
    return load_golden("cube_small")


@pytest.fixture(scope="session")
def c1_rows():
    return load_golden("c1_rows")


@pytest.fixture(scope="session")
def nodal_pairs():
    return load_golden("nodal_pairs")


@pytest.fixture(scope="session")
def traction_small():
    return load_golden("traction_small")


@pytest.fixture(scope="session")
def volume_small():
    return load_golden("volume_small")


@pytest.fixture(scope="session")
def volume_regions():
    return load_golden("volume_regions")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.lib()
    return orc


@pytest.fixture(scope="session")
def gpu():
    """Skips without a CUDA device; builds the library once if it is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mbem_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from mbem_gb300 import build
        build.build()
    _native.lib()
    return torch.device("cuda", 0)


def rel_err(a, b) -> float:
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


@pytest.fixture(scope="session")
def condense_small():
    return load_golden("condense_small")


@pytest.fixture(scope="session")
def compressed_small():
    return load_golden("compressed_small")


def golden_blocks(g: dict, key: str) -> list:
    """A block list stored flat (rows, cols and their offsets) as (rows, cols) pairs."""
    rows, cols, rp, cp = (g[f"{key}_{s}"] for s in ("rows", "cols", "rptr", "cptr"))
    return [(rows[rp[i]:rp[i + 1]], cols[cp[i]:cp[i + 1]]) for i in range(rp.size - 1)]
