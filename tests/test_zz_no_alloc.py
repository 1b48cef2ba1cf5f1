"""mbem_mixed_matvec_noalloc: the mixed-operator product for callers that
cannot allocate device memory (their host hands all device memory to its own
pool, or their loop must not enter the allocator). It keeps its scratch in a
fixed array inside the library instead of a caller workspace.

Checked through the C ABI against mbem_mixed_matvec (the workspace variant)
on two calls in a row, within the mixed-matvec tolerance of the other tests
(1e-13 relative); and its size limit is refused before any GPU work. This file
is collected last so that a run stopping at its first failure has run every
other test before it.
"""

import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_matvec_matches_workspace_variant_twice(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    from mbem_gb300.backends.dense import DenseBackend
    from mbem_gb300.cases import cube_fault_model
    from mbem_gb300.model import generate_system

    model, eps = cube_fault_model(6, 4)
    asm = DenseBackend(jump="calibrated", deflate=True, precision="mixed").assemble(generate_system(model), eps)
    op = asm.op
    n = op.n
    st = op.struct()
    work = torch.empty(2 * n * 4 + 64, dtype=torch.uint8, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(3)
    for _ in range(2):
        x = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        y_ref = torch.empty(n, dtype=torch.float64, device="cuda")
        y_new = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
        nat.call("mbem_mixed_matvec", ctypes.byref(st), ptr(x), ptr(y_ref), ptr(work), work.numel(),
                 stream_handle())
        nat.call("mbem_mixed_matvec_noalloc", ctypes.byref(st), ptr(x), ptr(y_new), stream_handle())
        torch.cuda.synchronize()
        # no bulk-copy wait of either product ran out of time
        nat.call("mbem_mixed_wait_check", stream_handle())
        assert torch.isfinite(y_new).all()
        assert rel_err(y_new.cpu().numpy(), y_ref.cpu().numpy()) < 1e-13


def test_noalloc_refuses_sizes_beyond_its_scratch(gpu):
    from mbem_gb300 import _native as nat
    from mbem_gb300._device import ptr, stream_handle
    cols = 262144 + 1
    A32 = torch.zeros((1, cols), dtype=torch.float32, device="cuda")
    x = torch.zeros(cols, dtype=torch.float64, device="cuda")
    y = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = nat.MixedOperator(1, cols, ptr(A32), cols, 0, None)
    with pytest.raises(nat.MbemError) as info:
        nat.call("mbem_mixed_matvec_noalloc", ctypes.byref(st), ptr(x), ptr(y), stream_handle())
    assert info.value.code == nat.ERR_SIZE
    assert "262144" in str(info.value)
