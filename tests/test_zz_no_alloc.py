"""The allocation-free masked dot product, checked against the allocating one.

ntg_glsc2_mask_noalloc serves callers that cannot allocate device memory
(another allocator owns the GPU's memory, memory is exhausted, or an
allocation's implicit synchronisation is not allowed mid-solve).  Its scratch
is a static device array shared by every call, so this test calls it twice
in a row with different data and compares each result with cuda_glsc2_mask,
through the C ABI.  The file sorts last so a run that stops at the first
failure has already run every other test; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(L, a, b, mask, out):
    st = L.ntg_glsc2_mask_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(mask.data_ptr()),
                                  int(mask.numel()), C.c_void_p(out.data_ptr()),
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


def test_noalloc_matches_allocating_entry_point(pkg, dev):
    L = pkg.lib()
    rng = np.random.default_rng(2024)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    for call, (n, m) in enumerate(((300_000, 120_000), (2_000_003, 1_500_001))):
        a = torch.from_numpy(rng.uniform(-1, 1, n)).to(dev)
        b = torch.from_numpy(rng.uniform(-1, 1, n)).to(dev)
        mask = torch.from_numpy(np.sort(rng.choice(n, m, replace=False)).astype(np.int32) + 1).to(dev)
        assert _run(L, a, b, mask, out) == 0, L.ntg_last_error()
        torch.cuda.synchronize()
        ref = pkg.glsc2_mask(a, b, mask)  # the allocating entry point
        got = float(out.item())
        assert abs(got - ref) <= 1e-13 * max(abs(ref), 1.0), (call, got, ref)


def test_noalloc_rejects_oversized_masks(pkg, dev):
    L = pkg.lib()
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    st = L.ntg_glsc2_mask_noalloc(None, None, None, 16_777_217, C.c_void_p(out.data_ptr()), None)
    assert st == 1
    assert b"exceeds the maximum" in L.ntg_last_error()


def test_noalloc_empty_mask_writes_zero(pkg, dev):
    L = pkg.lib()
    out = torch.full((1,), 7.0, dtype=torch.float64, device=dev)
    assert _run(L, out, out, torch.zeros(1, dtype=torch.int32, device=dev)[:0], out) == 0, L.ntg_last_error()
    torch.cuda.synchronize()
    assert float(out.item()) == 0.0
