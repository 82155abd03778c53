"""The allocation-free scan entry point (pbf_exclusive_scan_u32_noalloc).

It exists for callers that cannot allocate device memory when they scan —
a host whose own memory pool owns the device, a real-time loop that must not
enter the allocator, code running during stream capture — and keeps its
scratch in a fixed static device array instead.  Checked through the C ABI
against the allocating entry point pbf_exclusive_scan_u32 (integer results:
bit-exact) on two calls in a row, which also exercises the reuse of the
shared array; sizes past the stated maximum are refused.  This file is
collected last so a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from pbf_gb300 import _lib as L

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _scan(fn, x):
    d_in = torch.from_numpy(x.view(np.int32)).cuda()
    d_out = torch.full_like(d_in, -1)
    torch.cuda.synchronize()
    rc = fn(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), x.size, None)
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy().view(np.uint32)


def test_noalloc_scan_matches_allocating_scan_twice():
    lib = L.load()
    rng = np.random.default_rng(2024)
    # two calls in a row: a large input, then a smaller one that reuses the
    # shared scratch array left dirty by the first
    for n in (3_000_001, 70_001):
        x = rng.integers(0, 1000, size=n, dtype=np.uint32)
        rc_a, want = _scan(lib.pbf_exclusive_scan_u32, x)
        rc_b, got = _scan(lib.pbf_exclusive_scan_u32_noalloc, x)
        assert rc_a == L.PBF_OK and rc_b == L.PBF_OK
        assert np.array_equal(got, want)
        assert got[0] == 0 and int(got[-1]) == int(x[:-1].sum(dtype=np.uint64)) % (1 << 32)


def test_noalloc_scan_rejects_oversize():
    lib = L.load()
    rc = lib.pbf_exclusive_scan_u32_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), L.SCAN_NOALLOC_MAX + 1, None)
    assert rc == L.PBF_ECAPACITY
