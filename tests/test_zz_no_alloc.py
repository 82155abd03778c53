"""The allocation-free scan entry point (pbf_exclusive_scan_u32_noalloc).

It exists for callers that cannot allocate device memory when they scan —
a host whose own memory pool owns the device, a real-time loop that must not
enter the allocator — and keeps its scratch in a fixed static device array
instead.  Checked through the C ABI on two calls in a row (the second reuses
the shared array the first left dirty):
  - the whole output against an exclusive scan computed with np.cumsum, and
    against the allocating entry point pbf_exclusive_scan_u32 (integer
    results: bit-exact);
  - that the call allocates nothing from the device's default memory pool
    (its used-memory high-water mark, reset before the call, stays where it
    was; the allocating entry point moves it, which shows the probe works);
  - sizes past the stated maximum are refused.
This file is collected last so a failure here comes after every other test
has run.
"""
import ctypes

import numpy as np
import pytest

from pbf_gb300 import _lib as L

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8  # CUmemPool_attribute (cuda.h)


def _scan(fn, x):
    d_in = torch.from_numpy(x.view(np.int32)).cuda()
    d_out = torch.full_like(d_in, -1)
    torch.cuda.synchronize()
    rc = fn(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), x.size, None)
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy().view(np.uint32)


def _exclusive_cumsum(x):
    out = np.zeros(x.size, dtype=np.uint64)
    out[1:] = np.cumsum(x[:-1], dtype=np.uint64)
    return (out & 0xFFFFFFFF).astype(np.uint32)


class _DefaultPool:
    """The current device's default memory pool through the driver API: its
    used-memory high-water mark can be reset and read."""

    def __init__(self):
        self.drv = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.drv.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
        self.pool = ctypes.c_void_p()
        assert self.drv.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.drv.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def high(self):
        v = ctypes.c_uint64()
        assert self.drv.cuMemPoolGetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


def test_noalloc_scan_matches_cumsum_and_allocating_scan_twice():
    lib = L.load()
    rng = np.random.default_rng(2024)
    # two calls in a row: a large input, then a smaller one that reuses the
    # shared scratch array left dirty by the first
    for n in (3_000_001, 70_001):
        x = rng.integers(0, 1 << 20, size=n, dtype=np.uint32)
        want = _exclusive_cumsum(x)
        rc_a, alloc = _scan(lib.pbf_exclusive_scan_u32, x)
        rc_b, got = _scan(lib.pbf_exclusive_scan_u32_noalloc, x)
        assert rc_a == L.PBF_OK and rc_b == L.PBF_OK
        assert np.array_equal(got, want)
        assert np.array_equal(got, alloc)


def test_noalloc_scan_allocates_nothing():
    lib = L.load()
    pool = _DefaultPool()
    x = np.random.default_rng(7).integers(0, 50, size=1_000_003, dtype=np.uint32)
    d_in = torch.from_numpy(x.view(np.int32)).cuda()
    d_out = torch.empty_like(d_in)
    torch.cuda.synchronize()
    base = pool.high()
    pool.reset_high()
    before = pool.high()
    assert lib.pbf_exclusive_scan_u32_noalloc(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
                                              x.size, None) == L.PBF_OK
    torch.cuda.synchronize()
    assert pool.high() == before, "the allocation-free scan allocated from the default pool"
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), _exclusive_cumsum(x))
    # the probe sees the allocating entry point's scratch
    pool.reset_high()
    assert lib.pbf_exclusive_scan_u32(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), x.size,
                                      None) == L.PBF_OK
    torch.cuda.synchronize()
    assert pool.high() > before
    assert base >= 0


def test_noalloc_scan_rejects_oversize():
    lib = L.load()
    rc = lib.pbf_exclusive_scan_u32_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), L.SCAN_NOALLOC_MAX + 1, None)
    assert rc == L.PBF_ECAPACITY
