"""geon_shadow_bisect_dev_noalloc: the shadow bisection for callers that cannot
let the library allocate device memory while they run.

It keeps its working memory in a fixed array inside the library instead of
asking the allocator, so this test checks, through the C ABI, that it returns
the same results as geon_shadow_bisect_dev (which allocates its working
memory per call) on two calls in a row - the second call reuses the array the
first one left behind - and that requests larger than the array are refused.
The FP64 bisection is deterministic, so "the same" is bit for bit (tolerance
0, as the other FP64 parity tests); the mixed-precision run is held to the
same bar because both entry points run identical kernels on identical inputs.
It also checks the property the entry point exists for: once a first call has
loaded its array and kernels onto the device, a call takes no device memory
(the stream-ordered pool that the allocating entry point draws from does not
grow, and the device's free memory does not shrink), and the largest accepted
request (4096 brackets) gives the allocating entry point's results.
This file is collected last so that a failing run stopped at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, fn, m, lo, hi, iters, precision, torch):
    nb = lo.numel()
    ac = torch.full((nb,), np.nan, dtype=torch.float64, device="cuda")
    lo_o = torch.full((nb,), np.nan, dtype=torch.float64, device="cuda")
    hi_o = torch.full((nb,), np.nan, dtype=torch.float64, device="cuda")
    st = torch.full((nb,), -1, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    rc = getattr(lib, fn)(m.handle, 20.0, lo.data_ptr(), hi.data_ptr(), nb, iters, 0.01, 200000, precision,
                          ac.data_ptr(), lo_o.data_ptr(), hi_o.data_ptr(), st.data_ptr(), s.cuda_stream)
    assert rc == 0, lib.geon_last_error()
    torch.cuda.synchronize()
    return ac.cpu().numpy(), lo_o.cpu().numpy(), hi_o.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_noalloc_bisection_matches_allocating_entry_point(geon, precision):
    torch = pytest.importorskip("torch")
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    calls = [(np.radians(rng.uniform(13.0, 14.0, 24)), np.radians(rng.uniform(14.5, 15.5, 24)), 14),
             (np.radians(rng.uniform(12.0, 14.0, 7)), np.radians(rng.uniform(14.5, 16.0, 7)), 9)]
    for lo_h, hi_h, iters in calls:  # two calls in a row share the fixed scratch
        lo = torch.tensor(lo_h, device="cuda")
        hi = torch.tensor(hi_h, device="cuda")
        want = _run(lib, "geon_shadow_bisect_dev", m, lo, hi, iters, precision, torch)
        got = _run(lib, "geon_shadow_bisect_dev_noalloc", m, lo, hi, iters, precision, torch)
        for w, g in zip(want, got):
            assert np.array_equal(w, g)
        assert np.all(np.isfinite(got[0])) and np.all(got[3] > 0)


class _DevicePool:
    """Usage of the device's default stream-ordered memory pool (the pool that
    cudaMallocAsync draws from) and the device's free memory, read through the
    driver API."""
    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8  # CUmemPool_attribute

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuCtxGetDevice(ctypes.byref(dev)) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def attr(self, a):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, a, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def free_bytes(self):
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
        return free.value


def test_noalloc_call_takes_no_device_memory(geon):
    torch = pytest.importorskip("torch")
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(7)
    nb, iters = 64, 6
    lo = torch.tensor(np.radians(rng.uniform(13.0, 14.0, nb)), device="cuda")
    hi = torch.tensor(np.radians(rng.uniform(14.5, 15.5, nb)), device="cuda")
    out = [torch.empty(nb, dtype=torch.float64, device="cuda") for _ in range(3)]
    st = torch.empty(nb, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()

    def call(fn):
        rc = getattr(lib, fn)(m.handle, 20.0, lo.data_ptr(), hi.data_ptr(), nb, iters, 0.01, 200000, 1,
                              out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), st.data_ptr(), s.cuda_stream)
        assert rc == 0, lib.geon_last_error()
        torch.cuda.synchronize()

    call("geon_shadow_bisect_dev_noalloc")  # the first call on the device loads the array and the kernels
    pool = _DevicePool()
    # the probe sees the allocating entry point's working memory
    call("geon_shadow_bisect_dev")
    pool.reset_high()
    base = pool.attr(pool.USED_MEM_CURRENT)
    call("geon_shadow_bisect_dev")
    assert pool.attr(pool.USED_MEM_HIGH) > base
    # and none from the no-alloc entry point
    pool.reset_high()
    base = pool.attr(pool.USED_MEM_CURRENT)
    free0 = pool.free_bytes()
    call("geon_shadow_bisect_dev_noalloc")
    assert pool.attr(pool.USED_MEM_HIGH) == base
    assert pool.free_bytes() >= free0


@pytest.mark.parametrize("precision,iters", [(1, 6), (0, 2)], ids=["mixed", "fp64"])
def test_noalloc_largest_request(geon, precision, iters):
    torch = pytest.importorskip("torch")
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x4096)
    lo = torch.tensor(np.radians(rng.uniform(13.0, 14.0, 4096)), device="cuda")
    hi = torch.tensor(np.radians(rng.uniform(14.5, 15.5, 4096)), device="cuda")
    want = _run(lib, "geon_shadow_bisect_dev", m, lo, hi, iters, precision, torch)
    for _ in range(2):
        got = _run(lib, "geon_shadow_bisect_dev_noalloc", m, lo, hi, iters, precision, torch)
        for w, g in zip(want, got):
            assert np.array_equal(w, g)


def test_noalloc_refuses_oversized_requests(geon):
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    # 4097 brackets: refused before any device work, with a message naming the limit
    rc = lib.geon_shadow_bisect_dev_noalloc(m.handle, 20.0, ctypes.c_void_p(16), ctypes.c_void_p(16), 4097, 10,
                                            0.01, 1000, 0, ctypes.c_void_p(16), None, None, None, None)
    assert rc == -1
    assert b"4096" in lib.geon_last_error()
    # not a Schwarzschild metric
    mk = geon.Minkowski()
    rc = lib.geon_shadow_bisect_dev_noalloc(mk.handle, 20.0, ctypes.c_void_p(16), ctypes.c_void_p(16), 4, 10,
                                            0.01, 1000, 0, ctypes.c_void_p(16), None, None, None, None)
    assert rc == -1
