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
