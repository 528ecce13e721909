"""Host-side parts of the serving engine (geon_gb300/csrc/serve_host.h),
compiled for the host: the first-fit arena, the speculative bisection tree and
the shortest-remaining-first claim order, against Python models."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "geon_gb300", "csrc")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("serve_host") / "libserve_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "serve_host_harness.cpp"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    sz, vp = ctypes.c_size_t, ctypes.c_void_p
    lib.arena_new.restype = vp
    lib.arena_new.argtypes = [sz]
    lib.arena_free.argtypes = [vp]
    lib.arena_alloc.argtypes = [vp, sz, ctypes.POINTER(sz)]
    lib.arena_release.argtypes = [vp, sz, sz]
    lib.align_up.restype = sz
    lib.align_up.argtypes = [sz]
    lib.tree.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    ip, i64p, u64p, up = (ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64),
                          ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint))
    lib.order.argtypes = [ip, i64p, u64p, ip, ctypes.c_int, ctypes.c_int, sz, ip, up]
    return lib


def test_arena_first_fit_and_coalescing(host):
    """Random allocations and releases against a Python first-fit model: the
    same offsets, no overlap, and one free block of the whole arena at the end."""
    size = 1 << 24
    a = host.arena_new(size)
    free = {0: size}  # model: offset -> length
    live = {}
    rng = np.random.default_rng(3)

    def model_alloc(n):
        n = (max(n, 1) + 255) // 256 * 256
        for o in sorted(free):
            if free[o] >= n:
                rem = free.pop(o) - n
                if rem:
                    free[o + n] = rem
                return o, n
        return None, n

    def model_release(o, n):
        free[o] = n
        keys = sorted(free)
        merged = {}
        for k in keys:
            if merged:
                last = max(merged)
                if last + merged[last] == k:
                    merged[last] += free[k]
                    continue
            merged[k] = free[k]
        free.clear()
        free.update(merged)

    try:
        for step in range(3000):
            if live and (rng.random() < 0.45 or len(live) > 200):
                key = list(live)[rng.integers(len(live))]
                o, n, req = live.pop(key)
                host.arena_release(a, o, req)
                model_release(o, n)
            else:
                req = int(rng.integers(0, 1 << 18))
                off = ctypes.c_size_t()
                ok = host.arena_alloc(a, req, ctypes.byref(off))
                mo, n = model_alloc(req)
                assert bool(ok) == (mo is not None)
                if ok:
                    assert off.value == mo and off.value % 256 == 0
                    for o2, n2, _ in live.values():  # no overlap with live blocks
                        assert off.value + n <= o2 or o2 + n2 <= off.value
                    live[step] = (off.value, n, req)
        for o, n, req in live.values():
            host.arena_release(a, o, req)
            model_release(o, n)
        assert free == {0: size}
        off = ctypes.c_size_t()
        assert host.arena_alloc(a, size, ctypes.byref(off)) == 1 and off.value == 0  # fully coalesced
        assert host.arena_alloc(a, 1, ctypes.byref(off)) == 0
    finally:
        host.arena_free(a)
    assert host.align_up(0) == 0 and host.align_up(1) == 256 and host.align_up(256) == 256


def test_bisection_tree_matches_sequential_halvings(host):
    """Node i of the heap-ordered tree is the midpoint the sequential bisection
    (bin/validate_shadow.rs:70-77) reaches after the halvings that lead to it,
    formed by the same 0.5 * (lo + hi)."""
    rng = np.random.default_rng(5)
    for _ in range(20):
        lo, hi = np.radians(rng.uniform(13, 14)), np.radians(rng.uniform(14.5, 15.5))
        levels = int(rng.integers(1, 9))
        out = (ctypes.c_double * ((1 << levels) - 1))()
        host.tree(lo, hi, levels, out)
        got = np.array(out[:])
        for i in range(1, (1 << levels)):
            path = bin(i)[3:]  # bits below the leading 1: 0 = keep [lo, mid], 1 = keep [mid, hi]
            l, h = lo, hi
            for bit in path:
                mid = 0.5 * (l + h)
                if bit == "0":
                    h = mid
                else:
                    l = mid
            assert got[i - 1] == 0.5 * (l + h)


def test_claim_order_shortest_remaining_first(host):
    rng = np.random.default_rng(7)
    n, ncls, stride = 300, 8, 4096
    cls = rng.integers(0, ncls, n).astype(np.int32)
    left = rng.integers(-3, 50, n).astype(np.int64)  # <= 0: nothing left to claim
    ids = rng.permutation(n).astype(np.uint64)
    slot = np.arange(n, dtype=np.int32)
    out = np.full(ncls * stride, -1, np.int32)
    counts = np.zeros(ncls, np.uint32)
    host.order(cls.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), left.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
               ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), slot.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
               n, ncls, stride, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
               counts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)))
    for c in range(ncls):
        want = [s for _, _, s in sorted((int(left[i]), int(ids[i]), int(slot[i])) for i in range(n)
                                        if cls[i] == c and left[i] > 0)]
        assert counts[c] == len(want)
        assert list(out[c * stride:c * stride + counts[c]]) == want
