"""Launch-configuration autotuner for the mixed-precision trace kernel.

The library times each register-cap variant of the kernel on a calibration
render of a metric and keeps the fastest for that metric kind
(geon_autotune_mixed). This module runs it, and remembers the result per GPU
model in geon_gb300/_lib/autotune.json so later processes skip the calibration.
"""
import ctypes
import json
import os

from . import _ffi
from ._util import check

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")
CAPS = ("no register cap", "<=64 registers", "<=51 registers")
BLOCKS = (128, 64, 256)
# source 0 (camera rays, ray arrays): the register caps at 128 threads per block;
# source 1 (equatorial shadow rays): cap + 3 * block-size index
VARIANTS = tuple(f"{c}, {b} threads/block" for b in BLOCKS for c in CAPS)


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:  # noqa: BLE001 - any failure just disables the cache key
        return "unknown-gpu"


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def autotune(metric, n_rays=0, max_steps=20000, use_cache=True):
    """Pick the fastest variant per ray source for metric's kind.

    Returns {"variant": [camera/array source, equatorial source], "rates": ...}.
    """
    lib = _ffi.load()
    key = f"{_gpu_name()}|kind={metric.kind}|rays={n_rays}|steps={max_steps}|variants={len(VARIANTS)}"
    cache = _load() if use_cache else {}
    if key in cache:
        for src, v in enumerate(cache[key]["variant"]):
            if v >= 0:
                check(lib.geon_set_mixed_variant(metric.kind, src, int(v)))
        return cache[key]
    rates = (ctypes.c_double * 12)()
    best = (ctypes.c_int * 2)()
    check(lib.geon_autotune_mixed(metric.handle, int(n_rays), int(max_steps), rates, best))
    entry = {"variant": [int(best[0]), int(best[1])],
             "rates": {"camera": [float(r) for r in rates[:3]], "equatorial": [float(r) for r in rates[3:]]},
             "block_size": {"camera": 128, "equatorial": BLOCKS[int(best[1]) // 3] if best[1] >= 0 else None},
             "variants": list(VARIANTS), "calibration": {"rays": int(n_rays), "max_steps": int(max_steps)}}
    if use_cache:
        cache[key] = entry
        try:
            os.makedirs(os.path.dirname(CACHE), exist_ok=True)
            with open(CACHE, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return entry


def current_variant(kind, source=0):
    return _ffi.load().geon_get_mixed_variant(int(kind), int(source))
