"""C ABI checks that need no GPU: the library loads and exports every entry
point include/geon_gpu.h declares; argument errors are reported without CUDA."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if not hdr.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", hdr)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(geon_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from geon_gb300 import _ffi, build
    build.build()
    return _ffi.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ["geon_metric_create", "geon_trace", "geon_render", "geon_camera_tetrad",
                 "geon_riemann", "geon_einstein", "geon_nec_contraction", "geon_shadow_bisect"]:
        assert must in names


def test_every_declared_symbol_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_covers_header():
    from geon_gb300 import _ffi
    assert set(declared_functions()) <= set(_ffi.SIGNATURES)


def test_argument_errors_without_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.geon_metric_create(17, None, 0, ctypes.byref(h)) == -1
    assert b"unknown metric kind" in lib.geon_last_error()
    assert lib.geon_metric_create(1, None, 0, None) == -1
    p = (ctypes.c_double * 5)(1, 2, 3, 4, 5)
    assert lib.geon_metric_create(1, p, 5, ctypes.byref(h)) == -1


def test_render_config_default_matches_reference(lib):
    from geon_gb300 import _ffi
    c = _ffi.GeonRenderConfig()
    lib.geon_render_config_default(ctypes.byref(c))
    assert c.step == 0.05 and c.max_steps == 20000 and c.samples_per_axis == 1
    assert list(c.captured_rgb) == [0.0, 0.0, 0.0] and list(c.diverged_rgb) == [1.0, 0.0, 1.0]


def test_show_stars_flag(lib):
    lib.geon_set_show_stars(0)
    assert lib.geon_get_show_stars() == 0
    lib.geon_set_show_stars(1)
    assert lib.geon_get_show_stars() == 1
