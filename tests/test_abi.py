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


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes struct of the binding has the C header's size and field offsets."""
    import shutil
    import subprocess
    from geon_gb300 import _ffi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"geon_camera": _ffi.GeonCamera, "geon_render_config": _ffi.GeonRenderConfig,
               "geon_render_stats": _ffi.GeonRenderStats, "geon_grid": _ffi.GeonGrid,
               "geon_job": _ffi.GeonJob, "geon_server_stats": _ffi.GeonServerStats,
               "geon_render_item": _ffi.GeonRenderItem}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "geon_gpu.h"', "int main(void) {"]
    expect = []
    for cname, cls in structs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(ctypes.sizeof(cls))
        for fname, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {fname}));')
            expect.append(getattr(cls, fname).offset)
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect


def test_server_argument_errors_without_gpu(lib):
    from geon_gb300 import _ffi
    h = ctypes.c_void_p()
    assert lib.geon_server_create(16, ctypes.byref(h)) == -1
    assert lib.geon_server_create(1 << 20, None) == -1
    job = _ffi.GeonJob()
    jid = ctypes.c_uint64()
    assert lib.geon_server_submit(None, ctypes.byref(job), ctypes.byref(jid)) == -1
    assert lib.geon_server_poll(None, 1) == -1
    assert lib.geon_server_destroy(None) == 0


def test_adaptive_tolerance_setter_without_gpu(lib):
    import ctypes as C
    r, a = C.c_double(), C.c_double()
    lib.geon_get_adaptive_tolerance(C.byref(r), C.byref(a))
    assert (r.value, a.value) == (1e-10, 1e-12)
    assert lib.geon_set_adaptive_tolerance(-1.0, 1e-12) == -1
    assert lib.geon_set_adaptive_tolerance(0.0, 0.0) == -1
    assert lib.geon_set_adaptive_tolerance(1e-8, 1e-10) == 0
    lib.geon_get_adaptive_tolerance(C.byref(r), C.byref(a))
    assert (r.value, a.value) == (1e-8, 1e-10)
    assert lib.geon_set_adaptive_tolerance(1e-10, 1e-12) == 0


def test_server_tuning_argument_errors_without_gpu(lib):
    assert lib.geon_server_set_steps_per_launch(None, 1, 4096) == -1
    assert lib.geon_server_get_steps_per_launch(None, 1) == -1
    assert lib.geon_server_autotune(None, None, None) == -1


def test_render_batch_argument_errors_without_gpu(lib):
    from geon_gb300 import _ffi
    assert lib.geon_render_batch(None, 0) == 0  # nothing to do
    items = (_ffi.GeonRenderItem * 9)()
    assert lib.geon_render_batch(items, 9) == -1  # at most 8 items
    assert b"1 to 8" in lib.geon_last_error()
    items[0].render.precision = 2  # the adaptive stepper has no batched kernel
    assert lib.geon_render_batch(items, 1) == -1


def test_mixed_null_fix_and_sweep_order_flags_without_gpu(lib):
    assert lib.geon_get_mixed_null_fix() == 1 and lib.geon_get_sweep_order() == 1  # on by default
    lib.geon_set_mixed_null_fix(0)
    lib.geon_set_sweep_order(0)
    assert lib.geon_get_mixed_null_fix() == 0 and lib.geon_get_sweep_order() == 0
    lib.geon_set_mixed_null_fix(1)
    lib.geon_set_sweep_order(1)


def test_mixed_orbit_plane_flag_without_gpu(lib):
    assert lib.geon_get_mixed_orbit_plane() == 1  # on by default
    lib.geon_set_mixed_orbit_plane(0)
    assert lib.geon_get_mixed_orbit_plane() == 0
    lib.geon_set_mixed_orbit_plane(1)
    assert lib.geon_get_mixed_orbit_plane() == 1


def test_persistent_reserve_setters_without_gpu(lib):
    # plain stores, no CUDA: whole and fractional counts, and values that mean none
    for v in (0.0, 4.5, -1.0, float("nan"), 1e30):
        lib.geon_set_persistent_reserve_f(v)
    lib.geon_set_persistent_reserve(3)
    lib.geon_set_persistent_reserve(0)
