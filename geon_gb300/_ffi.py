"""ctypes binding of libgeon_gpu.so (the C ABI declared in include/geon_gpu.h).

The library is built in-tree by geon_gb300/build.py. There is no CPU fallback:
if the library is missing or a call fails, an exception says why.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgeon_gpu.so")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p

GEON_OK = 0
GEON_ERR_INVALID = -1
GEON_ERR_SINGULAR_METRIC = -2
GEON_ERR_NOT_TIMELIKE = -3
GEON_ERR_GRAM_SCHMIDT = -4
GEON_ERR_CUDA = -5
GEON_ERR_OOM = -6
GEON_ERR_ADMISSION = -7
GEON_ERR_TIMEOUT = -8
GEON_ERR_NOT_FOUND = -9
GEON_ERR_CANCELLED = -10
GEON_ERR_UNSUPPORTED = -11


class GeonCamera(ctypes.Structure):
    _fields_ = [("observer", ctypes.c_double * 4), ("fov_y_deg", ctypes.c_double),
                ("width", ctypes.c_int64), ("height", ctypes.c_int64),
                ("forward_sign", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class GeonRenderConfig(ctypes.Structure):
    _fields_ = [("step", ctypes.c_double), ("max_steps", ctypes.c_int64),
                ("captured_rgb", ctypes.c_float * 3), ("diverged_rgb", ctypes.c_float * 3),
                ("samples_per_axis", ctypes.c_int64), ("show_stars", ctypes.c_int32),
                ("precision", ctypes.c_int32)]


class GeonGrid(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3), ("n", ctypes.c_int64 * 3),
                ("t", ctypes.c_double)]


class GeonRenderStats(ctypes.Structure):
    _fields_ = [("captured", ctypes.c_int64), ("escaped", ctypes.c_int64),
                ("diverged", ctypes.c_int64), ("max_null_residual", ctypes.c_double),
                ("avg_steps", ctypes.c_double), ("total_steps", ctypes.c_int64)]


class GeonRenderItem(ctypes.Structure):
    _fields_ = [("metric", ctypes.c_void_p), ("camera", GeonCamera), ("render", GeonRenderConfig),
                ("rgb", ctypes.c_void_p), ("stats", ctypes.POINTER(GeonRenderStats)),
                ("pixel_class", ctypes.c_void_p), ("pixel_steps", ctypes.c_void_p)]


class GeonJob(ctypes.Structure):
    """geon_job: one serving request (pointers are plain addresses)."""
    _fields_ = [("type", ctypes.c_int32), ("metric_kind", ctypes.c_int32),
                ("metric_params", ctypes.c_double * 4), ("nparams", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("deadline_s", ctypes.c_double),
                ("camera", GeonCamera), ("render", GeonRenderConfig),
                ("rgb", c_void_p), ("render_stats", c_void_p), ("pixel_class", c_void_p),
                ("pixel_steps", c_void_p), ("rgb8", c_void_p),
                ("r_obs", ctypes.c_double), ("lo", ctypes.c_double), ("hi", ctypes.c_double),
                ("step", ctypes.c_double), ("max_steps", ctypes.c_int64), ("iters", ctypes.c_int32),
                ("rays_per_round", ctypes.c_int32), ("alpha_c", c_void_p), ("lo_out", c_void_p),
                ("hi_out", c_void_p), ("steps_out", c_void_p),
                ("grid", GeonGrid), ("nk", ctypes.c_int64), ("seed", ctypes.c_uint64),
                ("einstein", c_void_p), ("nec", c_void_p)]


class GeonServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("running", ctypes.c_int64),
                ("completed_by_type", ctypes.c_int64 * 3),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("p50_ms_by_type", ctypes.c_double * 3), ("p99_ms_by_type", ctypes.c_double * 3),
                ("ray_steps", ctypes.c_double), ("grid_points", ctypes.c_double), ("wall_s", ctypes.c_double),
                ("epochs", ctypes.c_int64), ("ray_steps_unfinished", ctypes.c_double)]


# name -> (restype, argtypes); every exported symbol of include/geon_gpu.h
SIGNATURES = {
    "geon_version": (ctypes.c_char_p, []),
    "geon_last_error": (ctypes.c_char_p, []),
    "geon_render_config_default": (None, [ctypes.POINTER(GeonRenderConfig)]),
    "geon_metric_create": (ctypes.c_int, [ctypes.c_int, c_double_p, ctypes.c_int, ctypes.POINTER(c_void_p)]),
    "geon_metric_destroy": (ctypes.c_int, [c_void_p]),
    "geon_metric_create_field": (ctypes.c_int, [ctypes.POINTER(GeonGrid), c_double_p, ctypes.c_int,
                                                ctypes.POINTER(c_void_p)]),
    "geon_metric_kind": (ctypes.c_int, [c_void_p]),
    "geon_metric_name": (ctypes.c_char_p, [c_void_p]),
    "geon_metric_g": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_metric_dg": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_metric_g_inv": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_metric_christoffel": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_metric_terminate": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_int32_p]),
    "geon_metric_asymptotic_direction": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_trace": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, ctypes.c_double, ctypes.c_int64,
                                  ctypes.c_int, c_int32_p, c_double_p, c_int64_p, c_double_p]),
    "geon_trace_dev": (ctypes.c_int, [c_void_p, c_void_p, c_size_t, ctypes.c_double, ctypes.c_int64,
                                      ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "geon_camera_tetrad": (ctypes.c_int, [c_void_p, c_double_p, c_double_p]),
    "geon_camera_ray_states": (ctypes.c_int, [ctypes.POINTER(GeonCamera), c_double_p, ctypes.c_double,
                                              ctypes.c_double, c_double_p]),
    "geon_render": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonCamera), ctypes.POINTER(GeonRenderConfig),
                                   c_float_p, ctypes.POINTER(GeonRenderStats)]),
    "geon_render_u8": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonCamera), ctypes.POINTER(GeonRenderConfig),
                                      c_void_p, c_void_p, ctypes.POINTER(GeonRenderStats)]),
    "geon_tonemap_u8": (ctypes.c_int, [c_void_p, c_size_t, c_void_p]),
    "geon_tonemap_u8_dev": (ctypes.c_int, [c_void_p, c_size_t, c_void_p, c_void_p]),
    "geon_render_ex": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonCamera), ctypes.POINTER(GeonRenderConfig),
                                      c_float_p, ctypes.POINTER(GeonRenderStats), c_int32_p, c_int64_p]),
    "geon_render_batch": (ctypes.c_int, [ctypes.POINTER(GeonRenderItem), c_size_t]),
    "geon_sky_sample": (ctypes.c_int, [c_double_p, c_size_t, ctypes.c_int, c_float_p]),
    "geon_set_show_stars": (None, [ctypes.c_int]),
    "geon_get_show_stars": (ctypes.c_int, []),
    "geon_set_mixed_band": (ctypes.c_int, [ctypes.c_int, ctypes.c_double]),
    "geon_get_mixed_band": (ctypes.c_double, [ctypes.c_int]),
    "geon_set_mixed_reproject": (None, [ctypes.c_int]),
    "geon_set_mixed_orbit_plane": (None, [ctypes.c_int]),
    "geon_get_mixed_orbit_plane": (ctypes.c_int, []),
    "geon_set_mixed_null_fix": (None, [ctypes.c_int]),
    "geon_set_sweep_order": (None, [ctypes.c_int]),
    "geon_get_sweep_order": (ctypes.c_int, []),
    "geon_get_mixed_null_fix": (ctypes.c_int, []),
    "geon_set_persistent_reserve": (None, [ctypes.c_int]),
    "geon_set_persistent_reserve_f": (None, [ctypes.c_double]),
    "geon_set_mixed_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "geon_get_mixed_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "geon_autotune_mixed": (ctypes.c_int, [c_void_p, ctypes.c_int64, ctypes.c_int64, c_double_p,
                                           ctypes.POINTER(ctypes.c_int)]),
    "geon_riemann": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_ricci": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_ricci_scalar": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_einstein": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_stress_energy": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p]),
    "geon_nec_contraction": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p, c_size_t,
                                            ctypes.c_int, c_double_p]),
    "geon_wec_contraction": (ctypes.c_int, [c_void_p, c_double_p, c_size_t, c_double_p, c_size_t,
                                            ctypes.c_int, c_double_p]),
    "geon_curvature_grid": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonGrid), c_size_t, ctypes.c_uint64,
                                           c_double_p, c_double_p, c_double_p]),
    "geon_curvature_grid_dev": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonGrid), c_size_t, ctypes.c_uint64,
                                               c_void_p, c_void_p, c_void_p, c_void_p]),
    "geon_equatorial_rays": (ctypes.c_int, [c_void_p, ctypes.c_double, c_double_p, c_size_t, c_double_p]),
    "geon_shadow_classify": (ctypes.c_int, [c_void_p, ctypes.c_double, c_double_p, c_size_t, ctypes.c_double,
                                            ctypes.c_int64, ctypes.c_int, c_int32_p, c_int64_p]),
    "geon_shadow_trace": (ctypes.c_int, [c_void_p, ctypes.c_double, c_double_p, c_size_t, ctypes.c_double,
                                         ctypes.c_int64, ctypes.c_int, c_int32_p, c_double_p, c_int64_p,
                                         c_double_p]),
    "geon_shadow_bisect": (ctypes.c_int, [c_void_p, ctypes.c_double, c_double_p, c_double_p, c_size_t,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                          c_double_p, c_double_p, c_double_p, c_int64_p]),
    "geon_shadow_classify_dev": (ctypes.c_int, [c_void_p, ctypes.c_double, c_void_p, c_size_t, ctypes.c_double,
                                                ctypes.c_int64, ctypes.c_int, c_void_p, c_void_p, c_void_p]),
    "geon_shadow_bisect_dev": (ctypes.c_int, [c_void_p, ctypes.c_double, c_void_p, c_void_p, c_size_t,
                                              ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                              c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "geon_shadow_bisect_dev_noalloc": (ctypes.c_int, [c_void_p, ctypes.c_double, c_void_p, c_void_p, c_size_t,
                                                      ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                                      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "geon_server_create": (ctypes.c_int, [c_size_t, ctypes.POINTER(c_void_p)]),
    "geon_server_submit": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonJob), ctypes.POINTER(ctypes.c_uint64)]),
    "geon_server_poll": (ctypes.c_int, [c_void_p, ctypes.c_uint64]),
    "geon_server_wait": (ctypes.c_int, [c_void_p, ctypes.c_uint64, ctypes.c_double]),
    "geon_server_wait_all": (ctypes.c_int, [c_void_p, ctypes.c_double]),
    "geon_server_cancel": (ctypes.c_int, [c_void_p, ctypes.c_uint64]),
    "geon_server_stats_get": (ctypes.c_int, [c_void_p, ctypes.POINTER(GeonServerStats)]),
    "geon_server_destroy": (ctypes.c_int, [c_void_p]),
    "geon_server_set_steps_per_launch": (ctypes.c_int, [c_void_p, ctypes.c_int, ctypes.c_int]),
    "geon_server_get_steps_per_launch": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "geon_server_autotune": (ctypes.c_int, [c_void_p, c_double_p, ctypes.POINTER(ctypes.c_int)]),
    "geon_energy_conditions": (ctypes.c_int, [c_double_p]),
    "geon_set_adaptive_tolerance": (ctypes.c_int, [ctypes.c_double, ctypes.c_double]),
    "geon_set_bisect_rays_per_round": (ctypes.c_int, [ctypes.c_int64]),
    "geon_get_bisect_rays_per_round": (ctypes.c_int64, []),
    "geon_get_adaptive_tolerance": (None, [c_double_p, c_double_p]),
    "geon_launch_count": (ctypes.c_ulonglong, []),
    "geon_probe_fma_peak": (ctypes.c_int, [ctypes.c_int, c_double_p]),
}

_lib = None


def load():
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run geon_gb300.build.build() "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
