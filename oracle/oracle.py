"""ctypes front end of the CPU FP64 oracle (test infrastructure only).

The oracle restates the geon reference (Rust) path in C++; see geon_oracle.h.
Only tests/, the smoke check and bench.py's CPU-baseline leg use this module,
and only as the checker, never as the thing measured or shipped.
"""
import ctypes

import numpy as np

from . import build as _build

LIBM = 0
GEON = 1
NUDGE = 2
KINDS = {"minkowski": 0, "schwarzschild": 1, "alcubierre": 2, "morris_thorne": 3}

_lib = None


class RenderStats(ctypes.Structure):
    _fields_ = [("captured", ctypes.c_int64), ("escaped", ctypes.c_int64),
                ("diverged", ctypes.c_int64), ("max_null_residual", ctypes.c_double),
                ("avg_steps", ctypes.c_double), ("total_steps", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _params(params):
    p = np.zeros(4, dtype=np.float64)
    p[: len(params)] = params
    return p


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def hardware_threads():
    return lib().orc_hardware_threads()


def geon_sincos(x):
    x, xp = _d(x)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().orc_geon_sincos(xp, ctypes.c_int64(x.size), _p(s, ctypes.c_double), _p(c, ctypes.c_double))
    return s, c


def geon_tanh(x):
    x, xp = _d(x)
    o = np.empty_like(x)
    lib().orc_geon_tanh(xp, ctypes.c_int64(x.size), _p(o, ctypes.c_double))
    return o


def geon_expm1(x):
    x, xp = _d(x)
    o = np.empty_like(x)
    lib().orc_geon_expm1(xp, ctypes.c_int64(x.size), _p(o, ctypes.c_double))
    return o


def inv4(m):
    m, mp = _d(m)
    o = np.empty(16)
    ok = lib().orc_inv4(mp, _p(o, ctypes.c_double))
    return o.reshape(4, 4) if ok else None


def _pointwise(fn, kind, params, math, x, width, name):
    x, xp = _d(np.asarray(x, dtype=np.float64).reshape(-1, 4))
    n = x.shape[0]
    out = np.empty((n, width))
    p, pp = _d(_params(params))
    rc = getattr(lib(), fn)(ctypes.c_int(kind), pp, ctypes.c_int(math), xp, ctypes.c_int64(n),
                            _p(out, ctypes.c_double))
    _check(rc, name)
    return out


def metric_g(kind, params, x, math=LIBM):
    return _pointwise("orc_metric_g", kind, params, math, x, 16, "g").reshape(-1, 4, 4)


def metric_dg(kind, params, x, math=LIBM):
    return _pointwise("orc_metric_dg", kind, params, math, x, 64, "dg").reshape(-1, 4, 4, 4)


def metric_g_inv(kind, params, x, math=LIBM):
    return _pointwise("orc_metric_g_inv", kind, params, math, x, 16, "g_inv").reshape(-1, 4, 4)


def metric_christoffel(kind, params, x, math=LIBM):
    return _pointwise("orc_metric_christoffel", kind, params, math, x, 64, "christoffel").reshape(-1, 4, 4, 4)


def metric_terminate(kind, params, x, math=LIBM):
    x, xp = _d(np.asarray(x, dtype=np.float64).reshape(-1, 4))
    out = np.empty(x.shape[0], dtype=np.int32)
    p, pp = _d(_params(params))
    lib().orc_metric_terminate(kind, pp, math, xp, ctypes.c_int64(x.shape[0]), _p(out, ctypes.c_int32))
    return out


def asymptotic_direction(kind, params, states, math=LIBM):
    s, sp = _d(np.asarray(states, dtype=np.float64).reshape(-1, 8))
    out = np.empty((s.shape[0], 3))
    p, pp = _d(_params(params))
    lib().orc_asymptotic_direction(kind, pp, math, sp, ctypes.c_int64(s.shape[0]), _p(out, ctypes.c_double))
    return out


def trace(kind, params, y0, step, max_steps, math=LIBM, nthreads=0):
    y0, yp = _d(np.asarray(y0, dtype=np.float64).reshape(-1, 8))
    n = y0.shape[0]
    term = np.empty(n, dtype=np.int32)
    yf = np.empty((n, 8))
    steps = np.empty(n, dtype=np.int64)
    resid = np.empty(n)
    p, pp = _d(_params(params))
    rc = lib().orc_trace(kind, pp, math, yp, ctypes.c_int64(n), ctypes.c_double(step),
                         ctypes.c_int64(max_steps), ctypes.c_int(nthreads), _p(term, ctypes.c_int32),
                         _p(yf, ctypes.c_double), _p(steps, ctypes.c_int64), _p(resid, ctypes.c_double))
    _check(rc, "trace")
    return term, yf, steps, resid


def field_set(lo, hi, n, samples, chart=0):
    """Register the sampled metric used as kind 4 (the GPU's GEON_FIELD)."""
    lo_, lp = _d(np.asarray(lo, dtype=np.float64))
    hi_, hp = _d(np.asarray(hi, dtype=np.float64))
    n_ = np.ascontiguousarray(np.asarray(n, dtype=np.int64))
    s_, sp = _d(np.asarray(samples, dtype=np.float64).reshape(-1, 10))
    rc = lib().orc_field_set(lp, hp, _p(n_, ctypes.c_int64), ctypes.c_int(chart), sp)
    _check(rc, "field_set")


def trace_adaptive(kind, params, y0, h0, max_steps, rtol=1e-10, atol=1e-12, math=LIBM, nthreads=0):
    """The GPU's adaptive (Dormand-Prince 5(4)) trace, restated."""
    y0, yp = _d(np.asarray(y0, dtype=np.float64).reshape(-1, 8))
    n = y0.shape[0]
    term = np.empty(n, dtype=np.int32)
    yf = np.empty((n, 8))
    steps = np.empty(n, dtype=np.int64)
    resid = np.empty(n)
    p, pp = _d(_params(params))
    rc = lib().orc_trace_adaptive(kind, pp, math, yp, ctypes.c_int64(n), ctypes.c_double(h0),
                                  ctypes.c_int64(max_steps), ctypes.c_double(rtol), ctypes.c_double(atol),
                                  ctypes.c_int(nthreads), _p(term, ctypes.c_int32), _p(yf, ctypes.c_double),
                                  _p(steps, ctypes.c_int64), _p(resid, ctypes.c_double))
    _check(rc, "trace_adaptive")
    return term, yf, steps, resid


def camera_tetrad(kind, params, observer, math=LIBM):
    o, op = _d(observer)
    out = np.empty(16)
    p, pp = _d(_params(params))
    rc = lib().orc_camera_tetrad(kind, pp, math, op, _p(out, ctypes.c_double))
    return rc, out.reshape(4, 4)


def camera_rays(tetrad, observer, fov_y_deg, width, height, row0=0, nrows=None, du=0.5, dv=0.5,
                forward_sign=1):
    nrows = height if nrows is None else nrows
    t, tp = _d(np.asarray(tetrad).reshape(16))
    o, op = _d(observer)
    out = np.empty((nrows * width, 8))
    lib().orc_camera_rays(tp, op, ctypes.c_double(fov_y_deg), ctypes.c_int64(width),
                          ctypes.c_int64(height), ctypes.c_int64(row0), ctypes.c_int64(nrows),
                          ctypes.c_double(du), ctypes.c_double(dv), ctypes.c_int(forward_sign),
                          _p(out, ctypes.c_double))
    return out


def sky_sample(dirs, show_stars=True):
    d, dp = _d(np.asarray(dirs, dtype=np.float64).reshape(-1, 3))
    out = np.empty((d.shape[0], 3), dtype=np.float32)
    lib().orc_sky_sample(dp, ctypes.c_int64(d.shape[0]), ctypes.c_int(int(show_stars)),
                         _p(out, ctypes.c_float))
    return out


def render(kind, params, observer, fov_y_deg, width, height, step=0.05, max_steps=20000,
           samples_per_axis=1, show_stars=True, forward_sign=1, row0=0, nrows=None, math=LIBM,
           nthreads=0):
    nrows = height if nrows is None else nrows
    o, op = _d(observer)
    rgb = np.empty((nrows, width, 3), dtype=np.float32)
    cls = np.empty((nrows, width), dtype=np.int32)
    pst = np.empty((nrows, width), dtype=np.int64)
    st = RenderStats()
    p, pp = _d(_params(params))
    rc = lib().orc_render(kind, pp, math, op, ctypes.c_double(fov_y_deg), ctypes.c_int64(width),
                          ctypes.c_int64(height), ctypes.c_int64(row0), ctypes.c_int64(nrows),
                          ctypes.c_double(step), ctypes.c_int64(max_steps),
                          ctypes.c_int64(samples_per_axis), ctypes.c_int(int(show_stars)),
                          ctypes.c_int(forward_sign), ctypes.c_int(nthreads),
                          _p(rgb, ctypes.c_float), _p(cls, ctypes.c_int32), _p(pst, ctypes.c_int64),
                          ctypes.byref(st))
    _check(rc, "render")
    return rgb, cls, pst, st.as_dict()


def tonemap_u8(rgb):
    """write_png's tonemap (render.rs:174-178) with libm powf."""
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint8)
    lib().orc_tonemap_u8(_p(a, ctypes.c_float), ctypes.c_int64(a.size), _p(out, ctypes.c_uint8))
    return out


WHAT = {"riemann": (0, 256), "ricci": (1, 16), "ricci_scalar": (2, 1), "einstein": (3, 16),
        "stress_energy": (4, 16)}


def curvature(kind, params, x, what, math=LIBM, faithful=False, nthreads=0):
    code, width = WHAT[what]
    x, xp = _d(np.asarray(x, dtype=np.float64).reshape(-1, 4))
    n = x.shape[0]
    out = np.empty((n, width))
    p, pp = _d(_params(params))
    rc = lib().orc_curvature(kind, pp, math, xp, ctypes.c_int64(n), ctypes.c_int(code),
                             ctypes.c_int(int(faithful)), ctypes.c_int(nthreads), _p(out, ctypes.c_double))
    _check(rc, what)
    shape = {256: (n, 4, 4, 4, 4), 16: (n, 4, 4), 1: (n,)}[width]
    return out.reshape(shape)


def nec(kind, params, x, k, math=LIBM, faithful=False, nthreads=0):
    """k: (nk, 4) shared by every point, or (n, nk, 4) per point. Returns (n, nk)."""
    x, xp = _d(np.asarray(x, dtype=np.float64).reshape(-1, 4))
    n = x.shape[0]
    k = np.asarray(k, dtype=np.float64)
    shared = k.ndim == 2
    nk = k.shape[0] if shared else k.shape[1]
    k, kp = _d(k)
    out = np.empty((n, nk))
    p, pp = _d(_params(params))
    rc = lib().orc_nec(kind, pp, math, xp, ctypes.c_int64(n), kp, ctypes.c_int64(nk),
                       ctypes.c_int(int(shared)), ctypes.c_int(int(faithful)), ctypes.c_int(nthreads),
                       _p(out, ctypes.c_double))
    _check(rc, "nec")
    return out


def equatorial_ray(mass, r_obs, alpha, math=LIBM):
    a, ap = _d(np.atleast_1d(alpha))
    out = np.empty((a.size, 8))
    lib().orc_equatorial_ray(ctypes.c_double(mass), ctypes.c_double(r_obs), ctypes.c_int(math), ap,
                             ctypes.c_int64(a.size), _p(out, ctypes.c_double))
    return out


def shadow_classify(schw_params, r_obs, alpha, step, max_steps, math=LIBM, nthreads=0):
    a, ap = _d(np.atleast_1d(alpha))
    term = np.empty(a.size, dtype=np.int32)
    steps = np.empty(a.size, dtype=np.int64)
    p, pp = _d(_params(schw_params))
    lib().orc_shadow_classify(pp, ctypes.c_double(r_obs), ctypes.c_int(math), ap, ctypes.c_int64(a.size),
                              ctypes.c_double(step), ctypes.c_int64(max_steps), ctypes.c_int(nthreads),
                              _p(term, ctypes.c_int32), _p(steps, ctypes.c_int64))
    return term, steps


def shadow_bisect(schw_params, r_obs, lo, hi, iters, step, max_steps, math=LIBM, nthreads=0):
    lo, lop = _d(np.atleast_1d(lo))
    hi, hip = _d(np.atleast_1d(hi))
    nb = lo.size
    ac = np.empty(nb)
    lo_o = np.empty(nb)
    hi_o = np.empty(nb)
    st = np.empty(nb, dtype=np.int64)
    p, pp = _d(_params(schw_params))
    lib().orc_shadow_bisect(pp, ctypes.c_double(r_obs), ctypes.c_int(math), lop, hip, ctypes.c_int64(nb),
                            ctypes.c_int(iters), ctypes.c_double(step), ctypes.c_int64(max_steps),
                            ctypes.c_int(nthreads), _p(ac, ctypes.c_double), _p(lo_o, ctypes.c_double),
                            _p(hi_o, ctypes.c_double), _p(st, ctypes.c_int64))
    return ac, lo_o, hi_o, st


def energy_conditions(math=LIBM):
    out = np.empty(128)
    n = lib().orc_energy_conditions(ctypes.c_int(math), _p(out, ctypes.c_double))
    return out[:n]
