"""Shadow validation (bin/validate_shadow.rs): equatorial rays, capture test and
batched bisection of the critical launch angle, on the GPU."""
import numpy as np

from . import _ffi
from ._util import check, dp, f64, i32p, i64p
from .geodesic import PRECISION, TraceResult
from .metric import CAPTURED


def equatorial_ray(metric, r_obs, alpha):
    a = f64(np.atleast_1d(alpha))
    out = np.empty((a.size, 8))
    check(_ffi.load().geon_equatorial_rays(metric.handle, float(r_obs), dp(a), a.size, dp(out)))
    return out[0] if np.ndim(alpha) == 0 else out


def classify(metric, r_obs, alpha, step=0.01, max_steps=200000, precision="fp64"):
    """Termination of the equatorial ray at each launch angle, and its steps."""
    a = f64(np.atleast_1d(alpha))
    term = np.empty(a.size, dtype=np.int32)
    steps = np.empty(a.size, dtype=np.int64)
    check(_ffi.load().geon_shadow_classify(metric.handle, float(r_obs), dp(a), a.size, float(step),
                                           int(max_steps), PRECISION[precision], i32p(term), i64p(steps)))
    return term, steps


def trace(metric, r_obs, alpha, step=0.01, max_steps=200000, precision="fp64"):
    """geodesic::trace of the equatorial ray at each launch angle, with the
    stepper classify() uses for them; a TraceResult per ray."""
    a = f64(np.atleast_1d(alpha))
    n = a.size
    term = np.empty(n, dtype=np.int32)
    yf = np.empty((n, 8))
    steps = np.empty(n, dtype=np.int64)
    resid = np.empty(n)
    check(_ffi.load().geon_shadow_trace(metric.handle, float(r_obs), dp(a), n, float(step), int(max_steps),
                                        PRECISION[precision], i32p(term), dp(yf), i64p(steps), dp(resid)))
    return TraceResult(term, yf, steps, resid)


def is_captured(metric, r_obs, alpha, step=0.01, max_steps=200000, precision="fp64"):
    term, _ = classify(metric, r_obs, alpha, step, max_steps, precision)
    return term[0] == CAPTURED if np.ndim(alpha) == 0 else term == CAPTURED


def bisect(metric, r_obs, lo, hi, iters=60, step=0.01, max_steps=200000, precision="fp64"):
    """Independent bisections (bin/validate_shadow.rs:70-79) of every [lo, hi].
    Returns (alpha_c, lo, hi, steps) arrays."""
    lo = f64(np.atleast_1d(lo))
    hi = f64(np.atleast_1d(hi))
    nb = lo.size
    ac, lo_o, hi_o = np.empty(nb), np.empty(nb), np.empty(nb)
    st = np.empty(nb, dtype=np.int64)
    check(_ffi.load().geon_shadow_bisect(metric.handle, float(r_obs), dp(lo), dp(hi), nb, int(iters),
                                         float(step), int(max_steps), PRECISION[precision], dp(ac),
                                         dp(lo_o), dp(hi_o), i64p(st)))
    return ac, lo_o, hi_o, st


def impact_parameter(metric, r_obs, alpha):
    """b = r_obs sin(alpha) / sqrt(1 - 2M/r_obs) (bin/validate_shadow.rs:78-79)."""
    f = 1.0 - 2.0 * metric.mass / r_obs
    return r_obs * np.sin(alpha) / np.sqrt(f)
