"""geodesic::trace (geodesic.rs:62-117) over batches of rays on the GPU."""
from dataclasses import dataclass

import numpy as np

from . import _ffi
from ._util import check, dp, i32p, i64p, points

FP64, MIXED, ADAPTIVE, FP64_FAST = 0, 1, 2, 3
PRECISION = {"fp64": FP64, "mixed": MIXED, "adaptive": ADAPTIVE, "fp64fast": FP64_FAST,
             FP64: FP64, MIXED: MIXED, ADAPTIVE: ADAPTIVE, FP64_FAST: FP64_FAST}


def set_adaptive_tolerance(rtol, atol):
    """Error tolerances of precision="adaptive" (FP64 Dormand-Prince 5(4))."""
    check(_ffi.load().geon_set_adaptive_tolerance(float(rtol), float(atol)))


def adaptive_tolerance():
    r, a = _ffi.ctypes.c_double(), _ffi.ctypes.c_double()
    _ffi.load().geon_get_adaptive_tolerance(_ffi.ctypes.byref(r), _ffi.ctypes.byref(a))
    return r.value, a.value


@dataclass
class TraceResult:
    """TraceResult (geodesic.rs:18-25), one entry per ray."""
    termination: np.ndarray  # int32: 0 Diverged, 1 Captured, 2 Escaped
    final_state: np.ndarray  # (n, 8)
    steps_taken: np.ndarray  # int64
    null_residual: np.ndarray


def trace(metric, y0, step, max_steps, precision="fp64"):
    """Integrate every ray of y0 ((8,) or (n, 8)) until termination."""
    a, single = points(y0, 8)
    n = a.shape[0]
    term = np.empty(n, dtype=np.int32)
    yf = np.empty((n, 8))
    steps = np.empty(n, dtype=np.int64)
    resid = np.empty(n)
    lib = _ffi.load()
    check(lib.geon_trace(metric.handle, dp(a), n, float(step), int(max_steps), PRECISION[precision],
                         i32p(term), dp(yf), i64p(steps), dp(resid)))
    if single:
        return TraceResult(int(term[0]), yf[0], int(steps[0]), float(resid[0]))
    return TraceResult(term, yf, steps, resid)


def trace_dev(metric, n, y0, step, max_steps, term, final_state, steps, resid, stream=0,
              precision="fp64"):
    """Stream-ordered variant on device memory: y0, term, final_state, steps and
    resid are CUDA device addresses (ints, e.g. torch's tensor.data_ptr()),
    stream a cudaStream_t handle (0 = legacy default stream)."""
    lib = _ffi.load()
    check(lib.geon_trace_dev(metric.handle, y0, int(n), float(step), int(max_steps),
                             PRECISION[precision], term, final_state, steps, resid, stream))


def pos(y):
    return np.asarray(y)[..., :4]


def mom(y):
    return np.asarray(y)[..., 4:]
