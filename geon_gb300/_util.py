"""Shared helpers: numpy <-> ctypes, status -> exception."""

import numpy as np

from . import _ffi


class GeonError(RuntimeError):
    """A failed library call. `status` is the GEON_ERR_* code."""

    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


# Messages of the reference's panics, for statuses that replace them.
PANICS = {
    _ffi.GEON_ERR_SINGULAR_METRIC: "metric became singular — coordinate chart broke down",
    _ffi.GEON_ERR_NOT_TIMELIKE: "observer is not in a timelike region (g_tt >= 0)",
    _ffi.GEON_ERR_GRAM_SCHMIDT: "Gram–Schmidt produced non-spacelike vector — chart broken at this point",
}


def check(rc):
    if rc != _ffi.GEON_OK:
        lib = _ffi.load()
        msg = lib.geon_last_error().decode(errors="replace")
        raise GeonError(rc, PANICS.get(rc, msg) if rc in PANICS else msg)


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def dp(a):
    return a.ctypes.data_as(_ffi.c_double_p)


def fp(a):
    return a.ctypes.data_as(_ffi.c_float_p)


def i32p(a):
    return a.ctypes.data_as(_ffi.c_int32_p)


def i64p(a):
    return a.ctypes.data_as(_ffi.c_int64_p)


def points(x, width):
    """Accept one point or a batch; return (contiguous (n, width) array, was_single)."""
    a = np.asarray(x, dtype=np.float64)
    single = a.ndim == 1
    return f64(a.reshape(-1, width)), single
