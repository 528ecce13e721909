"""sky::sample (sky.rs:107-120) and the SHOW_STARS flag (sky.rs:23)."""
import numpy as np

from . import _ffi
from ._util import check, dp, fp, points


def sample(dir_cart, show_stars=None):
    a, single = points(dir_cart, 3)
    out = np.empty((a.shape[0], 3), dtype=np.float32)
    flag = get_show_stars() if show_stars is None else int(bool(show_stars))
    check(_ffi.load().geon_sky_sample(dp(a), a.shape[0], flag, fp(out)))
    return out[0] if single else out


def set_show_stars(on):
    _ffi.load().geon_set_show_stars(int(bool(on)))


def get_show_stars():
    return bool(_ffi.load().geon_get_show_stars())
