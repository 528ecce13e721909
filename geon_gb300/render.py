"""render::render (render.rs:55-166) on the GPU, plus the host PNG writer."""
import struct
import zlib
from dataclasses import dataclass

import numpy as np

from . import _ffi
from ._util import check, fp, i32p, i64p
from .geodesic import PRECISION


@dataclass
class RenderConfig:
    """RenderConfig (render.rs:17-43) with the sky flag (None = global) and precision."""
    step: float = 0.05
    max_steps: int = 20000
    captured_rgb: tuple = (0.0, 0.0, 0.0)
    diverged_rgb: tuple = (1.0, 0.0, 1.0)
    samples_per_axis: int = 1
    show_stars: object = None
    precision: str = "fp64"

    def c_struct(self):
        c = _ffi.GeonRenderConfig()
        c.step = float(self.step)
        c.max_steps = int(self.max_steps)
        for i in range(3):
            c.captured_rgb[i] = float(self.captured_rgb[i])
            c.diverged_rgb[i] = float(self.diverged_rgb[i])
        c.samples_per_axis = int(self.samples_per_axis)
        c.show_stars = -1 if self.show_stars is None else int(bool(self.show_stars))
        c.precision = PRECISION[self.precision]
        return c


@dataclass
class RenderStats:
    """RenderStats (render.rs:45-53) plus the total ray-step count."""
    captured: int = 0
    escaped: int = 0
    diverged: int = 0
    max_null_residual: float = 0.0
    avg_steps: float = 0.0
    total_steps: int = 0


def render(metric, camera, cfg=None, with_classes=False):
    """Returns (pixels (height, width, 3) float32, RenderStats) [+ (class, steps) maps]."""
    cfg = cfg or RenderConfig()
    rgb = np.empty((camera.height, camera.width, 3), dtype=np.float32)
    cls = np.empty((camera.height, camera.width), dtype=np.int32)
    pst = np.empty((camera.height, camera.width), dtype=np.int64)
    st = _ffi.GeonRenderStats()
    lib = _ffi.load()
    check(lib.geon_render_ex(metric.handle, camera.c_struct(), cfg.c_struct(), fp(rgb), st,
                             i32p(cls), i64p(pst)))
    stats = RenderStats(st.captured, st.escaped, st.diverged, st.max_null_residual, st.avg_steps,
                        st.total_steps)
    if with_classes:
        return rgb, stats, cls, pst
    return rgb, stats


def render_batch(items):
    """Several renders traced by one persistent kernel launch (geon_render_batch):
    items is a list of (metric, camera, cfg); every cfg has the same precision.
    Returns a list of (pixels, RenderStats, class map, steps map), each equal to
    render(metric, camera, cfg, with_classes=True) of that item alone."""
    n = len(items)
    arr = (_ffi.GeonRenderItem * n)()
    outs = []
    for j, (metric, camera, cfg) in enumerate(items):
        cfg = cfg or RenderConfig()
        rgb = np.empty((camera.height, camera.width, 3), dtype=np.float32)
        cls = np.empty((camera.height, camera.width), dtype=np.int32)
        pst = np.empty((camera.height, camera.width), dtype=np.int64)
        st = _ffi.GeonRenderStats()
        arr[j].metric = metric.handle.value
        arr[j].camera = camera.c_struct()
        arr[j].render = cfg.c_struct()
        arr[j].rgb = rgb.ctypes.data
        arr[j].stats = _ffi.ctypes.pointer(st)
        arr[j].pixel_class = cls.ctypes.data
        arr[j].pixel_steps = pst.ctypes.data
        outs.append((rgb, st, cls, pst))
    check(_ffi.load().geon_render_batch(arr, n))
    return [(rgb, RenderStats(st.captured, st.escaped, st.diverged, st.max_null_residual, st.avg_steps,
                              st.total_steps), cls, pst) for rgb, st, cls, pst in outs]


def render_u8(metric, camera, cfg=None, with_float=False):
    """render() followed by write_png's tonemap on the GPU: (height, width, 3)
    uint8, the bytes write_png encodes [+ the float image], and RenderStats."""
    cfg = cfg or RenderConfig()
    rgb8 = np.empty((camera.height, camera.width, 3), dtype=np.uint8)
    rgb = np.empty((camera.height, camera.width, 3), dtype=np.float32) if with_float else None
    st = _ffi.GeonRenderStats()
    check(_ffi.load().geon_render_u8(metric.handle, camera.c_struct(), cfg.c_struct(), rgb8.ctypes.data,
                                     rgb.ctypes.data if rgb is not None else None, st))
    stats = RenderStats(st.captured, st.escaped, st.diverged, st.max_null_residual, st.avg_steps,
                        st.total_steps)
    return (rgb8, rgb, stats) if with_float else (rgb8, stats)


def tonemap(pixels):
    """write_png's tonemap (render.rs:169-183) on the GPU: clamp, ^(1/2.2), *255, round to u8."""
    a = np.ascontiguousarray(pixels, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint8)
    check(_ffi.load().geon_tonemap_u8(a.ctypes.data, a.size, out.ctypes.data))
    return out


def write_png(path, pixels, width, height):
    """Write an RGB PNG (host side, like the reference's image crate call). pixels:
    the float image (tonemapped on the GPU) or the uint8 bytes of render_u8."""
    px = np.asarray(pixels)
    img = (px if px.dtype == np.uint8 else tonemap(px)).reshape(height, width, 3)
    raw = b"".join(b"\x00" + img[j].tobytes() for j in range(height))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", width, height, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)
