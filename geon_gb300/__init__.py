"""geon_gb300: GB300-native geodesic ray tracing and curvature.

A drop-in for the hot path of the geon crate: the Metric functors (g, dg, g^-1,
Christoffel with the finite-difference fallbacks), the Camera tetrad, render()
with its RK4 null-geodesic trace, the shadow bisection and the curvature.rs
chain. The compute runs in hand-written sm_103a CUDA behind the C ABI of
include/geon_gpu.h; this package is the Python host side of that ABI. There is
no CPU fallback: without the built library every call raises.
"""
from . import accuracy, autotune, curvature, energy, shadow, sky
from ._ffi import load as _load
from ._util import GeonError
from .camera import Camera
from .geodesic import (ADAPTIVE, FP64, FP64_FAST, MIXED, TraceResult, adaptive_tolerance, mom, pos, set_adaptive_tolerance,
                       trace, trace_dev)
from .metric import (ALCUBIERRE, CAPTURED, CARTESIAN, DIVERGED, ESCAPED, FIELD, MINKOWSKI, MORRIS_THORNE,
                     SCHWARZSCHILD, SPHERICAL, Alcubierre, FieldMetric, Metric, Minkowski, MorrisThorne,
                     Schwarzschild, from_kind)
from .render import RenderConfig, RenderStats, render, render_batch, render_u8, tonemap, write_png
from .serve import Job, Server


def version():
    return _load().geon_version().decode()


def library_path():
    from ._ffi import LIB_PATH
    return LIB_PATH
