"""Metric handles: the reference's `trait Metric` (metric/mod.rs:19-109) and its
four implementations, evaluated on the GPU in FP64.

Each method takes one point (shape (4,)) or a batch (shape (n, 4)) and returns
the reference's array for each point; a batch is one device launch.
"""
import ctypes

import numpy as np

from . import _ffi
from ._util import check, dp, f64, i32p, points

MINKOWSKI, SCHWARZSCHILD, ALCUBIERRE, MORRIS_THORNE, FIELD = 0, 1, 2, 3, 4
CARTESIAN, SPHERICAL = 0, 1
DIVERGED, CAPTURED, ESCAPED = 0, 1, 2
TERMINATION = {DIVERGED: "Diverged", CAPTURED: "Captured", ESCAPED: "Escaped", -1: None}


class Metric:
    """A device metric functor (immutable after creation)."""

    kind = None

    def __init__(self, params=()):
        lib = _ffi.load()
        p = f64(list(params) if len(params) else [0.0])
        h = ctypes.c_void_p()
        check(lib.geon_metric_create(self.kind, dp(p), len(params), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.params = tuple(float(v) for v in params)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.geon_metric_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def name(self):
        return self._lib.geon_metric_name(self._h).decode()

    def _pw(self, fn, x, in_w, out_shape):
        a, single = points(x, in_w)
        n = a.shape[0]
        out = np.empty((n,) + out_shape)
        check(getattr(self._lib, fn)(self._h, dp(a), n, dp(out)))
        return out[0] if single else out

    def g(self, x):
        return self._pw("geon_metric_g", x, 4, (4, 4))

    def dg(self, x):
        return self._pw("geon_metric_dg", x, 4, (4, 4, 4))

    def g_inv(self, x):
        return self._pw("geon_metric_g_inv", x, 4, (4, 4))

    def christoffel(self, x):
        return self._pw("geon_metric_christoffel", x, 4, (4, 4, 4))

    def fd_step(self, x=None):
        return np.full(4, 1e-5)

    def terminate(self, x):
        a, single = points(x, 4)
        out = np.empty(a.shape[0], dtype=np.int32)
        check(self._lib.geon_metric_terminate(self._h, dp(a), a.shape[0], i32p(out)))
        return int(out[0]) if single else out

    def asymptotic_direction(self, x, p=None):
        """(x, p) for one ray, or an (n, 8) array of States."""
        if p is not None:
            s = np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 4),
                                np.asarray(p, dtype=np.float64).reshape(-1, 4)], axis=1)
            single = np.asarray(x).ndim == 1
        else:
            s, single = points(x, 8)
        out = np.empty((s.shape[0], 3))
        check(self._lib.geon_metric_asymptotic_direction(self._h, dp(f64(s)), s.shape[0], dp(out)))
        return out[0] if single else out


class Minkowski(Metric):
    """metric/minkowski.rs"""
    kind = MINKOWSKI

    def __init__(self):
        super().__init__(())


class Schwarzschild(Metric):
    """metric/schwarzschild.rs; Schwarzschild::new(mass) defaults (pad 1.001, escape 1000)."""
    kind = SCHWARZSCHILD

    def __init__(self, mass=1.0, horizon_pad=1.001, escape_radius=1000.0):
        super().__init__((mass, horizon_pad, escape_radius))
        self.mass, self.horizon_pad, self.escape_radius = self.params

    @classmethod
    def new(cls, mass):
        return cls(mass)


class Alcubierre(Metric):
    """metric/alcubierre.rs; Alcubierre::default() is (R=2, s=0.5, v=2, ship_x=0)."""
    kind = ALCUBIERRE

    def __init__(self, bubble_radius=2.0, bubble_thickness=0.5, ship_velocity=2.0, ship_x=0.0):
        super().__init__((bubble_radius, bubble_thickness, ship_velocity, ship_x))
        self.bubble_radius, self.bubble_thickness, self.ship_velocity, self.ship_x = self.params


class MorrisThorne(Metric):
    """metric/morris_thorne.rs; MorrisThorne::default() has throat_radius 1."""
    kind = MORRIS_THORNE

    def __init__(self, throat_radius=1.0):
        super().__init__((throat_radius,))
        self.throat_radius = self.params[0]


class FieldMetric(Metric):
    """A sampled (tensor-field) metric, geon_metric_create_field: the 10 unique
    components of a static g at the nodes of a regular grid over (x1, x2, x3),
    the control points of a uniform cubic B-spline (C2, so its curvature is
    meaningful). samples: (n0*n1*n2, 10) or (n2, n1, n0, 10), x fastest, in the
    order g00 g01 g02 g03 g11 g12 g13 g22 g23 g33. chart: CARTESIAN or SPHERICAL
    (how escape directions read the coordinates)."""
    kind = FIELD
    COMPONENTS = ((0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3))

    def __init__(self, lo, hi, n, samples, chart=CARTESIAN):
        lib = _ffi.load()
        grid = _ffi.GeonGrid()
        for a in range(3):
            grid.lo[a] = float(lo[a])
            grid.hi[a] = float(hi[a])
            grid.n[a] = int(n[a])
        nodes = int(n[0]) * int(n[1]) * int(n[2])
        s = f64(np.asarray(samples, dtype=np.float64).reshape(nodes, 10))
        h = ctypes.c_void_p()
        check(lib.geon_metric_create_field(grid, dp(s), int(chart), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.params = ()
        self.lo, self.hi, self.n, self.chart = tuple(lo), tuple(hi), tuple(int(v) for v in n), int(chart)
        self.samples = s

    @staticmethod
    def nodes(lo, hi, n, t=0.0):
        """The node positions (n0*n1*n2, 4), x fastest."""
        axes = [np.linspace(float(lo[a]), float(hi[a]), int(n[a])) if int(n[a]) > 1 else np.array([float(lo[a])])
                for a in range(3)]
        z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        return np.stack([np.full(x.size, float(t)), x.ravel(), y.ravel(), z.ravel()], axis=1)

    @classmethod
    def sample(cls, metric, lo, hi, n, chart=CARTESIAN, t=0.0):
        """Sample another metric's g at the grid nodes (on the GPU)."""
        g = metric.g(cls.nodes(lo, hi, n, t)).reshape(-1, 4, 4)
        comps = np.stack([g[:, i, j] for i, j in cls.COMPONENTS], axis=1)
        return cls(lo, hi, n, comps, chart)


def from_kind(kind, params=()):
    cls = {MINKOWSKI: Minkowski, SCHWARZSCHILD: Schwarzschild, ALCUBIERRE: Alcubierre,
           MORRIS_THORNE: MorrisThorne}[kind]
    return cls(*params)
