"""curvature.rs (Riemann -> Ricci -> R -> Einstein -> T -> T(k,k)) on the GPU, FP64."""
import numpy as np

from . import _ffi
from ._util import check, dp, f64, points


def _call(fn, metric, x, shape):
    a, single = points(x, 4)
    n = a.shape[0]
    out = np.empty((n,) + shape)
    check(getattr(_ffi.load(), fn)(metric.handle, dp(a), n, dp(out)))
    return out[0] if single else out


def riemann(metric, x):
    """R^rho_{sigma mu nu} as [rho][sigma][mu][nu] (curvature.rs:48-70)."""
    return _call("geon_riemann", metric, x, (4, 4, 4, 4))


def ricci(metric, x):
    return _call("geon_ricci", metric, x, (4, 4))


def ricci_scalar(metric, x):
    r = _call("geon_ricci_scalar", metric, x, ())
    return float(r) if np.ndim(r) == 0 else r


def einstein(metric, x):
    return _call("geon_einstein", metric, x, (4, 4))


def stress_energy(metric, x):
    return _call("geon_stress_energy", metric, x, (4, 4))


def nec_contraction(metric, x, k):
    """T_mu_nu k^mu k^nu. k: (4,) or (nk, 4) shared by all points, or (n, nk, 4)."""
    a, single = points(x, 4)
    n = a.shape[0]
    kk = np.asarray(k, dtype=np.float64)
    k_single = kk.ndim == 1
    if kk.ndim <= 2:
        kk = f64(kk.reshape(-1, 4))
        nk, shared = kk.shape[0], 1
    else:
        kk = f64(kk)
        nk, shared = kk.shape[1], 0
    out = np.empty((n, nk))
    check(_ffi.load().geon_nec_contraction(metric.handle, dp(a), n, dp(kk), nk, shared, dp(out)))
    if k_single:
        out = out[:, 0]
    return (float(out[0]) if k_single else out[0]) if single else out


def wec_contraction(metric, x, u):
    return nec_contraction(metric, x, u)


def _grid_desc(lo, hi, n, t):
    g = _ffi.GeonGrid()
    for i in range(3):
        g.lo[i] = float(lo[i])
        g.hi[i] = float(hi[i])
        g.n[i] = int(n[i])
    g.t = float(t)
    return g


def grid_into(metric, lo, hi, n, einstein, nec, k=None, t=0.0, nk=16, seed=0x5EED):
    """grid() into caller-owned host arrays (C-contiguous float64): einstein
    (N, 4, 4) or None, nec (N, nk) (None when nk is 0), k (N, nk, 4) or None.
    A caller that computes many grids reuses its arrays: host memory that a
    device copy has not written before costs the driver a first-use setup
    (about 40 ms for 512 MiB on GB300), a reused array only the copy."""
    npts = int(n[0]) * int(n[1]) * int(n[2])
    for a, shape in ((einstein, (npts, 4, 4)), (nec, (npts, nk)), (k, (npts, nk, 4))):
        if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous or a.size != int(np.prod(shape))):
            raise ValueError(f"output array must be C-contiguous float64 with {int(np.prod(shape))} elements")
    check(_ffi.load().geon_curvature_grid(metric.handle, _grid_desc(lo, hi, n, t), int(nk),
                                          int(seed) & 0xFFFFFFFFFFFFFFFF,
                                          dp(einstein) if einstein is not None else None,
                                          dp(nec) if nec is not None else None,
                                          dp(k) if k is not None else None))


def grid(metric, lo, hi, n, t=0.0, nk=16, seed=0x5EED, with_einstein=True, with_k=False):
    """Einstein tensor and T(k, k) for nk seeded null vectors per point over a
    regular grid (endpoints included). Returns (points (N, 4), einstein
    (N, 4, 4) or None, nec (N, nk), k (N, nk, 4) or None)."""
    npts = int(n[0]) * int(n[1]) * int(n[2])
    ein = np.empty((npts, 4, 4)) if with_einstein else None
    nec = np.empty((npts, nk)) if nk else None
    kk = np.empty((npts, nk, 4)) if (with_k and nk) else None
    grid_into(metric, lo, hi, n, ein, nec, kk, t=t, nk=nk, seed=seed)
    return grid_points(lo, hi, n, t), ein, nec, kk


def grid_dev(metric, lo, hi, n, einstein, nec, nk=16, seed=0x5EED, k_out=None, t=0.0, stream=0):
    """Device-pointer form of grid(): einstein (N*16 doubles, or None), nec
    (N*nk doubles) and k_out (N*nk*4 doubles, or None) are device addresses
    (ints, or objects with data_ptr()); the launch is queued on stream and not
    waited for."""
    g = _grid_desc(lo, hi, n, t)

    def ptr(a):
        if a is None:
            return None
        return a.data_ptr() if hasattr(a, "data_ptr") else int(a)
    check(_ffi.load().geon_curvature_grid_dev(metric.handle, g, int(nk), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                              ptr(einstein), ptr(nec), ptr(k_out), int(stream)))


def grid_points(lo, hi, n, t=0.0):
    """The points of a grid job, in its index order (x fastest)."""
    axes = []
    for i in range(3):
        if int(n[i]) > 1:
            step = (float(hi[i]) - float(lo[i])) / float(int(n[i]) - 1)
            axes.append(float(lo[i]) + np.arange(int(n[i]), dtype=np.float64) * step)
        else:
            axes.append(np.array([float(lo[i])]))
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    pts = np.stack([np.full(x.size, float(t)), x.ravel(), y.ravel(), z.ravel()], axis=1)
    return pts
