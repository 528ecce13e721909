"""The orbit-plane frame of the mixed renders (geon_gb300/csrc/orbit_frame.cuh),
compiled for the host: round trips, invariants, and the physics it relies on
(a ray of a spherically symmetric metric traced on the equator of its own
orbit frame ends where the full 8-component trace of the oracle ends)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "geon_gb300", "csrc")


@pytest.fixture(scope="module")
def frame(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("orbit") / "liborbit.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "orbit_frame_harness.cpp"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    d, f = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)
    lib.orbit_in_n.argtypes = [d, ctypes.c_long, d, f, f]
    lib.orbit_out_n.argtypes = [d, f, f, ctypes.c_long, d]

    def rin(y):
        y = np.ascontiguousarray(y, dtype=np.float64)
        n = len(y)
        yr, e1, e2 = np.empty((n, 8)), np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        lib.orbit_in_n(y.ctypes.data_as(d), n, yr.ctypes.data_as(d), e1.ctypes.data_as(f), e2.ctypes.data_as(f))
        return yr, e1, e2

    def rout(yr, e1, e2):
        yr = np.ascontiguousarray(yr, dtype=np.float64)
        y = np.empty_like(yr)
        lib.orbit_out_n(yr.ctypes.data_as(d), np.ascontiguousarray(e1).ctypes.data_as(f),
                        np.ascontiguousarray(e2).ctypes.data_as(f), len(yr), y.ctypes.data_as(d))
        return y
    return rin, rout


def random_states(n, seed):
    rng = np.random.default_rng(seed)
    y = np.zeros((n, 8))
    y[:, 0] = rng.uniform(-5, 5, n)
    y[:, 1] = rng.uniform(3, 40, n)
    y[:, 2] = rng.uniform(0.1, np.pi - 0.1, n)
    y[:, 3] = rng.uniform(-np.pi, np.pi, n)
    y[:, 4:] = rng.normal(size=(n, 4))
    return y


def test_round_trip_and_invariants(frame):
    rin, rout = frame
    y = random_states(2000, 1)
    yr, e1, e2 = rin(y)
    assert np.array_equal(yr[:, [0, 1, 4, 5]], y[:, [0, 1, 4, 5]])  # t, r and their momenta unchanged
    assert np.all(yr[:, 2] == np.pi / 2) and np.all(yr[:, 3] == 0.0) and np.all(yr[:, 6] == 0.0)
    # |w|^2 = (p^th)^2 + sin^2 th (p^ph)^2: the angular part of g(p, p) / r^2 is kept
    assert np.allclose(yr[:, 7] ** 2, y[:, 6] ** 2 + np.sin(y[:, 2]) ** 2 * y[:, 7] ** 2, rtol=1e-14)
    assert np.allclose(np.linalg.norm(e1, axis=1), 1, atol=1e-7) and np.allclose(np.linalg.norm(e2, axis=1), 1, atol=1e-7)
    assert np.abs(np.sum(e1 * e2, axis=1)).max() < 1e-7
    z = rout(yr, e1, e2)
    assert np.array_equal(z[:, [0, 1, 4, 5]], y[:, [0, 1, 4, 5]])
    assert np.abs(z[:, 2] - y[:, 2]).max() < 2e-7
    assert np.abs(np.angle(np.exp(1j * (z[:, 3] - y[:, 3])))).max() < 2e-6  # phi comes back in (-pi, pi]
    scale = np.abs(y[:, 6:8]).max(axis=1, keepdims=True) + 1e-300
    assert (np.abs(z[:, 6:8] - y[:, 6:8]) / scale).max() < 2e-6


def test_radial_ray(frame):
    rin, rout = frame
    y = np.array([[0.0, 20.0, 1.0, 0.3, 1.1, -1.0, 0.0, 0.0]])
    yr, e1, e2 = rin(y)
    assert yr[0, 7] == 0.0
    z = rout(yr, e1, e2)
    assert abs(z[0, 2] - 1.0) < 1e-7 and abs(z[0, 3] - 0.3) < 1e-7 and z[0, 6] == 0.0


def planar_schwarzschild(yr, m, h, max_steps, capture_r, escape_r):
    """FP64 RK4 of the equatorial Schwarzschild geodesic equation, per ray."""
    def rhs(s):
        t, r, ph, pt, pr, pp = s.T
        f = 1.0 - 2.0 * m / r
        gtr = m / (r * r * f)
        return np.stack([pt, pr, pp, -2.0 * gtr * pt * pr,
                         -(m * f / (r * r)) * pt * pt + gtr * pr * pr + (r - 2.0 * m) * pp * pp,
                         -2.0 / r * pr * pp], axis=1)
    s = yr[:, [0, 1, 3, 4, 5, 7]].copy()
    done = np.zeros(len(s), bool)
    term = np.zeros(len(s), int)
    for _ in range(max_steps):
        live = ~done
        if not live.any():
            break
        r = s[:, 1]
        cap, esc = live & (r < capture_r), live & (r > escape_r)
        term[cap], term[esc] = 1, 2
        done |= cap | esc
        live = ~done
        x = s[live]
        k1 = rhs(x)
        k2 = rhs(x + 0.5 * h * k1)
        k3 = rhs(x + 0.5 * h * k2)
        k4 = rhs(x + h * k3)
        s[live] = x + h / 6.0 * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)
    out = yr.copy()
    out[:, [0, 1, 3, 4, 5, 7]] = s
    return out, term


def test_planar_trace_matches_full_trace(frame, orc):
    """Camera rays of the config-1 Schwarzschild view (r 30M, fov 60): traced
    on the equator of their orbit frame and turned back, the escape directions
    agree with the oracle's 8-component trace (the two RK4 runs differ only in
    truncation error, h = 0.05). Rays whose 8-component trace runs away in the
    chart (theta -> +-1e11 near the polar axis: the coordinate singularity the
    reference shares) are the only exceptions; the orbit frame has no such
    singularity."""
    rin, rout = frame
    params = [1.0, 1.001, 100.0]
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    rc, tet = orc.camera_tetrad(1, params, obs, 0)
    y0 = orc.camera_rays(tet, obs, 60.0, 12, 12)
    term, yf, steps, resid = orc.trace(1, params, y0, 0.05, 20000, math=0)
    yr, e1, e2 = rin(y0)
    yrf, pterm = planar_schwarzschild(yr, 1.0, 0.05, 20000, 2.0 * 1.001, 100.0)
    assert np.mean(pterm == term) >= 0.97  # horizon-step accidents of the 8-component trace aside
    esc = (term == 2) & (pterm == 2)
    runaway = np.abs(yf[:, 2]) > 10.0
    assert runaway.sum() <= 4
    esc &= ~runaway
    assert esc.sum() > 100
    d_full = orc.asymptotic_direction(1, params, yf[esc], 0)
    d_plane = orc.asymptotic_direction(1, params, rout(yrf[esc], e1[esc], e2[esc]), 0)
    err = np.linalg.norm(d_full - d_plane, axis=1)
    assert np.median(err) < 1e-8 and err.max() < 1e-6


def planar_morris_thorne(yr, b0, h, n_steps):
    """FP64 RK4 of the equatorial Morris-Thorne geodesic equation, fixed steps."""
    def rhs(s):
        t, l, ph, pt, pl, pp = s.T
        return np.stack([pt, pl, pp, np.zeros_like(pt), l * pp * pp, -2.0 * l / (b0 * b0 + l * l) * pl * pp],
                        axis=1)
    s = yr[:, [0, 1, 3, 4, 5, 7]].copy()
    for _ in range(n_steps):
        k1 = rhs(s)
        k2 = rhs(s + 0.5 * h * k1)
        k3 = rhs(s + 0.5 * h * k2)
        k4 = rhs(s + h * k3)
        s = s + h / 6.0 * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)
    out = yr.copy()
    out[:, [0, 1, 3, 4, 5, 7]] = s
    return out


def test_planar_trace_matches_full_trace_morris_thorne(frame, orc):
    """Config-3 Morris-Thorne view (l 10, fov 90), 400 steps of h 0.05 (rays
    through the throat included): the final state turned back from the orbit
    frame equals the oracle's 8-component trace up to RK4 truncation."""
    rin, rout = frame
    obs = [0.0, 10.0, np.pi / 2, 0.0]
    rc, tet = orc.camera_tetrad(3, [1.0], obs, 0)
    y0 = orc.camera_rays(tet, obs, 90.0, 10, 10)
    term, yf, steps, resid = orc.trace(3, [1.0], y0, 0.05, 400, math=0)
    assert np.all(steps == 400)
    yr, e1, e2 = rin(y0)
    z = rout(planar_morris_thorne(yr, 1.0, 0.05, 400), e1, e2)
    sane = np.abs(yf[:, 2]) < 10.0
    assert sane.sum() >= 96
    # the two RK4 runs in different coordinates differ by their truncation
    # errors: ~3e-7 in l after 400 steps (2e-8 relative)
    assert np.abs(z[sane, 1] - yf[sane, 1]).max() < 1e-6 and np.abs(z[sane, 5] - yf[sane, 5]).max() < 1e-6
    assert np.abs(z[sane, 2] - yf[sane, 2]).max() < 1e-6
    assert np.abs(np.angle(np.exp(1j * (z[sane, 3] - yf[sane, 3])))).max() < 1e-6
