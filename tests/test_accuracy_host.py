"""Host logic of the FP64 arbiter (geon_gb300.accuracy): the orbit-plane frame
of a state is an exact rotation (the invariants of a spherically symmetric
metric are kept), and clean_escapes keeps only rays that ended at the escape
radius on the null cone."""
import types

import numpy as np

from geon_gb300 import accuracy


def _schwarzschild_invariants(y, m=1.0):
    r, th = y[:, 1], y[:, 2]
    f = 1.0 - 2.0 * m / r
    ang = y[:, 6] ** 2 + (np.sin(th) * y[:, 7]) ** 2  # (p^theta)^2 + sin^2 (p^phi)^2
    gpp = -f * y[:, 4] ** 2 + y[:, 5] ** 2 / f + r * r * ang
    return gpp, r ** 4 * ang  # g(p, p) and L^2


def test_orbit_frame_states_is_a_rotation():
    rng = np.random.default_rng(11)
    n = 2000
    y = np.stack([rng.uniform(0, 5, n), rng.uniform(3, 50, n), rng.uniform(0.05, np.pi - 0.05, n),
                  rng.uniform(-np.pi, np.pi, n), rng.uniform(0.5, 2, n), rng.uniform(-1, 1, n),
                  rng.uniform(-0.05, 0.05, n), rng.uniform(-0.05, 0.05, n)], axis=1)
    out = accuracy.orbit_frame_states(y)
    assert np.all(out[:, 2] == np.pi / 2) and np.all(out[:, 3] == 0.0) and np.all(out[:, 6] == 0.0)
    assert np.array_equal(out[:, [0, 1, 4, 5]], y[:, [0, 1, 4, 5]])
    assert np.all(out[:, 7] >= 0.0)
    g0, l0 = _schwarzschild_invariants(y)
    g1, l1 = _schwarzschild_invariants(out)
    assert np.allclose(l1, l0, rtol=1e-12, atol=0.0)
    assert np.allclose(g1, g0, rtol=1e-12, atol=1e-12)


def test_orbit_frame_states_radial_ray():
    y = np.array([[0.0, 20.0, 1.0, 0.3, 1.0, -0.9, 0.0, 0.0]])
    out = accuracy.orbit_frame_states(y)
    assert out[0, 7] == 0.0 and out[0, 2] == np.pi / 2


def test_clean_escapes():
    m = types.SimpleNamespace(kind=1, escape_radius=100.0, mass=1.0)  # Schwarzschild
    fs = np.zeros((5, 8))
    fs[:, 1] = [100.5, 100.5, 1e30, 100.5, 150.0]
    fs[:, 4] = 1.0
    res = types.SimpleNamespace(termination=np.array([2, 2, 2, 1, 2]), final_state=fs,
                                null_residual=np.array([1e-12, 1e-3, 1e-12, 1e-12, 1e-12]))
    # on the cone at the escape radius; off the cone; flung to 1e30; captured; past 1.1 r_esc
    assert list(accuracy.clean_escapes(m, res)) == [True, False, False, False, False]
