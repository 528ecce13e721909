"""Pin the CPU oracle to the reference's own known answers (CPU only).

The reference has no test suite; its validation is the printed output of
bin/energy_conditions.rs (committed as docs/energy_conditions.txt) and of
bin/validate_shadow.rs (quoted in README.md:43-50). tests/golden/ holds those
numbers; the oracle must reproduce every printed digit.
"""
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def fmt(v):
    # Rust's {:+.4e} prints e.g. +1.7073e-3 / -2.4626e-2 / +0.0000e0
    s = "%+.4e" % v
    mant, exp = s.split("e")
    return f"{mant}e{int(exp)}"


def golden_values(ec):
    vals = [r["value"] for r in ec["minkowski"]] + [r["value"] for r in ec["schwarzschild"]]
    return vals


@pytest.mark.parametrize("math", [0, 1], ids=["libm", "geon"])
def test_energy_conditions_printed_digits(orc, math):
    ec = json.load(open(os.path.join(GOLD, "energy_conditions.json"), encoding="utf-8"))
    out = orc.energy_conditions(math)
    assert len(out) == 99
    got_mink = out[0:2]
    got_schw = out[2:8]
    alc = out[8:49]
    mt = out[52:93]
    pairs = list(zip(got_mink, [r["value"] for r in ec["minkowski"]]))
    pairs += list(zip(got_schw, [r["value"] for r in ec["schwarzschild"]]))
    pairs += list(zip(alc[::4], [r["value"] for r in ec["alcubierre"]]))
    pairs += list(zip(mt[::4], [r["value"] for r in ec["morris_thorne"]]))
    pairs += [(out[49], ec["alcubierre_min"]), (out[51], ec["alcubierre_integral"]),
              (out[93], ec["morris_thorne_min"])]
    pairs += list(zip(out[95:99], ec["morris_thorne_throat_T_diag"]))
    assert len(pairs) == 2 + 6 + 11 + 11 + 3 + 4
    for got, want in pairs:
        assert fmt(got) == fmt(want), (got, want)
    # "at x = {:.2}": the minimum sits at x = +2.40 (not -2.40) in the reference's run
    assert "%.2f" % out[50] == "%.2f" % ec["alcubierre_min_at"]
    assert "%.2f" % out[94] == "%.2f" % ec["morris_thorne_min_at"]
    # Morris-Thorne throat: T_tt = -1/(8 pi) to the printed digits (README.md:72)
    assert fmt(out[95]) == fmt(-1.0 / (8.0 * np.pi))


@pytest.mark.parametrize("math", [0, 1], ids=["libm", "geon"])
def test_validate_shadow_b_c(orc, math):
    g = json.load(open(os.path.join(GOLD, "validate_shadow.json"), encoding="utf-8"))
    ac, lo, hi, st = orc.shadow_bisect([1.0, 1.001, 1000.0], 20.0, [0.0], [np.pi / 2 - 1e-3], 60, 0.01,
                                       200000, math=math)
    f = 1.0 - 2.0 / 20.0
    b_c = 20.0 * np.sin(ac[0]) / np.sqrt(f)
    b_an = np.sqrt(3.0) * 3.0
    assert "%.6f" % b_c == "%.6f" % g["b_c_measured"]
    assert "%.4f" % np.degrees(ac[0]) == "%.4f" % g["alpha_c_measured_deg"]
    assert "%.2e" % (abs(b_c - b_an) / b_an) == "%.2e" % g["rel_err"]


def test_minkowski_null_residual(orc):
    # README.md:50: Minkowski rays stay on the null cone to ~5e-16.
    rc, tet = orc.camera_tetrad(0, [], [0.0, 20.0, 0.0, 0.0])
    assert rc == 0
    y0 = orc.camera_rays(tet, [0.0, 20.0, 0.0, 0.0], 60.0, 16, 16)
    # from r = 20 through the origin to r > 1000 takes > 20000 steps of 0.05
    term, yf, steps, resid = orc.trace(0, [], y0, 0.05, 30000)
    assert np.all(term == 2)
    assert resid.max() < 2e-15


def test_inv4_matches_linear_algebra(orc):
    rng = np.random.default_rng(1)
    for _ in range(200):
        m = rng.normal(size=(4, 4)) + 4 * np.eye(4)
        inv = orc.inv4(m)
        np.testing.assert_allclose(inv, np.linalg.inv(m), rtol=1e-11, atol=1e-13)
    assert orc.inv4(np.zeros((4, 4))) is None


def test_geon_math_close_to_libm(orc):
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-60, 60, 100000), rng.uniform(1.55, 1.6, 20000), [np.pi / 2, 0.0]])
    s, c = orc.geon_sincos(x)
    us = np.abs(s.view(np.int64) - np.sin(x).view(np.int64))
    uc = np.abs(c.view(np.int64) - np.cos(x).view(np.int64))
    assert us.max() <= 1 and uc.max() <= 1
    assert (us == 0).mean() > 0.97 and (uc == 0).mean() > 0.97
    assert c[-2] == np.cos(np.pi / 2)  # 6.123233995736766e-17, as glibc
    # tanh (and expm1) follow the libm's own method: equal bit for bit
    t = np.concatenate([rng.uniform(-25, 25, 100000), rng.uniform(-1.2, 1.2, 100000),
                        np.ldexp(rng.uniform(-1, 1, 20000), -rng.integers(0, 60, 20000)),
                        [0.0, -0.0, 22.0, -22.0, 1.0, -1.0, np.inf, -np.inf]])
    # (math.tanh is the platform libm's; numpy's tanh is its own SIMD code)
    libm_tanh = np.array([math.tanh(v) for v in t])
    assert np.array_equal(orc.geon_tanh(t).view(np.int64), libm_tanh.view(np.int64))
    e = np.concatenate([rng.uniform(-50, 50, 100000), rng.uniform(-2, 2, 100000), [0.0, 709.0, -800.0]])
    libm_expm1 = np.array([math.expm1(v) for v in e])
    assert np.array_equal(orc.geon_expm1(e).view(np.int64), libm_expm1.view(np.int64))


def test_math_mode_floor(orc):
    """A 1-ulp change in libm moves the FD curvature of the reference by ~1e-7:
    the geon-math oracle sits inside that floor."""
    a = orc.energy_conditions(0)
    b = orc.energy_conditions(1)
    c = orc.energy_conditions(2)
    floor = np.abs(a - c).max()
    assert 1e-9 < floor < 1e-6
    assert np.abs(a - b).max() <= 2 * floor


def test_faithful_curvature_equals_single_riemann(orc):
    x = np.array([[0.0, 2.3, 0.4, -0.2], [0.0, -1.7, 0.1, 0.9]])
    k = np.array([[1.0, 1.0, 0.0, 0.0], [1.0, 0.0, 1.0, 0.0]])
    a = orc.nec(2, [2.0, 0.5, 2.0, 0.0], x, k, math=0, faithful=True)
    b = orc.nec(2, [2.0, 0.5, 2.0, 0.0], x, k, math=0, faithful=False)
    assert np.array_equal(a, b)


def test_oracle_tonemap_known_values(orc):
    """write_png's tonemap (render.rs:174-178): clamp, ^(1/2.2) in f32, *255, round, saturating cast."""
    x = np.array([0.0, 1.0, 0.5, -1.0, 2.0, np.nan, np.inf, -np.inf, 0.214, 1e-30], dtype=np.float32)
    assert orc.tonemap_u8(x).tolist() == [0, 255, 186, 0, 255, 0, 255, 0, 127, 0]
    # every byte value is reached, monotonically, over [0, 1]
    v = np.linspace(0.0, 1.0, 100001, dtype=np.float32)
    t = orc.tonemap_u8(v)
    assert np.all(np.diff(t.astype(int)) >= 0) and set(t.tolist()) == set(range(256))


def test_energy_conditions_report_format(orc):
    """The report formatter (geon_gb300/energy.py) on the oracle's numbers gives the
    reference's committed stdout of bin/energy_conditions.rs, line for line, in the
    libm mode and in the deterministic-math mode the GPU shares."""
    import json
    import os
    from geon_gb300 import energy
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "energy_conditions_stdout.json"),
                          encoding="utf-8"))["lines"]
    for math in (orc.LIBM, orc.GEON):
        assert energy.report(orc.energy_conditions(math)) == gold


def test_oracle_adaptive_matches_fixed_step_physics(orc):
    """The adaptive restatement on the validate_shadow rays: far fewer steps, the
    same escape directions, and no class change except the fixed step's horizon
    accidents and rays within 0.05 deg of the critical angle 14.269 deg."""
    p = [1.0, 1.001, 1000.0]
    alpha = np.radians(np.linspace(10.0, 20.0, 97))
    y0 = orc.equatorial_ray(1.0, 20.0, alpha, math=orc.GEON)
    tf, yff, sf, _ = orc.trace(1, p, y0, 0.01, 200000, math=orc.GEON)
    ta, yfa, sa, _ = orc.trace_adaptive(1, p, y0, 0.01, 200000, math=orc.GEON)
    assert sa.sum() * 100 < sf.sum()
    # a fixed-step ray "escaping" from inside the photon sphere was thrown by the horizon step
    thrown = (tf == 2) & (np.degrees(alpha) < 14.269)
    diff = np.where(ta != tf)[0]
    assert np.all(thrown[diff] | (np.abs(np.degrees(alpha[diff]) - 14.269) < 0.05))
    esc = (tf == 2) & (ta == 2)
    da = orc.asymptotic_direction(1, p, yfa[esc])
    df = orc.asymptotic_direction(1, p, yff[esc])
    assert np.max(np.arccos(np.clip(np.sum(da * df, axis=1), -1, 1))) < 1e-6


def _affine_samples(nodes):
    # g = eta + a linear function of (x, y, z): reproduced exactly by the B-spline
    x, y, z = nodes[:, 1], nodes[:, 2], nodes[:, 3]
    comps = np.zeros((len(nodes), 10))
    comps[:, 0] = -1.0 + 0.01 * x - 0.02 * z
    comps[:, 1] = 0.03 * y
    comps[:, 4] = 1.0 + 0.02 * y
    comps[:, 6] = -0.01 * x
    comps[:, 7] = 1.0 + 0.015 * z
    comps[:, 9] = 1.0 - 0.01 * x + 0.005 * y
    return comps


def _grid_nodes(lo, hi, n):
    axes = [np.linspace(lo[a], hi[a], n[a]) for a in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([np.zeros(x.size), x.ravel(), y.ravel(), z.ravel()], axis=1)


def test_oracle_field_reproduces_affine_metric(orc):
    """The sampled metric's B-spline reproduces an affine field exactly (up to
    rounding) inside the grid, and a constant field gives zero curvature."""
    lo, hi, n = (-1.0, -2.0, 0.0), (1.0, 2.0, 1.5), (9, 11, 7)
    nodes = _grid_nodes(lo, hi, n)
    orc.field_set(lo, hi, n, _affine_samples(nodes))
    rng = np.random.default_rng(3)
    x = np.stack([np.zeros(50), rng.uniform(-0.7, 0.7, 50), rng.uniform(-1.5, 1.5, 50), rng.uniform(0.3, 1.1, 50)], 1)
    g = orc.metric_g(4, [], x, math=orc.GEON).reshape(-1, 4, 4)
    want = _affine_samples(x)
    idx = ((0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3))
    for q, (i, j) in enumerate(idx):
        assert np.max(np.abs(g[:, i, j] - want[:, q])) < 1e-14
        assert np.array_equal(g[:, i, j], g[:, j, i])
    flat = np.zeros((len(nodes), 10))
    flat[:, 0], flat[:, 4], flat[:, 7], flat[:, 9] = -1.0, 1.0, 1.0, 1.0
    orc.field_set(lo, hi, n, flat)
    rs = orc.curvature(4, [], x, "ricci_scalar", math=orc.GEON)
    assert np.max(np.abs(rs)) < 1e-5
