"""Curvature grid jobs (the batch form of bin/energy_conditions.rs): bit-exact
against the oracle on the same points and null vectors, and the reference's own
physics checks at BASELINE's curvature configurations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GEON_MATH = 1


def test_grid_matches_oracle_alcubierre(geon, orc):
    params = [2.0, 0.125, 0.5, 0.0]
    m = geon.Alcubierre(*params)
    lo, hi, n = (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0), (7, 5, 3)
    pts, ein, nec, k = geon.curvature.grid(m, lo, hi, n, nk=5, seed=1234, with_k=True)
    assert np.array_equal(ein, orc.curvature(2, params, pts, "einstein", math=GEON_MATH))
    assert np.array_equal(nec, orc.nec(2, params, pts, k, math=GEON_MATH))
    g = orc.metric_g(2, params, pts, GEON_MATH)
    kk = np.einsum("pij,pqi,pqj->pq", g, k, k)
    assert np.abs(kk).max() < 1e-13  # null in the local metric
    assert np.all(np.abs(k[..., 0] - k[..., 0].mean()) < 10)
    pts2, ein2, nec2, k2 = geon.curvature.grid(m, lo, hi, n, nk=5, seed=1234, with_k=True)
    assert np.array_equal(nec, nec2) and np.array_equal(k, k2)  # deterministic stream
    _, _, nec3, _ = geon.curvature.grid(m, lo, hi, n, nk=5, seed=99)
    assert not np.array_equal(nec, nec3)


def test_grid_into_reused_arrays(geon):
    """grid_into fills caller-owned arrays (reused across calls) with grid()'s
    bits, and refuses arrays of the wrong size or layout."""
    m = geon.Alcubierre(2.0, 0.125, 0.5, 0.0)
    lo, hi, n = (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0), (6, 5, 4)
    _, ein, nec, k = geon.curvature.grid(m, lo, hi, n, nk=3, seed=5, with_k=True)
    e2, n2, k2 = np.full_like(ein, np.nan), np.full_like(nec, np.nan), np.full_like(k, np.nan)
    for _ in range(2):
        geon.curvature.grid_into(m, lo, hi, n, e2, n2, k2, nk=3, seed=5)
        assert np.array_equal(e2, ein) and np.array_equal(n2, nec) and np.array_equal(k2, k)
    geon.curvature.grid_into(m, lo, hi, n, None, n2, nk=3, seed=5)
    assert np.array_equal(n2, nec)
    with pytest.raises(ValueError):
        geon.curvature.grid_into(m, lo, hi, n, e2[:-1], n2, nk=3)
    with pytest.raises(ValueError):
        geon.curvature.grid_into(m, lo, hi, n, e2, np.asfortranarray(n2.reshape(-1, 3)[:, ::-1]), nk=3)
    with pytest.raises(ValueError):
        geon.curvature.grid_into(m, lo, hi, n, e2.astype(np.float32), n2, nk=3)


def test_grid_morris_thorne_throat_energy_density(geon):
    """Config 4b: b0 = 1, 4096 points over l in [-5, 5]; T_tt at the throat vs -1/(8 pi)."""
    m = geon.MorrisThorne(1.0)
    pts, ein, nec, _ = geon.curvature.grid(m, (-5.0, np.pi / 2, 0.0), (5.0, np.pi / 2, 0.0), (4096, 1, 1), nk=16)
    t_tt = ein[:, 0, 0] / (8.0 * np.pi)
    at0 = geon.curvature.stress_energy(m, [0.0, 0.0, np.pi / 2, 0.0])[0, 0]
    assert abs(at0 - (-1.0 / (8.0 * np.pi))) < 1e-6
    mid = np.argmin(np.abs(pts[:, 1]))
    assert abs(t_tt[mid] - (-1.0 / (8.0 * np.pi))) < 1e-4
    # NEC: violated by every throat point for some null direction (the radial
    # ones: rho + p_r < 0) and never clearly satisfied (tangential: rho + p_t = 0)
    near = np.abs(pts[:, 1]) < 0.5
    assert np.all(nec[near].min(axis=1) < -1e-3)
    assert np.all(nec[near] < 1e-6)  # rho + p_t = 0 up to the ~1e-7 FD noise of T


def test_grid_schwarzschild_vacuum(geon):
    """Config 4c: 1e5 seeded points r in [3, 50], theta in [0.1, pi-0.1]: vacuum."""
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    n = 100000
    x = np.stack([np.zeros(n), rng.uniform(3, 50, n), rng.uniform(0.1, np.pi - 0.1, n),
                  rng.uniform(0, 2 * np.pi, n)], axis=1)
    ric = geon.curvature.ricci(m, x)
    rs = geon.curvature.ricci_scalar(m, x)
    # FD-of-analytic-Gamma noise: ~1e-12 on the equator, growing as 1/sin^2 theta
    w = np.sin(x[:, 2]) ** 2
    assert np.percentile(np.abs(rs), 50) < 1e-10
    assert np.max(np.abs(rs) * w) < 1e-7
    assert np.max(np.abs(ric).max(axis=(1, 2)) * w / (1 + x[:, 1] ** 2)) < 1e-9


@pytest.mark.parametrize("kind,params,lo,hi", [
    (0, [], (-3.0, -3.0, -3.0), (3.0, 3.0, 3.0)),
    (1, [1.0, 1.001, 100.0], (3.0, 0.3, -3.0), (40.0, 2.8, 3.0)),
    (2, [2.0, 0.5, 2.0, 0.0], (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0)),
    (3, [1.0], (-5.0, 0.3, -3.0), (5.0, 2.8, 3.0)),
], ids=["minkowski", "schwarzschild", "alcubierre_default", "morris_thorne"])
def test_grid_matches_oracle_all_metrics(geon, orc, kind, params, lo, hi):
    """Every metric's stencil (the slots a metric depends on, shared positions)
    against the oracle's per-point chain, at t != 0 and a ragged last block."""
    m = geon.from_kind(kind, params)
    pts, ein, nec, k = geon.curvature.grid(m, lo, hi, (5, 4, 3), t=1.5, nk=3, seed=77, with_k=True)
    assert np.array_equal(ein, orc.curvature(kind, params, pts, "einstein", math=GEON_MATH))
    # v = 2: inside the bubble g_tt > 0, no static observer, k and T(k, k) NaN
    assert np.array_equal(nec, orc.nec(kind, params, pts, k, math=GEON_MATH), equal_nan=True)
    if kind == 2:
        assert np.isnan(nec).any() and not np.isnan(nec).all()
