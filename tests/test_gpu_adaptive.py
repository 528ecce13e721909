"""Adaptive stepping (precision="adaptive", FP64 Dormand-Prince 5(4)): the GPU
equals the oracle's restatement bit for bit (terminations, final states, step
counts, residuals) on every metric; it classifies the shadow sweep like the
fixed-step FP64 path once the reference's horizon accidents are mapped to
Captured, and its bisection finds b_c within 1e-6 with a small fraction of the
steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHW = [1.0, 1.001, 1000.0]


def same(r, o):
    t, yf, st, rs = o
    assert np.array_equal(r.termination, t)
    assert np.array_equal(r.steps_taken, st)
    assert np.array_equal(r.final_state.view(np.uint64), yf.view(np.uint64))
    assert np.array_equal(r.null_residual.view(np.uint64), rs.view(np.uint64))


def test_adaptive_shadow_rays_bit_exact(geon, orc):
    m = geon.Schwarzschild(*SCHW)
    alpha = np.radians(np.linspace(10.0, 20.0, 513))
    y0 = geon.shadow.equatorial_ray(m, 20.0, alpha)
    r = geon.trace(m, y0, 0.01, 200000, precision="adaptive")
    same(r, orc.trace_adaptive(1, SCHW, y0, 0.01, 200000, math=orc.GEON))


@pytest.mark.parametrize("kind,params,obs,fov,fwd", [
    (0, [], [0.0, 20.0, 0.0, 0.0], 60.0, 1),
    (1, [1.0, 1.001, 100.0], [0.0, 30.0, np.pi / 2, 0.0], 60.0, 1),
    (2, [2.0, 0.125, 0.5, 0.0], [0.0, -10.0, 0.0, 0.0], 90.0, -1),
    (3, [1.0], [0.0, 10.0, np.pi / 2, 0.0], 90.0, 1),
])
def test_adaptive_camera_rays_bit_exact(geon, orc, kind, params, obs, fov, fwd):
    m = geon.from_kind(kind, params)
    cam = geon.Camera(obs, fov, 24, 16, forward_sign=fwd)
    y0 = cam.ray_states(cam.tetrad(m))
    r = geon.trace(m, y0, 0.05, 20000, precision="adaptive")
    same(r, orc.trace_adaptive(kind, params, y0, 0.05, 20000, math=orc.GEON))


def test_adaptive_tolerance_changes_the_integration(geon, orc):
    m = geon.Schwarzschild(*SCHW)
    y0 = geon.shadow.equatorial_ray(m, 20.0, np.radians(np.linspace(12.0, 16.0, 65)))
    rtol0, atol0 = geon.adaptive_tolerance()
    try:
        geon.set_adaptive_tolerance(1e-7, 1e-9)
        r = geon.trace(m, y0, 0.01, 200000, precision="adaptive")
        same(r, orc.trace_adaptive(1, SCHW, y0, 0.01, 200000, 1e-7, 1e-9, math=orc.GEON))
    finally:
        geon.set_adaptive_tolerance(rtol0, atol0)


def test_adaptive_classification_and_b_c(geon):
    m = geon.Schwarzschild(*SCHW)
    rng = np.random.default_rng(11)
    alpha = np.radians(rng.uniform(10.0, 20.0, 4096))
    y0 = geon.shadow.equatorial_ray(m, 20.0, alpha)
    fixed = geon.trace(m, y0, 0.01, 200000, precision="fp64")
    ad = geon.trace(m, y0, 0.01, 200000, precision="adaptive")
    # where the adaptive and fixed-step classes differ, the independent FP64
    # arbiter sides with the adaptive integration (the fixed step's horizon
    # accidents), except for rays within 0.01 deg of the critical angle
    dis = np.flatnonzero(fixed.termination != ad.termination)
    arb = geon.accuracy.arbiter_classes(m, y0[dis], 0.01, 200000)
    bad = dis[arb != ad.termination[dis]]
    assert np.all(np.abs(np.degrees(alpha[bad]) - 14.269) < 1e-2)
    assert ad.steps_taken.sum() * 50 < fixed.steps_taken.sum()
    ac, _, _, _ = geon.shadow.bisect(m, 20.0, 0.0, np.pi / 2 - 1e-3, iters=60, precision="adaptive")
    b_c = geon.shadow.impact_parameter(m, 20.0, ac[0])
    assert abs(b_c - 3.0 * np.sqrt(3.0)) / (3.0 * np.sqrt(3.0)) <= 1e-6


def test_adaptive_render(geon):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 64, 48)
    rgb, st, cls, pst = geon.render(m, cam, geon.RenderConfig(precision="adaptive"), with_classes=True)
    rgb64, st64, cls64, _ = geon.render(m, cam, geon.RenderConfig(precision="fp64"), with_classes=True)
    assert st.total_steps * 5 < st64.total_steps
    assert np.mean(cls != cls64) < 0.05
