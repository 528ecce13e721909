"""GEON_FP64_FAST: FP64 RK4 in the reference's chart, with its stage points,
termination tests, NaN guard and step cap, but held to the tolerance of the
reference's own CUDA kernel (cuda/schwarzschild_render.cu:3-5: equal to the
CPU code "up to associativity") instead of to its bits.

Bars, the FP64 parity path's own against the reference run with glibc:
classes equal except on rays the reference's fixed step does not settle (the
photon-sphere separatrix, and its horizon and polar-axis accidents, decided by
the independent FP64 arbiter of geon_gb300.accuracy), at most 2e-3 of the
rays; escape directions within 1e-10 on >= 99.5 % of the escaped rays; the
critical impact parameter within 1e-6 of 3 sqrt(3) M. Metrics other than
Schwarzschild run the parity stepper, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHW = [1.0, 1.001, 100.0]
LIBM = 0


def test_fast_render_vs_libm_reference(geon, orc):
    m = geon.Schwarzschild(*SCHW)
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    rc, tet = orc.camera_tetrad(1, SCHW, obs, orc.LIBM)
    y0 = orc.camera_rays(tet, obs, 60.0, 96, 96)
    res = geon.trace(m, y0, 0.05, 20000, precision="fp64fast")
    term, yf, steps, resid = orc.trace(1, SCHW, y0, 0.05, 20000, math=orc.LIBM)
    assert np.mean(res.termination != term) <= 2e-3
    # both see a clean escape (the reference's fixed step flings some captured
    # rays to r ~ 1e30 as "Escaped": their final states carry no direction)
    ref = geon.TraceResult(term, yf, steps, resid)
    esc = geon.accuracy.clean_escapes(m, res) & geon.accuracy.clean_escapes(m, ref)
    d_gpu = m.asymptotic_direction(res.final_state[esc])
    d_ref = orc.asymptotic_direction(1, SCHW, yf[esc], orc.LIBM)
    err = np.nan_to_num(np.linalg.norm(d_gpu - d_ref, axis=1), nan=np.inf)
    assert np.mean(err <= 1e-10) >= 0.995
    assert np.median(err) <= 1e-12


def test_fast_matches_fp64_path_config1(geon):
    m = geon.Schwarzschild(*SCHW)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 128, 128)
    y0 = cam.ray_states(cam.tetrad(m))
    ex = geon.trace(m, y0, 0.05, 20000, precision="fp64")
    fa = geon.trace(m, y0, 0.05, 20000, precision="fp64fast")
    dis = np.flatnonzero(ex.termination != fa.termination)
    arb = geon.accuracy.arbiter_classes(m, y0[dis], 0.05, 20000)
    # disagreements on rays the parity path classifies right are the fast mode's own
    assert np.sum(arb == ex.termination[dis]) <= 2e-3 * len(y0)
    same = ex.termination == fa.termination
    assert np.mean(ex.steps_taken[same] == fa.steps_taken[same]) >= 0.99
    esc = geon.accuracy.clean_escapes(m, ex) & geon.accuracy.clean_escapes(m, fa)
    d_ex = m.asymptotic_direction(ex.final_state[esc])
    d_fa = m.asymptotic_direction(fa.final_state[esc])
    err = np.linalg.norm(d_ex - d_fa, axis=1)
    assert np.mean(err <= 1e-10) >= 0.995
    # the render runs the same stepper
    rgb, st, cls, pst = geon.render(m, cam, geon.RenderConfig(precision="fp64fast"), with_classes=True)
    assert np.array_equal(cls.ravel(), fa.termination)
    assert st.total_steps == int(fa.steps_taken.sum())


def test_fast_equatorial_rays(geon):
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    alpha = np.radians(rng.uniform(10.0, 20.0, 8192))
    ex = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="fp64")
    fa = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="fp64fast")
    y0 = geon.shadow.equatorial_ray(m, 20.0, alpha)
    dis = np.flatnonzero(ex.termination != fa.termination)
    arb = geon.accuracy.arbiter_classes(m, y0[dis], 0.01, 200000)
    assert np.sum(arb == ex.termination[dis]) <= 2e-3 * len(alpha)
    esc = geon.accuracy.clean_escapes(m, ex) & geon.accuracy.clean_escapes(m, fa)
    assert np.abs(ex.steps_taken[esc] - fa.steps_taken[esc]).max() <= 1
    d_ex = m.asymptotic_direction(ex.final_state[esc])
    d_fa = m.asymptotic_direction(fa.final_state[esc])
    err = np.linalg.norm(d_ex - d_fa, axis=1)
    assert np.mean(err <= 1e-10) >= 0.995
    t, s = geon.shadow.classify(m, 20.0, alpha, 0.01, 200000, precision="fp64fast")
    assert np.array_equal(t, fa.termination) and np.array_equal(s, fa.steps_taken)


def test_fast_bisection_b_c(geon):
    m = geon.Schwarzschild(1.0)
    ac, lo, hi, st = geon.shadow.bisect(m, 20.0, 0.0, np.pi / 2 - 1e-3, iters=60, precision="fp64fast")
    b_c = geon.shadow.impact_parameter(m, 20.0, ac[0])
    assert abs(b_c - 3.0 * np.sqrt(3.0)) / (3.0 * np.sqrt(3.0)) <= 1e-6


@pytest.mark.parametrize("kind,params", [(3, [1.0]), (2, [2.0, 0.125, 0.5, 0.0]), (0, [])],
                         ids=["morris_thorne", "alcubierre", "minkowski"])
def test_fast_other_metrics_run_the_parity_stepper(geon, kind, params):
    m = geon.from_kind(kind, params)
    obs = [0.0, 10.0, np.pi / 2, 0.0] if kind == 3 else [0.0, -10.0, 0.0, 0.0]
    cam = geon.Camera(obs, 90.0, 16, 16, forward_sign=1 if kind == 3 else -1)
    y0 = cam.ray_states(cam.tetrad(m))
    a = geon.trace(m, y0, 0.05, 3000, precision="fp64")
    b = geon.trace(m, y0, 0.05, 3000, precision="fp64fast")
    assert np.array_equal(a.termination, b.termination) and np.array_equal(a.final_state, b.final_state)
