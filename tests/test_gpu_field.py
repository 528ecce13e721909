"""Sampled (tensor-field) metric, GEON_FIELD: g from B-spline control points on
a grid, then the reference's generic finite-difference chain. The GPU equals
the oracle's restatement bit for bit (functors, curvature, FP64 and adaptive
traces); a field sampled from the analytic Alcubierre metric reproduces its
Einstein tensor and NEC to the spline's O(spacing^2) accuracy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALC = [2.0, 0.5, 2.0, 0.0]  # energy_conditions.rs's bubble (R 2, thickness 0.5, v 2)
LO, HI, N = (0.6, -0.8, -0.8), (3.4, 0.8, 0.8), (71, 41, 41)  # spacing 0.04 around the +x bubble wall


@pytest.fixture(scope="module")
def sampled(geon):
    alc = geon.Alcubierre(*ALC)
    return alc, geon.FieldMetric.sample(alc, LO, HI, N)


@pytest.fixture
def field(sampled, orc):
    orc.field_set(LO, HI, N, sampled[1].samples, 0)  # the oracle's kind-4 metric for this test
    return sampled


def interior_points(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([np.zeros(n), rng.uniform(0.8, 3.2, n), rng.uniform(-0.6, 0.6, n), rng.uniform(-0.6, 0.6, n)], 1)


def test_field_functors_bit_exact(geon, orc, field):
    _, f = field
    x = interior_points(300, 1)
    x[:5, 1] = [LO[0], HI[0], 5.0, -3.0, 1.0]  # edges and beyond (clamped nodes)
    assert np.array_equal(f.g(x), orc.metric_g(4, [], x, math=orc.GEON).reshape(-1, 4, 4))
    assert np.array_equal(f.g_inv(x), orc.metric_g_inv(4, [], x, math=orc.GEON).reshape(-1, 4, 4))
    assert np.array_equal(f.christoffel(x), orc.metric_christoffel(4, [], x, math=orc.GEON).reshape(-1, 4, 4, 4))
    assert np.array_equal(f.terminate(x), orc.metric_terminate(4, [], x, math=orc.GEON))


def test_field_curvature_bit_exact(geon, orc, field):
    _, f = field
    x = interior_points(64, 2)
    assert np.array_equal(geon.curvature.einstein(f, x).reshape(-1, 16),
                          orc.curvature(4, [], x, "einstein", math=orc.GEON).reshape(-1, 16))
    k = np.array([1.0, 1.0, 0.0, 0.0])
    assert np.array_equal(geon.curvature.nec_contraction(f, x, k),
                          orc.nec(4, [], x, k.reshape(1, 4), math=orc.GEON).reshape(-1))


def test_field_curvature_matches_analytic_metric(geon, field):
    alc, f = field
    # the bin's null vector along the axis, through the bubble wall at x = 2
    x = np.stack([np.zeros(41), np.linspace(1.2, 2.8, 41), np.zeros(41), np.zeros(41)], 1)
    k = np.array([1.0, 1.0, 0.0, 0.0])
    nf = geon.curvature.nec_contraction(f, x, k)
    na = geon.curvature.nec_contraction(alc, x, k)
    assert np.max(np.abs(nf - na)) < 0.02 * np.max(np.abs(na))
    gf = geon.curvature.einstein(f, x)
    ga = geon.curvature.einstein(alc, x)
    assert np.max(np.abs(gf - ga)) < 0.02 * np.max(np.abs(ga))


@pytest.mark.parametrize("precision", ["fp64", "adaptive"])
def test_field_trace_bit_exact(geon, orc, field, precision):
    _, f = field
    cam = geon.Camera([0.0, 3.2, 0.0, 0.0], 60.0, 12, 8)  # outside the bubble, looking into its wall
    y0 = cam.ray_states(cam.tetrad(f))
    r = geon.trace(f, y0, 0.02, 5000, precision=precision)
    if precision == "fp64":
        t, yf, st, rs = orc.trace(4, [], y0, 0.02, 5000, math=orc.GEON)
    else:
        t, yf, st, rs = orc.trace_adaptive(4, [], y0, 0.02, 5000, math=orc.GEON)
    assert np.array_equal(r.termination, t) and np.array_equal(r.steps_taken, st)
    assert np.array_equal(r.final_state.view(np.uint64), yf.view(np.uint64))
    if precision == "fp64":
        # the fixed step carries every ray through the superluminal (v = 2) wall
        # and out of the sampled box; the adaptive step resolves the wall's
        # blueshift (|p| grows without bound there) and ends those rays Diverged
        assert np.all(r.termination == 2)


def test_field_spherical_chart_render(geon, orc):
    sch = geon.Schwarzschild(1.0, 1.001, 100.0)
    lo, hi, n = (2.5, 0.4, -0.6), (14.0, 2.74, 0.6), (116, 48, 25)
    f = geon.FieldMetric.sample(sch, lo, hi, n, chart=geon.SPHERICAL)
    orc.field_set(lo, hi, n, f.samples, 1)
    obs = [0.0, 10.0, np.pi / 2, 0.0]
    cam = geon.Camera(obs, 30.0, 10, 8)
    rgb, st, cls, pst = geon.render(f, cam, geon.RenderConfig(max_steps=3000), with_classes=True)
    orgb, ocls, opst, ost = orc.render(4, [], obs, 30.0, 10, 8, 0.05, 3000, math=orc.GEON)
    assert np.array_equal(cls, ocls) and np.array_equal(pst, opst) and np.array_equal(rgb, orgb)
    assert st.captured > 0 and st.escaped > 0


def test_field_mixed_precision_unsupported(geon, field):
    _, f = field
    with pytest.raises(geon.GeonError) as e:
        geon.trace(f, np.zeros((1, 8)), 0.05, 10, precision="mixed")
    assert e.value.status == -11
