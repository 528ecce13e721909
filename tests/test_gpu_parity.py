"""GPU parity: the FP64 device path against the CPU oracle, through the C ABI.

Bar: with the deterministic sin/cos/tanh (oracle math mode GEON), every FP64
result is bit-identical to the oracle (np.array_equal; +0 and -0 compare equal).
Against the reference-faithful libm mode the tolerances of the task apply:
identical capture/escape classes except chaotic photon-sphere rays, final
direction within 1e-10 relative, curvature within 1e-9 where the reference's
own 1-ulp floor allows (Schwarzschild), within the measured floor otherwise.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEON_MATH, LIBM = 1, 0
GOLD = os.path.join(os.path.dirname(__file__), "golden")

# (kind, params, observer, fov, forward_sign)
SCHW = (1, [1.0, 1.001, 100.0])
ALC_CFG3 = (2, [2.0, 0.125, 0.5, 0.0])
ALC_DEF = (2, [2.0, 0.5, 2.0, 0.0])
MT = (3, [1.0])
MINK = (0, [])


def make(geon, kind, params):
    return geon.from_kind(kind, params)


def sample_points(kind, n, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 4))
    x[:, 0] = rng.uniform(-5, 5, n)
    if kind == 1:
        x[:, 1] = rng.uniform(2.5, 50, n)
        x[:, 2] = rng.uniform(0.1, np.pi - 0.1, n)
        x[:, 3] = rng.uniform(-np.pi, np.pi, n)
    elif kind == 3:
        x[:, 1] = rng.uniform(-10, 10, n)
        x[:, 2] = rng.uniform(0.1, np.pi - 0.1, n)
        x[:, 3] = rng.uniform(-np.pi, np.pi, n)
    else:
        x[:, 1:] = rng.uniform(-5, 5, (n, 3))
    return x


ALL = [MINK, SCHW, ALC_CFG3, ALC_DEF, MT]
IDS = ["minkowski", "schwarzschild", "alcubierre_sigma8", "alcubierre_default", "morris_thorne"]


@pytest.mark.parametrize("kind,params", ALL, ids=IDS)
def test_metric_functors_bitexact(geon, orc, kind, params):
    m = make(geon, kind, params)
    x = sample_points(kind, 300, 10 + kind)
    assert np.array_equal(m.g(x), orc.metric_g(kind, params, x, GEON_MATH).reshape(-1, 4, 4))
    assert np.array_equal(m.dg(x), orc.metric_dg(kind, params, x, GEON_MATH))
    assert np.array_equal(m.g_inv(x), orc.metric_g_inv(kind, params, x, GEON_MATH))
    assert np.array_equal(m.christoffel(x), orc.metric_christoffel(kind, params, x, GEON_MATH))
    assert np.array_equal(m.terminate(x), orc.metric_terminate(kind, params, x, GEON_MATH))
    st = np.concatenate([x, np.random.default_rng(3).normal(size=(300, 4))], axis=1)
    # angles far outside [0, 2pi): rays that graze the chart's pole reach them
    st[:6, 2] = [1e17, -3e100, 2.5e300, 4.5e15, -9.1e15, 7.0]
    st[:6, 3] = [-2e16, 1e200, 3.0, -1e300, 2.0**53 + 2, 2.0**54 + 6]
    # (t^2 overflows for the largest angles: both sides give the same NaN)
    assert np.array_equal(m.asymptotic_direction(st), orc.asymptotic_direction(kind, params, st, GEON_MATH),
                          equal_nan=True)


def camera_for(kind):
    if kind == 1:
        return [0.0, 30.0, np.pi / 2, 0.0], 60.0, 1
    if kind == 3:
        return [0.0, 10.0, np.pi / 2, 0.0], 90.0, 1
    if kind == 2:
        return [0.0, -10.0, 0.0, 0.0], 90.0, -1
    return [0.0, 20.0, 0.0, 0.0], 60.0, 1


@pytest.mark.parametrize("kind,params", ALL, ids=IDS)
def test_tetrad_and_camera_rays_bitexact(geon, orc, kind, params):
    m = make(geon, kind, params)
    obs, fov, fs = camera_for(kind)
    cam = geon.Camera(obs, fov, 37, 23, forward_sign=fs)
    tet = cam.tetrad(m)
    rc, otet = orc.camera_tetrad(kind, params, obs, GEON_MATH)
    assert rc == 0 and np.array_equal(tet, otet)
    for du, dv in [(0.5, 0.5), (0.25, 0.75)]:
        ys = cam.ray_states(tet, du, dv)
        oys = orc.camera_rays(otet, obs, fov, 37, 23, du=du, dv=dv, forward_sign=fs)
        assert np.array_equal(ys, oys)


@pytest.mark.parametrize("kind,params,size,max_steps", [
    (*MINK, 24, 30000), (*SCHW, 48, 20000), (*ALC_CFG3, 12, 4000), (*ALC_DEF, 12, 4000), (*MT, 12, 4000)],
    ids=IDS)
def test_trace_bitexact(geon, orc, kind, params, size, max_steps):
    m = make(geon, kind, params)
    obs, fov, fs = camera_for(kind)
    rc, tet = orc.camera_tetrad(kind, params, obs, GEON_MATH)
    y0 = orc.camera_rays(tet, obs, fov, size, size, forward_sign=fs)
    res = geon.trace(m, y0, 0.05, max_steps)
    term, yf, steps, resid = orc.trace(kind, params, y0, 0.05, max_steps, math=GEON_MATH)
    assert np.array_equal(res.termination, term)
    assert np.array_equal(res.steps_taken, steps)
    assert np.array_equal(res.final_state, yf)
    assert np.array_equal(res.null_residual, resid)


def test_trace_edge_cases(geon, orc):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    p = [1.0, 1.001, 100.0]
    y = orc.equatorial_ray(1.0, 20.0, np.array([0.1, 0.3, 1.2]), GEON_MATH)
    cases = np.concatenate([
        y,
        [[0.0, 1.5, np.pi / 2, 0.0, 1.0, -1.0, 0.0, 0.0]],     # starts inside the capture radius
        [[0.0, 150.0, np.pi / 2, 0.0, 1.0, 1.0, 0.0, 0.0]],    # starts beyond escape
        [[0.0, np.nan, np.pi / 2, 0.0, 1.0, 1.0, 0.0, 0.0]],   # non-finite r: Diverged at once
        [[0.0, 20.0, np.pi / 2, 0.0, 1.0, -1e300, 0.0, 0.0]],  # overflows: NaN guard
    ])
    for max_steps in [0, 1, 7, 5000]:
        res = geon.trace(m, cases, 0.05, max_steps)
        term, yf, steps, resid = orc.trace(1, p, cases, 0.05, max_steps, math=GEON_MATH)
        assert np.array_equal(res.termination, term)
        assert np.array_equal(res.steps_taken, steps)
        assert np.array_equal(res.final_state, yf, equal_nan=True)
        assert np.array_equal(res.null_residual, resid, equal_nan=True)
    empty = geon.trace(m, np.zeros((0, 8)), 0.05, 10)
    assert empty.termination.shape == (0,)


def test_render_config1_bitexact(geon, orc):
    """Config 1: Schwarzschild M=1, 256x256, r_obs 30, fov 60, h 0.05, cap 20000, escape 100M."""
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    cam = geon.Camera(obs, 60.0, 256, 256)
    rgb, st, cls, pst = geon.render(m, cam, geon.RenderConfig(show_stars=True), with_classes=True)
    orgb, ocls, opst, ost = orc.render(1, SCHW[1], obs, 60.0, 256, 256, math=GEON_MATH)
    assert np.array_equal(cls, ocls)
    assert np.array_equal(pst, opst)
    assert np.array_equal(rgb, orgb)
    assert (st.captured, st.escaped, st.diverged) == (ost["captured"], ost["escaped"], ost["diverged"])
    assert st.max_null_residual == ost["max_null_residual"]
    assert st.avg_steps == ost["avg_steps"] and st.total_steps == ost["total_steps"]


def test_render_supersampled_and_flags(geon, orc):
    m = geon.Schwarzschild(1.0)
    obs = [0.0, 20.0, np.pi / 2, 0.0]
    cam = geon.Camera(obs, 60.0, 40, 24)
    for show in (True, False):
        rgb, st, cls, pst = geon.render(m, cam, geon.RenderConfig(samples_per_axis=2, show_stars=show),
                                        with_classes=True)
        orgb, ocls, opst, ost = orc.render(1, [1.0, 1.001, 1000.0], obs, 60.0, 40, 24, samples_per_axis=2,
                                           show_stars=show, math=GEON_MATH)
        assert np.array_equal(cls, ocls) and np.array_equal(pst, opst) and np.array_equal(rgb, orgb)
        assert st.total_steps == ost["total_steps"] and st.avg_steps == ost["avg_steps"]
    # RenderConfig colours: pixels whose samples were all captured take captured_rgb
    rgb2, _ = geon.render(m, cam, geon.RenderConfig(samples_per_axis=2, captured_rgb=(0.25, 0.5, 0.75)))
    full_cap = np.all(rgb == 0.0, axis=-1)
    assert full_cap.any()
    assert np.array_equal(rgb2[full_cap], np.broadcast_to(np.float32([0.25, 0.5, 0.75]), rgb2[full_cap].shape))


@pytest.mark.parametrize("kind,params", [ALC_CFG3, MT], ids=["alcubierre_sigma8", "morris_thorne"])
def test_render_exotic_bitexact(geon, orc, kind, params):
    m = make(geon, kind, params)
    obs, fov, fs = camera_for(kind)
    cam = geon.Camera(obs, fov, 16, 16, forward_sign=fs)
    cfg = geon.RenderConfig(max_steps=3000)
    rgb, st, cls, pst = geon.render(m, cam, cfg, with_classes=True)
    orgb, ocls, opst, ost = orc.render(kind, params, obs, fov, 16, 16, max_steps=3000, forward_sign=fs,
                                       math=GEON_MATH)
    assert np.array_equal(cls, ocls) and np.array_equal(pst, opst) and np.array_equal(rgb, orgb)


def test_render_vs_libm_reference(geon, orc):
    """Against the reference-faithful oracle (glibc sin/cos): same classes except
    rays on the photon-sphere separatrix, escape directions within 1e-10."""
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    rc, tet = orc.camera_tetrad(1, SCHW[1], obs, LIBM)
    y0 = orc.camera_rays(tet, obs, 60.0, 96, 96)
    res = geon.trace(m, y0, 0.05, 20000)
    term, yf, steps, resid = orc.trace(1, SCHW[1], y0, 0.05, 20000, math=LIBM)
    mism = res.termination != term
    assert mism.mean() <= 2e-3
    esc = (res.termination == 2) & (term == 2)
    d_gpu = m.asymptotic_direction(res.final_state[esc])
    d_ref = orc.asymptotic_direction(1, SCHW[1], yf[esc], LIBM)
    err = np.nan_to_num(np.linalg.norm(d_gpu - d_ref, axis=1), nan=np.inf)
    # rays that graze the polar axis of the chart run away numerically (in the
    # reference too); they are the only ones allowed past 1e-10
    assert np.mean(err <= 1e-10) >= 0.995
    assert np.median(err) <= 1e-12


@pytest.mark.parametrize("params", [ALC_CFG3[1], ALC_DEF[1]], ids=["alcubierre_sigma8", "alcubierre_default"])
def test_alcubierre_equals_libm_reference(geon, orc, params):
    """tanh follows the libm's own method, so the Alcubierre path (tanh, sqrt and
    IEEE arithmetic only) equals the reference run with glibc bit for bit: the
    curvature chain, the grid job and the FP64 trace."""
    m = geon.Alcubierre(*params)
    x = sample_points(2, 40, 77)
    for what, fn in [("riemann", geon.curvature.riemann), ("einstein", geon.curvature.einstein),
                     ("stress_energy", geon.curvature.stress_energy)]:
        assert np.array_equal(fn(m, x), orc.curvature(2, params, x, what, math=LIBM)), what
    pts, ein, nec, k = geon.curvature.grid(m, (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0), (9, 7, 5), nk=4, seed=3,
                                           with_k=True)
    assert np.array_equal(ein, orc.curvature(2, params, pts, "einstein", math=LIBM))
    assert np.array_equal(nec, orc.nec(2, params, pts, k, math=LIBM), equal_nan=True)
    obs, fov, fs = camera_for(2)
    cam = geon.Camera(obs, fov, 24, 24, forward_sign=fs)
    y0 = cam.ray_states(cam.tetrad(m))
    res = geon.trace(m, y0, 0.05, 3000)
    term, yf, steps, resid = orc.trace(2, params, y0, 0.05, 3000, math=LIBM)
    assert np.array_equal(res.termination, term) and np.array_equal(res.steps_taken, steps)
    assert np.array_equal(res.final_state, yf)


def test_sky_sample_matches(geon, orc):
    rng = np.random.default_rng(7)
    d = rng.normal(size=(200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for show in (True, False):
        assert np.array_equal(geon.sky.sample(d, show), orc.sky_sample(d, show))


@pytest.mark.parametrize("kind,params", ALL, ids=IDS)
def test_curvature_bitexact(geon, orc, kind, params):
    m = make(geon, kind, params)
    x = sample_points(kind, 40, 20 + kind)
    for what, fn in [("riemann", geon.curvature.riemann), ("ricci", geon.curvature.ricci),
                     ("ricci_scalar", geon.curvature.ricci_scalar), ("einstein", geon.curvature.einstein),
                     ("stress_energy", geon.curvature.stress_energy)]:
        assert np.array_equal(fn(m, x), orc.curvature(kind, params, x, what, math=GEON_MATH)), what
    k = np.random.default_rng(5).normal(size=(40, 3, 4))
    assert np.array_equal(geon.curvature.nec_contraction(m, x, k), orc.nec(kind, params, x, k, math=GEON_MATH))


def test_schwarzschild_curvature_vs_libm(geon, orc):
    """Analytic Gamma: one FD level, so GPU (own sin/cos) and glibc agree to ~1e-12."""
    m = geon.Schwarzschild(1.0)
    x = sample_points(1, 200, 31)
    a = geon.curvature.einstein(m, x)
    b = orc.curvature(1, [1.0, 1.001, 1000.0], x, "einstein", math=LIBM)
    assert np.abs(a - b).max() <= 1e-9
    # vacuum: R ~ 1e-13 on the equator (docs/energy_conditions.txt:6-11), FD noise
    # grows as 1/sin^2(theta) towards the poles (g^phiphi)
    rs = geon.curvature.ricci_scalar(m, x)
    assert np.abs(rs).max() <= 1e-7
    assert np.abs(rs - orc.curvature(1, [1.0, 1.001, 1000.0], x, "ricci_scalar", math=LIBM)).max() <= 1e-9


def test_energy_conditions_on_gpu(geon):
    """bin/energy_conditions.rs through the GPU library, to the printed digits."""
    ec = json.load(open(os.path.join(GOLD, "energy_conditions.json"), encoding="utf-8"))

    def fmt(v):
        mant, exp = ("%+.4e" % v).split("e")
        return f"{mant}e{int(exp)}"

    mk = geon.Minkowski()
    assert fmt(geon.curvature.nec_contraction(mk, [0, 1, 1, 1], [1, 1, 0, 0])) == fmt(ec["minkowski"][0]["value"])
    sch = geon.Schwarzschild(1.0)
    got = []
    for r in (5.0, 10.0, 30.0):
        f = 1.0 - 2.0 / r
        x = [0.0, r, np.pi / 2, 0.0]
        got += [geon.curvature.nec_contraction(sch, x, [1 / np.sqrt(f), -np.sqrt(f), 0, 0]),
                geon.curvature.ricci_scalar(sch, x)]
    assert [fmt(v) for v in got] == [fmt(r["value"]) for r in ec["schwarzschild"]]
    alc = geon.Alcubierre(2.0, 0.5, 2.0, 0.0)
    xs = np.array([[0.0, -4.0 + 0.2 * n, 0.0, 0.0] for n in range(41)])
    nec = geon.curvature.nec_contraction(alc, xs, [1.0, 1.0, 0.0, 0.0])
    assert [fmt(v) for v in nec[::4]] == [fmt(r["value"]) for r in ec["alcubierre"]]
    xi = []
    xp = -5.0
    while xp <= 5.0:
        xi.append([0.0, xp, 0.0, 0.0])
        xp += 0.05
    vals = geon.curvature.nec_contraction(alc, np.array(xi), [1.0, 1.0, 0.0, 0.0])
    integral = 0.0
    for v in vals:
        if v < 0.0:
            integral += v * 0.05
    assert fmt(integral) == fmt(ec["alcubierre_integral"])
    mt = geon.MorrisThorne(1.0)
    xs = np.array([[0.0, -4.0 + 0.2 * n, np.pi / 2, 0.0] for n in range(41)])
    nec = geon.curvature.nec_contraction(mt, xs, [1.0, 1.0, 0.0, 0.0])
    assert [fmt(v) for v in nec[::4]] == [fmt(r["value"]) for r in ec["morris_thorne"]]
    t = geon.curvature.stress_energy(mt, [0.0, 0.0, np.pi / 2, 0.0])
    assert [fmt(t[i, i]) for i in range(4)] == [fmt(v) for v in ec["morris_thorne_throat_T_diag"]]


def test_shadow_classify_bitexact(geon, orc):
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    alpha = np.radians(rng.uniform(10.0, 20.0, 512))
    t, s = geon.shadow.classify(m, 20.0, alpha, 0.01, 200000)
    ot, os_ = orc.shadow_classify([1.0, 1.001, 1000.0], 20.0, alpha, 0.01, 200000, math=GEON_MATH)
    assert np.array_equal(t, ot) and np.array_equal(s, os_)
    y = geon.shadow.equatorial_ray(m, 20.0, alpha)
    assert np.array_equal(y, orc.equatorial_ray(1.0, 20.0, alpha, GEON_MATH))


def test_shadow_bisect_equals_sequential(geon, orc):
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    lo = np.radians(rng.uniform(13.0, 14.0, 6))
    hi = np.radians(rng.uniform(14.5, 15.5, 6))
    ac, l, h, st = geon.shadow.bisect(m, 20.0, lo, hi, iters=21, step=0.01, max_steps=200000)
    oac, ol, oh, ost = orc.shadow_bisect([1.0, 1.001, 1000.0], 20.0, lo, hi, 21, 0.01, 200000, math=GEON_MATH)
    assert np.array_equal(ac, oac) and np.array_equal(l, ol) and np.array_equal(h, oh)
    assert np.array_equal(st, ost)


def test_validate_shadow_on_gpu(geon):
    """bin/validate_shadow.rs end to end on the GPU: b_c = 5.196151, rel err 3.55e-7."""
    g = json.load(open(os.path.join(GOLD, "validate_shadow.json"), encoding="utf-8"))
    m = geon.Schwarzschild(1.0)
    assert geon.shadow.is_captured(m, 20.0, 0.0)
    assert not geon.shadow.is_captured(m, 20.0, np.pi / 2 - 1e-3)
    ac, lo, hi, st = geon.shadow.bisect(m, 20.0, 0.0, np.pi / 2 - 1e-3, iters=60)
    b_c = geon.shadow.impact_parameter(m, 20.0, ac[0])
    b_an = 3.0 * np.sqrt(3.0)
    assert "%.6f" % b_c == "%.6f" % g["b_c_measured"]
    assert "%.2e" % (abs(b_c - b_an) / b_an) == "%.2e" % g["rel_err"]
    assert abs(b_c - b_an) / b_an <= 1e-6


def test_errors_map_reference_panics(geon):
    from geon_gb300._util import GeonError
    inside = geon.Camera([0.0, 1.5, np.pi / 2, 0.0], 60.0, 8, 8)
    with pytest.raises(GeonError) as e:
        inside.tetrad(geon.Schwarzschild(1.0))
    assert e.value.status == -3
    mt = geon.MorrisThorne(1.0)
    with pytest.raises(GeonError) as e:
        mt.christoffel([0.0, 1.0, 0.0, 0.0])  # theta = 0: g_phiphi = 0, g singular
    assert e.value.status == -2


def test_trace_dev_with_device_buffers(geon, orc):
    torch = pytest.importorskip("torch")
    m = geon.Schwarzschild(1.0)
    y0 = orc.equatorial_ray(1.0, 20.0, np.radians(np.linspace(10, 20, 333)), GEON_MATH)
    d_y0 = torch.tensor(y0, device="cuda")
    n = y0.shape[0]
    d_term = torch.empty(n, dtype=torch.int32, device="cuda")
    d_yf = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    d_st = torch.empty(n, dtype=torch.int64, device="cuda")
    d_res = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    geon.trace_dev(m, n, d_y0.data_ptr(), 0.01, 200000, d_term.data_ptr(), d_yf.data_ptr(), d_st.data_ptr(),
                   d_res.data_ptr(), stream=stream.cuda_stream)
    torch.cuda.synchronize()
    term, yf, steps, resid = orc.trace(1, [1.0, 1.001, 1000.0], y0, 0.01, 200000, math=GEON_MATH)
    assert np.array_equal(d_term.cpu().numpy(), term)
    assert np.array_equal(d_yf.cpu().numpy(), yf)
    assert np.array_equal(d_st.cpu().numpy(), steps)


def test_bisection_width_does_not_change_results(geon):
    """The speculative width (rays per round) changes how many halvings one round
    replays, never the result: every width gives the sequential loop's bits."""
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(21)
    lo = np.radians(rng.uniform(13.0, 14.0, 8))
    hi = np.radians(rng.uniform(14.5, 15.5, 8))
    ref = geon.shadow.bisect(m, 20.0, lo, hi, iters=23)
    try:
        for width in (1, 100, 65536):
            assert lib.geon_set_bisect_rays_per_round(width) == 0
            got = geon.shadow.bisect(m, 20.0, lo, hi, iters=23)
            for a, b in zip(ref, got):
                assert np.array_equal(a, b)
    finally:
        lib.geon_set_bisect_rays_per_round(16384)
