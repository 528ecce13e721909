"""Mixed-precision path (FP32 bulk, compensated state) against the FP64 path,
which is the reference's algorithm bit for bit.

Classes: every ray on which the two disagree is traced again by the
independent FP64 arbiter (geon_gb300.accuracy: 16 sub-steps per step,
termination tested at every sub-step, orbit-plane frame for the spherically
symmetric metrics), and so is a sample of the rays on which they agree. The
mixed class must equal the arbiter's on all but a fraction < 1e-4 of the rays,
the task's bound, at the reference's step cap (20,000 for renders, 200,000 for
the shadow sweep). Directions: escape directions of rays both paths call
Escaped, per metric below. b_c within 1e-6 of 3 sqrt(3) M."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISMATCH = 1e-4  # classification mismatch bound against the arbiter


def geon_accuracy():
    from geon_gb300 import accuracy
    return accuracy


def _directions_close(m, r64, rmx, median, p99):
    # rays both paths see escape cleanly (the reference's fixed step also
    # flings some captured rays to r ~ 1e30 as "Escaped"; those carry no direction)
    esc = geon_accuracy().clean_escapes(m, r64) & geon_accuracy().clean_escapes(m, rmx)
    d64 = m.asymptotic_direction(r64.final_state[esc])
    dmx = m.asymptotic_direction(rmx.final_state[esc])
    ang = np.arccos(np.clip(np.sum(d64 * dmx, axis=1), -1.0, 1.0))
    assert esc.sum() > 0
    assert np.median(ang) < median
    assert np.quantile(ang, 0.99) < p99
    return ang


def test_mixed_shadow_sweep_matches_fp64(geon):
    m = geon.Schwarzschild(1.0)
    rng = np.random.default_rng(0x5EED)
    alpha = np.radians(rng.uniform(10.0, 20.0, 16384))
    r64 = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="fp64")
    rmx = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="mixed")  # the planar step the sweep times
    y0 = geon.shadow.equatorial_ray(m, 20.0, alpha)
    rep = geon.accuracy.class_report(m, y0, 0.01, 200000, rmx.termination, r64.termination)
    # The reference's fixed step at the horizon flings ~8 % of the captured rays
    # to r ~ 1e30 (reported Escaped); the arbiter confirms every one a capture.
    assert rep["disagreements_arbiter_sides_with_trace"] == rep["disagreements"]
    assert rep["mismatch_vs_arbiter"] < MISMATCH
    assert rep["agreeing_rays_arbiter_differs"] == 0
    esc = geon.accuracy.clean_escapes(m, r64) & (rmx.termination == 2)
    assert np.abs(rmx.steps_taken[esc] - r64.steps_taken[esc]).max() <= 1
    # every mixed escape is clean: the mixed path flings no ray off its geodesic
    assert np.array_equal(geon.accuracy.clean_escapes(m, rmx), rmx.termination == 2)
    # compensated null re-projection (default on): the FP64 path's null drift
    assert np.max(rmx.null_residual[esc]) < 1e-11
    _directions_close(m, r64, rmx, 1e-6, 1e-3)
    t, s = geon.shadow.classify(m, 20.0, alpha, 0.01, 200000, precision="mixed")
    assert np.array_equal(t, rmx.termination) and np.array_equal(s, rmx.steps_taken)


def test_mixed_bisection_b_c(geon):
    m = geon.Schwarzschild(1.0)
    ac, lo, hi, st = geon.shadow.bisect(m, 20.0, 0.0, np.pi / 2 - 1e-3, iters=60, precision="mixed")
    b_c = geon.shadow.impact_parameter(m, 20.0, ac[0])
    assert abs(b_c - 3.0 * np.sqrt(3.0)) / (3.0 * np.sqrt(3.0)) <= 1e-6


def test_mixed_bisection_early_decision_equals_full_traces(geon):
    """Bisection rounds of the mixed path end a ray as soon as its class is
    settled (outward beyond 3.3M with the escape radius within the steps left,
    or inward inside 2.9M); the halvings must be the ones the full traces give
    (geon_shadow_classify runs each ray to its end)."""
    m = geon.Schwarzschild(1.0)
    lo0 = np.radians([13.1, 13.6, 14.0, 14.2])
    hi0 = np.radians([14.9, 15.3, 14.5, 14.35])
    lo, hi = lo0.copy(), hi0.copy()
    for _ in range(24):  # bin/validate_shadow.rs:70-77, all brackets at once
        mid = 0.5 * (lo + hi)
        cap = geon.shadow.is_captured(m, 20.0, mid, precision="mixed")
        lo = np.where(cap, mid, lo)
        hi = np.where(cap, hi, mid)
    ac, lo_b, hi_b, st = geon.shadow.bisect(m, 20.0, lo0, hi0, iters=24, precision="mixed")
    assert np.array_equal(lo_b, lo) and np.array_equal(hi_b, hi)
    assert np.array_equal(ac, 0.5 * (lo + hi))


def test_mixed_render_schwarzschild(geon):
    """BASELINE config-1 view (r 30M, fov 60, h 0.05, cap 20000, escape 100M) at 128^2."""
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 128, 128)
    y0 = cam.ray_states(cam.tetrad(m))
    r64 = geon.trace(m, y0, 0.05, 20000, precision="fp64")
    rmx = geon.trace(m, y0, 0.05, 20000, precision="mixed")
    rep = geon.accuracy.class_report(m, y0, 0.05, 20000, rmx.termination, r64.termination)
    assert rep["mismatch_vs_arbiter"] < MISMATCH
    assert rep["agreeing_rays_arbiter_differs"] == 0
    # directions differ by the RK4 truncation error of the orbit-plane frame
    # against the chart's (~1e-6 at h = 0.05), more near the photon sphere
    _directions_close(m, r64, rmx, 1e-6, 1e-3)
    # the render's pixel classes are the traced classes (one sample per pixel)
    rgbmx, stmx, cls, _ = geon.render(m, cam, geon.RenderConfig(precision="mixed"), with_classes=True)
    assert np.array_equal(cls.ravel(), rmx.termination)
    rgb64, st64 = geon.render(m, cam, geon.RenderConfig(precision="fp64"))
    same_cls = cls.ravel() == r64.termination
    assert np.mean(np.any(rgb64.reshape(-1, 3)[same_cls] != rgbmx.reshape(-1, 3)[same_cls], axis=-1)) < 0.03


@pytest.mark.parametrize("band,reproject,bound", [(4.0, 0, 2e-3), (0.0, 1, 3e-2)], ids=["band4", "reproject"])
def test_mixed_chart_options(geon, band, reproject, bound):
    """The opt-in FP64 band and null re-projection step in the (theta, phi)
    chart (no orbit-plane frame). Measured: the band keeps the default's
    accuracy at 3.4x the cost; re-projection at FP32 precision replaces the
    compensated p^t by an FP32 one and loses accuracy; hence their bounds."""
    lib = geon._load()
    lib.geon_set_mixed_band(1, band)
    lib.geon_set_mixed_reproject(reproject)
    try:
        m = geon.Schwarzschild(1.0, 1.001, 100.0)
        cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 64, 64)
        y0 = cam.ray_states(cam.tetrad(m))
        r64 = geon.trace(m, y0, 0.05, 20000, precision="fp64")
        rmx = geon.trace(m, y0, 0.05, 20000, precision="mixed")
        rep = geon.accuracy.class_report(m, y0, 0.05, 20000, rmx.termination, r64.termination)
        assert rep["mismatch_vs_arbiter"] <= bound
    finally:
        lib.geon_set_mixed_band(1, 0.0)
        lib.geon_set_mixed_reproject(0)


@pytest.mark.parametrize("kind,params,obs,fov,fs,med,p99", [
    (3, [1.0], [0.0, 10.0, np.pi / 2, 0.0], 90.0, 1, 1e-5, 1e-3),
    (2, [2.0, 0.125, 0.5, 0.0], [0.0, -10.0, 0.0, 0.0], 90.0, -1, 1e-5, 1e-3),
    (0, [], [0.0, 20.0, 0.0, 0.0], 60.0, 1, 1e-6, 1e-5)], ids=["morris_thorne", "alcubierre", "minkowski"])
def test_mixed_exotic_classes_and_directions(geon, kind, params, obs, fov, fs, med, p99):
    """BASELINE config-3 views (fov 90, h 0.05, cap 20000) at 128^2."""
    m = geon.from_kind(kind, params)
    cam = geon.Camera(obs, fov, 128, 128, forward_sign=fs)
    y0 = cam.ray_states(cam.tetrad(m))
    r64 = geon.trace(m, y0, 0.05, 20000, precision="fp64")
    rmx = geon.trace(m, y0, 0.05, 20000, precision="mixed")
    rep = geon.accuracy.class_report(m, y0, 0.05, 20000, rmx.termination, r64.termination)
    assert rep["mismatch_vs_arbiter"] < MISMATCH
    assert rep["agreeing_rays_arbiter_differs"] == 0
    if np.any((r64.termination == 2) & (rmx.termination == 2)):
        _directions_close(m, r64, rmx, med, p99)


def test_mixed_orbit_plane_opt_out(geon):
    """geon_set_mixed_orbit_plane(0) returns to the chart step; the default is on."""
    lib = geon._load()
    assert lib.geon_get_mixed_orbit_plane() == 1
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 32, 32)
    y0 = cam.ray_states(cam.tetrad(m))
    a = geon.trace(m, y0, 0.05, 20000, precision="mixed")
    lib.geon_set_mixed_orbit_plane(0)
    try:
        b = geon.trace(m, y0, 0.05, 20000, precision="mixed")
    finally:
        lib.geon_set_mixed_orbit_plane(1)
    assert not np.array_equal(a.final_state, b.final_state)
    c = geon.trace(m, y0, 0.05, 20000, precision="mixed")
    assert np.array_equal(a.final_state, c.final_state) and np.array_equal(a.termination, c.termination)


def test_mixed_null_fix_opt_out(geon):
    """geon_set_mixed_null_fix(0) leaves p^t to the RK4 alone: the null drift
    of the FP32 right-hand sides (~1e-8) comes back; classes do not change."""
    lib = geon._load()
    assert lib.geon_get_mixed_null_fix() == 1
    m = geon.Schwarzschild(1.0)
    alpha = np.radians(np.linspace(15.0, 19.0, 512))
    on = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="mixed")
    lib.geon_set_mixed_null_fix(0)
    try:
        off = geon.shadow.trace(m, 20.0, alpha, 0.01, 200000, precision="mixed")
    finally:
        lib.geon_set_mixed_null_fix(1)
    esc = geon.accuracy.clean_escapes(m, on) & geon.accuracy.clean_escapes(m, off)
    assert esc.sum() > 400
    assert np.max(on.null_residual[esc]) < 1e-11 < 1e-9 < np.max(off.null_residual[esc])
    assert np.array_equal(on.termination, off.termination)


def test_shadow_dev_api(geon):
    torch = pytest.importorskip("torch")
    lib = geon._load()
    m = geon.Schwarzschild(1.0)
    lo = torch.tensor(np.radians([13.1, 13.7]), device="cuda")
    hi = torch.tensor(np.radians([14.9, 15.4]), device="cuda")
    ac = torch.empty(2, dtype=torch.float64, device="cuda")
    st = torch.empty(2, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    assert lib.geon_shadow_bisect_dev(m.handle, 20.0, lo.data_ptr(), hi.data_ptr(), 2, 12, 0.01, 200000, 0,
                                      ac.data_ptr(), None, None, st.data_ptr(), s.cuda_stream) == 0
    torch.cuda.synchronize()
    ref, _, _, rst = geon.shadow.bisect(m, 20.0, lo.cpu().numpy(), hi.cpu().numpy(), iters=12)
    assert np.array_equal(ac.cpu().numpy(), ref) and np.array_equal(st.cpu().numpy(), rst)


def test_mixed_trace_edge_cases(geon):
    """The reference's loop structure in the mixed path (geodesic.rs:62-117):
    the termination test before every step, the step cap with steps_taken =
    max_steps, the NaN guard keeping the pre-step state; the same classes and
    counts as the FP64 path on rays that end at once or at the cap. One
    documented difference: a step with a stage at or inside 2M is a horizon
    step in the mixed path (Captured, the step counted, the state kept), also
    when the stage radius is -inf; the FP64 path, like the reference, lets
    that step overflow and its NaN guard reports Diverged."""
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    y = geon.shadow.equatorial_ray(m, 20.0, np.array([0.1, 0.3, 1.2]))
    cases = np.concatenate([
        y,
        [[0.0, 1.5, np.pi / 2, 0.0, 1.0, -1.0, 0.0, 0.0]],     # starts inside the capture radius
        [[0.0, 150.0, np.pi / 2, 0.0, 1.0, 1.0, 0.0, 0.0]],    # starts beyond escape
        [[0.0, np.nan, np.pi / 2, 0.0, 1.0, 1.0, 0.0, 0.0]],   # non-finite r: Diverged at once
        [[0.0, 20.0, np.pi / 2, 0.0, 1.0, -1e300, 0.0, 0.0]],  # p^r overflows FP32: stage radius -inf
        [[0.0, 20.0, 1.0, 0.3, 1.0, -0.5, 0.01, 0.02]],        # off the equator (orbit-plane frame)
    ])
    same = np.arange(len(cases)) != 6
    for max_steps in [0, 1, 7, 16, 17]:
        r64 = geon.trace(m, cases, 0.05, max_steps, precision="fp64")
        rmx = geon.trace(m, cases, 0.05, max_steps, precision="mixed")
        assert np.array_equal(rmx.termination[same], r64.termination[same]), max_steps
        assert np.array_equal(rmx.steps_taken[same], r64.steps_taken[same]), max_steps
        if max_steps == 0:  # no test and no step: every ray Diverged with its loaded state
            assert np.all(rmx.termination == 0) and np.all(rmx.steps_taken == 0)
        else:
            assert rmx.termination[4] == 2 and rmx.final_state[4, 1] == 150.0
            assert rmx.termination[5] == 0 and np.isnan(rmx.final_state[5, 1])
            assert rmx.termination[6] == 1 and rmx.steps_taken[6] == 1  # horizon step, state kept
        assert rmx.final_state[6, 1] == 20.0
    r64 = geon.trace(m, cases, 0.05, 5000, precision="fp64")
    rmx = geon.trace(m, cases, 0.05, 5000, precision="mixed")
    assert np.array_equal(rmx.termination[same], r64.termination[same])
    esc = r64.termination == 2
    assert np.abs(rmx.steps_taken[esc] - r64.steps_taken[esc]).max() <= 1
    # ray 7 is timelike (g(p, p) = -0.47): no null re-projection, its invariant
    # kept as the FP64 path keeps it
    assert r64.null_residual[7] > 0.4
    assert abs(rmx.null_residual[7] - r64.null_residual[7]) <= 1e-6 * r64.null_residual[7]
    # null rays are re-projected (every 16 steps; at h = 0.05 the drift of the
    # steps since the last one stays below 1e-10)
    assert np.all(rmx.null_residual[[1, 2]] < 1e-10)
    empty = geon.trace(m, np.zeros((0, 8)), 0.05, 10, precision="mixed")
    assert empty.termination.shape == (0,)
