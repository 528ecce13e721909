"""Serving engine: each request's result is the one the single-call API gives,
bit for bit, whether it runs alone or in a mix of other requests (renders of
every metric, bisections, curvature grids, both precisions); admission by the
memory budget; cancellation and deadlines; latency statistics."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R_OBS = 20.0


def metrics(geon):
    return {
        "minkowski": (geon.Minkowski(), [0.0, 20.0, 0.0, 0.0], 60.0, 1),
        "schwarzschild": (geon.Schwarzschild(1.0, 1.001, 100.0), [0.0, 30.0, np.pi / 2, 0.0], 60.0, 1),
        "alcubierre": (geon.Alcubierre(2.0, 0.125, 0.5, 0.0), [0.0, -10.0, 0.0, 0.0], 90.0, -1),
        "morris_thorne": (geon.MorrisThorne(1.0), [0.0, 10.0, np.pi / 2, 0.0], 90.0, 1),
    }


def single_render(geon, m, cam, cfg):
    rgb, stats, cls, pst = geon.render(m, cam, cfg, with_classes=True)
    return rgb, stats, cls, pst


def same_render(a, b):
    rgb_a, st_a, cls_a, pst_a = a
    rgb_b, st_b, cls_b, pst_b = b
    assert np.array_equal(rgb_a.view(np.uint32), rgb_b.view(np.uint32))
    assert np.array_equal(cls_a, cls_b) and np.array_equal(pst_a, pst_b)
    assert (st_a.captured, st_a.escaped, st_a.diverged, st_a.total_steps) == \
        (st_b.captured, st_b.escaped, st_b.diverged, st_b.total_steps)
    assert st_a.max_null_residual == st_b.max_null_residual


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_render_alone_equals_single_call(geon, precision):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 96, 64)
    cfg = geon.RenderConfig(precision=precision, show_stars=True)
    ref = single_render(geon, m, cam, cfg)
    with geon.Server(1 << 30) as srv:
        got = srv.submit_render(m, cam, cfg).result(timeout=120)
    same_render(ref, got)


def test_bisect_alone_equals_single_call(geon):
    m = geon.Schwarzschild(1.0)
    for precision in ("fp64", "mixed"):
        ac, lo, hi, st = geon.shadow.bisect(m, R_OBS, 13.0 * np.pi / 180, 15.5 * np.pi / 180, iters=40,
                                            precision=precision)
        with geon.Server(1 << 26) as srv:
            r = srv.submit_bisect(m, R_OBS, 13.0 * np.pi / 180, 15.5 * np.pi / 180, iters=40,
                                  precision=precision).result(timeout=120)
        assert r["alpha_c"] == ac[0] and r["lo"] == lo[0] and r["hi"] == hi[0]
        assert r["steps"] == st[0]


def test_mix_equals_alone(geon):
    """Renders of the four metrics in both precisions, bisections and curvature
    grids submitted together; every result equals its single-call result."""
    ms = metrics(geon)
    expected, jobs = [], []
    with geon.Server(4 << 30) as srv:
        for name, (m, obs, fov, fwd) in ms.items():
            for precision in ("fp64", "mixed"):
                w, h = (40, 32) if name in ("alcubierre", "morris_thorne") else (64, 48)
                cam = geon.Camera(obs, fov, w, h, forward_sign=fwd)
                cfg = geon.RenderConfig(precision=precision, show_stars=True,
                                        max_steps=4000 if name in ("alcubierre", "morris_thorne") else 20000)
                jobs.append(("render", srv.submit_render(m, cam, cfg)))
                expected.append(("render", (m, cam, cfg)))
        sch = geon.Schwarzschild(1.0)
        brackets = [(13.0, 15.5), (13.5, 14.5), (10.0, 20.0)]
        for i, (lo, hi) in enumerate(brackets):
            precision = "fp64" if i % 2 == 0 else "mixed"
            jobs.append(("bisect", srv.submit_bisect(sch, R_OBS, np.radians(lo), np.radians(hi), iters=30,
                                                     precision=precision, rays_per_round=7 if i == 2 else 31)))
            expected.append(("bisect", (np.radians(lo), np.radians(hi), precision)))
        for m in (ms["schwarzschild"][0], ms["morris_thorne"][0], ms["alcubierre"][0]):
            lo, hi, n = (-3.0, -3.0, -3.0), (3.0, 3.0, 3.0), (9, 8, 7)
            if m.kind in (1, 3):
                lo, hi = (4.0, 0.5, 0.0), (8.0, 2.5, 3.0)
            jobs.append(("curv", srv.submit_curvature(m, lo, hi, n, nk=8, seed=77)))
            expected.append(("curv", (m, lo, hi, n)))
        srv.wait_all(timeout=600)
        stats = srv.stats()
        results = [j.result() for _, j in jobs]
    assert stats["completed"] == len(jobs) and stats["failed"] == 0
    assert stats["launches"] > 1
    for (kind, args), got in zip(expected, results):
        if kind == "render":
            m, cam, cfg = args
            same_render(single_render(geon, m, cam, cfg), got)
        elif kind == "bisect":
            lo, hi, precision = args
            ac, l, h, st = geon.shadow.bisect(sch, R_OBS, lo, hi, iters=30, precision=precision)
            assert (got["alpha_c"], got["lo"], got["hi"], got["steps"]) == (ac[0], l[0], h[0], st[0])
        else:
            m, lo, hi, n = args
            _, ein, nec, _ = geon.curvature.grid(m, lo, hi, n, nk=8, seed=77)
            assert np.array_equal(ein, got[0]) and np.array_equal(nec, got[1])


def test_admission_budget(geon):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 64, 64)
    cfg = geon.RenderConfig(precision="mixed")
    ref = single_render(geon, m, cam, cfg)
    # room for one 64x64 request at a time (~230 KB of buffers each)
    with geon.Server(300 << 10) as srv:
        jobs = [srv.submit_render(m, cam, cfg) for _ in range(4)]
        for j in jobs:
            same_render(ref, j.result(timeout=120))
        big = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 1024, 1024)
        with pytest.raises(geon.GeonError) as e:
            srv.submit_render(m, big, cfg)
        assert e.value.status == -7  # GEON_ERR_ADMISSION
        assert srv.stats()["completed"] == 4


def test_cancel_and_deadline(geon):
    m = geon.Alcubierre(2.0, 0.125, 0.5, 0.0)
    big = geon.Camera([0.0, -10.0, 0.0, 0.0], 90.0, 512, 512, forward_sign=-1)
    cfg = geon.RenderConfig(precision="fp64")
    sch = geon.Schwarzschild(1.0, 1.001, 100.0)
    small = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 32, 32)
    with geon.Server(1 << 30) as srv:
        a = srv.submit_render(m, big, cfg)
        b = srv.submit_render(m, big, cfg, deadline_s=0.05)
        a.cancel()
        assert a.wait(timeout=120) == -10   # GEON_ERR_CANCELLED
        assert b.wait(timeout=120) == -8    # GEON_ERR_TIMEOUT
        # the server keeps serving, with correct results
        got = srv.submit_render(sch, small, geon.RenderConfig(precision="mixed")).result(timeout=120)
        same_render(single_render(geon, sch, small, geon.RenderConfig(precision="mixed")), got)
        st = srv.stats()
        assert st["failed"] == 2 and st["completed"] == 1


def test_bad_request_fails_alone(geon):
    sch = geon.Schwarzschild(1.0)
    inside = geon.Camera([0.0, 1.5, np.pi / 2, 0.0], 60.0, 16, 16)  # r < 2M: g_tt >= 0
    ok = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 16, 16)
    with geon.Server(1 << 26) as srv:
        bad = srv.submit_render(sch, inside)
        good = srv.submit_render(sch, ok)
        assert bad.wait(timeout=60) == -3  # GEON_ERR_NOT_TIMELIKE
        same_render(single_render(geon, sch, ok, geon.RenderConfig()), good.result(timeout=60))


def test_latency_stats(geon):
    sch = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 32, 32)
    with geon.Server(1 << 28) as srv:
        js = [srv.submit_render(sch, cam, geon.RenderConfig(precision="mixed")) for _ in range(6)]
        js += [srv.submit_curvature(sch, (4.0, 1.0, 0.0), (6.0, 2.0, 1.0), (4, 4, 4), nk=4)]
        srv.wait_all(timeout=120)
        st = srv.stats()
        total = sum(j.result()[1].total_steps for j in js[:6])
    assert st["completed"] == 7 and st["by_type"]["render"]["completed"] == 6
    assert st["by_type"]["curvature"]["completed"] == 1 and st["grid_points"] == 64
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    assert st["ray_steps"] == total


def test_many_jobs_per_class(geon):
    """Twenty renders of different sizes in the same two classes, in flight at
    once with bisections: every ray is claimed exactly once."""
    sch = geon.Schwarzschild(1.0, 1.001, 100.0)
    rng = np.random.default_rng(5)
    cases = []
    with geon.Server(1 << 30) as srv:
        jobs = []
        for i in range(20):
            w, h = int(rng.integers(8, 48)), int(rng.integers(8, 48))
            r = float(rng.uniform(12.0, 40.0))
            cam = geon.Camera([0.0, r, np.pi / 2, 0.0], float(rng.uniform(40.0, 90.0)), w, h)
            cfg = geon.RenderConfig(precision="mixed" if i % 2 else "fp64", show_stars=True)
            jobs.append(srv.submit_render(sch, cam, cfg))
            cases.append((cam, cfg))
        bis = [srv.submit_bisect(geon.Schwarzschild(1.0), R_OBS, np.radians(13.0), np.radians(15.5), iters=20,
                                 precision=p) for p in ("fp64", "mixed", "fp64", "mixed")]
        srv.wait_all(timeout=300)
        for j, (cam, cfg) in zip(jobs, cases):
            same_render(single_render(geon, sch, cam, cfg), j.result())
        for j, p in zip(bis, ("fp64", "mixed", "fp64", "mixed")):
            ac, lo, hi, st = geon.shadow.bisect(geon.Schwarzschild(1.0), R_OBS, np.radians(13.0),
                                                np.radians(15.5), iters=20, precision=p)
            assert j.result()["alpha_c"] == ac[0] and j.result()["steps"] == st[0]


def test_steps_per_launch_autotune(geon):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 64, 48)
    cfg = geon.RenderConfig(precision="mixed", show_stars=True)
    with geon.Server(1 << 30) as srv:
        assert srv.steps_per_launch("mixed") == 4096 and srv.steps_per_launch("fp64") == 128
        tuned = srv.autotune()
        for p in ("fp64", "mixed"):
            assert tuned[p]["steps"] in tuned[p]["rates"]
            assert all(r > 0 for r in tuned[p]["rates"].values())
            assert srv.steps_per_launch(p) == tuned[p]["steps"]
        srv.set_steps_per_launch("mixed", 100)  # any budget gives the same bits
        got = srv.submit_render(m, cam, cfg).result(timeout=120)
        with pytest.raises(geon.GeonError):
            srv.set_steps_per_launch("mixed", 0)
    same_render(single_render(geon, m, cam, cfg), got)
