"""Device tonemap (write_png, render.rs:169-183) against the oracle's libm
version: bit-exact bytes on rendered images, on every byte boundary and on a
uniform sample of all f32 values in [0, 1], plus the special values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def boundary_values():
    # f32 values within 8 ulps of each rounding boundary ((k + 0.5) / 255)^2.2
    out = []
    for k in range(255):
        b = np.float32(((k + 0.5) / 255.0) ** 2.2)
        bits = b.view(np.uint32)
        out.append((bits + np.arange(-8, 9, dtype=np.int64)).astype(np.uint32).view(np.float32))
    return np.concatenate(out)


def test_tonemap_matches_oracle(geon, orc):
    sweep = (np.arange(0, 0x3F800001, 997, dtype=np.int64).astype(np.uint32)).view(np.float32)
    special = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, -1e-45, 1e-45, 1.0000001, 255.0, -3.0],
                       dtype=np.float32)
    x = np.concatenate([sweep, boundary_values(), special])
    assert np.array_equal(geon.tonemap(x), orc.tonemap_u8(x))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_render_u8_equals_tonemapped_render(geon, orc, precision):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 96, 64)
    cfg = geon.RenderConfig(precision=precision, samples_per_axis=2)
    rgb, st = geon.render(m, cam, cfg)
    rgb8, rgbf, st8 = geon.render_u8(m, cam, cfg, with_float=True)
    assert np.array_equal(rgbf.view(np.uint32), rgb.view(np.uint32))
    assert np.array_equal(rgb8, orc.tonemap_u8(rgb))
    assert st8.total_steps == st.total_steps


def test_fp64_render_u8_matches_oracle_pipeline(geon, orc):
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    rgb8, st = geon.render_u8(m, geon.Camera(obs, 60.0, 64, 48), geon.RenderConfig())
    orgb, _, _, _ = orc.render(1, [1.0, 1.001, 100.0], obs, 60.0, 64, 48, math=orc.GEON)
    assert np.array_equal(rgb8, orc.tonemap_u8(orgb))


def test_served_render_u8(geon, orc):
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 48, 32)
    cfg = geon.RenderConfig(precision="mixed")
    with geon.Server(1 << 26) as srv:
        rgb, st, cls, pst, rgb8 = srv.submit_render(m, cam, cfg, with_u8=True).result(timeout=120)
    assert np.array_equal(rgb8, orc.tonemap_u8(rgb))
