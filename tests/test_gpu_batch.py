"""geon_render_batch: several renders traced by one persistent kernel launch
(one device work queue over every image's rays, lanes refilled across images
and metric kinds). Each image must equal its single render (geon_render_ex)
bit for bit: pixels, classes, per-pixel steps and statistics, in both
precisions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _items(geon, precision, size, max_steps):
    cfg = geon.RenderConfig(precision=precision, max_steps=max_steps, show_stars=True)
    return [
        (geon.Alcubierre(2.0, 0.125, 0.5, 0.0), geon.Camera([0.0, -10.0, 0.0, 0.0], 90.0, size, size - 8,
                                                            forward_sign=-1), cfg),
        (geon.MorrisThorne(1.0), geon.Camera([0.0, 10.0, np.pi / 2, 0.0], 90.0, size + 8, size), cfg),
        (geon.Schwarzschild(1.0, 1.001, 100.0), geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, size, size),
         geon.RenderConfig(precision=precision, max_steps=max_steps, samples_per_axis=2)),
        (geon.Minkowski(), geon.Camera([0.0, 20.0, 0.0, 0.0], 60.0, 16, 16), cfg),
    ]


@pytest.mark.parametrize("precision,size,max_steps", [("mixed", 96, 20000), ("fp64", 24, 3000)])
def test_render_batch_equals_single_renders(geon, precision, size, max_steps):
    items = _items(geon, precision, size, max_steps)
    out = geon.render_batch(items)
    assert len(out) == len(items)
    for (m, cam, cfg), (rgb, st, cls, pst) in zip(items, out):
        rgb1, st1, cls1, pst1 = geon.render(m, cam, cfg, with_classes=True)
        assert np.array_equal(rgb, rgb1)
        assert np.array_equal(cls, cls1) and np.array_equal(pst, pst1)
        assert (st.captured, st.escaped, st.diverged, st.total_steps) == \
            (st1.captured, st1.escaped, st1.diverged, st1.total_steps)
        assert st.max_null_residual == st1.max_null_residual


def test_render_batch_rejects_mixed_precisions(geon):
    m = geon.Schwarzschild(1.0)
    cam = geon.Camera([0.0, 30.0, np.pi / 2, 0.0], 60.0, 8, 8)
    with pytest.raises(geon.GeonError):
        geon.render_batch([(m, cam, geon.RenderConfig(precision="mixed")),
                           (m, cam, geon.RenderConfig(precision="fp64"))])
