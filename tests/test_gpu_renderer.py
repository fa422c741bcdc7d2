"""CudaFractalRenderer mirror (chaos_renderer): renderQuality then renderFast
frames through the C ABI, against the oracle's main/advanced + compose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle.oracle import MANDELBROT  # noqa: E402
from tests.test_gpu_reference_mode import rect_for, zoom_at  # noqa: E402


def test_quality_then_fast(cuda, oracle):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    w, h = 200, 120
    pal = default_palette()
    m = cg.Module("mandelbrot")
    r = cg.Renderer(m)
    r.initialize(w, h, pal)
    rect = rect_for((-0.748, 0.1), 0.0014, w, h)
    model = cg.RenderingModel(max_iterations=800, max_super_sampling=3.0, use_adaptive_super_sampling=1,
                              use_sample_reuse=1, use_foveated_rendering=0, arith=cg.ARITH_PARITY,
                              sample_reuse_cache_dirty=1, mouse_focus_x=120, mouse_focus_y=40)
    model.left_bottom_x, model.left_bottom_y, model.right_top_x, model.right_top_y = rect
    r.render_quality(model)
    assert model.floating_point_precision == cg.PRECISION_SINGLE
    assert model.sample_reuse_cache_dirty == 0
    prev = oracle.render_main(MANDELBROT, False, cg.ARITH_PARITY, w, h, rect, 800, 3.0, 1)
    assert np.array_equal(r.read_output(), oracle.compose(prev, pal, 3.0))

    # zoom in about the mouse for a few frames (the serving-like fast path)
    for _ in range(3):
        new = zoom_at(rect, (120, 40), w, h)
        model.left_bottom_x, model.left_bottom_y, model.right_top_x, model.right_top_y = new
        model.zooming, model.zooming_in = 1, 1
        r.render_fast(model)
        want = oracle.render_advanced(MANDELBROT, False, cg.ARITH_PARITY, w, h, new, 800, 3.0, 8 | 16 | 32 | 1, rect,
                                      prev, (120, 40))
        assert np.array_equal(r.read_output(), oracle.compose(want, pal, 3.0))
        prev, rect = want, new
    r.free_resources()
    r.close()


def test_double_precision_selected_for_deep_view(cuda, oracle):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    w, h = 64, 48
    pal = default_palette()
    r = cg.Renderer(cg.Module("mandelbrot"))
    r.initialize(w, h, pal)
    rect = rect_for((-0.551042868375875, 0.62714332109057), 8.00592947491907e-09, w, h)  # premade view M5
    model = cg.RenderingModel(max_iterations=3000, max_super_sampling=1.0, arith=cg.ARITH_PARITY)
    model.left_bottom_x, model.left_bottom_y, model.right_top_x, model.right_top_y = rect
    r.render_quality(model)
    assert model.floating_point_precision == cg.PRECISION_DOUBLE
    want = oracle.render_main(MANDELBROT, True, cg.ARITH_PARITY, w, h, rect, 3000, 1.0, 0)
    assert np.array_equal(r.read_output(), oracle.compose(want, pal, 1.0))
