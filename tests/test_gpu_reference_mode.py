"""GPU parity of the reference-mode kernels (fractalRenderMain / Advanced /
UnderSampled / compose semantics) in the C ABI library against the oracle's
lock-step restatement.  Every pixel record field must match bit for bit."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle.oracle import JULIA, MANDELBROT  # noqa: E402
from tests.gpu_util import pitched, read_pixels, same_pixels, upload_pixels  # noqa: E402

M1 = (-0.748, 0.1, 0.0014)  # premade view M1 (PresenterFX.java:244-252): centre, zoom (plane height)


def rect_for(center, zoom, w, h):
    """Model.setPlaneSegmentFromCenter (J/rendering/Model.java:247-256)."""
    rw = 1.0 / h * w
    return (center[0] - rw * zoom / 2, center[1] - zoom / 2, center[0] + rw * zoom / 2, center[1] + zoom / 2)


def zoom_at(rect, where, w, h, into=True):
    """RenderingController.zoomAt (J/rendering/RenderingController.java:130-150), ZOOM_COEFF = 0.977f."""
    sw, sh = rect[2] - rect[0], rect[3] - rect[1]
    rel_top = where[1] / h
    rel_btm = 1 - rel_top
    rel_left = where[0] / w
    rel_rght = 1 - rel_left
    cx, cy = rect[0] + sw * rel_left, rect[1] + sh * rel_btm
    z = float(np.float32(0.977)) if into else 2.0 - float(np.float32(0.977))
    return (cx - sw * rel_left * z, cy - sh * rel_btm * z, cx + sw * rel_rght * z, cy + sh * rel_top * z)


CASES = [
    # (w, h, max_ss, flags)
    (64, 48, 1.0, 1),
    (100, 37, 2.0, 1),
    (100, 37, 3.4, 0),
    (257, 131, 4.6, 1),
    (65, 66, 5.0, 1),
    (48, 40, 7.0, 0),
    (48, 40, 12.0, 1),
    (33, 29, 17.0, 1),
]


@pytest.mark.parametrize("w,h,max_ss,flags", CASES)
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("arith", [0, 1])
def test_main_mandelbrot(cuda, oracle, w, h, max_ss, flags, dbl, arith):
    import chaos_gb300 as cg
    rect = rect_for(M1[:2], M1[2], w, h)
    buf, pitch = pitched(cuda, w, h)
    with cg.Module("mandelbrot") as m:
        m.render_main(buf.data_ptr(), pitch, w, h, rect, 600, max_ss, flags, double=dbl, arith=arith)
    got = read_pixels(buf, w)
    want = oracle.render_main(MANDELBROT, dbl, arith, w, h, rect, 600, max_ss, flags)
    bad = same_pixels(got, want)
    assert not bad.any(), (int(bad.sum()), got[bad][:3], want[bad][:3])


@pytest.mark.parametrize("dbl", [False, True])
def test_main_julia(cuda, oracle, dbl):
    import chaos_gb300 as cg
    w, h = 120, 90
    rect = rect_for((0.0, 0.0), 2.2, w, h)
    buf, pitch = pitched(cuda, w, h)
    with cg.Module("julia") as m:
        m.set_custom_params("-0.8;0.156")
        m.render_main(buf.data_ptr(), pitch, w, h, rect, 900, 4.0, 1, double=dbl, arith=cg.ARITH_PARITY)
    got = read_pixels(buf, w)
    want = oracle.render_main(JULIA, dbl, cg.ARITH_PARITY, w, h, rect, 900, 4.0, 1, julia_c=(-0.8, 0.156))
    assert not same_pixels(got, want).any()




@pytest.mark.parametrize("flags", [8 | 16 | 32 | 1, 8 | 16 | 1, 8 | 1, 8 | 16 | 32, 4 | 16 | 32 | 1, 4 | 8 | 16 | 32 | 1])
@pytest.mark.parametrize("dbl", [False, True])
def test_advanced_zoom_step(cuda, oracle, flags, dbl):
    """One renderFast step: previous frame from fractalRenderMain, plane zoomed by
    RenderingController.zoomAt about the focus, advanced kernel reusing it."""
    import chaos_gb300 as cg
    w, h = 160, 96
    focus = (97, 31)
    old = rect_for(M1[:2], M1[2], w, h)
    new = zoom_at(old, focus, w, h)
    prev = oracle.render_main(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, old, 600, 3.0, 1)
    inbuf, in_pitch = upload_pixels(cuda, prev)
    out, pitch = pitched(cuda, w, h)
    with cg.Module("mandelbrot") as m:
        m.render_advanced(out.data_ptr(), pitch, w, h, new, 600, 3.0, flags, old, inbuf.data_ptr(), in_pitch, focus,
                          double=dbl, arith=cg.ARITH_PARITY)
    got = read_pixels(out, w)
    want = oracle.render_advanced(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, new, 600, 3.0, flags, old, prev, focus)
    bad = same_pixels(got, want)
    if flags & 4:
        # foveation calls atanf: CUDA's and the C library's may differ in the
        # last place, which can move a whole 8x4 tile across a threshold
        assert bad.mean() < 0.02, bad.mean()
    else:
        assert not bad.any(), (int(bad.sum()), got[bad][:3], want[bad][:3])


def test_under_sampled(cuda, oracle):
    import chaos_gb300 as cg
    w, h = 130, 70
    rect = rect_for(M1[:2], M1[2], w, h)
    buf, pitch = pitched(cuda, w, h)
    with cg.Module("mandelbrot") as m:
        m.render_under_sampled(buf.data_ptr(), pitch, w, h, rect, 500, 4)
    got = read_pixels(buf, w)
    want = oracle.render_under_sampled(MANDELBROT, cg.ARITH_PARITY, w, h, rect, 500, 4)
    assert not same_pixels(got, want).any()


@pytest.mark.parametrize("visualize", [False, True])
def test_compose(cuda, oracle, visualize):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    from oracle.oracle import PIXEL_DTYPE
    rng = np.random.default_rng(2)
    w, h = 131, 77
    pix = np.zeros((h, w), dtype=PIXEL_DTYPE)
    pix["value"] = rng.uniform(0, 5000, (h, w)).astype(np.float32)
    pix["weight"] = rng.integers(0, 80, (h, w)).astype(np.float32)
    pix["is_reused"] = rng.integers(0, 2, (h, w))
    pix["weight_of_new_samples"] = rng.integers(0, 70, (h, w)).astype(np.float32)
    pal = default_palette()
    torch = cuda
    inbuf, pitch = upload_pixels(torch, pix)
    out = torch.zeros((h, w + 3), dtype=torch.int32, device="cuda:0")
    dpal = torch.from_numpy(pal.view(np.int32)).to("cuda:0")
    with cg.Module("mandelbrot") as m:
        m.write_constant("VISUALIZE_SAMPLE_COUNT", b"\1" if visualize else b"\0")
        m.compose(inbuf.data_ptr(), pitch, out.data_ptr(), 4 * (w + 3), w, h, dpal.data_ptr(), len(pal), 9.5)
    got = out.cpu().numpy().view(np.uint32)[:, :w]
    want = oracle.compose(pix, pal, 9.5, visualize)
    assert np.array_equal(got, want)


def test_rejects_bad_arguments_on_gpu(cuda):
    import chaos_gb300 as cg
    buf, pitch = pitched(cuda, 16, 8)
    with cg.Module("mandelbrot") as m:
        with pytest.raises(cg.ChaosError):
            m.render_main(buf.data_ptr(), pitch, 16, 8, (-2, -1, 1, math.inf), 100, 1.0, 0)
        m.render_main(buf.data_ptr(), pitch, 16, 8, (-2, -1, 1, 1), 100, 1.0, 0)  # still usable
