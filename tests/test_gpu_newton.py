"""Newton modules (newton wired / generic / colored by iterations): the
library's kernels and the drop-in module files against the oracle, and the
drop-in modules against the reference's own Newton cubins (--fmad=false)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tests.gpu_util import (MODULE_KERNELS, Driver, java_grid, main_params, pitched, read_pixels,  # noqa: E402
                            same_pixels, upload_pixels)
from tests.test_gpu_reference_mode import rect_for, zoom_at  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEFAULT = ([1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378], [-1, 0, 0, 1], 11)
OTHER = ([-1.7692923542386314, 0, 0.884646177119315707620204, 0.589742805022205501647280, 0.884646177119315707,
          -0.589742805022205501], [2, -2, 0, 1], 7)
OTHER_JSON = ('{"colorMagnifier": 7, "coefficients": [1, 0, -2, 2], "roots": [[-1.7692923542386314, 0], '
              '[0.884646177119315707620204, 0.589742805022205501647280], [0.884646177119315707, -0.589742805022205501]]}')
NAMES = {2: "newton_wired", 3: "newton_generic", 4: "newton_iterations"}


@pytest.mark.parametrize("kind", [2, 3, 4])
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("other", [False, True])
def test_library_main_matches_oracle(cuda, oracle, kind, dbl, other):
    import chaos_gb300 as cg
    w, h = 120, 75
    rect = rect_for((0.1, -0.05), 3.0, w, h)
    buf, pitch = pitched(cuda, w, h)
    m = cg.Module(NAMES[kind])
    roots, coeffs, mag = DEFAULT
    if other and kind != 2:
        m.set_custom_params(OTHER_JSON)
        roots, coeffs, mag = OTHER
    m.render_main(buf.data_ptr(), pitch, w, h, rect, 200, 3.0, 1, double=dbl)
    got = read_pixels(buf, w)
    oracle.set_newton(roots, coeffs, mag)
    want = oracle.render_main(kind, dbl, 1, w, h, rect, 200, 3.0, 1)
    oracle.set_newton()
    bad = same_pixels(got, want)
    assert not bad.any(), (int(bad.sum()), got[bad][:3], want[bad][:3])
    # compose with the module's colouring
    from chaos_gb300.palette import default_palette
    pal = default_palette()
    out = cuda.zeros((h, w), dtype=cuda.int32, device="cuda:0")
    dpal = cuda.from_numpy(pal.view(np.int32)).to("cuda:0")
    m.compose(buf.data_ptr(), pitch, out.data_ptr(), 4 * w, w, h, dpal.data_ptr(), len(pal), 3.0)
    mode = 1 if kind in (2, 3) else 2
    assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle.compose_mode(want, pal, mode, mag))


@pytest.mark.parametrize("kind", [2, 3, 4])
def test_library_advanced_matches_oracle(cuda, oracle, kind):
    import chaos_gb300 as cg
    w, h, focus = 96, 64, (30, 40)
    old = rect_for((0.1, -0.05), 3.0, w, h)
    new = zoom_at(old, focus, w, h)
    oracle.set_newton(*DEFAULT)
    prev = oracle.render_main(kind, False, 1, w, h, old, 200, 2.0, 1)
    inbuf, in_pitch = upload_pixels(cuda, prev)
    out, pitch = pitched(cuda, w, h)
    m = cg.Module(NAMES[kind])
    m.render_advanced(out.data_ptr(), pitch, w, h, new, 200, 2.0, 8 | 16 | 32 | 1, old, inbuf.data_ptr(), in_pitch,
                      focus)
    want = oracle.render_advanced(kind, False, 1, w, h, new, 200, 2.0, 8 | 16 | 32 | 1, old, prev, focus)
    assert not same_pixels(read_pixels(out, w), want).any()


@pytest.fixture(scope="module")
def drv(cuda, native):
    return Driver()


def _replay(drv, cuda, path, kind, w, h, rect, dbl, params):
    mod = drv.load(path)
    try:
        roots, coeffs, mag = params
        if kind in (3, 4):
            assert drv.write_constant(mod, "roots", np.array(roots, dtype=np.float64).tobytes()) == 48
            assert drv.write_constant(mod, "coefficients", np.array(coeffs, dtype=np.float64).tobytes()) == 32
        if kind == 4:
            assert drv.write_constant(mod, "colorMagnifier", np.int32(mag).tobytes()) == 4
        fn = drv.function(mod, "fractalRenderMainDouble" if dbl else "fractalRenderMainFloat")
        for k in MODULE_KERNELS:
            drv.function(mod, k)
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        drv.launch(fn, grid, block, main_params(buf.data_ptr(), pitch, w, h, rect, 200, 3.0, 1, dbl))
        return read_pixels(buf, w)
    finally:
        drv.unload(mod)


@pytest.mark.parametrize("kind", [2, 3, 4])
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("parity_dir", [True, False])
def test_dropin_newton_matches_reference_and_oracle(drv, cuda, oracle, kind, dbl, parity_dir):
    """The Newton modules of both module directories are rounded operation by
    operation: the reference built with --fmad=false, bit for bit."""
    import chaos_gb300 as cg
    w, h = 100, 60
    rect = rect_for((0.1, -0.05), 3.0, w, h)
    params = OTHER if kind != 2 else DEFAULT
    directory = cg.DROPIN_PARITY_DIR if parity_dir else cg.DROPIN_DIR
    ours = _replay(drv, cuda, os.path.join(directory, NAMES[kind] + ".ptx"), kind, w, h, rect, dbl, params)
    oracle.set_newton(*params)
    want = oracle.render_main(kind, dbl, 1, w, h, rect, 200, 3.0, 1)
    oracle.set_newton()
    assert not same_pixels(ours, want).any()
    ref_path = os.path.join(ROOT, "oracle", "_ref", f"ref_{NAMES[kind]}_nofma.cubin")
    if not os.path.exists(ref_path):
        pytest.skip("reference Newton cubin not built")
    ref = _replay(drv, cuda, ref_path, kind, w, h, rect, dbl, params)
    bad = same_pixels(ours, ref)
    assert not bad.any(), (int(bad.sum()), ours[bad][:3], ref[bad][:3])
