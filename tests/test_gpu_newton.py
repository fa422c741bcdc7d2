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
def test_dropin_newton_matches_reference_and_oracle(drv, cuda, oracle, kind, dbl):
    """The Newton modules of cudaKernels_parity are rounded operation by
    operation: the oracle and the reference built with --fmad=false, bit for
    bit."""
    import chaos_gb300 as cg
    w, h = 100, 60
    rect = rect_for((0.1, -0.05), 3.0, w, h)
    params = OTHER if kind != 2 else DEFAULT
    ours = _replay(drv, cuda, os.path.join(cg.DROPIN_PARITY_DIR, NAMES[kind] + ".ptx"), kind, w, h, rect, dbl, params)
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


def _replay_advanced(drv, cuda, path, kind, w, h, new, old, prev, focus, flags, dbl, params):
    from tests.gpu_util import advanced_params
    mod = drv.load(path)
    try:
        roots, coeffs, mag = params
        if kind in (3, 4):
            drv.write_constant(mod, "roots", np.array(roots, dtype=np.float64).tobytes())
            drv.write_constant(mod, "coefficients", np.array(coeffs, dtype=np.float64).tobytes())
        if kind == 4:
            drv.write_constant(mod, "colorMagnifier", np.int32(mag).tobytes())
        fn = drv.function(mod, "fractalRenderAdvancedDouble" if dbl else "fractalRenderAdvancedFloat")
        inbuf, in_pitch = upload_pixels(cuda, prev)
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        drv.launch(fn, grid, block, advanced_params(buf.data_ptr(), pitch, w, h, new, 200, 3.0, flags, old,
                                                    inbuf.data_ptr(), in_pitch, focus, dbl))
        return read_pixels(buf, w)
    finally:
        drv.unload(mod)


@pytest.mark.parametrize("kind", [2, 3, 4])
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("view", [0, 1, 2])
def test_default_build_newton_modules_are_the_reference_default_build(drv, cuda, kind, dbl, view):
    """cudaKernels/newton_*.ptx against the reference's Newton modules as nvcc
    builds them by default (contraction on, the build the Java application
    loads): main frames and a zoom step with reuse, record for record, on
    seeded views and both parameter sets."""
    import chaos_gb300 as cg
    rng = np.random.default_rng(300 + 10 * kind + view)
    w, h = int(rng.integers(40, 121)), int(rng.integers(30, 91))
    centre = (float(rng.uniform(-1.0, 1.0)), float(rng.uniform(-1.0, 1.0)))
    zoom = 10 ** float(rng.uniform(-3 if not dbl else -9, 0.5))
    rect = rect_for(centre, zoom, w, h)
    if not dbl:
        rect = tuple(float(v) for v in np.float32(rect))
    params = (OTHER if view % 2 else DEFAULT) if kind != 2 else DEFAULT
    ref_path = os.path.join(ROOT, "oracle", "_ref", f"ref_{NAMES[kind]}.cubin")
    if not os.path.exists(ref_path):
        pytest.skip("reference Newton cubin not built")
    ours_path = os.path.join(cg.DROPIN_DIR, NAMES[kind] + ".ptx")
    ref = _replay(drv, cuda, ref_path, kind, w, h, rect, dbl, params)
    ours = _replay(drv, cuda, ours_path, kind, w, h, rect, dbl, params)
    bad = same_pixels(ours, ref)
    assert not bad.any(), ("main", kind, dbl, view, int(bad.sum()), ours[bad][:3], ref[bad][:3])
    focus = (int(rng.integers(0, w)), int(rng.integers(0, h)))
    new = zoom_at(rect, focus, w, h, into=bool(view != 1))
    if not dbl:
        new = tuple(float(v) for v in np.float32(new))
    flags = 8 | 16 | (32 if view != 1 else 0) | 1 | (4 if view == 2 else 0)
    ref_a = _replay_advanced(drv, cuda, ref_path, kind, w, h, new, rect, ref, focus, flags, dbl, params)
    ours_a = _replay_advanced(drv, cuda, ours_path, kind, w, h, new, rect, ref, focus, flags, dbl, params)
    bad = same_pixels(ours_a, ref_a)
    assert not bad.any(), ("advanced", kind, dbl, view, int(bad.sum()), ours_a[bad][:3], ref_a[bad][:3])
