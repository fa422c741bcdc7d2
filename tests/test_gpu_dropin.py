"""The drop-in CUDA module files, loaded the way the Java host loads them.

tests/gpu_util.Driver replays JCuda's calls: cuModuleLoad of
<cudaKernelsDir>/<fractal>.ptx, cuModuleGetFunction for the seven kernels,
cuModuleGetGlobal + memcpy for the __constant__ symbols, cuLaunchKernel with a
void** parameter array and the 32x32 block shape.  Results are compared with
the oracle; where the reference's own kernels were built for sm_103a
(oracle/_ref/ref_<fractal>[_nofma].cubin) they are run the same way, which pins
the oracle's lock-step restatement to the reference itself.  The modules in
cudaKernels_parity match the reference built with --fmad=false, the
escape-time modules in cudaKernels the reference as nvcc builds it by default
(contraction on), record for record."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle.oracle import JULIA, MANDELBROT  # noqa: E402
from tests.gpu_util import (MODULE_KERNELS, Driver, advanced_params, java_grid, main_params, pitched,  # noqa: E402
                            read_pixels, same_pixels, upload_pixels)
from tests.test_gpu_reference_mode import M1, rect_for, zoom_at  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

# Parameter offsets and sizes (CUDA parameter ABI) of the reference's entry
# points, from the Java marshalling (RenderingKernel/KernelMain/KernelAdvanced/
# KernelCompose): (offset, size) per parameter.
LAYOUT = {
    "fractalRenderMainFloat": [(0, 8), (8, 8), (16, 8), (24, 16), (40, 4), (44, 4), (48, 4)],
    "fractalRenderMainDouble": [(0, 8), (8, 8), (16, 8), (24, 32), (56, 4), (60, 4), (64, 4)],
    "fractalRenderAdvancedFloat": [(0, 8), (8, 8), (16, 8), (24, 16), (40, 4), (44, 4), (48, 4), (52, 16), (72, 8),
                                   (80, 8), (88, 8)],
    "fractalRenderAdvancedDouble": [(0, 8), (8, 8), (16, 8), (24, 32), (56, 4), (60, 4), (64, 4), (72, 32), (104, 8),
                                    (112, 8), (120, 8)],
    "compose": [(0, 8), (8, 8), (16, 8), (24, 8), (32, 8), (40, 4), (44, 4), (48, 8), (56, 4), (60, 4)],
    "fractalRenderUnderSampled": [(0, 8), (8, 8), (16, 4), (20, 4), (24, 4), (28, 4), (32, 4), (36, 4), (40, 4),
                                  (44, 4)],
}


@pytest.fixture(scope="module")
def drv(cuda, native):
    return Driver()


def module_path(fractal, parity):
    import chaos_gb300 as cg
    return os.path.join(cg.DROPIN_PARITY_DIR if parity else cg.DROPIN_DIR, fractal + ".ptx")


def param_layout(drv, fn, n):
    import ctypes as C
    out = []
    for i in range(n):
        off, size = C.c_size_t(), C.c_size_t()
        rc = drv.cu.cuFuncGetParamInfo(fn, C.c_size_t(i), C.byref(off), C.byref(size))
        assert rc == 0, (i, rc)
        out.append((off.value, size.value))
    return out


@pytest.mark.parametrize("fractal", ["mandelbrot", "julia"])
@pytest.mark.parametrize("parity", [False, True])
def test_module_exports_reference_interface(drv, fractal, parity):
    mod = drv.load(module_path(fractal, parity))
    try:
        fns = {k: drv.function(mod, k) for k in MODULE_KERNELS}
        for name, layout in LAYOUT.items():
            assert param_layout(drv, fns[name], len(layout)) == layout, name
        assert drv.global_(mod, "VISUALIZE_SAMPLE_COUNT")[1] == 1
        if fractal == "julia":
            assert drv.global_(mod, "julia_c")[1] == 16
    finally:
        drv.unload(mod)


def replay_main(drv, cuda, path, w, h, rect, max_iter, max_ss, flags, dbl, julia_c=None):
    mod = drv.load(path)
    try:
        if julia_c is not None:
            drv.write_constant(mod, "julia_c", np.array(julia_c, dtype=np.float64).tobytes())
        drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")
        fn = drv.function(mod, "fractalRenderMainDouble" if dbl else "fractalRenderMainFloat")
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        drv.launch(fn, grid, block, main_params(buf.data_ptr(), pitch, w, h, rect, max_iter, max_ss, flags, dbl))
        return read_pixels(buf, w)
    finally:
        drv.unload(mod)


def replay_advanced(drv, cuda, path, w, h, rect, max_iter, max_ss, flags, old, prev, focus, dbl):
    mod = drv.load(path)
    try:
        fn = drv.function(mod, "fractalRenderAdvancedDouble" if dbl else "fractalRenderAdvancedFloat")
        inbuf, in_pitch = upload_pixels(cuda, prev)
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        drv.launch(fn, grid, block, advanced_params(buf.data_ptr(), pitch, w, h, rect, max_iter, max_ss, flags, old,
                                                    inbuf.data_ptr(), in_pitch, focus, dbl))
        return read_pixels(buf, w)
    finally:
        drv.unload(mod)


MAIN_CASES = [(96, 64, 1.0, 1), (100, 37, 4.6, 1), (70, 45, 3.0, 0), (65, 66, 9.0, 1)]


@pytest.mark.parametrize("w,h,max_ss,flags", MAIN_CASES)
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("parity", [True, False])
def test_dropin_main_matches_oracle(drv, cuda, oracle, w, h, max_ss, flags, dbl, parity):
    import chaos_gb300 as cg
    rect = rect_for(M1[:2], M1[2], w, h)
    got = replay_main(drv, cuda, module_path("mandelbrot", parity), w, h, rect, 600, max_ss, flags, dbl)
    arith = cg.ARITH_PARITY if parity else cg.ARITH_CONTRACTED
    want = oracle.render_main(MANDELBROT, dbl, arith, w, h, rect, 600, max_ss, flags)
    assert not same_pixels(got, want).any()


def test_dropin_julia_constant(drv, cuda, oracle):
    import chaos_gb300 as cg
    w, h = 90, 60
    rect = rect_for((0.0, 0.0), 2.0, w, h)
    got = replay_main(drv, cuda, module_path("julia", True), w, h, rect, 900, 2.0, 1, False, julia_c=(0.285, 0.01))
    want = oracle.render_main(JULIA, False, cg.ARITH_PARITY, w, h, rect, 900, 2.0, 1, julia_c=(0.285, 0.01))
    assert not same_pixels(got, want).any()


@pytest.mark.parametrize("dbl", [False, True])
def test_dropin_advanced_matches_oracle(drv, cuda, oracle, dbl):
    import chaos_gb300 as cg
    w, h, focus = 128, 80, (40, 50)
    old = rect_for(M1[:2], M1[2], w, h)
    new = zoom_at(old, focus, w, h)
    prev = oracle.render_main(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, old, 600, 3.0, 1)
    got = replay_advanced(drv, cuda, module_path("mandelbrot", True), w, h, new, 600, 3.0, 8 | 16 | 32 | 1, old, prev,
                          focus, dbl)
    want = oracle.render_advanced(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, new, 600, 3.0, 8 | 16 | 32 | 1, old, prev,
                                  focus)
    assert not same_pixels(got, want).any()


def ref_cubin(fractal, nofma=True):
    p = os.path.join(REF_DIR, f"ref_{fractal}{'_nofma' if nofma else ''}.cubin")
    if not os.path.exists(p):
        pytest.skip(f"reference cubin not built ({p})")
    return p


def test_reference_cubin_interface_matches(drv):
    """The reference's own module has the parameter layout the drop-in copies."""
    mod = drv.load(ref_cubin("mandelbrot"))
    try:
        fns = {k: drv.function(mod, k) for k in MODULE_KERNELS}
        for name, layout in LAYOUT.items():
            assert param_layout(drv, fns[name], len(layout)) == layout, name
    finally:
        drv.unload(mod)


@pytest.mark.parametrize("w,h,max_ss,flags", MAIN_CASES + [(48, 40, 12.0, 1), (33, 29, 17.0, 1)])
@pytest.mark.parametrize("dbl", [False, True])
def test_reference_kernel_pins_oracle_main(drv, cuda, oracle, w, h, max_ss, flags, dbl):
    """The reference's fractalRenderMain (built --fmad=false) = the oracle = our parity module."""
    import chaos_gb300 as cg
    rect = rect_for(M1[:2], M1[2], w, h)
    ref = replay_main(drv, cuda, ref_cubin("mandelbrot"), w, h, rect, 600, max_ss, flags, dbl)
    want = oracle.render_main(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, rect, 600, max_ss, flags)
    bad = same_pixels(ref, want)
    assert not bad.any(), (int(bad.sum()), ref[bad][:3], want[bad][:3])
    ours = replay_main(drv, cuda, module_path("mandelbrot", True), w, h, rect, 600, max_ss, flags, dbl)
    assert not same_pixels(ours, ref).any()


@pytest.mark.parametrize("flags", [8 | 16 | 32 | 1, 8 | 1, 4 | 8 | 16 | 32 | 1])
@pytest.mark.parametrize("dbl", [False, True])
def test_reference_kernel_pins_oracle_advanced(drv, cuda, oracle, flags, dbl):
    import chaos_gb300 as cg
    w, h, focus = 128, 80, (40, 50)
    old = rect_for(M1[:2], M1[2], w, h)
    new = zoom_at(old, focus, w, h)
    prev = oracle.render_main(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, old, 600, 3.0, 1)
    ref = replay_advanced(drv, cuda, ref_cubin("mandelbrot"), w, h, new, 600, 3.0, flags, old, prev, focus, dbl)
    ours = replay_advanced(drv, cuda, module_path("mandelbrot", True), w, h, new, 600, 3.0, flags, old, prev, focus,
                           dbl)
    assert not same_pixels(ours, ref).any()  # same CUDA atanf on both sides: exact even with foveation
    want = oracle.render_advanced(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, new, 600, 3.0, flags, old, prev, focus)
    bad = same_pixels(ref, want)
    if flags & 4:
        assert bad.mean() < 0.02
    else:
        assert not bad.any(), (int(bad.sum()), ref[bad][:3], want[bad][:3])


def test_reference_julia_pins_oracle(drv, cuda, oracle):
    import chaos_gb300 as cg
    w, h = 90, 60
    rect = rect_for((0.0, 0.0), 2.0, w, h)
    ref = replay_main(drv, cuda, ref_cubin("julia"), w, h, rect, 900, 4.0, 1, True, julia_c=(-0.4, 0.6))
    want = oracle.render_main(JULIA, True, cg.ARITH_PARITY, w, h, rect, 900, 4.0, 1, julia_c=(-0.4, 0.6))
    assert not same_pixels(ref, want).any()


CONTRACTED_ADV_FLAGS = [8 | 16 | 32 | 1, 8 | 1, 4 | 8 | 16 | 32 | 1, 4 | 16 | 32 | 1]


@pytest.mark.parametrize("w,h,max_ss,flags", MAIN_CASES + [(48, 40, 12.0, 1), (33, 29, 17.0, 1), (257, 131, 4.6, 1)])
@pytest.mark.parametrize("dbl", [False, True])
def test_contracted_module_is_the_reference_default_build_main(drv, cuda, oracle, w, h, max_ss, flags, dbl):
    """cudaKernels/mandelbrot = the reference's module as nvcc builds it by
    default (ref_mandelbrot.cubin), record for record; the oracle's contracted
    restatement gives the same records."""
    import chaos_gb300 as cg
    rect = rect_for(M1[:2], M1[2], w, h)
    ref = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=False), w, h, rect, 600, max_ss, flags, dbl)
    ours = replay_main(drv, cuda, module_path("mandelbrot", False), w, h, rect, 600, max_ss, flags, dbl)
    bad = same_pixels(ours, ref)
    assert not bad.any(), (int(bad.sum()), ours[bad][:3], ref[bad][:3])
    want = oracle.render_main(MANDELBROT, dbl, cg.ARITH_CONTRACTED, w, h, rect, 600, max_ss, flags)
    assert not same_pixels(ref, want).any()


@pytest.mark.parametrize("flags", CONTRACTED_ADV_FLAGS)
@pytest.mark.parametrize("dbl", [False, True])
def test_contracted_module_is_the_reference_default_build_advanced(drv, cuda, oracle, flags, dbl):
    """Sample reuse, the blend near the zoom centre and foveation as the
    reference's default build computes them (the same CUDA atanf on both
    sides, so foveated tiles agree exactly as well)."""
    import chaos_gb300 as cg
    w, h, focus = 128, 80, (40, 50)
    old = rect_for(M1[:2], M1[2], w, h)
    new = zoom_at(old, focus, w, h)
    prev = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=False), w, h, old, 600, 3.0, 1, dbl)
    ref = replay_advanced(drv, cuda, ref_cubin("mandelbrot", nofma=False), w, h, new, 600, 3.0, flags, old, prev, focus,
                          dbl)
    ours = replay_advanced(drv, cuda, module_path("mandelbrot", False), w, h, new, 600, 3.0, flags, old, prev, focus,
                           dbl)
    bad = same_pixels(ours, ref)
    assert not bad.any(), (int(bad.sum()), ours[bad][:3], ref[bad][:3])
    want = oracle.render_advanced(MANDELBROT, dbl, cg.ARITH_CONTRACTED, w, h, new, 600, 3.0, flags, old, prev, focus)
    assert same_pixels(ref, want).mean() < (0.02 if flags & 4 else 1e-9)  # CUDA vs C-library atanf


@pytest.mark.parametrize("dbl", [False, True])
def test_contracted_julia_module_is_the_reference_default_build(drv, cuda, dbl):
    w, h = 90, 60
    rect = rect_for((0.0, 0.0), 2.0, w, h)
    ref = replay_main(drv, cuda, ref_cubin("julia", nofma=False), w, h, rect, 900, 4.0, 1, dbl, julia_c=(-0.4, 0.6))
    ours = replay_main(drv, cuda, module_path("julia", False), w, h, rect, 900, 4.0, 1, dbl, julia_c=(-0.4, 0.6))
    assert not same_pixels(ours, ref).any()


def test_contracted_library_call_matches_the_default_build(drv, cuda):
    """The C ABI's render_main with CHAOS_ARITH_CONTRACTED = the reference's
    default build (binary64, adaptive super-sampling)."""
    import chaos_gb300 as cg
    from tests.gpu_util import pitched, read_pixels
    w, h = 100, 37
    rect = rect_for(M1[:2], M1[2], w, h)
    ref = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=False), w, h, rect, 600, 4.6, 1, True)
    buf, pitch = pitched(cuda, w, h)
    cg.Module("mandelbrot").render_main(buf.data_ptr(), pitch, w, h, rect, 600, 4.6, 1, double=True,
                                        arith=cg.ARITH_CONTRACTED)
    cuda.cuda.synchronize()
    assert not same_pixels(read_pixels(buf, w), ref).any()


def replay_under_sampled(drv, cuda, path, w, h, rect, max_iter, level):
    import ctypes as C
    mod = drv.load(path)
    try:
        fn = drv.function(mod, "fractalRenderUnderSampled")
        buf, pitch = pitched(cuda, w, h)
        params = [C.c_uint64(buf.data_ptr()), C.c_int64(pitch), C.c_uint32(w), C.c_uint32(h)] + \
                 [C.c_float(v) for v in rect] + [C.c_uint32(max_iter), C.c_uint32(level)]
        grid, block = java_grid((w + level - 1) // level, (h + level - 1) // level)
        drv.launch(fn, grid, block, params)
        return read_pixels(buf, w)
    finally:
        drv.unload(mod)


@pytest.mark.parametrize("parity", [True, False])
def test_under_sampled_is_the_reference_build(drv, cuda, parity):
    """fractalRenderUnderSampled of each drop-in module against the reference
    built the same way (--fmad=false / default contraction)."""
    w, h, level = 150, 97, 3
    rect = tuple(float(v) for v in np.float32(rect_for(M1[:2], M1[2], w, h)))
    ref = replay_under_sampled(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, rect, 700, level)
    ours = replay_under_sampled(drv, cuda, module_path("mandelbrot", parity), w, h, rect, 700, level)
    bad = same_pixels(ours, ref)
    assert not bad.any(), (int(bad.sum()), ours[bad][:3], ref[bad][:3])


def _random_view(rng, dbl):
    """A seeded view near the set's boundary: centre from a short list of
    boundary regions, plane height log-uniform (down to 1e-12 in binary64,
    1e-5 in binary32), frame 8..96 pixels a side, maxIter 50..3000, maxSS
    1..20, adaptive sampling on or off."""
    centres = [(-0.748, 0.1), (-0.74364388703715, 0.13182590420531), (0.3004395381261789, -0.5705143370804123),
               (-1.25066, 0.02012), (-0.1011, 0.9563), (0.285, 0.01)]
    c = centres[rng.integers(len(centres))]
    zoom = 10 ** rng.uniform(-12 if dbl else -5, -1)
    w, h = int(rng.integers(8, 97)), int(rng.integers(8, 97))
    return (c, zoom, w, h, int(rng.integers(50, 3001)), float(rng.uniform(1.0, 20.0)), int(rng.integers(0, 2)))


@pytest.mark.parametrize("seed", range(40))
def test_random_main_views_against_both_reference_builds(drv, cuda, seed):
    """Seeded random views: cudaKernels = the reference's default build and
    cudaKernels_parity = its --fmad=false build, record for record."""
    rng = np.random.default_rng(1000 + seed)
    for dbl in (False, True):
        c, zoom, w, h, mi, mss, flags = _random_view(rng, dbl)
        rect = rect_for(c, zoom, w, h)
        if not dbl:
            rect = tuple(float(v) for v in np.float32(rect))
        for parity in (False, True):
            ref = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, rect, mi, mss, flags, dbl)
            ours = replay_main(drv, cuda, module_path("mandelbrot", parity), w, h, rect, mi, mss, flags, dbl)
            bad = same_pixels(ours, ref)
            assert not bad.any(), (seed, dbl, parity, (c, zoom, w, h, mi, mss, flags), int(bad.sum()))


@pytest.mark.parametrize("seed", range(40))
def test_random_advanced_frames_against_both_reference_builds(drv, cuda, seed):
    """Seeded zoom steps with random flags (reuse, zooming in or out,
    foveation, adaptive) and focus, previous frame from the same build."""
    rng = np.random.default_rng(2000 + seed)
    for dbl in (False, True):
        c, zoom, w, h, mi, mss, _ = _random_view(rng, dbl)
        w, h = max(w, 24), max(h, 16)
        focus = (int(rng.integers(0, w)), int(rng.integers(0, h)))
        old = rect_for(c, zoom, w, h)
        into = bool(rng.integers(0, 2))
        new = zoom_at(old, focus, w, h, into=into)
        flags = 8 | 16 | (32 if into else 0) | int(rng.integers(0, 2)) | (4 if rng.integers(0, 2) else 0)
        if not dbl:
            old = tuple(float(v) for v in np.float32(old))
            new = tuple(float(v) for v in np.float32(new))
        for parity in (False, True):
            prev = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, old, mi, mss, 1, dbl)
            ref = replay_advanced(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, new, mi, mss, flags, old, prev,
                                  focus, dbl)
            ours = replay_advanced(drv, cuda, module_path("mandelbrot", parity), w, h, new, mi, mss, flags, old, prev,
                                   focus, dbl)
            bad = same_pixels(ours, ref)
            assert not bad.any(), (seed, dbl, parity, flags, (c, zoom, w, h, mi, mss), int(bad.sum()))


@pytest.mark.parametrize("seed", range(20))
def test_random_julia_views_against_both_reference_builds(drv, cuda, seed):
    """Julia modules on seeded views and constants, both builds."""
    rng = np.random.default_rng(3000 + seed)
    consts = [(-0.4, 0.6), (0.285, 0.01), (-0.8, 0.156), (-0.7269, 0.1889), (0.355, 0.355)]
    for dbl in (False, True):
        jc = consts[rng.integers(len(consts))]
        c = (float(rng.uniform(-0.8, 0.8)), float(rng.uniform(-0.8, 0.8)))
        zoom = 10 ** rng.uniform(-9 if dbl else -4, 0.3)
        w, h = int(rng.integers(8, 97)), int(rng.integers(8, 97))
        mi, mss, flags = int(rng.integers(50, 2001)), float(rng.uniform(1.0, 12.0)), int(rng.integers(0, 2))
        rect = rect_for(c, zoom, w, h)
        if not dbl:
            rect = tuple(float(v) for v in np.float32(rect))
        for parity in (False, True):
            ref = replay_main(drv, cuda, ref_cubin("julia", nofma=parity), w, h, rect, mi, mss, flags, dbl, julia_c=jc)
            ours = replay_main(drv, cuda, module_path("julia", parity), w, h, rect, mi, mss, flags, dbl, julia_c=jc)
            bad = same_pixels(ours, ref)
            assert not bad.any(), (seed, dbl, parity, jc, (c, zoom, w, h, mi, mss, flags), int(bad.sum()))


@pytest.mark.parametrize("case", ["zoom_in_f32", "zoom_out_f32", "zoom_in_f64", "pan_f64"])
def test_large_reuse_frames_match_both_reference_builds(drv, cuda, case):
    """Frames large enough for the library's persistent reuse kernel to claim
    strips of several tiles and read each group of four in row order
    (3840x2160) against the reference's own
    fractalRenderAdvanced in the Java launch shape: the library with the
    rounded arithmetic against the --fmad=false build and with the
    contracted arithmetic against the default build, record for record.
    The previous frame is the reference's own fractalRenderMain of the old
    plane (maxIter small: the reuse path is what is checked)."""
    import chaos_gb300 as cg
    w, h, mi, mss = 3840, 2160, 150, 2.0
    dbl = case.endswith("f64")
    rng = np.random.default_rng(hash(case) % 1000)
    focus = (int(rng.integers(w // 4, 3 * w // 4)), int(rng.integers(h // 4, 3 * h // 4)))
    old = rect_for((-0.748, 0.1), 0.0014, w, h)
    if case == "pan_f64":
        dx = (old[2] - old[0]) * 0.013
        new = (old[0] + dx, old[1] - dx / 3, old[2] + dx, old[3] - dx / 3)
        flags = 8 | 16 | 1
    else:
        into = case.startswith("zoom_in")
        new = zoom_at(old, focus, w, h, into=into)
        flags = 8 | 16 | (32 if into else 0) | 1 | 4
    if not dbl:
        old = tuple(float(v) for v in np.float32(old))
        new = tuple(float(v) for v in np.float32(new))
    for parity in (True, False):
        prev = replay_main(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, old, mi, mss, 1, dbl)
        ref = replay_advanced(drv, cuda, ref_cubin("mandelbrot", nofma=parity), w, h, new, mi, mss, flags, old, prev,
                              focus, dbl)
        inbuf, in_pitch = upload_pixels(cuda, prev)
        buf, pitch = pitched(cuda, w, h)
        cg.Module("mandelbrot").render_advanced(buf.data_ptr(), pitch, w, h, new, mi, mss, flags, old,
                                                inbuf.data_ptr(), in_pitch, focus, double=dbl,
                                                arith=cg.ARITH_PARITY if parity else cg.ARITH_CONTRACTED)
        cuda.cuda.synchronize()
        got = read_pixels(buf, w)
        assert float(got["is_reused"].mean()) > 0.9  # the reuse path carries the frame
        bad = same_pixels(got, ref)
        assert not bad.any(), (case, parity, int(bad.sum()), got[bad][:3], ref[bad][:3])
