"""The drop-in module against the reference's own kernels on the same GPU:
same inputs, same launch shape (32x32 blocks on the default stream, as the
Java host launches), identical pixel records, and the time of each launch.

oracle/build_ref.sh builds the reference's mandelbrot module from its source
for sm_103a twice: with nvcc's default contraction (the build the Java
application loads; the drop-in's cudaKernels module reproduces it) and with
--fmad=false (the rounding of the parity module, cudaKernels_parity).  Workloads, both in the reference's own sampling
(fractalRenderMain: sample 0 at the pixel corner, then the diagonal / grid
pattern with warp votes):

* C2 view: binary64, pixel 1e-10/3840 around the seeded boundary centre of
  the 3840x2160 workload (bisection along the ray of seed 2), maxIter 20000,
  maxSS 4, adaptive sampling on; the central 1920x1080 of the frame;
* C1 view: binary32, 1024x1024 over [-2, 1] x [-1.5, 1.5], maxIter 1000,
  maxSS 1;
* a renderFast frame (fractalRenderAdvancedFloat): 3840x2160 around the
  premade view M1, zoomed in 1/0.977 at a seeded focus from the previous
  frame, with sample reuse, foveation and adaptive sampling (the Java
  renderer's flags while zooming in).

The same frames also go through the C ABI (chaos_render_main_f64/_f32).
Each kernel runs once untimed, then back to back (enough launches for
~50 ms, at most 20) between CUDA events; the mean is reported.  The times
are printed as one JSON line per view (run pytest with -s to see them)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tests.gpu_util import (Driver, advanced_params, java_grid, main_params, pitched, read_pixels,  # noqa: E402
                            same_pixels, upload_pixels)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

C2_FULL_W, C2_SPAN, C2_MAX_ITER, C2_SEED = 3840, 1e-10, 20000, 2
C2_W, C2_H = 1920, 1080


@pytest.fixture(scope="module")
def drv(cuda, native):
    return Driver()


def _cubin(name):
    p = os.path.join(REF_DIR, name)
    if not os.path.exists(p):
        pytest.skip(f"reference cubin not built ({p})")
    return p


def _ours(parity):
    import chaos_gb300 as cg
    return os.path.join(cg.DROPIN_PARITY_DIR if parity else cg.DROPIN_DIR, "mandelbrot.ptx")


def _timed(cuda, run, stream=None):
    """Mean time of back-to-back launches of `run` (ms): one untimed launch,
    then enough launches for ~50 ms (1 to 20) between one pair of events, so
    that the host's launch gap before the first one weighs little on a
    0.1 ms kernel."""
    import time
    cuda.cuda.synchronize()
    t0 = time.perf_counter()
    run()
    cuda.cuda.synchronize()
    reps = max(1, min(20, int(0.05 / max(time.perf_counter() - t0, 1e-6))))
    e0, e1 = cuda.cuda.Event(enable_timing=True), cuda.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    cuda.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _timed_main(drv, cuda, path, w, h, rect, max_iter, max_ss, flags, dbl):
    """fractalRenderMain{Float,Double} of a module in the Java launch shape on
    the default stream; (pixels of the last launch, mean ms)."""
    mod = drv.load(path)
    try:
        drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")
        fn = drv.function(mod, "fractalRenderMainDouble" if dbl else "fractalRenderMainFloat")
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        params = main_params(buf.data_ptr(), pitch, w, h, rect, max_iter, max_ss, flags, dbl)
        drv.launch(fn, grid, block, params)
        buf.zero_()
        ms = _timed(cuda, lambda: drv.launch(fn, grid, block, params, sync=False))
        return read_pixels(buf, w), ms
    finally:
        drv.unload(mod)


def _timed_library(cuda, w, h, rect, max_iter, max_ss, flags, dbl):
    """The same render through the C ABI (chaos_render_main_f64/_f32, parity
    arithmetic) on the current stream; (pixels, ms)."""
    import chaos_gb300 as cg
    module = cg.Module("mandelbrot")
    buf, pitch = pitched(cuda, w, h)
    stream = cuda.cuda.current_stream()

    def run():
        module.render_main(buf.data_ptr(), pitch, w, h, rect, max_iter, max_ss, flags, double=dbl,
                           arith=cg.ARITH_PARITY, stream=stream)

    run()
    buf.zero_()
    ms = _timed(cuda, run, stream)
    return read_pixels(buf, w), ms


def _compare(drv, cuda, name, w, h, rect, max_iter, max_ss, flags, dbl):
    ref_nofma, t_ref_nofma = _timed_main(drv, cuda, _cubin("ref_mandelbrot_nofma.cubin"), w, h, rect, max_iter,
                                         max_ss, flags, dbl)
    ref_fma, t_ref_fma = _timed_main(drv, cuda, _cubin("ref_mandelbrot.cubin"), w, h, rect, max_iter, max_ss, flags,
                                     dbl)
    ours_par, t_par = _timed_main(drv, cuda, _ours(True), w, h, rect, max_iter, max_ss, flags, dbl)
    ours_con, t_con = _timed_main(drv, cuda, _ours(False), w, h, rect, max_iter, max_ss, flags, dbl)
    lib_par, t_lib = _timed_library(cuda, w, h, rect, max_iter, max_ss, flags, dbl)
    line = {"view": name, "width": w, "height": h, "max_iter": max_iter, "max_ss": max_ss,
            "ms": {"reference_nofma": t_ref_nofma, "dropin_parity": t_par, "reference_default": t_ref_fma,
                   "dropin_contracted": t_con,
                   "library_parity": t_lib},
            "speedup": {"parity_vs_reference_nofma": t_ref_nofma / t_par,
                        "contracted_vs_reference_default": t_ref_fma / t_con,
                        "library_parity_vs_reference_nofma": t_ref_nofma / t_lib},
            "records_differing": {"parity_vs_reference_nofma": float(same_pixels(ours_par, ref_nofma).mean()),
                                  "contracted_vs_reference_default": float(same_pixels(ours_con, ref_fma).mean()),
                                  "library_parity_vs_reference_nofma": float(same_pixels(lib_par, ref_nofma).mean())}}
    print(json.dumps(line), flush=True)
    return line


def test_c2_view_dropin_vs_reference_kernel(drv, cuda):
    """The parity module equals the reference built with --fmad=false record for
    record and is faster than it on the deep binary64 view."""
    import chaos_gb300 as cg
    from chaos_gb300.workloads import boundary_point
    cx, cy = boundary_point(C2_SEED, max_iter=C2_MAX_ITER)
    ps = C2_SPAN / C2_FULL_W
    rect = (cx - C2_W / 2 * ps, cy - C2_H / 2 * ps, cx + C2_W / 2 * ps, cy + C2_H / 2 * ps)
    line = _compare(drv, cuda, "C2 central 1920x1080, reference sampling", C2_W, C2_H, rect, C2_MAX_ITER, 4.0,
                    cg.FLAG_ADAPTIVE_SS, True)
    assert line["records_differing"]["parity_vs_reference_nofma"] == 0.0
    assert line["records_differing"]["library_parity_vs_reference_nofma"] == 0.0
    assert line["records_differing"]["contracted_vs_reference_default"] == 0.0
    assert line["speedup"]["parity_vs_reference_nofma"] > 1.0
    assert line["speedup"]["contracted_vs_reference_default"] > 1.0


def test_c1_view_dropin_vs_reference_kernel(drv, cuda):
    line = _compare(drv, cuda, "C1 1024x1024 binary32, reference sampling", 1024, 1024, (-2.0, -1.5, 1.0, 1.5), 1000,
                    1.0, 0, False)
    assert line["records_differing"]["parity_vs_reference_nofma"] == 0.0
    assert line["records_differing"]["contracted_vs_reference_default"] == 0.0
    assert line["speedup"]["parity_vs_reference_nofma"] > 1.0


def _timed_advanced(drv, cuda, path, w, h, rect, max_iter, max_ss, flags, old, in_ptr, in_pitch, focus):
    """fractalRenderAdvancedFloat of a module in the Java launch shape; (pixels, mean ms)."""
    mod = drv.load(path)
    try:
        drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")
        fn = drv.function(mod, "fractalRenderAdvancedFloat")
        buf, pitch = pitched(cuda, w, h)
        grid, block = java_grid(w, h)
        params = advanced_params(buf.data_ptr(), pitch, w, h, rect, max_iter, max_ss, flags, old, in_ptr, in_pitch,
                                 focus, False)
        drv.launch(fn, grid, block, params)
        buf.zero_()
        ms = _timed(cuda, lambda: drv.launch(fn, grid, block, params, sync=False))
        return read_pixels(buf, w), ms
    finally:
        drv.unload(mod)


def test_reuse_frame_dropin_vs_reference_kernel(drv, cuda):
    """renderFast's kernel, fractalRenderAdvancedFloat, on a zoom-in frame that
    reuses the previous one: the drop-in modules equal the reference's two
    builds record for record, and each is faster than the build it mirrors."""
    import chaos_gb300 as cg
    from tests.test_gpu_reference_mode import M1, rect_for, zoom_at
    w, h, mi, mss = 3840, 2160, 400, 2.0
    focus = (1700, 900)
    old = tuple(float(v) for v in np.float32(rect_for(M1[:2], M1[2], w, h)))
    new = tuple(float(v) for v in np.float32(zoom_at(old, focus, w, h, into=True)))
    flags = (cg.FLAG_SAMPLE_REUSE | cg.FLAG_IS_ZOOMING | cg.FLAG_ZOOMING_IN | cg.FLAG_ADAPTIVE_SS |
             cg.FLAG_FOVEATION)
    line = {"view": "renderFast 3840x2160 around M1, zoom-in 1/0.977 with reuse + foveation", "ms": {},
            "speedup": {}, "records_differing": {}}
    for parity in (True, False):
        ref_path = _cubin("ref_mandelbrot_nofma.cubin" if parity else "ref_mandelbrot.cubin")
        # the previous frame: the reference's own renderQuality of the old plane
        mod = drv.load(ref_path)
        try:
            drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")
            fn = drv.function(mod, "fractalRenderMainFloat")
            prev, prev_pitch = pitched(cuda, w, h)
            grid, block = java_grid(w, h)
            drv.launch(fn, grid, block, main_params(prev.data_ptr(), prev_pitch, w, h, old, mi, mss, 1, False))
        finally:
            drv.unload(mod)
        ref, t_ref = _timed_advanced(drv, cuda, ref_path, w, h, new, mi, mss, flags, old, prev.data_ptr(),
                                     prev_pitch, focus)
        ours, t_ours = _timed_advanced(drv, cuda, _ours(parity), w, h, new, mi, mss, flags, old, prev.data_ptr(),
                                       prev_pitch, focus)
        name = "parity_vs_reference_nofma" if parity else "contracted_vs_reference_default"
        line["ms"][name] = [t_ours, t_ref]
        line["speedup"][name] = t_ref / t_ours
        line["records_differing"][name] = float(same_pixels(ours, ref).mean())
        assert float(ours["is_reused"].mean()) > 0.5  # the reuse path carries the frame
    print(json.dumps(line), flush=True)
    for name in line["speedup"]:
        assert line["records_differing"][name] == 0.0, name
        assert line["speedup"][name] > 1.0, name
