"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-side logic (module registry, custom parameters,
constants, precision selection, argument validation) behaves like the
reference's Java layer."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "chaos_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(chaos_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native):
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_binding_covers_header(native):
    from chaos_gb300._native import SIGNATURES

    assert sorted(SIGNATURES) == header_functions()


def test_version_and_fractals(native):
    import chaos_gb300 as cg

    assert "sm_103a" in cg.version()
    assert cg.available_fractals() == ["mandelbrot", "julia", "newton wired", "newton generic",
                                       "newton colored by iterations"]


def test_module_registry(native):
    import chaos_gb300 as cg

    with cg.Module("mandelbrot") as m:
        assert m.fractal_name == "mandelbrot"
        assert m.default_view() == (-0.5, 0.0, 2.0, 1600, 5.0)  # ModuleMandelbrot.java:20-25
    with pytest.raises(cg.ChaosError) as e:
        cg.Module("newton_wired_typo")
    assert e.value.code == 3 and "Unknown fractal" in e.value.message


def test_julia_custom_params_and_constants(native):
    import chaos_gb300 as cg

    m = cg.Module("julia")
    m.set_custom_params("-0.4;0.6")
    m.set_custom_params("-1.77578 ;0")  # PresenterFX J3 preset, whitespace tolerated like Double.parseDouble
    m.set_custom_params("0.285,0.01")
    for bad in ("", "1.0", "a;b"):
        with pytest.raises(cg.ChaosError) as e:
            m.set_custom_params(bad)
        assert e.value.code == 1
    m.write_constant("julia_c", np.array([-0.8, 0.156]).tobytes())
    with pytest.raises(cg.ChaosError) as e:
        m.write_constant("julia_c", b"\0" * 8)
    assert e.value.code == 1
    m.write_constant("VISUALIZE_SAMPLE_COUNT", b"\1")
    with pytest.raises(cg.ChaosError) as e:
        m.write_constant("roots", b"\0" * 48)
    assert e.value.code == 4
    mm = cg.Module("mandelbrot")
    with pytest.raises(cg.ChaosError) as e:
        mm.write_constant("julia_c", b"\0" * 16)  # cuModuleGetGlobal: not in this module
    assert e.value.code == 4
    mm.set_custom_params("anything")  # ModuleMandelbrot ignores its parameters


def _java_ulp_float(v):
    f = abs(float(np.float32(v)))
    if f < 2.0 ** -126:
        return 2.0 ** -149
    return 2.0 ** (math.frexp(f)[1] - 24)


def _java_ulp_double(v):
    d = abs(v)
    if d < 2.0 ** -1022:
        return 2.0 ** -1074
    return 2.0 ** (math.frexp(d)[1] - 53)


def _java_precision(rect, w, h):
    pw = abs(rect[2] - rect[0]) / w
    ph = abs(rect[3] - rect[1]) / h
    p = 0
    if pw < _java_ulp_float(rect[0]) or ph < _java_ulp_float(rect[1]):
        p = 1
    if pw < _java_ulp_double(rect[0]) or ph < _java_ulp_double(rect[1]):
        p = 2
    return p


def test_select_precision(native):
    import chaos_gb300 as cg

    rng = np.random.default_rng(3)
    cases = [(-2.0, -1.0, 1.0, 1.0), (-0.75, 0.1, -0.7499, 0.1001), (0.0, 0.0, 1e-300, 1e-300)]
    for _ in range(300):
        cx, cy = rng.uniform(-2, 1), rng.uniform(-1.2, 1.2)
        span = 10.0 ** rng.uniform(-18, 0.5)
        cases.append((cx - span, cy - span / 2, cx + span, cy + span / 2))
    for r in cases:
        assert cg.select_precision(r, 1280, 720) == _java_precision(r, 1280, 720), r


def test_argument_validation_without_gpu(native):
    """Every check below fails before any CUDA call (no GPU needed)."""
    import chaos_gb300 as cg

    m = cg.Module("mandelbrot")
    good = dict(out_ptr=0x10000, pitch=16 * 64, width=64, height=32, rect=(-2, -1, 1, 1), max_iter=100, max_ss=1.0,
                flags=0)
    for bad, code in [(dict(width=0), 1), (dict(pitch=16 * 63), 1), (dict(out_ptr=0), 1), (dict(max_ss=0.5), 1),
                      (dict(max_iter=0), 1), (dict(rect=(float("nan"), -1, 1, 1)), 1), (dict(width=65535 * 32 + 1), 1)]:
        kw = dict(good)
        kw.update(bad)
        for dbl in (False, True):
            with pytest.raises(cg.ChaosError) as e:
                m.render_main(double=dbl, **kw)
            assert e.value.code == code, (bad, e.value)
    with pytest.raises(cg.ChaosError) as e:
        m.render_advanced(0x10000, 16 * 64, 64, 32, (-2, -1, 1, 1), 100, 1.0, 0, (-2, -1, 1, 1), 0x10000, 16 * 64,
                          (0, 0))
    assert e.value.code == 1 and "overlap" in e.value.message
    with pytest.raises(cg.ChaosError) as e:
        m.render_under_sampled(0x10000, 16 * 64, 64, 32, (-2, -1, 1, 1), 100, 0)
    assert e.value.code == 1
    with pytest.raises(cg.ChaosError) as e:
        m.compose(0x10000, 16 * 64, 0x20000, 4 * 64, 64, 32, 0, 0, 1.0)
    assert e.value.code == 1 and "palette" in e.value.message
    d = cg.FrameDesc(width=64, height=64, max_iterations=10, samples_per_pixel=2, sample_mode=cg.SAMPLES_CENTER,
                     tier=cg.TIER_F32, pixel_size=0.01)
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(d, cg.FrameOut())
    assert e.value.code == 1
    d.samples_per_pixel, d.sample_mode, d.pixel_size = 4, cg.SAMPLES_JITTER, 0.0
    with pytest.raises(cg.ChaosError):
        cg.render_frame(d, cg.FrameOut())
    d.pixel_size, d.tier = 0.01, 7
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(d, cg.FrameOut())
    assert e.value.code == 8
    # the contracted arithmetic is for the reference-mode calls only
    d.tier, d.arith = cg.TIER_F32, cg.ARITH_CONTRACTED
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(d, cg.FrameOut())
    assert e.value.code == 8 and "ARITH" in e.value.message


def test_renderer_state_machine_without_gpu(native):
    import chaos_gb300 as cg

    r = cg.Renderer(cg.Module("mandelbrot"))
    model = cg.RenderingModel(left_bottom_x=-2, left_bottom_y=-1, right_top_x=1, right_top_y=1, max_iterations=100,
                              max_super_sampling=1)
    with pytest.raises(cg.ChaosError) as e:
        r.render_quality(model)
    assert e.value.code == 5 and "initialized first" in e.value.message
    with pytest.raises(cg.ChaosError) as e:
        r.free_resources()
    assert e.value.code == 5


def test_struct_layouts_match_header(native, tmp_path):
    """ctypes layouts of the ABI structs equal what the C compiler computes from the header."""
    import shutil
    import subprocess

    import chaos_gb300 as cg

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"chaos_rendering_model": cg.RenderingModel, "chaos_frame_desc": cg.FrameDesc,
               "chaos_frame_out": cg.FrameOut, "chaos_viewport": cg.Viewport, "chaos_batch_config": cg.BatchConfig,
               "chaos_session_desc": cg.SessionDesc, "chaos_frame_record": cg.FrameRecord}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append('printf("chaos_pixel_info size %zu\\n", sizeof(chaos_pixel_info));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        *key, val = line.split()
        got[tuple(key)] = int(val)
    assert got[("chaos_pixel_info", "size")] == 16
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_newton_module_params(native):
    import chaos_gb300 as cg
    for name, shown in (("newton_generic", "newton generic"), ("newton colored by iterations",
                                                              "newton colored by iterations")):
        m = cg.Module(name)
        assert m.fractal_name == shown
        assert m.default_view()[3] == 200
        m.set_custom_params('{ "coefficients" : [1, 0, -2, 2], "roots" : [ [-1.7692923542386314,0], '
                            '[0.884646177119315707620204,0.589742805022205501647280] , '
                            '[0.884646177119315707,-0.589742805022205501] ] }')
        for bad, msg in (('{"coefficients": [1, 2, 3], "roots": [[1,0],[2,0],[3,0]]}', "4 coefficients"),
                         ('{"coefficients": [1, 2, 3, 4], "roots": [[1,0],[2,0]]}', "3 roots"),
                         ('{"coefficients": [1, 2, 3, 4], "roots": [[1,0],[2],[3,0]]}', "[real, imag]"),
                         ('not json', "JSON")):
            with pytest.raises(cg.ChaosError) as e:
                m.set_custom_params(bad)
            assert msg in e.value.message
        m.write_constant("roots", np.zeros(6).tobytes())
        m.write_constant("coefficients", np.zeros(4).tobytes())
        with pytest.raises(cg.ChaosError):
            m.write_constant("roots", np.zeros(3).tobytes())
    it = cg.Module("newton_iterations")
    it.write_constant("colorMagnifier", np.int32(5).tobytes())
    it.set_custom_params('{"colorMagnifier": 3, "coefficients": [1, 0, 0, -1], "roots": [[1,0],[-0.5,0.8],[-0.5,-0.8]]}')
    w = cg.Module("newton wired")
    w.set_custom_params("anything")  # ModuleNewtonWired ignores its parameters
    with pytest.raises(cg.ChaosError) as e:
        w.write_constant("roots", np.zeros(6).tobytes())
    assert e.value.code == 4


def test_pixel_divmod_by_magic_number():
    """The kernels split a pixel index n into (n / w, n % w) as q = mulhi(n,
    floor(2^32 / w)) plus one correction (chaos_device.cuh divmod_magic):
    exact for every 32-bit n, here on random and edge cases."""
    import random
    rng = random.Random(3)
    divisors = [1, 2, 3, 7, 255, 256, 1000, 1023, 1920, 3840, 4095, 65535, 65536, 99991, 2**31 - 1, 2**31, 2**32 - 1]
    divisors += [rng.randrange(1, 1 << 20) for _ in range(200)]
    for d in divisors:
        m = 0xFFFFFFFF if d <= 1 else (1 << 32) // d
        for n in [0, 1, d - 1, d, d + 1, 2**31 - 1, 2**32 - 1] + [rng.randrange(0, 1 << 32) for _ in range(50)]:
            n &= 0xFFFFFFFF
            q = (n * m) >> 32
            r = (n - q * d) & 0xFFFFFFFF
            if r >= d:
                q += 1
                r -= d
            assert (q, r) == divmod(n, d), (n, d)
