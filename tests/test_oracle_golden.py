"""The oracle against the reference's own outputs (committed golden vectors).

tests/golden/reference_golden.json was produced by the reference's
src/main/cuda/fractals/{mandelbrot,julia}.cu host-built by oracle/build_ref.sh
(tests/golden/make_golden.py).  These tests run on any CPU."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.oracle import ARITH_PARITY, JULIA, MANDELBROT

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.mark.parametrize("dbl,tag", [(0, "f32"), (1, "f64")])
def test_c1_known_answer(oracle, golden, dbl, tag):
    c1 = golden["c1"]
    total, counts = oracle.escape_grid(MANDELBROT, dbl, ARITH_PARITY, c1["w"], c1["h"], c1["x0"], c1["y0"], c1["dx"],
                                       c1["dy"], c1["max_iter"])
    assert int(total) == c1[f"total_{tag}"]
    assert int((counts == c1["max_iter"]).sum()) == c1[f"interior_{tag}"]
    assert hashlib.sha256(counts.astype("<u4").tobytes()).hexdigest() == c1[f"sha256_{tag}"]
    assert counts[300:332, 600:632].tolist() == c1[f"crop_{tag}"]


def test_c1_survey_numbers(golden):
    # the figures the survey measured with the reference's code (FP32 and FP64, no contraction)
    assert golden["c1"]["total_f32"] == 181_032_650 and golden["c1"]["interior_f32"] == 175_986
    assert golden["c1"]["total_f64"] == 181_040_256 and golden["c1"]["interior_f64"] == 176_008


def test_mandelbrot_points(oracle, golden):
    bad = []
    for p in golden["mandelbrot_points"]:
        f = oracle.compute_fractal(MANDELBROT, 0, ARITH_PARITY, p["max_iter"], np.float32(p["x"]), np.float32(p["y"]))
        d = oracle.compute_fractal(MANDELBROT, 1, ARITH_PARITY, p["max_iter"], p["x"], p["y"])
        if f != p["f32"] or d != p["f64"]:
            bad.append((p, f, d))
    assert not bad, bad[:5]


def test_julia_points(oracle, golden):
    bad = []
    for p in golden["julia_points"]:
        c = tuple(p["c"])
        f = oracle.compute_fractal(JULIA, 0, ARITH_PARITY, p["max_iter"], np.float32(p["x"]), np.float32(p["y"]), c)
        d = oracle.compute_fractal(JULIA, 1, ARITH_PARITY, p["max_iter"], p["x"], p["y"], c)
        if f != p["f32"] or d != p["f64"]:
            bad.append((p, f, d))
    assert not bad, bad[:5]


def test_colorize_default_palette(oracle, golden):
    from chaos_gb300.palette import default_palette

    pal = default_palette()
    assert hashlib.sha256(pal.astype("<u4").tobytes()).hexdigest() == golden["default_palette_sha256"]
    from oracle.oracle import PIXEL_DTYPE

    cases = golden["colorize_default_palette"]
    pix = np.zeros((1, len(cases)), dtype=PIXEL_DTYPE)
    pix["value"][0] = [c["value"] for c in cases]
    pix["weight"][0] = 1
    got = oracle.compose(pix, pal, 1.0)[0]
    assert got.tolist() == [c["rgba"] for c in cases]


def test_oracle_matches_reference_live(oracle, reference):
    """Where the reference builds on this host: extra random points, bit for bit."""
    rng = np.random.default_rng(7)
    xs = rng.uniform(-2.2, 0.8, 4000)
    ys = rng.uniform(-1.3, 1.3, 4000)
    for x, y in zip(xs, ys):
        for dbl in (0, 1):
            xv, yv = (x, y) if dbl else (np.float32(x), np.float32(y))
            assert oracle.compute_fractal(MANDELBROT, dbl, ARITH_PARITY, 500, xv, yv) == reference.mandelbrot(dbl, 500,
                                                                                                             xv, yv)
    c = (-0.8, 0.156)
    for x, y in zip(xs[:1000] * 0.6, ys[:1000]):
        for dbl in (0, 1):
            xv, yv = (x, y) if dbl else (np.float32(x), np.float32(y))
            assert oracle.compute_fractal(JULIA, dbl, ARITH_PARITY, 300, xv, yv, c) == reference.julia(dbl, 300, xv,
                                                                                                      yv, c)


def test_newton_points(oracle, golden):
    bad = []
    prms = golden["newton_params"]
    for p in golden["newton_points"]:
        prm = prms[p["params"]]
        oracle.set_newton(prm["roots"], prm["coefficients"], prm["magnifier"])
        f = oracle.compute_fractal(p["kind"], 0, 1, p["max_iter"], np.float32(p["x"]), np.float32(p["y"]))
        d = oracle.compute_fractal(p["kind"], 1, 1, p["max_iter"], p["x"], p["y"])
        if f != p["f32"] or d != p["f64"]:
            bad.append((p, f, d))
    oracle.set_newton()
    assert len(golden["newton_points"]) == 288 and not bad, bad[:5]


def test_newton_colorize(oracle, golden):
    from chaos_gb300.palette import default_palette
    from oracle.oracle import PIXEL_DTYPE
    pal = default_palette()
    for kind, mode, mag in ((2, 1, 1), (3, 1, 1), (4, 2, 11)):
        cases = [c for c in golden["newton_colorize"] if c["kind"] == kind]
        pix = np.zeros((1, len(cases)), dtype=PIXEL_DTYPE)
        pix["value"][0] = [c["value"] for c in cases]
        got = oracle.compose_mode(pix, pal, mode, mag)[0]
        assert got.tolist() == [c["rgba"] for c in cases], kind


def test_rounded_step_doubling_identity():
    """The kernels' rounded step computes (2x)*y + cy as fma(2, x*y, cy): equal
    whenever x*y rounds to at least 2^-1021 (the kernels take the literal form
    below that).  Checked on random and edge operands with the C library's fma."""
    import ctypes

    import numpy as np
    libm = ctypes.CDLL("libm.so.6")
    libm.fma.restype = ctypes.c_double
    libm.fma.argtypes = [ctypes.c_double] * 3
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-2, 2, 3000), rng.standard_normal(1000) * 1e-150,
                         np.ldexp(rng.uniform(1, 2, 1000), rng.integers(-520, -500, 1000))])
    ys = np.concatenate([rng.uniform(-2, 2, 3000), rng.standard_normal(1000) * 1e-150,
                         np.ldexp(rng.uniform(1, 2, 1000), rng.integers(-520, -500, 1000))])
    cys = np.concatenate([rng.uniform(-2, 2, 3000), rng.uniform(-1e-300, 1e-300, 1000),
                          np.ldexp(rng.uniform(-2, 2, 1000), rng.integers(-1030, -1000, 1000))])
    checked = 0
    for x, y, cy in zip(xs.tolist(), ys.tolist(), cys.tolist()):
        p = x * y
        if p != 0.0 and abs(p) < 2.0 ** -1021:
            continue  # the literal form runs there
        assert libm.fma(2.0, p, cy) == (2.0 * x) * y + cy, (x, y, cy)
        checked += 1
    assert checked > 4000


def test_rounded_batch_tier_is_the_reference_loop(oracle, reference):
    """The oracle's batch viewport in the rounded binary64 tier (5) gives the
    reference's computeFractal<double> counts at the same sample points.  The
    view is dyadic (pixel 2^-9, centre (-0.75, 0.09375)), so each sample point
    is one rounded add whether formed with an fma or not."""
    w = h = 48
    ps, cx, cy, mi = 2.0 ** -9, -0.75, 0.09375, 3000
    o = oracle.batch_viewport(w, h, 1, 0, mi, 5, 1, (cx, cy), ps)
    q = np.arange(w * h)
    xs = cx + ((q % w) + 0.5 - w / 2) * ps
    ys = cy - ((q // w) + 0.5 - h / 2) * ps
    total, want = reference.points_d(xs, ys, mi)
    assert np.array_equal(o["counts"], want)
    assert o["total"] == total
    assert 0 < (want == mi).sum() < len(want)  # interior and exterior both present


def test_contracted_oracle_matches_the_reference_default_build(oracle):
    """The oracle's ARITH_CONTRACTED restatement against pixel records the
    reference's own default (contraction-on) sm_103a build produced
    (tests/golden/contracted_golden.npz, tests/golden/make_contracted_golden.py):
    main frames at maxSS 1..17 and zoom steps with sample reuse, every record
    bit for bit."""
    import json
    import os
    from oracle.oracle import ARITH_CONTRACTED, MANDELBROT, PIXEL_DTYPE
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "contracted_golden.npz")
    g = np.load(path)
    meta = json.loads(g["meta"].tobytes().decode())
    for m in meta["main"]:
        got = oracle.render_main(MANDELBROT, m["dbl"], ARITH_CONTRACTED, m["w"], m["h"], tuple(m["rect"]),
                                 m["max_iter"], m["max_ss"], m["flags"])
        want = g[m["name"]]
        bad = (got.view(np.uint8).reshape(m["h"], m["w"], 16) != want).any(axis=2)
        assert not bad.any(), (m["name"], int(bad.sum()))
    for m in meta["advanced"]:
        prev = np.ascontiguousarray(g[m["name"] + "_prev"]).view(PIXEL_DTYPE).reshape(m["h"], m["w"])
        got = oracle.render_advanced(MANDELBROT, m["dbl"], ARITH_CONTRACTED, m["w"], m["h"], tuple(m["new"]),
                                     m["max_iter"], m["max_ss"], m["flags"], tuple(m["old"]), prev, tuple(m["focus"]))
        want = g[m["name"]]
        bad = (got.view(np.uint8).reshape(m["h"], m["w"], 16) != want).any(axis=2)
        assert not bad.any(), (m["name"], int(bad.sum()))
