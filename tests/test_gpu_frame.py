"""GPU parity of the frame path (chaos_render_frame) against the oracle.

Escape counts and pixel-iteration totals: bit-exact (same arithmetic, FMA or
not, on both sides).  Smooth values: within 2 ulp of the value + 2e-6 (CUDA's
log2f and the C library's may differ in the last place).  RGBA: every channel
within 1 LSB (a last-place difference in the smooth value can move a rounding
boundary of the interpolated palette)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle.oracle import JULIA, MANDELBROT  # noqa: E402


def run_frame(cuda, w, h, max_iter, spp, mode, tier, arith, fractal=0, seed=0, center=(-0.5, 0.0), ps=None,
              julia_c=(0.0, 0.0), palette=None, interior=0xFF000000, stream=None):
    import chaos_gb300 as cg
    torch = cuda
    n = w * h
    counts = torch.zeros(n * spp, dtype=torch.int32, device="cuda:0")
    smooth = torch.zeros(n * spp, dtype=torch.float32, device="cuda:0")
    pitch = 16 * w + 64
    pix = torch.zeros((h, pitch), dtype=torch.uint8, device="cuda:0")
    total = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    out = cg.FrameOut(counts=counts.data_ptr(), smooth=smooth.data_ptr(), pixels=pix.data_ptr(), pixels_pitch=pitch,
                      total_iterations=total.data_ptr())
    rgba = None
    if palette is not None:
        pal = torch.from_numpy(np.ascontiguousarray(palette, dtype=np.uint32).view(np.int32)).to("cuda:0")
        rgba = torch.zeros(n, dtype=torch.int32, device="cuda:0")
        out.rgba, out.palette, out.palette_len, out.interior_rgba = rgba.data_ptr(), pal.data_ptr(), len(palette), interior
    desc = cg.FrameDesc(width=w, height=h, max_iterations=max_iter, samples_per_pixel=spp, sample_mode=mode, tier=tier,
                        arith=arith, fractal=fractal, seed=seed, center_x=center[0], center_y=center[1],
                        pixel_size=ps if ps is not None else 3.0 / w, julia_cx=julia_c[0], julia_cy=julia_c[1])
    cg.render_frame(desc, out, stream=stream)
    from tests.gpu_util import read_pixels
    return {"counts": counts.cpu().numpy().view(np.uint32).reshape(n, spp),
            "smooth": smooth.cpu().numpy().reshape(n, spp),
            "pixels": read_pixels(pix, w).reshape(n),
            "rgba": rgba.cpu().numpy().view(np.uint32) if rgba is not None else None,
            "total": int(total.item())}


def check_smooth(a, b):
    tol = 2 * np.spacing(np.abs(b).astype(np.float32)) + 2e-6
    bad = np.abs(a - b) > tol
    assert not bad.any(), (int(bad.sum()), a[bad][:5], b[bad][:5])


def check_rgba(a, b):
    da = a.view(np.uint8).astype(np.int16)
    db = b.view(np.uint8).astype(np.int16)
    assert np.abs(da - db).max() <= 1
    assert (a != b).mean() < 0.01


@pytest.mark.parametrize("tier,total,interior", [(0, 181_032_650, 175_986), (1, 181_040_256, 176_008)])
def test_c1_known_answer_parity(cuda, oracle, tier, total, interior):
    """C1 (1024^2 pixel centres of [-2,1]x[-1.5,1.5], maxIter 1000) with rounded
    arithmetic reproduces the reference's own totals."""
    import chaos_gb300 as cg
    g = run_frame(cuda, 1024, 1024, 1000, 1, cg.SAMPLES_CENTER, tier, cg.ARITH_PARITY)
    assert g["total"] == total
    assert int((g["counts"] == 1000).sum()) == interior
    o = oracle.frame(1024, 1024, 1000, 1, 0, tier == 1, cg.ARITH_PARITY, MANDELBROT, 0, (-0.5, 0.0), 3.0 / 1024)
    assert np.array_equal(g["counts"], o["counts"])
    check_smooth(g["smooth"], o["smooth"])


@pytest.mark.parametrize("tier", [0, 1])
def test_c1_fma_matches_oracle(cuda, oracle, tier):
    import chaos_gb300 as cg
    g = run_frame(cuda, 1024, 1024, 1000, 1, cg.SAMPLES_CENTER, tier, cg.ARITH_FMA)
    o = oracle.frame(1024, 1024, 1000, 1, 0, tier == 1, cg.ARITH_FMA, MANDELBROT, 0, (-0.5, 0.0), 3.0 / 1024)
    assert np.array_equal(g["counts"], o["counts"])
    assert g["total"] == o["total"]


@pytest.mark.parametrize("tier", [0, 1])
@pytest.mark.parametrize("arith", [0, 1])
def test_jittered_frame_with_palette(cuda, oracle, tier, arith):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(256, seed=11)
    w, h, spp, mi = 333, 201, 4, 2000
    center, ps = (-0.748, 0.1), 0.0014 / 201
    g = run_frame(cuda, w, h, mi, spp, cg.SAMPLES_JITTER, tier, arith, seed=1234, center=center, ps=ps, palette=pal)
    o = oracle.frame(w, h, mi, spp, 1, tier == 1, arith, MANDELBROT, 1234, center, ps, palette=pal)
    assert np.array_equal(g["counts"], o["counts"])
    assert g["total"] == o["total"]
    check_smooth(g["smooth"], o["smooth"])
    assert np.array_equal(g["pixels"]["weight"], o["pixels"]["weight"])
    check_smooth(g["pixels"]["value"], o["pixels"]["value"])
    check_rgba(g["rgba"], o["rgba"])


def test_julia_frame_and_stream(cuda, oracle):
    import chaos_gb300 as cg
    torch = cuda
    s = torch.cuda.Stream()
    g = run_frame(cuda, 400, 300, 900, 1, cg.SAMPLES_CENTER, cg.TIER_F32, cg.ARITH_FMA, fractal=JULIA,
                  center=(0.0, 0.0), ps=3.0 / 400, julia_c=(-0.8, 0.156), stream=s)
    o = oracle.frame(400, 300, 900, 1, 0, False, cg.ARITH_FMA, JULIA, 0, (0.0, 0.0), 3.0 / 400, julia_c=(-0.8, 0.156))
    assert np.array_equal(g["counts"], o["counts"])


def test_tiny_and_ragged_frames(cuda, oracle):
    import chaos_gb300 as cg
    for w, h in [(1, 1), (1, 37), (33, 1), (7, 5)]:
        g = run_frame(cuda, w, h, 300, 3, cg.SAMPLES_JITTER, cg.TIER_F32, cg.ARITH_FMA, seed=5, ps=0.01)
        o = oracle.frame(w, h, 300, 3, 1, False, cg.ARITH_FMA, MANDELBROT, 5, (-0.5, 0.0), 0.01)
        assert np.array_equal(g["counts"], o["counts"]), (w, h)


@pytest.mark.parametrize("center", [(0.0, 0.0), (-0.75, 0.0), (-1.25, 0.0), (0.0, 0.75)])
@pytest.mark.parametrize("tier", [0, 1])
@pytest.mark.parametrize("arith", [0, 1])
def test_axis_pixels_exact(cuda, oracle, center, tier, arith):
    """Odd-sized frames whose middle row and column sit exactly on the axes
    (c = x + 0i, c = 0 + iy): x or x*y is exactly 0 on every step there, the
    case where the binary64 kernels fall back from the fused six-op rounded
    step and the integer doubling to the literal step."""
    import chaos_gb300 as cg
    w, h, mi = 101, 77, 700
    ps = 0.9 / w
    g = run_frame(cuda, w, h, mi, 1, cg.SAMPLES_CENTER, tier, arith, center=center, ps=ps)
    o = oracle.frame(w, h, mi, 1, 0, tier == 1, arith, MANDELBROT, 0, center, ps)
    assert np.array_equal(g["counts"], o["counts"])
    assert g["total"] == int(o["counts"].astype(np.int64).sum())


@pytest.mark.parametrize("arith", [0, 1])
def test_julia_through_origin_exact(cuda, oracle, arith):
    """Julia frames whose pixel grid contains z0 = 0 and the axes."""
    import chaos_gb300 as cg
    w, h = 81, 61
    for jc in ((-0.8, 0.156), (0.0, 0.8), (-1.0, 0.0)):
        g = run_frame(cuda, w, h, 500, 1, cg.SAMPLES_CENTER, cg.TIER_F64, arith, fractal=JULIA, center=(0.0, 0.0),
                      ps=3.0 / w, julia_c=jc)
        o = oracle.frame(w, h, 500, 1, 0, True, arith, JULIA, 0, (0.0, 0.0), 3.0 / w, julia_c=jc)
        assert np.array_equal(g["counts"], o["counts"]), jc


@pytest.mark.parametrize("tier", [0, 1])
def test_c1_cycles_skip_iterations_not_counts(cuda, tier):
    """Most C1 interior pixels settle on an exact cycle of the rounded
    iteration: the frame kernel stops them at a repeated state and reports the
    iterations it did not run apart, while the counts (and so the reference's
    known answer) stay the same."""
    import chaos_gb300 as cg
    torch = cuda
    n = 1024 * 1024
    counts = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    total = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    skipped = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    desc = cg.FrameDesc(width=1024, height=1024, max_iterations=1000, samples_per_pixel=1,
                        sample_mode=cg.SAMPLES_CENTER, tier=tier, arith=cg.ARITH_PARITY, fractal=cg.MANDELBROT,
                        seed=0, center_x=-0.5, center_y=0.0, pixel_size=3.0 / 1024)
    cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr(), total_iterations=total.data_ptr(),
                                      cycle_skipped=skipped.data_ptr()))
    want_total, want_interior = (181_032_650, 175_986) if tier == 0 else (181_040_256, 176_008)
    assert int(total.item()) == want_total
    assert int((counts.cpu().numpy() == 1000).sum()) == want_interior
    # binary32 cycles show up sooner (fewer states; a checkpoint every 16 steps
    # against every 128 in binary64): more than half, resp. a third, of the
    # work (a numpy restatement of the binary64 checkpoints gives 69,847,176)
    assert int(skipped.item()) > (want_total // 2 if tier == 0 else want_total // 3)
