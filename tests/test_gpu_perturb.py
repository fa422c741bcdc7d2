"""Deep-zoom tier (perturbation) against the high-precision oracle.

Escape counts of a perturbation frame are not bit-identical to any other
arithmetic; the bar is the escape-count mismatch rate against the oracle's
multi-word direct iteration at the same sample points (stated per test)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISIUREWICZ_I = ("0.0", "1.0")  # c = i: preperiodic, on the set boundary


def perturb_frame(cuda, orbit, w, h, max_iter, spp, mode, tier, ps, seed=3, palette=None):
    import chaos_gb300 as cg
    torch = cuda
    n = w * h
    counts = torch.zeros(n * spp, dtype=torch.int32, device="cuda:0")
    smooth = torch.zeros(n * spp, dtype=torch.float32, device="cuda:0")
    total = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    rebases = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    out = cg.FrameOut(counts=counts.data_ptr(), smooth=smooth.data_ptr(), total_iterations=total.data_ptr(),
                      rebases=rebases.data_ptr())
    if palette is not None:
        pal = torch.from_numpy(np.ascontiguousarray(palette, dtype=np.uint32).view(np.int32)).to("cuda:0")
        rgba = torch.zeros(n, dtype=torch.int32, device="cuda:0")
        out.rgba, out.palette, out.palette_len, out.interior_rgba = rgba.data_ptr(), pal.data_ptr(), len(palette), 0xFF000000
    desc = cg.FrameDesc(width=w, height=h, max_iterations=max_iter, samples_per_pixel=spp, sample_mode=mode,
                        tier=tier, fractal=cg.MANDELBROT, seed=seed, pixel_size=ps)
    cg.render_frame_perturb(desc, orbit, out)
    c = counts.cpu().numpy().view(np.uint32)
    assert int(total.item()) == int(c.astype(np.int64).sum())
    return c, smooth.cpu().numpy(), int(rebases.item())


def hp_counts(oracle, centre, w, h, spp, mode, seed, ps, bits, max_iter, pix=None):
    if pix is None:
        dcx, dcy = oracle.frame_offsets(w, h, spp, mode, seed, ps, 0, w * h)
    else:
        parts = [oracle.frame_offsets(w, h, spp, mode, seed, ps, int(p), 1) for p in pix]
        dcx = np.concatenate([p[0] for p in parts])
        dcy = np.concatenate([p[1] for p in parts])
    return oracle.hp_escape_batch(centre[0], centre[1], dcx, dcy, bits, max_iter)[0]


@pytest.mark.parametrize("span,bits", [(1e-60, 384), (1e-200, 832)])
def test_misiurewicz_deep_f64(cuda, oracle, span, bits):
    import chaos_gb300 as cg
    w, h, mi = 192, 108, 3000
    ps = span / w
    orbit = cg.Orbit(*MISIUREWICZ_I, bits, mi)
    assert orbit.info()["escaped_at"] == mi  # c = i never escapes
    got, _, _ = perturb_frame(cuda, orbit, w, h, mi, 1, cg.SAMPLES_JITTER, cg.TIER_PERTURB_F64, ps)
    want = hp_counts(oracle, MISIUREWICZ_I, w, h, 1, 1, 3, ps, bits, mi)
    rate = float((got != want).mean())
    assert rate <= 0.005, rate
    assert np.abs(got.astype(np.int64) - want).max() <= 2 or rate < 0.001


def test_shallow_f32_and_f64_match_hp(cuda, oracle):
    """Span 1e-6 at the premade view M1: binary32 differences track the oracle."""
    import chaos_gb300 as cg
    from fractions import Fraction
    w, h, mi, bits = 160, 90, 2000, 192
    ps = 1e-6 / w
    centre = (cg.to_hex_fixed(Fraction(-0.748), bits), cg.to_hex_fixed(Fraction(0.1), bits))
    orbit = cg.Orbit(*centre, bits, mi)
    want = hp_counts(oracle, centre, w, h, 2, 1, 9, ps, bits, mi)
    for tier, bar in ((cg.TIER_PERTURB_F64, 0.005), (cg.TIER_PERTURB_F32, 0.01)):
        got, _, _ = perturb_frame(cuda, orbit, w, h, mi, 2, cg.SAMPLES_JITTER, tier, ps, seed=9)
        rate = float((got != want).mean())
        assert rate <= bar, (tier, rate)


def test_rebasing_when_reference_escapes(cuda, oracle):
    """A centre outside the set: its orbit ends early, so interior samples must
    rebase to the orbit start to keep going."""
    import chaos_gb300 as cg
    from fractions import Fraction
    w, h, mi, bits = 128, 96, 1500, 192
    centre = (cg.to_hex_fixed(Fraction(-0.7455), bits), cg.to_hex_fixed(Fraction(0.1133), bits))
    ps = 2e-3 / w
    orbit = cg.Orbit(*centre, bits, mi)
    info = orbit.info()
    want = hp_counts(oracle, centre, w, h, 1, 0, 0, ps, bits, mi)
    got, smooth, rebases = perturb_frame(cuda, orbit, w, h, mi, 1, cg.SAMPLES_CENTER, cg.TIER_PERTURB_F64, ps)
    assert rebases > 0
    assert float((got != want).mean()) <= 0.005
    assert info["escaped_at"] < mi or (want == mi).any()


def test_hp_golden_points_through_the_kernel(cuda, oracle):
    """The mpmath-pinned golden cases at c = i, rendered as 1x1 frames whose
    single sample sits at the case's offset (pixel centre of a 1x1 frame is the
    frame centre, so the orbit centre is shifted by the offset instead)."""
    import chaos_gb300 as cg
    cases = [c for c in json.load(open(os.path.join(os.path.dirname(__file__), "golden", "hp_golden.json")))["cases"]
             if c["centre"] == "misiurewicz-i"]
    from fractions import Fraction
    for c in cases:
        cx = cg.to_hex_fixed(Fraction(c["dcx"]), c["bits"])
        cy = cg.to_hex_fixed(1 + Fraction(c["dcy"]), c["bits"])
        orbit = cg.Orbit(cx, cy, c["bits"], c["max_iter"])
        got, _, _ = perturb_frame(cuda, orbit, 1, 1, c["max_iter"], 1, cg.SAMPLES_CENTER, cg.TIER_PERTURB_F64,
                                  c["span"] / 1920)
        assert int(got[0]) == c["count"]
