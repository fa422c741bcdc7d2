"""Batched viewports (chaos_batch_*): one CUDA-graph launch over viewports of
uneven size, iteration limit and precision tier, against the oracle's
restatement per viewport.  Escape counts and totals bit-exact; smooth values
within 2 ulp + 2e-6; RGBA within 1 LSB."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (w, h, spp, mode, max_iter, tier, centre, span)
VIEWS = [
    (96, 64, 1, 0, 800, 255, (-0.5, 0.0), 3.0),              # auto -> binary32
    (64, 48, 2, 1, 2500, 255, (-0.748, 0.1), 1.4e-5),        # auto -> float-float
    (80, 40, 1, 1, 3000, 255, (-0.74364388703715, 0.13182590420531), 8e-12),  # auto -> binary64
    (33, 17, 3, 1, 1200, 0, (-0.235125, 0.827215), 4e-4),     # forced binary32
    (40, 30, 1, 0, 1500, 2, (-0.925, 0.266), 3e-3),           # forced float-float
    (8, 8, 1, 0, 500, 1, (0.3, 0.02), 0.5),                   # forced binary64
    (128, 72, 1, 0, 4000, 255, (-0.57675236, 0.4625193), 3e-8),
    (1, 1, 4, 1, 100, 255, (-1.95, 0.0), 1e-3),               # |c| > 1.9975 corner: every step tested
]


def build(cuda, views, palette, config=None):
    import chaos_gb300 as cg
    torch = cuda
    bufs, vps = [], []
    for w, h, spp, mode, mi, tier, c, span in views:
        counts = torch.zeros(w * h * spp, dtype=torch.int32, device="cuda:0")
        smooth = torch.zeros(w * h * spp, dtype=torch.float32, device="cuda:0")
        rgba = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
        bufs.append((counts, smooth, rgba))
        vps.append(cg.Viewport(width=w, height=h, max_iterations=mi, samples_per_pixel=spp, sample_mode=mode,
                               tier=tier, seed=17 + w, center_x=c[0], center_y=c[1], pixel_size=span / w,
                               counts=counts.data_ptr(), smooth=smooth.data_ptr(), rgba=rgba.data_ptr()))
    pal = torch.from_numpy(np.ascontiguousarray(palette, dtype=np.uint32).view(np.int32)).to("cuda:0")
    b = cg.Batch(vps, pal.data_ptr(), len(palette), 0xFF000000, config)
    return b, bufs, pal


def run(cuda, b, bufs):
    torch = cuda
    b.launch()
    torch.cuda.synchronize()
    return [(c.cpu().numpy().view(np.uint32), s.cpu().numpy(), r.cpu().numpy().view(np.uint32)) for c, s, r in bufs]


def test_batch_matches_oracle(cuda, oracle):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(256, seed=5)
    b, bufs, _ = build(cuda, VIEWS, pal)
    tiers = b.tiers()
    want_tiers = [cg.auto_tier(v[6][0], v[6][1], v[7] / v[0]) if v[5] == 255 else v[5] for v in VIEWS]
    assert tiers == want_tiers
    assert tiers[0] == cg.TIER_F32 and tiers[1] == cg.TIER_FLOATFLOAT and tiers[2] == cg.TIER_F64
    got = run(cuda, b, bufs)
    for k, ((w, h, spp, mode, mi, _, c, span), (counts, smooth, rgba)) in enumerate(zip(VIEWS, got)):
        o = oracle.batch_viewport(w, h, spp, mode, mi, tiers[k], 17 + w, c, span / w, palette=pal)
        assert np.array_equal(counts, o["counts"]), (k, int((counts != o["counts"]).sum()))
        tol = 2 * np.spacing(np.abs(o["smooth"])) + 2e-6
        assert (np.abs(smooth - o["smooth"]) <= tol).all(), k
        d = np.abs(rgba.view(np.uint8).astype(int) - o["rgba"].view(np.uint8).astype(int))
        assert d.max() <= 1, k
    assert b.read_total() == sum(int(c.astype(np.int64).sum()) for c, _, _ in got)
    # the graph relaunches to the same result
    again = run(cuda, b, bufs)
    for (c1, s1, r1), (c2, s2, r2) in zip(got, again):
        assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    b.close()


@pytest.mark.parametrize("threads,block,chunk", [(128, 8, 4), (512, 32, 1), (64, 16, 16)])
def test_batch_launch_config_does_not_change_results(cuda, oracle, threads, block, chunk):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(64, seed=1)
    cfg = cg.BatchConfig((threads, threads, threads), (block, block, block), (chunk, chunk, chunk))
    b, bufs, _ = build(cuda, VIEWS[:6], pal, cfg)
    got = run(cuda, b, bufs)
    b2, bufs2, _ = build(cuda, VIEWS[:6], pal)
    ref = run(cuda, b2, bufs2)
    for (c1, _, r1), (c2, _, r2) in zip(got, ref):
        assert np.array_equal(c1, c2) and np.array_equal(r1, r2)


def test_batch_rejects_bad_config(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    with pytest.raises(cg.ChaosError):
        build(cuda, VIEWS[:2], seeded_palette(16), cg.BatchConfig((100, 0, 0), (0, 0, 0)))
    with pytest.raises(cg.ChaosError):
        build(cuda, VIEWS[:2], seeded_palette(16), cg.BatchConfig((0, 0, 0), (12, 0, 0)))
    with pytest.raises(cg.ChaosError):
        build(cuda, VIEWS[:2], seeded_palette(16), cg.BatchConfig((0, 0, 0), (0, 0, 0), (0, 65, 0)))


# binary64 rounded as the reference's computeFractal<double> (tier 5), beside a
# binary32 viewport; the 31x31 view has a sample row on the real axis (y = 0,
# products 0: the literal-step redo)
ROUNDED_VIEWS = [
    (80, 40, 1, 1, 3000, 5, (-0.74364388703715, 0.13182590420531), 8e-12),
    (64, 48, 2, 1, 2500, 5, (-0.748, 0.1), 1.4e-5),
    (40, 30, 1, 0, 1500, 5, (-0.925, 0.266), 3e-3),
    (31, 31, 1, 0, 800, 5, (-0.5, 0.0), 2.5),
    (1, 1, 4, 1, 100, 5, (-1.95, 0.0), 1e-3),
    (33, 17, 3, 1, 1200, 0, (-0.235125, 0.827215), 4e-4),
]


def test_batch_rounded_binary64_matches_oracle(cuda, oracle):
    """Tier F64_ROUNDED gives the FP64 oracle's escape counts bit for bit."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(256, seed=3)
    b, bufs, _ = build(cuda, ROUNDED_VIEWS, pal)
    assert b.tiers() == [cg.TIER_F64_ROUNDED] * 5 + [cg.TIER_F32]
    got = run(cuda, b, bufs)
    for k, ((w, h, spp, mode, mi, tier, c, span), (counts, smooth, rgba)) in enumerate(zip(ROUNDED_VIEWS, got)):
        o = oracle.batch_viewport(w, h, spp, mode, mi, tier, 17 + w, c, span / w, palette=pal)
        assert np.array_equal(counts, o["counts"]), (k, int((counts != o["counts"]).sum()))
        tol = 2 * np.spacing(np.abs(o["smooth"])) + 2e-6
        assert (np.abs(smooth - o["smooth"]) <= tol).all(), k
        d = np.abs(rgba.view(np.uint8).astype(int) - o["rgba"].view(np.uint8).astype(int))
        assert d.max() <= 1, k
    assert b.read_total() == sum(int(c.astype(np.int64).sum()) for c, _, _ in got)
    b.close()


def test_floatfloat_tier_accuracy_against_rounded_binary64(cuda):
    """Float-float (about 48 bits) on views where that is ample: its escape
    counts differ from the FP64 oracle's (the rounded binary64 tier) on few
    pixels, no more than the fused binary64 tier's do plus a small margin.  A
    broken double-word step (one that drops its normalisation, for instance)
    shows up here even though it would still match its own restatement."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    views = [(128, 96, 1, 0, 2000, (-0.748, 0.1), 1.4e-5),
             (96, 96, 1, 0, 3000, (-0.925, 0.266), 3e-4),
             (128, 64, 1, 0, 3000, (-0.74364388703715, 0.13182590420531), 1e-9)]
    pal = seeded_palette(16)
    counts = {}
    for tier in (cg.TIER_FLOATFLOAT, cg.TIER_F64, cg.TIER_F64_ROUNDED):
        b, bufs, _ = build(cuda, [(w, h, spp, m, mi, tier, c, sp) for w, h, spp, m, mi, c, sp in views], pal)
        counts[tier] = [c for c, _, _ in run(cuda, b, bufs)]
        b.close()
    n = sum(len(c) for c in counts[cg.TIER_F64_ROUNDED])

    def mismatch(t):
        return sum(int((a != r).sum()) for a, r in zip(counts[t], counts[cg.TIER_F64_ROUNDED])) / n

    ff, fused = mismatch(cg.TIER_FLOATFLOAT), mismatch(cg.TIER_F64)
    print("float-float / fused binary64 mismatch vs rounded binary64:", ff, fused)
    assert ff <= 2 * fused + 0.01, (ff, fused)


def test_batch_rejects_mixed_binary64_arithmetic(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    views = [(8, 8, 1, 0, 100, cg.TIER_F64, (0.3, 0.02), 0.5), (8, 8, 1, 0, 100, cg.TIER_F64_ROUNDED, (0.3, 0.02), 0.5)]
    with pytest.raises(cg.ChaosError):
        build(cuda, views, seeded_palette(16))


def test_autotune_picks_a_shape_and_caches_it(cuda, tmp_path):
    """The autotuner returns a shape from its search space for each tier slot
    present, the batch built with it gives the default shape's bits, and a
    second call with the same cache file times nothing."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(64, seed=2)
    views = VIEWS[:6]
    b, bufs, _ = build(cuda, views, pal)
    ref = run(cuda, b, bufs)
    tiers = b.tiers()
    b.close()
    cache = str(tmp_path / "tune.txt")
    vps = [cg.Viewport(width=w, height=h, max_iterations=mi, samples_per_pixel=spp, sample_mode=mode, tier=t,
                       seed=17 + w, center_x=c[0], center_y=c[1], pixel_size=span / w)
           for w, h, spp, mode, mi, t, c, span in views]
    cfg, hit = cg.autotune_batch(vps, cache)
    assert not hit
    slots = {0: 0, 2: 1, 1: 2}  # tier id -> config slot
    for t in set(tiers):
        k = slots[t]
        assert cfg.block_threads[k] in (128, 256, 512) and cfg.escape_block[k] in (8, 16, 32)
        assert cfg.chunk[k] in (1, 2, 4)
    assert cfg.fp64_warps_per_sm in (8, 12, 16)  # binary64 shares the batch with other tiers here
    cfg2, hit2 = cg.autotune_batch(vps, cache)
    assert hit2 and bytes(cfg2) == bytes(cfg)
    assert len(open(cache).read().splitlines()) == len(set(tiers)) + 1  # + the shared launch
    b2, bufs2, _ = build(cuda, views, pal, cfg)
    got = run(cuda, b2, bufs2)
    for (c1, _, r1), (c2, _, r2) in zip(ref, got):
        assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    b2.close()


DEEP_VIEWS = [
    (64, 36, 1, 0, 600, 254, (-0.5, 0.0), 3.0),                                 # auto-deep -> binary32
    (48, 32, 1, 1, 2000, 254, (-0.748, 0.1), 1.4e-5),                           # auto-deep -> float-float
    (80, 45, 1, 1, 3000, 254, (-0.74364388703715, 0.13182590420531), 8e-12),    # auto-deep -> perturbation, binary32
    (40, 24, 2, 1, 3000, 4, (0.0, 1.0), 4e-36),                                   # forced perturbation, binary64 (c = i)
]


def orbit_bits(ps):
    """The orbit precision a batch picks for a perturbation viewport: -log2(pixel) + 96 bits, in 64-bit words."""
    import math
    return int(min(1536, max(128, math.ceil((-math.log2(ps) + 96) / 64) * 64)))


def test_batch_perturbation_matches_single_frames(cuda):
    """Perturbation viewports inside a batch graph give the same bits as the
    single-frame perturbation entry point with an orbit of the same centre and
    precision (that entry point is held to the multi-word oracle by its own
    tests); the other tiers still match plain batches."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    torch = cuda
    pal = seeded_palette(128, seed=9)
    b, bufs, dpal = build(cuda, DEEP_VIEWS, pal)
    tiers = b.tiers()
    assert tiers == [cg.TIER_F32, cg.TIER_FLOATFLOAT, cg.TIER_PERTURB_F32, cg.TIER_PERTURB_F64]
    got = run(cuda, b, bufs)
    for k in (2, 3):
        w, h, spp, mode, mi, _, c, span = DEEP_VIEWS[k]
        ps = span / w
        bits = orbit_bits(ps)
        orbit = cg.Orbit(cg.to_hex_fixed(c[0], bits), cg.to_hex_fixed(c[1], bits), bits, mi)
        counts = torch.zeros(w * h * spp, dtype=torch.int32, device="cuda:0")
        smooth = torch.zeros(w * h * spp, dtype=torch.float32, device="cuda:0")
        rgba = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
        out = cg.FrameOut(counts=counts.data_ptr(), smooth=smooth.data_ptr(), rgba=rgba.data_ptr(),
                          palette=dpal.data_ptr(), palette_len=len(pal), interior_rgba=0xFF000000)
        desc = cg.FrameDesc(width=w, height=h, max_iterations=mi, samples_per_pixel=spp, sample_mode=mode,
                            tier=tiers[k], fractal=cg.MANDELBROT, seed=17 + w, pixel_size=ps)
        cg.render_frame_perturb(desc, orbit, out)
        orbit.close()
        gc, gs, gr = got[k]
        assert np.array_equal(gc, counts.cpu().numpy().view(np.uint32)), k
        assert np.array_equal(gs.view(np.uint32), smooth.cpu().numpy().view(np.uint32)), k
        assert np.array_equal(gr, rgba.cpu().numpy().view(np.uint32)), k
        assert len(np.unique(gc)) > 4, k  # the view shows structure
    # the shallow viewports equal the same viewports in a plain batch
    b2, bufs2, _ = build(cuda, [v[:5] + (255,) + v[6:] for v in DEEP_VIEWS[:2]], pal)
    ref = run(cuda, b2, bufs2)
    for (c1, _, r1), (c2, _, r2) in zip(got[:2], ref):
        assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    assert b.read_total() == sum(int(c.astype(np.int64).sum()) for c, _, _ in got)
    again = run(cuda, b, bufs)
    for (c1, _, _), (c2, _, _) in zip(got, again):
        assert np.array_equal(c1, c2)
    b.close()
    b2.close()


def test_batch_rejects_perturbation_below_binary64_range(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    v = (16, 16, 1, 0, 100, cg.TIER_PERTURB_F32, (-0.74, 0.13), 1e-295 * 16)
    with pytest.raises(cg.ChaosError):
        build(cuda, [v], seeded_palette(16))


def test_c4_deep_viewports_against_multiword_oracle(cuda, oracle):
    """The C4 viewports that plain tier choice sends to binary64 (pixel below
    |c| * 2^-42), rendered by the binary64 tier and by perturbation, against the
    multi-word oracle at sampled pixels.  Near the set boundary at these depths
    binary64 iteration is itself off (the point c rounds to a double and the
    orbit is chaotic), so the bar is that perturbation, which keeps c exact,
    is no further from the oracle than binary64."""
    import chaos_gb300 as cg
    from chaos_gb300.workloads import c4_viewports
    torch = cuda
    specs = [s for s in c4_viewports()
             if cg.auto_tier(s["center"][0], s["center"][1], s["span"] / s["width"]) == cg.TIER_F64]
    assert len(specs) == 9
    views = [(s["width"], s["height"], 1, cg.SAMPLES_CENTER, s["max_iter"], 0, s["center"], s["span"]) for s in specs]
    rates = {}
    for tier in (cg.TIER_F64, cg.TIER_AUTO_DEEP):
        bufs, vps = [], []
        for s, v in zip(specs, views):
            counts = torch.zeros(v[0] * v[1], dtype=torch.int32, device="cuda:0")
            bufs.append(counts)
            vps.append(cg.Viewport(width=v[0], height=v[1], max_iterations=v[4], samples_per_pixel=1,
                                   sample_mode=cg.SAMPLES_CENTER, tier=tier, seed=s["seed"], center_x=v[6][0],
                                   center_y=v[6][1], pixel_size=v[7] / v[0], counts=counts.data_ptr()))
        b = cg.Batch(vps)
        b.launch()
        torch.cuda.synchronize()
        bad = n = 0
        for s, v, counts in zip(specs, views, bufs):
            w, h, ps = v[0], v[1], v[7] / v[0]
            pix = np.sort(np.random.default_rng(s["seed"]).choice(w * h, 384, replace=False))
            parts = [oracle.frame_offsets(w, h, 1, cg.SAMPLES_CENTER, s["seed"], ps, int(p), 1) for p in pix]
            bits = orbit_bits(ps) + 64
            want = oracle.hp_escape_batch(cg.to_hex_fixed(v[6][0], bits), cg.to_hex_fixed(v[6][1], bits),
                                          np.concatenate([p[0] for p in parts]),
                                          np.concatenate([p[1] for p in parts]), bits, v[4])[0]
            got = counts.cpu().numpy().view(np.uint32)[pix]
            bad += int((got != want).sum())
            n += len(pix)
        rates[tier] = bad / n
        b.close()
    print("c4 deep viewports, escape-count mismatch vs multi-word oracle:",
          {"f64": rates[cg.TIER_F64], "perturbation": rates[cg.TIER_AUTO_DEEP]})
    assert rates[cg.TIER_AUTO_DEEP] <= rates[cg.TIER_F64] + 0.01
