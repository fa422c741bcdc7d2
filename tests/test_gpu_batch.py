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


@pytest.mark.parametrize("threads,block", [(128, 8), (512, 32), (64, 16)])
def test_batch_launch_config_does_not_change_results(cuda, oracle, threads, block):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(64, seed=1)
    cfg = cg.BatchConfig((threads, threads, threads), (block, block, block))
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
