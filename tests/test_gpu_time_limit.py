"""Time limits of the persistent kernels (frames, perturbation frames,
batches): a launch that runs past its limit stops at its warps' next round,
completes with CHAOS_ERR_TIMEOUT (synchronous calls) or STATUS_TIMEOUT in its
status word, and leaves the context usable: the next launch, without a limit,
matches the oracle."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# a deep binary64 view whose full frame takes ~0.5 s (every sample runs
# thousands of iterations and none cycles): the limits below end it early
DEEP_SEED, DEEP_SPAN, DEEP_MAX_ITER = 2, 1e-10, 20000
LIMIT_S = 0.02


def deep_desc(cg, w=1920, h=1080, limit=LIMIT_S):
    from chaos_gb300.workloads import boundary_point
    cx, cy = boundary_point(DEEP_SEED, max_iter=DEEP_MAX_ITER)
    return cg.FrameDesc(width=w, height=h, max_iterations=DEEP_MAX_ITER, samples_per_pixel=1,
                        sample_mode=cg.SAMPLES_CENTER, tier=cg.TIER_F64, arith=cg.ARITH_PARITY, fractal=cg.MANDELBROT,
                        seed=0, center_x=cx, center_y=cy, pixel_size=DEEP_SPAN / w, time_limit_s=limit)


def small_frame_matches_oracle(cuda, oracle):
    import chaos_gb300 as cg
    torch = cuda
    w, h, mi = 256, 192, 500
    counts = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
    desc = cg.FrameDesc(width=w, height=h, max_iterations=mi, samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                        tier=cg.TIER_F64, arith=cg.ARITH_PARITY, fractal=cg.MANDELBROT, seed=0, center_x=-0.5,
                        center_y=0.0, pixel_size=3.0 / w)
    cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr()))
    o = oracle.frame(w, h, mi, 1, 0, True, cg.ARITH_PARITY, cg.MANDELBROT, 0, (-0.5, 0.0), 3.0 / w)
    return np.array_equal(counts.cpu().numpy().view(np.uint32), o["counts"].reshape(-1))


def test_frame_time_limit_then_next_frame(cuda, oracle):
    import chaos_gb300 as cg
    torch = cuda
    desc = deep_desc(cg)
    counts = torch.zeros(desc.width * desc.height, dtype=torch.int32, device="cuda:0")
    out = cg.FrameOut(counts=counts.data_ptr())
    t0 = time.perf_counter()
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(desc, out)
    wall = time.perf_counter() - t0
    assert e.value.code == 7, e.value  # CHAOS_ERR_TIMEOUT
    assert wall < 0.3, wall  # the frame alone takes ~0.5 s
    assert small_frame_matches_oracle(cuda, oracle)


def test_frame_time_limit_async_status_word(cuda, oracle):
    import chaos_gb300 as cg
    torch = cuda
    desc = deep_desc(cg)
    counts = torch.zeros(desc.width * desc.height, dtype=torch.int32, device="cuda:0")
    # an unsynchronised frame with a limit needs a status word
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr()), sync=False)
    assert e.value.code == 1  # CHAOS_ERR_INVALID_ARGUMENT
    status = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr(), status=status.data_ptr()), sync=False)
    torch.cuda.synchronize()
    assert int(status.item()) & cg.STATUS_TIMEOUT
    assert small_frame_matches_oracle(cuda, oracle)


def test_frame_within_its_limit_is_complete(cuda, oracle):
    """A limit the frame stays inside changes nothing."""
    import chaos_gb300 as cg
    torch = cuda
    w, h, mi = 320, 200, 1000
    counts = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
    total = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    desc = cg.FrameDesc(width=w, height=h, max_iterations=mi, samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                        tier=cg.TIER_F32, arith=cg.ARITH_FMA, fractal=cg.MANDELBROT, seed=0, center_x=-0.5,
                        center_y=0.0, pixel_size=3.0 / w, time_limit_s=30.0)
    cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr(), total_iterations=total.data_ptr()))
    o = oracle.frame(w, h, mi, 1, 0, False, cg.ARITH_FMA, cg.MANDELBROT, 0, (-0.5, 0.0), 3.0 / w)
    assert np.array_equal(counts.cpu().numpy().view(np.uint32), o["counts"].reshape(-1))
    assert int(total.item()) == o["total"]


def test_frame_rejects_a_negative_limit(cuda):
    import chaos_gb300 as cg
    torch = cuda
    counts = torch.zeros(64, dtype=torch.int32, device="cuda:0")
    desc = deep_desc(cg, w=8, h=8, limit=-1.0)
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame(desc, cg.FrameOut(counts=counts.data_ptr()))
    assert e.value.code == 1  # CHAOS_ERR_INVALID_ARGUMENT


def test_perturbation_frame_time_limit(cuda, oracle):
    import chaos_gb300 as cg
    torch = cuda
    w = h = 2048
    orbit = cg.Orbit("0.0", "1.0", 384, 3000)  # c = i, preperiodic
    counts = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
    desc = cg.FrameDesc(width=w, height=h, max_iterations=3000, samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                        tier=cg.TIER_PERTURB_F64, fractal=cg.MANDELBROT, seed=0, pixel_size=1e-60 / w,
                        time_limit_s=1e-4)
    with pytest.raises(cg.ChaosError) as e:
        cg.render_frame_perturb(desc, orbit, cg.FrameOut(counts=counts.data_ptr()))
    assert e.value.code == 7
    assert small_frame_matches_oracle(cuda, oracle)


def test_batch_time_limit_then_next_batch(cuda, oracle):
    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    from chaos_gb300.workloads import boundary_point
    torch = cuda
    pal = seeded_palette(256, seed=5)
    dpal = torch.from_numpy(np.ascontiguousarray(pal, dtype=np.uint32).view(np.int32)).to("cuda:0")
    cx, cy = boundary_point(DEEP_SEED, max_iter=DEEP_MAX_ITER)
    w, h = 1920, 1080
    counts = torch.zeros(w * h, dtype=torch.int32, device="cuda:0")
    heavy = [cg.Viewport(width=w, height=h, max_iterations=DEEP_MAX_ITER, samples_per_pixel=1,
                         sample_mode=cg.SAMPLES_CENTER, tier=cg.TIER_F64_ROUNDED, seed=1, center_x=cx, center_y=cy,
                         pixel_size=DEEP_SPAN / w, counts=counts.data_ptr())]
    b = cg.Batch(heavy, dpal.data_ptr(), len(pal), 0xFF000000, cg.BatchConfig(time_limit_s=LIMIT_S))
    t0 = time.perf_counter()
    b.launch()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    assert b.read_status() & cg.STATUS_TIMEOUT
    assert wall < 0.3, wall
    b.close()
    # the next batch, without a limit: complete and equal to the oracle
    sw, sh, mi = 96, 64, 800
    sc = torch.zeros(sw * sh, dtype=torch.int32, device="cuda:0")
    small = [cg.Viewport(width=sw, height=sh, max_iterations=mi, samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                         tier=cg.TIER_F32, seed=3, center_x=-0.5, center_y=0.0, pixel_size=3.0 / sw,
                         counts=sc.data_ptr())]
    b2 = cg.Batch(small, dpal.data_ptr(), len(pal), 0xFF000000)
    b2.launch()
    torch.cuda.synchronize()
    assert b2.read_status() == 0
    o = oracle.batch_viewport(sw, sh, 1, 0, mi, cg.TIER_F32, 3, (-0.5, 0.0), 3.0 / sw, palette=pal)
    assert np.array_equal(sc.cpu().numpy().view(np.uint32), o["counts"])
    b2.close()
