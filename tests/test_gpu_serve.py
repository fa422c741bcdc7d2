"""Serving (chaos_server_*): concurrent zoom sessions with device-resident
reuse buffers, admitted by an HBM budget.  A session's frames are bit-exact
whether it runs alone or mixed with others; a session's frame chain equals
the oracle's renderQuality/renderFast restatement."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLAGS_ADAPTIVE, FLAGS_FOVEATION, FLAGS_REUSE = 1, 4, 8


def desc(cg, w, h, target, max_iter=800, flags=FLAGS_ADAPTIVE | FLAGS_REUSE | FLAGS_FOVEATION, span=3.0,
         center=(-0.5, 0.0), arith=None):
    return cg.SessionDesc(width=w, height=h, max_iterations=max_iter, max_super_sampling=2.0, flags=flags,
                          fractal=cg.MANDELBROT, arith=cg.ARITH_FMA if arith is None else arith,
                          center_x=center[0], center_y=center[1], span=span, target_x=target[0],
                          target_y=target[1], zoom_per_frame=1.02)


SESSIONS = [(256, 144, (-0.7453, 0.1127)), (320, 180, (-0.1011, 0.9563)), (200, 200, (0.2925, 0.0148))]


def test_same_alone_and_in_mix(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    frames = 6
    mix = cg.Server(1 << 30, default_palette())
    ids = [mix.open(desc(cg, w, h, t)) for w, h, t in SESSIONS]
    for f in range(frames):  # interleaved, never waiting: frames of different sessions overlap
        for sid in ids:
            mix.submit(sid)
    mix.drain()
    mixed = [mix.read(sid) for sid in ids]
    recs = mix.records()
    assert len(recs) == frames * len(ids) and all(r[4] >= r[2] for r in recs)
    mix.close()
    for k, (w, h, t) in enumerate(SESSIONS):
        alone = cg.Server(1 << 30, default_palette())
        sid = alone.open(desc(cg, w, h, t))
        for f in range(frames):
            alone.submit(sid)
            alone.drain()
        img, iters = alone.read(sid)
        assert np.array_equal(img, mixed[k][0]), k
        assert iters == mixed[k][1] and iters > 0
        alone.close()


def test_session_chain_matches_oracle(cuda, oracle):
    """renderQuality then renderFast frames, restated with the oracle's kernels."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    from oracle.oracle import MANDELBROT
    w, h, tgt, mi = 160, 96, (-0.7453, 0.1127), 600
    flags = FLAGS_ADAPTIVE | FLAGS_REUSE
    pal = default_palette()
    srv = cg.Server(1 << 28, pal)
    sid = srv.open(desc(cg, w, h, tgt, max_iter=mi, flags=flags, arith=cg.ARITH_PARITY))
    cx, cy, span = -0.5, 0.0, 3.0
    prev_pix, prev_rect = None, None
    for f in range(4):
        if f:
            cx = tgt[0] + (cx - tgt[0]) / 1.02
            cy = tgt[1] + (cy - tgt[1]) / 1.02
            span /= 1.02
        hw, hh = 0.5 * span, 0.5 * span * h / w
        rect = (cx - hw, cy - hh, cx + hw, cy + hh)
        dbl = cg.select_precision(rect, w, h) != cg.PRECISION_SINGLE
        if f == 0:
            pix = oracle.render_main(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, rect, mi, 2.0, flags & 1)
        else:
            fx = min(max((tgt[0] - rect[0]) / (rect[2] - rect[0]) * w, 0.0), w - 1.0)
            fy = min(max((rect[3] - tgt[1]) / (rect[3] - rect[1]) * h, 0.0), h - 1.0)
            pix = oracle.render_advanced(MANDELBROT, dbl, cg.ARITH_PARITY, w, h, rect, mi, 2.0, flags | 16 | 32,
                                         prev_rect, prev_pix, (int(fx), int(fy)))
        srv.submit(sid)
        img, _ = srv.read(sid)
        assert np.array_equal(img, oracle.compose(pix, pal, 2.0)), f
        prev_pix, prev_rect = pix, rect
    srv.close()


def test_admission_by_hbm_budget(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    d = desc(cg, 1920, 1080, (-0.7453, 0.1127))
    need = cg.Server.session_bytes(d)
    srv = cg.Server(2 * need + need // 2, default_palette())
    a = srv.open(d)
    b = srv.open(d)
    assert srv.usage() == (2 * need, 2 * need + need // 2)
    with pytest.raises(cg.ChaosError) as e:
        srv.open(d)
    assert e.value.code == 6
    srv.close_session(a)
    c = srv.open(d)
    srv.submit(b)
    srv.submit(c)
    srv.drain()
    assert srv.usage()[0] == 2 * need
    srv.close()


def test_trace_replay_records_latency(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    srv = cg.Server(1 << 30, default_palette())
    ids = [srv.open(desc(cg, w, h, t)) for w, h, t in SESSIONS]
    rng = np.random.default_rng(3)
    sess, arr = [], []
    for sid in ids:
        t = 0.0
        while True:
            t += rng.exponential(1 / 60)
            if t > 0.4:
                break
            sess.append(sid)
            arr.append(t)
    order = np.argsort(arr)
    srv.run_trace(np.array(sess)[order], np.array(arr)[order])
    recs = srv.records()
    assert len(recs) == len(sess)
    for sid in ids:
        mine = [r for r in recs if r[0] == sid]
        assert [r[1] for r in mine] == list(range(len(mine)))
        assert all(r[4] >= r[2] >= 0 for r in mine)
    srv.close()


def test_deep_session_goes_on_by_perturbation(cuda):
    """A session zooming past binary64 (where the reference's renderer stops)
    renders by perturbation around its target with the target's orbit held by
    the session: the served image equals a perturbation frame rendered
    directly at the same offset, pixel size and orbit precision, composed with
    the same palette."""
    import math

    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    from chaos_gb300.workloads import boundary_point
    torch = cuda
    w, h, mi, z, frames = 320, 180, 3000, 4.0, 9
    target = boundary_point(21, 3000)
    center = (target[0] + 2e-13, target[1] - 1e-13)
    pal = default_palette()
    srv = cg.Server(1 << 28, pal)
    d = cg.SessionDesc(width=w, height=h, max_iterations=mi, max_super_sampling=2.0, flags=FLAGS_REUSE,
                       fractal=cg.MANDELBROT, arith=cg.ARITH_FMA, center_x=center[0], center_y=center[1],
                       span=4e-12, target_x=target[0], target_y=target[1], zoom_per_frame=z)
    sid = srv.open(d)
    for _ in range(frames):
        srv.submit(sid)
    srv.drain()
    recs = srv.records()
    precs = [r[5] for r in recs]
    assert precs[0] == cg.PRECISION_DOUBLE and precs[-1] == cg.PRECISION_TOO_BIG, precs
    img, iters = srv.read(sid)
    # the same frame, rendered directly: the server's offset and span after `frames` frames
    off_x, off_y, span = center[0] - target[0], center[1] - target[1], 4e-12
    for _ in range(frames - 1):
        off_x, off_y, span = off_x / z, off_y / z, span / z
    ps = span / w
    bits = int(min(1536, max(128, math.ceil((-math.log2(ps) + 96) / 64) * 64)))
    orbit = cg.Orbit(cg.to_hex_fixed(target[0], bits), cg.to_hex_fixed(target[1], bits), bits, mi)
    pitch = 16 * w
    pix = torch.zeros((h, pitch), dtype=torch.uint8, device="cuda:0")
    desc_ = cg.FrameDesc(width=w, height=h, max_iterations=mi, samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                         tier=cg.TIER_PERTURB_F64, fractal=cg.MANDELBROT, seed=0, center_x=off_x, center_y=off_y,
                         pixel_size=ps)
    cg.render_frame_perturb(desc_, orbit, cg.FrameOut(pixels=pix.data_ptr(), pixels_pitch=pitch))
    dpal = torch.from_numpy(np.ascontiguousarray(pal, dtype=np.uint32).view(np.int32)).to("cuda:0")
    rgba = torch.zeros((h, w), dtype=torch.int32, device="cuda:0")
    with cg.Module("mandelbrot") as m:
        m.compose(pix.data_ptr(), pitch, rgba.data_ptr(), 4 * w, w, h, dpal.data_ptr(), len(pal), 1.0)
    torch.cuda.synchronize()
    want = rgba.cpu().numpy().view(np.uint32).reshape(-1)
    assert np.array_equal(img.reshape(-1), want)
    assert len(np.unique(want)) > 8  # the view shows structure
    orbit.close()
    srv.close()
