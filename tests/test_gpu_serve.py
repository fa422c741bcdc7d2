"""Serving (chaos_server_*): concurrent zoom sessions with device-resident
reuse buffers.  Frame requests queue and are admitted per request as frame
slots and HBM budget free up; admitted frames of all sessions render together
in one launch.  A session's frames are bit-exact whether it runs alone or
mixed with others; a session's frame chain equals the oracle's
renderQuality/renderFast restatement; queued frames wait for memory and are
admitted when a session closes; frames past the wait limit or the launch time
limit, and frames of a session closed while they run, end with the matching
status and leave the server usable."""
import time

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


def test_floatfloat_session_chain_matches_oracle(cuda, oracle):
    """A CHAOS_ARITH_FMA session whose frames the selector puts in binary64
    runs them with the float-float escape loop (precision FLOATFLOAT): its
    renderQuality / renderFast chain equals the oracle's restatement with the
    same float-float step."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    from oracle.oracle import ARITH_FLOATFLOAT, MANDELBROT
    w, h, tgt, mi, span0 = 160, 96, (-0.7453, 0.1127), 1500, 4e-6
    flags = FLAGS_ADAPTIVE | FLAGS_REUSE
    pal = default_palette()
    srv = cg.Server(1 << 28, pal)
    center = (tgt[0] + 1e-6, tgt[1] - 5e-7)
    sid = srv.open(desc(cg, w, h, tgt, max_iter=mi, flags=flags, span=span0, center=center))
    cx, cy, span = center[0], center[1], span0
    prev_pix, prev_rect = None, None
    for f in range(4):
        if f:
            cx = tgt[0] + (cx - tgt[0]) / 1.02
            cy = tgt[1] + (cy - tgt[1]) / 1.02
            span /= 1.02
        hw, hh = 0.5 * span, 0.5 * span * h / w
        rect = (cx - hw, cy - hh, cx + hw, cy + hh)
        assert cg.select_precision(rect, w, h) == cg.PRECISION_DOUBLE
        if f == 0:
            pix = oracle.render_main(MANDELBROT, True, ARITH_FLOATFLOAT, w, h, rect, mi, 2.0, flags & 1)
        else:
            fx = min(max((tgt[0] - rect[0]) / (rect[2] - rect[0]) * w, 0.0), w - 1.0)
            fy = min(max((rect[3] - tgt[1]) / (rect[3] - rect[1]) * h, 0.0), h - 1.0)
            pix = oracle.render_advanced(MANDELBROT, True, ARITH_FLOATFLOAT, w, h, rect, mi, 2.0, flags | 16 | 32,
                                         prev_rect, prev_pix, (int(fx), int(fy)))
        srv.submit(sid)
        img, _ = srv.read(sid)
        got = srv.frame_state(sid)
        assert got["precision"] == cg.PRECISION_FLOATFLOAT
        assert np.array_equal(img, oracle.compose(pix, pal, 2.0)), f
        prev_pix, prev_rect = pix, rect
    assert all(r[5] == cg.PRECISION_FLOATFLOAT for r in srv.records())
    srv.close()


def _wait_queue(srv, pred, limit=60.0):
    t0 = time.time()
    while not pred(*srv.queue()):
        assert time.time() - t0 < limit, srv.queue()
        time.sleep(0.002)


def _alone(cg, d, frames, pal):
    srv = cg.Server(1 << 30, pal)
    sid = srv.open(d)
    for _ in range(frames):
        srv.submit(sid)
    srv.drain()
    img, iters = srv.read(sid)
    srv.close()
    return img, iters


def test_admission_waits_for_memory_and_slots(cuda):
    """A full server queues the next session's frame instead of refusing it;
    closing a session frees its memory and admits the waiting frame, whose
    image equals the same session rendered alone."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    pal = default_palette()
    descs = [desc(cg, 480, 270, t) for t in ((-0.7453, 0.1127), (-0.1011, 0.9563), (0.2925, 0.0148))]
    need = cg.Server.session_bytes(descs[0])
    srv = cg.Server(2 * need + need // 2, pal)
    with pytest.raises(cg.ChaosError) as e:  # alone larger than the whole budget: refused at once
        srv.open(desc(cg, 4096, 4096, (0.0, 0.0)))
    assert e.value.code == 6
    a, b, c = (srv.open(d) for d in descs)
    assert srv.usage() == (0, 2 * need + need // 2)  # nothing allocated before a frame is admitted
    for sid in (a, b, c):
        srv.submit(sid)
    _wait_queue(srv, lambda waiting, in_flight: waiting == 1 and in_flight == 0)
    assert srv.usage()[0] == 2 * need
    recs = srv.records()
    assert [r[3] >= 0 for r in recs] == [True, True, False]  # c's frame not admitted
    srv.submit(a)  # a resident session goes on while c waits
    _wait_queue(srv, lambda waiting, in_flight: waiting == 1 and in_flight == 0)
    srv.close_session(a)
    srv.drain()
    recs = srv.records()
    assert all(r[6] == 0 for r in recs), recs
    rc_ = [r for r in recs if r[0] == c]
    assert len(rc_) == 1 and rc_[0][3] >= rc_[0][2] and rc_[0][4] >= rc_[0][3]
    assert srv.usage()[0] == 2 * need
    img, iters = srv.read(c)
    want, want_iters = _alone(cg, descs[2], 1, pal)
    assert np.array_equal(img, want) and iters == want_iters
    srv.close()


def test_frame_slots_bound_frames_in_flight(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    srv = cg.Server(1 << 30, default_palette())
    srv.configure(max_frames_in_flight=1)
    ids = [srv.open(desc(cg, w, h, t)) for w, h, t in SESSIONS]
    for _ in range(2):
        for sid in ids:
            srv.submit(sid)
    srv.drain()
    recs = sorted(srv.records(), key=lambda r: r[3])
    assert len(recs) == 6 and all(r[6] == 0 for r in recs)
    for prev, nxt in zip(recs, recs[1:]):  # one frame at a time: admitted after the previous one finished
        assert nxt[3] >= prev[4]
    srv.close()


def test_wait_limit_expires_queued_frame(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    d = desc(cg, 480, 270, (-0.7453, 0.1127))
    need = cg.Server.session_bytes(d)
    srv = cg.Server(need + need // 2, default_palette())
    srv.configure(max_wait_s=0.05)
    a, b = srv.open(d), srv.open(d)
    srv.submit(a)
    srv.submit(b)  # no memory for b while a stays open
    srv.drain()
    recs = srv.records()
    assert recs[0][6] == 0 and recs[1][6] == 7  # CHAOS_ERR_TIMEOUT
    assert recs[1][4] - recs[1][2] >= 0.05 and recs[1][3] < 0
    srv.close()


HEAVY = dict(w=1920, h=1080, max_iter=20000)


def _heavy(cg):
    from chaos_gb300.workloads import boundary_point
    t = boundary_point(2, 20000)
    return cg.SessionDesc(width=HEAVY["w"], height=HEAVY["h"], max_iterations=HEAVY["max_iter"],
                          max_super_sampling=4.0, flags=FLAGS_ADAPTIVE, fractal=cg.MANDELBROT,
                          arith=cg.ARITH_PARITY, center_x=t[0], center_y=t[1], span=1e-10 / 2, target_x=t[0],
                          target_y=t[1], zoom_per_frame=1.02)


def test_launch_time_limit_stops_frames(cuda):
    """A launch that runs past frame_time_limit_s stops taking tiles: its frame
    ends with CHAOS_ERR_TIMEOUT well before the frame's full time, and the
    next frames render correctly."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    pal = default_palette()
    srv = cg.Server(4 << 30, pal)
    srv.configure(frame_time_limit_s=0.005)
    sid = srv.open(_heavy(cg))
    srv.submit(sid)
    srv.drain()
    r = srv.records()[0]
    assert r[6] == 7, r  # CHAOS_ERR_TIMEOUT
    assert r[7] < 500.0, r  # the full frame takes seconds
    srv.configure(frame_time_limit_s=0.0)
    small = desc(cg, 256, 144, SESSIONS[0][2])
    s2 = srv.open(small)
    for _ in range(3):
        srv.submit(s2)
    srv.drain()
    img, iters = srv.read(s2)
    want, want_iters = _alone(cg, small, 3, pal)
    assert np.array_equal(img, want) and iters == want_iters
    assert all(r[6] == 0 for r in srv.records()[1:])
    srv.close()


def test_close_cancels_frames_on_the_gpu(cuda):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    pal = default_palette()
    srv = cg.Server(4 << 30, pal)
    sid = srv.open(_heavy(cg))
    srv.submit(sid)
    _wait_queue(srv, lambda waiting, in_flight: in_flight == 1)
    t0 = time.time()
    srv.close_session(sid)
    closed_in = time.time() - t0
    r = srv.records()[0]
    assert r[6] == 5, r  # CHAOS_ERR_STATE: cancelled
    assert closed_in < 1.0 and r[7] < 1000.0, (closed_in, r)
    assert srv.usage()[0] == 0
    small = desc(cg, 256, 144, SESSIONS[1][2])
    s2 = srv.open(small)
    srv.submit(s2)
    srv.drain()
    img, iters = srv.read(s2)
    want, want_iters = _alone(cg, small, 1, pal)
    assert np.array_equal(img, want) and iters == want_iters
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
        assert all(r[4] >= r[3] >= r[2] >= 0 and r[6] == 0 and r[7] > 0 for r in mine)
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
