"""chaos_render_frame_host_noalloc: the frame entry point for callers that may
not allocate GPU memory (a process whose GPU memory is budgeted before it
serves frames, a JNI/Panama binding without a CUDA allocator).

It is checked through the C ABI against chaos_render_frame_host, the entry
point that allocates its device buffers: two different frames in a row must
give the same RGBA image and pixel-iteration count bit for bit (the same
kernel runs on both sides), so the shared scratch array carries nothing from
one call into the next.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _desc(cg, w, h, spp, mode, tier, arith, center, ps, seed, fractal=0, julia=(0.0, 0.0)):
    return cg.FrameDesc(width=w, height=h, max_iterations=1500, samples_per_pixel=spp, sample_mode=mode, tier=tier,
                        arith=arith, fractal=fractal, seed=seed, center_x=center[0], center_y=center[1],
                        pixel_size=ps, julia_cx=julia[0], julia_cy=julia[1])


def _noalloc(cg, desc, palette, interior):
    out = np.zeros(desc.width * desc.height, dtype=np.uint32)
    total = C.c_ulonglong(0)
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    rc = cg.lib().chaos_render_frame_host_noalloc(C.byref(desc), pal.ctypes.data_as(C.c_void_p), len(pal), interior,
                                                  out.ctypes.data_as(C.c_void_p), C.byref(total), None)
    return rc, out, total.value


def _allocating(cg, desc, palette, interior):
    out = np.zeros(desc.width * desc.height, dtype=np.uint32)
    total = C.c_ulonglong(0)
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    rc = cg.lib().chaos_render_frame_host(C.byref(desc), pal.ctypes.data_as(C.c_void_p), len(pal), interior,
                                          out.ctypes.data_as(C.c_void_p), C.byref(total), None)
    assert rc == 0, cg.lib().chaos_last_error()
    return out, total.value


def test_noalloc_matches_allocating_entry_point(cuda, native):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette, seeded_palette
    frames = [
        (_desc(cg, 640, 360, 2, cg.SAMPLES_JITTER, cg.TIER_F32, cg.ARITH_FMA, (-0.748, 0.1), 0.0014 / 640, 7),
         seeded_palette(256, seed=3), 0xFF000000),
        (_desc(cg, 333, 201, 1, cg.SAMPLES_CENTER, cg.TIER_F64, cg.ARITH_PARITY, (-0.5, 0.0), 3.0 / 333, 0),
         default_palette(), 0xFF202020),
    ]
    for desc, pal, interior in frames:  # two calls in a row, different frames
        rc, got, got_total = _noalloc(cg, desc, pal, interior)
        assert rc == 0, cg.lib().chaos_last_error()
        want, want_total = _allocating(cg, desc, pal, interior)
        assert got_total == want_total and got_total > 0
        assert np.array_equal(got, want)


def test_noalloc_rejects_frames_beyond_its_scratch(cuda, native):
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    desc = _desc(cg, 4096, 4096, 1, cg.SAMPLES_CENTER, cg.TIER_F32, cg.ARITH_FMA, (-0.5, 0.0), 3.0 / 4096, 0)
    rc, _, _ = _noalloc(cg, desc, default_palette(), 0xFF000000)
    assert rc == 1
    assert "scratch limit" in cg.lib().chaos_last_error().decode()
    small = _desc(cg, 64, 48, 1, cg.SAMPLES_CENTER, cg.TIER_F32, cg.ARITH_FMA, (-0.5, 0.0), 3.0 / 64, 0)
    rc, _, _ = _noalloc(cg, small, np.zeros(4097, dtype=np.uint32), 0)
    assert rc == 1
    rc, got, total = _noalloc(cg, small, default_palette(), 0xFF000000)  # still usable afterwards
    assert rc == 0 and total > 0


def test_noalloc_leaves_device_memory_unchanged(cuda, native):
    """After one call has set the entry point up (address look-up, kernel
    loaded), further calls -- the same frame again and a larger one on the
    same kernel -- take no device memory: the device's free bytes
    (cudaMemGetInfo) are the same before and after."""
    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    torch = cuda
    small = _desc(cg, 64, 48, 1, cg.SAMPLES_CENTER, cg.TIER_F32, cg.ARITH_FMA, (-0.5, 0.0), 3.0 / 64, 0)
    large = _desc(cg, 1920, 1080, 1, cg.SAMPLES_CENTER, cg.TIER_F32, cg.ARITH_FMA, (-0.75, 0.1), 0.01 / 1920, 0)
    pal = default_palette()
    rc, _, _ = _noalloc(cg, small, pal, 0xFF000000)  # set-up call
    assert rc == 0, cg.lib().chaos_last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for desc in (small, large):
        rc, _, total = _noalloc(cg, desc, pal, 0xFF000000)
        assert rc == 0 and total > 0, cg.lib().chaos_last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
