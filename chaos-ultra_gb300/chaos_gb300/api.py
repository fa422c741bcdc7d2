"""Thin object layer over the C ABI (names follow the reference's Java classes)."""
import ctypes as C

from ._native import (ARITH_FMA, BatchConfig, FrameDesc, FrameOut, FrameRecord, RenderingModel, ServedFrame,
                      ServerConfig, SessionDesc, Viewport,
                      _D4, _F4, check, lib)


def version():
    return lib().chaos_version().decode()


def available_fractals():
    return lib().chaos_available_fractals().decode().split(",")


def select_precision(rect, width, height):
    """RenderingKernel.isSegmentBoundsAt{Float,Double}Limit -> PRECISION_*."""
    return lib().chaos_select_precision(_D4(*rect), width, height)


def _stream(stream):
    if stream is None:
        return None
    return C.c_void_p(int(getattr(stream, "cuda_stream", stream)))


class Module:
    """FractalRenderingModule of one fractal (J/cudarenderer/FractalRenderingModule.java)."""

    def __init__(self, fractal_name):
        h = C.c_void_p()
        check(lib().chaos_module_open(fractal_name.encode(), C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().chaos_module_close(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def fractal_name(self):
        return lib().chaos_module_fractal_name(self.handle).decode()

    def write_constant(self, name, data: bytes):
        buf = C.create_string_buffer(bytes(data), len(data))
        check(lib().chaos_module_write_constant(self.handle, name.encode(), buf, len(data)))

    def set_custom_params(self, text):
        check(lib().chaos_module_set_custom_params(self.handle, text.encode()))

    def default_view(self):
        cx, cy, z = C.c_double(), C.c_double(), C.c_double()
        mi, ss = C.c_uint32(), C.c_float()
        check(lib().chaos_module_default_view(self.handle, C.byref(cx), C.byref(cy), C.byref(z), C.byref(mi),
                                              C.byref(ss)))
        return cx.value, cy.value, z.value, mi.value, ss.value

    # fractalRenderMain{Float,Double}
    def render_main(self, out_ptr, pitch, width, height, rect, max_iter, max_ss, flags, double=False,
                    arith=ARITH_FMA, stream=None):
        L = lib()
        if double:
            check(L.chaos_render_main_f64(self.handle, out_ptr, pitch, width, height, _D4(*rect), max_iter, max_ss,
                                          flags, arith, _stream(stream)))
        else:
            check(L.chaos_render_main_f32(self.handle, out_ptr, pitch, width, height, _F4(*rect), max_iter, max_ss,
                                          flags, arith, _stream(stream)))

    # fractalRenderAdvanced{Float,Double}
    def render_advanced(self, out_ptr, pitch, width, height, rect, max_iter, max_ss, flags, rect_reused, in_ptr,
                        in_pitch, focus, double=False, arith=ARITH_FMA, stream=None):
        L = lib()
        if double:
            check(L.chaos_render_advanced_f64(self.handle, out_ptr, pitch, width, height, _D4(*rect), max_iter,
                                              max_ss, flags, _D4(*rect_reused), in_ptr, in_pitch, focus[0], focus[1],
                                              arith, _stream(stream)))
        else:
            check(L.chaos_render_advanced_f32(self.handle, out_ptr, pitch, width, height, _F4(*rect), max_iter,
                                              max_ss, flags, _F4(*rect_reused), in_ptr, in_pitch, focus[0], focus[1],
                                              arith, _stream(stream)))

    def compose(self, in_ptr, pitch, out_ptr, out_pitch, width, height, palette_ptr, palette_len, max_ss,
                stream=None):
        check(lib().chaos_compose(self.handle, in_ptr, pitch, out_ptr, out_pitch, width, height, palette_ptr,
                                  palette_len, max_ss, _stream(stream)))

    def render_under_sampled(self, out_ptr, pitch, width, height, rect, max_iter, level, stream=None):
        check(lib().chaos_render_under_sampled(self.handle, out_ptr, pitch, width, height, _F4(*rect), max_iter,
                                               level, _stream(stream)))

    def debug(self):
        check(lib().chaos_debug(self.handle))


class Renderer:
    """CudaFractalRenderer with a headless RGBA8 output (J/cudarenderer/CudaFractalRenderer.java)."""

    def __init__(self, module: Module):
        h = C.c_void_p()
        check(lib().chaos_renderer_create(module.handle, C.byref(h)))
        self.handle = h
        self.module = module

    def initialize(self, width, height, palette):
        import numpy as np
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        check(lib().chaos_renderer_initialize(self.handle, width, height, pal.ctypes.data_as(C.c_void_p), len(pal)))
        self.width, self.height = width, height

    def free_resources(self):
        check(lib().chaos_renderer_free_resources(self.handle))

    def render_quality(self, model: RenderingModel):
        check(lib().chaos_renderer_render_quality(self.handle, C.byref(model)))

    def render_fast(self, model: RenderingModel):
        check(lib().chaos_renderer_render_fast(self.handle, C.byref(model)))

    def output(self):
        rgba, rp, prim, pp = C.c_void_p(), C.c_long(), C.c_void_p(), C.c_long()
        check(lib().chaos_renderer_output(self.handle, C.byref(rgba), C.byref(rp), C.byref(prim), C.byref(pp)))
        return rgba.value, rp.value, prim.value, pp.value

    def read_output(self):
        import numpy as np
        out = np.zeros((self.height, self.width), dtype=np.uint32)
        check(lib().chaos_renderer_read_output(self.handle, out.ctypes.data_as(C.c_void_p)))
        return out

    def close(self):
        if self.handle:
            lib().chaos_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_frame(desc: FrameDesc, out: FrameOut, stream=None, sync=True):
    fn = lib().chaos_render_frame if sync else lib().chaos_render_frame_async
    check(fn(C.byref(desc), C.byref(out), _stream(stream)))


def render_frame_host(desc: FrameDesc, palette, interior_rgba, rgba_host, stream=None):
    """chaos_render_frame_host: palette and image in host memory (numpy arrays).
    Returns the frame's pixel-iteration count."""
    import numpy as np
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    assert rgba_host.dtype == np.uint32 and rgba_host.flags.c_contiguous
    total = C.c_ulonglong()
    check(lib().chaos_render_frame_host(C.byref(desc), pal.ctypes.data_as(C.c_void_p), len(pal), interior_rgba,
                                        rgba_host.ctypes.data_as(C.c_void_p), C.byref(total), _stream(stream)))
    return total.value


def measure_fma_peak(tier):
    """Measured FMA throughput (FLOP/s, FMA = 2) of the current device for TIER_F32 / TIER_F64."""
    v = C.c_double()
    check(lib().chaos_measure_fma_peak(tier, C.byref(v)))
    return v.value


class Orbit:
    """Reference orbit of a deep-zoom centre (chaos_orbit_create).  Centres are
    "[-]I.hex" fixed-point strings (see to_hex_fixed)."""

    def __init__(self, center_x, center_y, bits, max_iterations):
        h = C.c_void_p()
        check(lib().chaos_orbit_create(center_x.encode(), center_y.encode(), bits, max_iterations, C.byref(h)))
        self.handle = h

    def info(self):
        n, e, b = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().chaos_orbit_info(self.handle, C.byref(n), C.byref(e), C.byref(b)))
        return {"stored": n.value, "escaped_at": e.value, "bits": b.value}

    def close(self):
        if self.handle:
            lib().chaos_orbit_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_frame_perturb(desc: FrameDesc, orbit: Orbit, out: FrameOut, stream=None, sync=True):
    fn = lib().chaos_render_frame_perturb if sync else lib().chaos_render_frame_perturb_async
    check(fn(C.byref(desc), orbit.handle, C.byref(out), _stream(stream)))


def to_hex_fixed(value, bits):
    """A real number (int/float/fractions.Fraction/decimal string handled by
    fractions.Fraction) as "[-]I.hex" with `bits` fraction bits, truncated."""
    from fractions import Fraction
    v = Fraction(value)
    neg = v < 0
    v = abs(v)
    ip = int(v)
    frac = v - ip
    digits = (bits + 3) // 4
    f = int(frac * (1 << (4 * digits)))
    return ("-" if neg else "") + f"{ip}." + format(f, f"0{digits}x")


class Batch:
    """Many viewports in one CUDA-graph launch (chaos_batch_*)."""

    def __init__(self, viewports, palette_ptr=None, palette_len=0, interior_rgba=0xFF000000, config=None):
        arr = (Viewport * len(viewports))(*viewports)
        h = C.c_void_p()
        cfg = C.byref(config) if config is not None else None
        check(lib().chaos_batch_create(arr, len(viewports), palette_ptr, palette_len, interior_rgba, cfg,
                                       C.byref(h)))
        self.handle = h
        self.n = len(viewports)

    def launch(self, stream=None):
        check(lib().chaos_batch_launch(self.handle, _stream(stream)))

    def tiers(self):
        t = (C.c_uint32 * self.n)()
        check(lib().chaos_batch_tiers(self.handle, t, self.n))
        return list(t)

    def total_ptr(self):
        p = C.c_void_p()
        check(lib().chaos_batch_total(self.handle, C.byref(p)))
        return p.value

    def read_total(self):
        t = C.c_ulonglong()
        check(lib().chaos_batch_read_total(self.handle, C.byref(t)))
        return t.value

    def read_cycle_skipped(self):
        """Iterations of the last launch proven interior by a repeated state and not run."""
        t = C.c_ulonglong()
        check(lib().chaos_batch_read_cycle_skipped(self.handle, C.byref(t)))
        return t.value

    def read_status(self):
        """STATUS_* bits of the last launch (0, or STATUS_TIMEOUT when the config's time limit ran out)."""
        t = C.c_uint32()
        check(lib().chaos_batch_read_status(self.handle, C.byref(t)))
        return t.value

    def close(self):
        if self.handle:
            lib().chaos_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_batch(viewports, cache_path=None):
    """chaos_batch_autotune: the fastest launch shape per tier for these
    viewports, as (BatchConfig, from_cache)."""
    arr = (Viewport * len(viewports))(*viewports)
    cfg = BatchConfig()
    hit = C.c_uint32(0)
    check(lib().chaos_batch_autotune(arr, len(viewports), cache_path.encode() if cache_path else None,
                                     C.byref(cfg), C.byref(hit)))
    return cfg, bool(hit.value)


def auto_tier(center_x, center_y, pixel_size):
    return lib().chaos_batch_auto_tier(center_x, center_y, pixel_size)


class Server:
    """Concurrent zoom sessions admitted by an HBM budget (chaos_server_*)."""

    def __init__(self, hbm_budget_bytes, palette):
        import numpy as np
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        h = C.c_void_p()
        check(lib().chaos_server_create(hbm_budget_bytes, pal.ctypes.data_as(C.c_void_p), len(pal), C.byref(h)))
        self.handle = h
        self.shapes = {}

    def open(self, desc: SessionDesc):
        sid = C.c_uint32()
        check(lib().chaos_server_open(self.handle, C.byref(desc), C.byref(sid)))
        self.shapes[sid.value] = (desc.height, desc.width)
        return sid.value

    @staticmethod
    def session_bytes(desc: SessionDesc):
        b = C.c_size_t()
        check(lib().chaos_server_session_bytes(C.byref(desc), C.byref(b)))
        return b.value

    def close_session(self, sid):
        """Drop the session's queued frames, cancel those on the GPU, release its buffers."""
        check(lib().chaos_server_close(self.handle, sid))
        self.shapes.pop(sid, None)

    def submit(self, sid, arrival_s=None):
        if arrival_s is None:
            arrival_s = self.clock()
        check(lib().chaos_server_submit(self.handle, sid, arrival_s))

    def drain(self):
        check(lib().chaos_server_drain(self.handle))

    def run_trace(self, sessions, arrivals):
        import numpy as np
        s = np.ascontiguousarray(sessions, dtype=np.uint32)
        a = np.ascontiguousarray(arrivals, dtype=np.float64)
        check(lib().chaos_server_run_trace(self.handle, s.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p),
                                           len(s)))

    def records(self):
        """(session, frame, arrival_s, start_s, done_s, precision, status, gpu_ms) per frame, oldest first;
        start_s is the admission into a launch."""
        n = C.c_uint32()
        check(lib().chaos_server_records(self.handle, None, 0, C.byref(n)))
        buf = (FrameRecord * max(1, n.value))()
        check(lib().chaos_server_records(self.handle, buf, n.value, C.byref(n)))
        return [(r.session, r.frame, r.arrival_s, r.start_s, r.done_s, r.precision, r.status, r.gpu_ms)
                for r in buf[:n.value]]

    def configure(self, **kw):
        """Set chaos_server_config fields (max_frames_in_flight, max_launches_in_flight, max_wait_s,
        frame_time_limit_s, call_timeout_s); the others keep their values."""
        cfg = ServerConfig()
        check(lib().chaos_server_get_config(self.handle, C.byref(cfg)))
        for k, v in kw.items():
            setattr(cfg, k, v)
        check(lib().chaos_server_configure(self.handle, C.byref(cfg)))

    def config(self):
        cfg = ServerConfig()
        check(lib().chaos_server_get_config(self.handle, C.byref(cfg)))
        return {k: getattr(cfg, k) for k, _ in ServerConfig._fields_}

    def queue(self):
        """(frames waiting for admission, frames on the GPU)."""
        w, f = C.c_uint32(), C.c_uint32()
        check(lib().chaos_server_queue(self.handle, C.byref(w), C.byref(f)))
        return w.value, f.value

    def frame_state(self, sid):
        """The session's latest finished frame (chaos_served_frame) as a dict."""
        f = ServedFrame()
        check(lib().chaos_server_frame_state(self.handle, sid, C.byref(f)))
        out = {k: getattr(f, k) for k, _ in ServedFrame._fields_ if k != "pad_"}
        out["rect"], out["rect_reused"] = tuple(f.rect), tuple(f.rect_reused)
        return out

    def read(self, sid):
        import numpy as np
        h, w = self.shapes[sid]
        out = np.zeros((h, w), dtype=np.uint32)
        it = C.c_ulonglong()
        check(lib().chaos_server_read(self.handle, sid, out.ctypes.data_as(C.c_void_p), C.byref(it)))
        return out, it.value

    def usage(self):
        u, b = C.c_size_t(), C.c_size_t()
        check(lib().chaos_server_usage(self.handle, C.byref(u), C.byref(b)))
        return u.value, b.value

    def clock(self):
        return lib().chaos_server_clock(self.handle)

    def close(self):
        if self.handle:
            lib().chaos_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
