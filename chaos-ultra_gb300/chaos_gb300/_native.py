"""ctypes declarations of libchaos_gb300.so (include/chaos_gb300.h).

The library is built in-tree by chaos-ultra_gb300/build_native.py.  There is
no Python or CPU fallback: if the shared library is missing, loading fails
with ChaosError.
"""
import ctypes as C
import os
import threading

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libchaos_gb300.so")
DROPIN_DIR = os.path.join(PKG_ROOT, "cudaKernels")
DROPIN_PARITY_DIR = os.path.join(PKG_ROOT, "cudaKernels_parity")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_UNKNOWN_FRACTAL = 3
ERR_NOT_FOUND = 4
ERR_STATE = 5
ERR_OUT_OF_MEMORY = 6
ERR_TIMEOUT = 7
STATUS_TIMEOUT = 1
ERR_UNSUPPORTED = 8

FLAG_ADAPTIVE_SS = 1 << 0
FLAG_VISUALIZE_SAMPLE_COUNT = 1 << 1
FLAG_FOVEATION = 1 << 2
FLAG_SAMPLE_REUSE = 1 << 3
FLAG_IS_ZOOMING = 1 << 4
FLAG_ZOOMING_IN = 1 << 5

ARITH_FMA = 0
ARITH_PARITY = 1
ARITH_CONTRACTED = 2  # the reference module as nvcc builds it by default (reference-mode calls)

PRECISION_SINGLE = 0
PRECISION_DOUBLE = 1
PRECISION_TOO_BIG = 2
PRECISION_FLOATFLOAT = 3  # served frames: binary64 by the selector, escape loop in float-float

SAMPLES_CENTER = 0
SAMPLES_JITTER = 1
TIER_F32 = 0
TIER_F64 = 1
TIER_FLOATFLOAT = 2
TIER_PERTURB_F32 = 3
TIER_PERTURB_F64 = 4
TIER_F64_ROUNDED = 5  # batches: binary64 rounded as the reference's computeFractal<double>

MANDELBROT = 0
JULIA = 1


class ChaosError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"chaos_gb300 error {code}: {message}")
        self.code = code
        self.message = message


class RenderingModel(C.Structure):
    _fields_ = [
        ("left_bottom_x", C.c_double), ("left_bottom_y", C.c_double),
        ("right_top_x", C.c_double), ("right_top_y", C.c_double),
        ("max_iterations", C.c_uint32), ("max_super_sampling", C.c_float),
        ("use_adaptive_super_sampling", C.c_uint8), ("visualise_sample_count", C.c_uint8),
        ("use_foveated_rendering", C.c_uint8), ("use_sample_reuse", C.c_uint8),
        ("zooming", C.c_uint8), ("zooming_in", C.c_uint8), ("sample_reuse_cache_dirty", C.c_uint8),
        ("pad_", C.c_uint8),
        ("mouse_focus_x", C.c_int32), ("mouse_focus_y", C.c_int32),
        ("arith", C.c_int32), ("floating_point_precision", C.c_int32),
    ]


class FrameDesc(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("max_iterations", C.c_uint32),
        ("samples_per_pixel", C.c_uint32), ("sample_mode", C.c_uint32), ("tier", C.c_uint32),
        ("arith", C.c_int32), ("fractal", C.c_uint32), ("seed", C.c_uint64),
        ("center_x", C.c_double), ("center_y", C.c_double), ("pixel_size", C.c_double),
        ("julia_cx", C.c_double), ("julia_cy", C.c_double), ("time_limit_s", C.c_double),
    ]


class FrameOut(C.Structure):
    _fields_ = [
        ("counts", C.c_void_p), ("smooth", C.c_void_p), ("pixels", C.c_void_p), ("pixels_pitch", C.c_long),
        ("rgba", C.c_void_p), ("palette", C.c_void_p), ("palette_len", C.c_uint32),
        ("interior_rgba", C.c_uint32), ("total_iterations", C.c_void_p), ("rebases", C.c_void_p),
        ("cycle_skipped", C.c_void_p), ("status", C.c_void_p),
    ]


class Viewport(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("max_iterations", C.c_uint32),
        ("samples_per_pixel", C.c_uint32), ("sample_mode", C.c_uint32), ("tier", C.c_uint32),
        ("seed", C.c_uint64), ("center_x", C.c_double), ("center_y", C.c_double), ("pixel_size", C.c_double),
        ("counts", C.c_void_p), ("smooth", C.c_void_p), ("rgba", C.c_void_p),
    ]


class BatchConfig(C.Structure):
    _fields_ = [("block_threads", C.c_uint32 * 3), ("escape_block", C.c_uint32 * 3), ("chunk", C.c_uint32 * 3),
                ("fp64_warps_per_sm", C.c_uint32), ("time_limit_s", C.c_double)]


TIER_AUTO = 255
TIER_AUTO_DEEP = 254


class SessionDesc(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("max_iterations", C.c_uint32),
        ("max_super_sampling", C.c_float), ("flags", C.c_uint32), ("fractal", C.c_uint32), ("arith", C.c_int32),
        ("pad_", C.c_uint32), ("center_x", C.c_double), ("center_y", C.c_double), ("span", C.c_double),
        ("target_x", C.c_double), ("target_y", C.c_double), ("zoom_per_frame", C.c_double),
        ("julia_cx", C.c_double), ("julia_cy", C.c_double),
    ]


SESSION_FLAG_BINARY64 = 1 << 16


class FrameRecord(C.Structure):
    _fields_ = [("session", C.c_uint32), ("frame", C.c_uint32), ("arrival_s", C.c_double), ("start_s", C.c_double),
                ("done_s", C.c_double), ("precision", C.c_int32), ("status", C.c_int32), ("gpu_ms", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("max_frames_in_flight", C.c_uint32), ("max_launches_in_flight", C.c_uint32),
                ("max_wait_s", C.c_double), ("frame_time_limit_s", C.c_double), ("call_timeout_s", C.c_double)]


class ServedFrame(C.Structure):
    _fields_ = [("frame", C.c_uint32), ("precision", C.c_int32), ("advanced", C.c_uint32), ("flags", C.c_uint32),
                ("arith", C.c_int32), ("max_iterations", C.c_uint32), ("max_super_sampling", C.c_float),
                ("focus_x", C.c_uint32), ("focus_y", C.c_uint32), ("pad_", C.c_uint32),
                ("rect", C.c_double * 4), ("rect_reused", C.c_double * 4),
                ("pixels", C.c_void_p), ("pixels_pitch", C.c_long),
                ("previous", C.c_void_p), ("previous_pitch", C.c_long)]

_F4 = C.c_float * 4
_D4 = C.c_double * 4
_vp = C.c_void_p
_u32 = C.c_uint32
_int = C.c_int
_long = C.c_long

# name -> (restype, argtypes); every symbol declared in include/chaos_gb300.h
SIGNATURES = {
    "chaos_last_error": (C.c_char_p, []),
    "chaos_version": (C.c_char_p, []),
    "chaos_available_fractals": (C.c_char_p, []),
    "chaos_module_open": (_int, [C.c_char_p, C.POINTER(_vp)]),
    "chaos_module_close": (_int, [_vp]),
    "chaos_module_fractal_name": (C.c_char_p, [_vp]),
    "chaos_module_write_constant": (_int, [_vp, C.c_char_p, _vp, C.c_size_t]),
    "chaos_module_set_custom_params": (_int, [_vp, C.c_char_p]),
    "chaos_module_default_view": (_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(_u32), C.POINTER(C.c_float)]),
    "chaos_render_main_f32": (_int, [_vp, _vp, _long, _u32, _u32, _F4, _u32, C.c_float, _u32, _int, _vp]),
    "chaos_render_main_f64": (_int, [_vp, _vp, _long, _u32, _u32, _D4, _u32, C.c_float, _u32, _int, _vp]),
    "chaos_render_advanced_f32": (_int, [_vp, _vp, _long, _u32, _u32, _F4, _u32, C.c_float, _u32, _F4, _vp, _long,
                                         _u32, _u32, _int, _vp]),
    "chaos_render_advanced_f64": (_int, [_vp, _vp, _long, _u32, _u32, _D4, _u32, C.c_float, _u32, _D4, _vp, _long,
                                         _u32, _u32, _int, _vp]),
    "chaos_compose": (_int, [_vp, _vp, _long, _vp, _long, _u32, _u32, _vp, _u32, C.c_float, _vp]),
    "chaos_render_under_sampled": (_int, [_vp, _vp, _long, _u32, _u32, _F4, _u32, _u32, _vp]),
    "chaos_debug": (_int, [_vp]),
    "chaos_select_precision": (_int, [_D4, _u32, _u32]),
    "chaos_renderer_create": (_int, [_vp, C.POINTER(_vp)]),
    "chaos_renderer_initialize": (_int, [_vp, _u32, _u32, _vp, _u32]),
    "chaos_renderer_free_resources": (_int, [_vp]),
    "chaos_renderer_render_quality": (_int, [_vp, C.POINTER(RenderingModel)]),
    "chaos_renderer_render_fast": (_int, [_vp, C.POINTER(RenderingModel)]),
    "chaos_renderer_output": (_int, [_vp, C.POINTER(_vp), C.POINTER(_long), C.POINTER(_vp), C.POINTER(_long)]),
    "chaos_renderer_read_output": (_int, [_vp, _vp]),
    "chaos_renderer_destroy": (_int, [_vp]),
    "chaos_render_frame_async": (_int, [C.POINTER(FrameDesc), C.POINTER(FrameOut), _vp]),
    "chaos_render_frame": (_int, [C.POINTER(FrameDesc), C.POINTER(FrameOut), _vp]),
    "chaos_render_frame_host": (_int, [C.POINTER(FrameDesc), _vp, _u32, _u32, _vp, C.POINTER(C.c_ulonglong), _vp]),
    "chaos_measure_fma_peak": (_int, [_u32, C.POINTER(C.c_double)]),
    "chaos_batch_auto_tier": (_u32, [C.c_double, C.c_double, C.c_double]),
    "chaos_batch_create": (_int, [C.POINTER(Viewport), _u32, _vp, _u32, _u32, C.POINTER(BatchConfig),
                                  C.POINTER(_vp)]),
    "chaos_batch_autotune": (_int, [C.POINTER(Viewport), _u32, C.c_char_p, C.POINTER(BatchConfig), C.POINTER(_u32)]),
    "chaos_batch_launch": (_int, [_vp, _vp]),
    "chaos_batch_tiers": (_int, [_vp, C.POINTER(_u32), _u32]),
    "chaos_batch_total": (_int, [_vp, C.POINTER(_vp)]),
    "chaos_batch_read_total": (_int, [_vp, C.POINTER(C.c_ulonglong)]),
    "chaos_batch_destroy": (_int, [_vp]),
    "chaos_server_create": (_int, [C.c_size_t, _vp, _u32, C.POINTER(_vp)]),
    "chaos_server_session_bytes": (_int, [C.POINTER(SessionDesc), C.POINTER(C.c_size_t)]),
    "chaos_server_open": (_int, [_vp, C.POINTER(SessionDesc), C.POINTER(_u32)]),
    "chaos_server_close": (_int, [_vp, _u32]),
    "chaos_server_submit": (_int, [_vp, _u32, C.c_double]),
    "chaos_server_drain": (_int, [_vp]),
    "chaos_server_run_trace": (_int, [_vp, _vp, _vp, _u32]),
    "chaos_server_records": (_int, [_vp, _vp, _u32, C.POINTER(_u32)]),
    "chaos_server_read": (_int, [_vp, _u32, _vp, C.POINTER(C.c_ulonglong)]),
    "chaos_server_usage": (_int, [_vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "chaos_server_clock": (C.c_double, [_vp]),
    "chaos_server_destroy": (_int, [_vp]),
    "chaos_batch_read_cycle_skipped": (_int, [_vp, C.POINTER(C.c_ulonglong)]),
    "chaos_batch_read_status": (_int, [_vp, C.POINTER(C.c_uint32)]),
    "chaos_server_configure": (_int, [_vp, C.POINTER(ServerConfig)]),
    "chaos_server_get_config": (_int, [_vp, C.POINTER(ServerConfig)]),
    "chaos_server_queue": (_int, [_vp, C.POINTER(_u32), C.POINTER(_u32)]),
    "chaos_server_frame_state": (_int, [_vp, _u32, C.POINTER(ServedFrame)]),
    "chaos_render_frame_host_noalloc": (_int, [C.POINTER(FrameDesc), _vp, _u32, _u32, _vp,
                                               C.POINTER(C.c_ulonglong), _vp]),
    "chaos_orbit_create": (_int, [C.c_char_p, C.c_char_p, _u32, _u32, C.POINTER(_vp)]),
    "chaos_orbit_info": (_int, [_vp, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "chaos_orbit_destroy": (_int, [_vp]),
    "chaos_render_frame_perturb_async": (_int, [C.POINTER(FrameDesc), _vp, C.POINTER(FrameOut), _vp]),
    "chaos_render_frame_perturb": (_int, [C.POINTER(FrameDesc), _vp, C.POINTER(FrameOut), _vp]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """The loaded library (loaded once).  Raises ChaosError if it is not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ChaosError(ERR_UNSUPPORTED, f"{LIB_PATH} is not built; run __graft_entry__.build()")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc):
    if rc != OK:
        msg = lib().chaos_last_error().decode(errors="replace")
        raise ChaosError(rc, msg)
    return rc
