"""chaos_gb300 -- GB300 (sm_103a) escape-time renderer, a drop-in for
chaos-ultra's fractal-kernel path.

Python face of libchaos_gb300.so: `Module` mirrors FractalRenderingModule and
its kernels, `Renderer` mirrors CudaFractalRenderer (renderQuality /
renderFast), `render_frame` is the jittered-supersampling frame path, `Batch`
renders many viewports in one CUDA-graph launch, `Server` serves concurrent
zoom sessions, `Orbit` / `render_frame_perturb` are the deep-zoom tier.
Device buffers are passed as raw device pointers (e.g. torch tensor
data_ptr()).
"""
from ._native import (ARITH_CONTRACTED, ARITH_FMA, ARITH_PARITY, DROPIN_DIR, DROPIN_PARITY_DIR, FLAG_ADAPTIVE_SS, FLAG_FOVEATION,
                      FLAG_IS_ZOOMING, FLAG_SAMPLE_REUSE, FLAG_VISUALIZE_SAMPLE_COUNT, FLAG_ZOOMING_IN, JULIA,
                      LIB_PATH, MANDELBROT, PRECISION_DOUBLE, PRECISION_FLOATFLOAT, PRECISION_SINGLE, PRECISION_TOO_BIG, SAMPLES_CENTER,
                      SAMPLES_JITTER, SESSION_FLAG_BINARY64, STATUS_TIMEOUT, TIER_AUTO, TIER_AUTO_DEEP, TIER_F32, TIER_F64, TIER_F64_ROUNDED, TIER_FLOATFLOAT,
                      TIER_PERTURB_F32, TIER_PERTURB_F64, BatchConfig, ChaosError, FrameDesc, FrameOut, FrameRecord,
                      RenderingModel, ServedFrame, ServerConfig, SessionDesc, Viewport, lib)
from .api import (Batch, Module, Orbit, Renderer, Server, auto_tier, autotune_batch, available_fractals,
                  measure_fma_peak, render_frame, render_frame_host, render_frame_perturb, select_precision,
                  to_hex_fixed, version)

__all__ = [
    "ARITH_CONTRACTED", "ARITH_FMA", "ARITH_PARITY", "DROPIN_DIR", "DROPIN_PARITY_DIR", "FLAG_ADAPTIVE_SS", "FLAG_FOVEATION",
    "FLAG_IS_ZOOMING", "FLAG_SAMPLE_REUSE", "FLAG_VISUALIZE_SAMPLE_COUNT", "FLAG_ZOOMING_IN", "JULIA", "LIB_PATH",
    "MANDELBROT", "PRECISION_DOUBLE", "PRECISION_FLOATFLOAT", "PRECISION_SINGLE", "PRECISION_TOO_BIG", "SAMPLES_CENTER", "SAMPLES_JITTER",
    "SESSION_FLAG_BINARY64", "STATUS_TIMEOUT", "TIER_AUTO", "TIER_AUTO_DEEP", "TIER_F32", "TIER_F64", "TIER_F64_ROUNDED", "TIER_FLOATFLOAT", "TIER_PERTURB_F32", "TIER_PERTURB_F64",
    "BatchConfig", "ChaosError", "FrameDesc", "FrameOut", "FrameRecord", "RenderingModel", "ServedFrame", "ServerConfig",
    "SessionDesc", "Viewport",
    "lib", "Batch", "Module", "Orbit", "Renderer", "Server", "auto_tier", "autotune_batch", "available_fractals",
    "measure_fma_peak", "render_frame", "render_frame_host", "render_frame_perturb", "select_precision",
    "to_hex_fixed", "version",
]
