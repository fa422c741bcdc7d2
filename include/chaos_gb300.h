/*
 * chaos_gb300.h -- C ABI of libchaos_gb300.so, the GB300 (sm_103a) escape-time
 * renderer that stands in for chaos-ultra's fractal-kernel path.
 *
 * Two ways in:
 *   1. The drop-in CUDA module files cudaKernels/<fractal>.ptx (cubin images;
 *      cuModuleLoad reads cubin as well as PTX).  They export the seven kernels
 *      the Java host resolves by name, with the reference's parameter layout and
 *      __constant__ symbols, so FractalRenderingModule loads them unchanged.
 *   2. This library: plain C functions (pointers, sizes, a cudaStream_t passed as
 *      void*), int status returns, no exceptions and no device traps, for a
 *      thin JNI or Panama binding on the Java side.
 *
 * Reference paths are relative to the chaos-ultra root; J/ stands for
 * src/main/java/cz/cuni/mff/cgg/teichmaa/chaosultra/ and gen.cu for
 * src/main/cuda/fractalRendererGeneric.cu.
 *
 * Threading: calls on one chaos_module / chaos_renderer are not thread-safe
 * (the reference makes every CUDA call from one thread, J/cudarenderer/
 * CudaHelpers.java:47-49).  Kernels are enqueued on the stream passed in
 * (NULL = the legacy default stream); functions without "_async" in their name
 * synchronise that stream before returning, as the reference does after every
 * launch (J/cudarenderer/CudaFractalRenderer.java:255-261).
 */
#ifndef CHAOS_GB300_H
#define CHAOS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define CHAOS_OK 0
#define CHAOS_ERR_INVALID_ARGUMENT 1 /* bad size, pointer, NaN/inf plane bound, ... */
#define CHAOS_ERR_CUDA 2             /* a CUDA runtime call failed; see chaos_last_error() */
#define CHAOS_ERR_UNKNOWN_FRACTAL 3  /* CudaFractalRendererProvider.getRenderer: "Unknown fractal" */
#define CHAOS_ERR_NOT_FOUND 4        /* unknown constant name (cuModuleGetGlobal NOT_FOUND) */
#define CHAOS_ERR_STATE 5            /* renderer not initialised / already initialised */
#define CHAOS_ERR_OUT_OF_MEMORY 6    /* allocation or HBM budget refused */
#define CHAOS_ERR_TIMEOUT 7          /* a bounded device wait gave up */
#define CHAOS_ERR_UNSUPPORTED 8      /* valid request this library does not implement */

/* Message of the last failing call on this thread ("" if none). */
const char *chaos_last_error(void);
/* Library version string. */
const char *chaos_version(void);

/* ---- shared types ------------------------------------------------------- */

/* pixel_info_t, src/main/cuda/helpers.cuh:106-130: 16 bytes, 4-byte aligned. */
typedef struct chaos_pixel_info {
    float value;                 /* averaged escape value */
    float weight;                /* number of samples (may decay under reuse) */
    uint8_t is_reused;           /* set when sample reuse produced the value */
    uint8_t pad_[3];
    float weight_of_new_samples; /* freshly computed weight when is_reused */
} chaos_pixel_info;

/* Kernel flag bits, gen.cu:157-161 / J/cudarenderer/KernelMain.java:12-13,
 * KernelAdvanced.java:17-20 (bit 1, "visualise sample count", is host-side). */
#define CHAOS_FLAG_ADAPTIVE_SS (1u << 0)
#define CHAOS_FLAG_VISUALIZE_SAMPLE_COUNT (1u << 1)
#define CHAOS_FLAG_FOVEATION (1u << 2)
#define CHAOS_FLAG_SAMPLE_REUSE (1u << 3)
#define CHAOS_FLAG_IS_ZOOMING (1u << 4)
#define CHAOS_FLAG_ZOOMING_IN (1u << 5)

/* Arithmetic of the escape loop.
 * CHAOS_ARITH_PARITY rounds every product and sum (the reference kernel built
 * with nvcc --fmad=false): escape counts are bit-identical to it.
 * CHAOS_ARITH_CONTRACTED is the reference module as nvcc builds it by default
 * (contraction on, the build the Java application loads): y' = fma(2x, y, cy),
 * the sample's x coordinate and parts of the reuse path fused, everything
 * else rounded; pixel records are bit-identical to that build.  Reference-mode
 * calls (render_main / render_advanced, the renderer) only.
 * CHAOS_ARITH_FMA uses fused multiply-adds, 4 FP ops per iteration; counts are
 * bit-identical to the oracle's fma restatement and differ from PARITY only
 * where rounding decides an escape. */
#define CHAOS_ARITH_FMA 0
#define CHAOS_ARITH_PARITY 1
#define CHAOS_ARITH_CONTRACTED 2

/* ---- module level: FractalRenderingModule + its seven kernels ----------- */

typedef struct chaos_module chaos_module;

/* Open the module of a registered fractal: "mandelbrot", "julia",
 * "newton_wired" / "newton wired", "newton_generic" / "newton generic",
 * "newton_iterations" / "newton colored by iterations" (module file name or
 * the name the Java GUI shows).  The Newton modules' kernels always use
 * rounded arithmetic (the `arith` argument does not apply to them).
 * Replaces FractalRenderingModule.initialize (J/cudarenderer/
 * FractalRenderingModule.java:73-100) + CudaFractalRendererProvider.getRenderer
 * (J/cudarenderer/CudaFractalRendererProvider.java:47-66). */
int chaos_module_open(const char *fractal_name, chaos_module **out);
int chaos_module_close(chaos_module *m);
/* Registered fractal names, comma separated (getAvailableFractals, :37-39). */
const char *chaos_available_fractals(void);
/* Fractal name of an open module (getFractalName). */
const char *chaos_module_fractal_name(const chaos_module *m);

/* Write a module constant by name, size must equal the symbol's size
 * ("VISUALIZE_SAMPLE_COUNT": 1 byte, gen.cu:14; "julia_c": 2 doubles,
 * julia.cu:3; "roots": 6 doubles, "coefficients": 4 doubles (c0..c3),
 * newton_generic.cu:7-8; "colorMagnifier": int, newton_iterations.cu:9).
 * Replaces writeToConstantMemory (FractalRenderingModule.java:163-227). */
int chaos_module_write_constant(chaos_module *m, const char *name, const void *src, size_t size);
/* Fractal custom parameters as the GUI sends them: "-0.4;0.6" for Julia
 * (ModuleJulia.setFractalCustomParameters, J/cudarenderer/modules/ModuleJulia.java:28-37);
 * {"coefficients": [a3, a2, a1, a0], "roots": [[re, im], [re, im], [re, im]],
 * "colorMagnifier": n} for the generic Newton modules
 * (ModuleNewtonGeneric.java:30-65, ModuleNewtonIterations.java:15-24). */
int chaos_module_set_custom_params(chaos_module *m, const char *text);
/* Default view of the module (supplyDefaultValues, ModuleMandelbrot.java:20-25,
 * ModuleJulia.java:40-49): centre, zoom (plane height), maxIterations, maxSS. */
int chaos_module_default_view(const chaos_module *m, double *center_x, double *center_y, double *zoom,
                              uint32_t *max_iterations, float *max_super_sampling);

/* fractalRenderMainFloat / fractalRenderMainDouble, gen.cu:384-405.
 * out: pitched width x height array of chaos_pixel_info (device memory, pitch
 * in bytes, >= 16*width).  rect = {left_bottom.x, left_bottom.y, right_top.x,
 * right_top.y}.  max_super_sampling in [1, 64].  Persistent warps take 8x4
 * pixel tiles from a work counter (each warp one tile at a time, the vote
 * group of the reference's adaptive super-sampling). */
int chaos_render_main_f32(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                          const float rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                          int arith, void *stream);
int chaos_render_main_f64(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                          const double rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                          int arith, void *stream);

/* fractalRenderAdvancedFloat / fractalRenderAdvancedDouble, gen.cu:423-448:
 * foveation + sample reuse from `in` (the previous frame, plane rect_reused).
 * in and out must not overlap. */
int chaos_render_advanced_f32(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                              const float rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                              const float rect_reused[4], const chaos_pixel_info *in, long in_pitch, uint32_t focus_x,
                              uint32_t focus_y, int arith, void *stream);
int chaos_render_advanced_f64(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                              const double rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                              const double rect_reused[4], const chaos_pixel_info *in, long in_pitch,
                              uint32_t focus_x, uint32_t focus_y, int arith, void *stream);

/* compose, gen.cu:455-475, with a headless output: out_rgba is a pitched
 * width x height array of RGBA8 words (R in the low byte), the palette a device
 * array of palette_len words (the one-row palette surface of the reference).
 * The module's VISUALIZE_SAMPLE_COUNT constant selects the sample-count ramp. */
int chaos_compose(chaos_module *m, const chaos_pixel_info *in, long pitch, uint32_t *out_rgba, long out_pitch,
                  uint32_t width, uint32_t height, const uint32_t *palette, uint32_t palette_len,
                  float max_super_sampling, void *stream);

/* fractalRenderUnderSampled, gen.cu:478-503 (float plane, every level-th pixel). */
int chaos_render_under_sampled(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                               const float rect[4], uint32_t max_iterations, uint32_t level, void *stream);

/* debug, gen.cu:505-512: prints the fractal's greeting from the device. */
int chaos_debug(chaos_module *m);

/* ---- precision selection (RenderingKernel.isSegmentBoundsAt*Limit) ----- */

#define CHAOS_PRECISION_SINGLE 0
#define CHAOS_PRECISION_DOUBLE 1
#define CHAOS_PRECISION_TOO_BIG 2
/* Served frames only (chaos_frame_record.precision): a frame the selector puts
 * in binary64, rendered with the escape loop in float-float. */
#define CHAOS_PRECISION_FLOATFLOAT 3
/* J/cudarenderer/RenderingKernel.java:124-138 + CudaFractalRenderer.updateFloatPrecision
 * (:409-419): single while the pixel is at least ulp((float)left_bottom) on both
 * axes, double below that, "too big" below ulp((double)left_bottom). */
int chaos_select_precision(const double rect[4], uint32_t width, uint32_t height);

/* ---- renderer level: CudaFractalRenderer (renderQuality / renderFast) --- */

/* RenderingModel fields the renderer reads (J/rendering/model/*.java). */
typedef struct chaos_rendering_model {
    double left_bottom_x, left_bottom_y, right_top_x, right_top_y; /* PlaneSegment */
    uint32_t max_iterations;
    float max_super_sampling;
    uint8_t use_adaptive_super_sampling;
    uint8_t visualise_sample_count;
    uint8_t use_foveated_rendering;
    uint8_t use_sample_reuse;
    uint8_t zooming;
    uint8_t zooming_in;
    uint8_t sample_reuse_cache_dirty;
    uint8_t pad_;
    int32_t mouse_focus_x, mouse_focus_y;
    int32_t arith; /* CHAOS_ARITH_* for this frame */
    int32_t floating_point_precision; /* out: CHAOS_PRECISION_* chosen for the frame */
} chaos_rendering_model;

typedef struct chaos_renderer chaos_renderer;

/* new CudaFractalRenderer(module) (J/cudarenderer/CudaFractalRenderer.java:65-77). */
int chaos_renderer_create(chaos_module *m, chaos_renderer **out);
/* initializeRendering(GLParams) with a headless output: allocates the two
 * pitched sample-reuse buffers (DeviceMemoryDoubleBuffer2D.reallocate,
 * J/cudarenderer/DeviceMemoryDoubleBuffer2D.java:37-41) and a width x height
 * RGBA8 output, and copies the palette (host array) to the device. */
int chaos_renderer_initialize(chaos_renderer *r, uint32_t width, uint32_t height, const uint32_t *palette,
                              uint32_t palette_len);
int chaos_renderer_free_resources(chaos_renderer *r);
/* renderQuality (CudaFractalRenderer.java:187-206): main kernel + compose. */
int chaos_renderer_render_quality(chaos_renderer *r, chaos_rendering_model *model);
/* renderFast (CudaFractalRenderer.java:159-184): advanced kernel reusing the
 * previous frame, buffer swap, compose; falls back to renderQuality when the
 * reuse cache is dirty. */
int chaos_renderer_render_fast(chaos_renderer *r, chaos_rendering_model *model);
/* Device pointers of the current output (RGBA8, pitch in bytes) and of the
 * primary reuse buffer. */
int chaos_renderer_output(const chaos_renderer *r, const uint32_t **rgba, long *rgba_pitch,
                          const chaos_pixel_info **primary, long *primary_pitch);
/* Copy the RGBA8 output to host memory (width*height words, row-major). */
int chaos_renderer_read_output(const chaos_renderer *r, uint32_t *host_rgba);
int chaos_renderer_destroy(chaos_renderer *r);

/* ---- frame level: per-sample escape counts, jittered supersampling ------ */

#define CHAOS_SAMPLES_CENTER 0 /* one sample at each pixel centre */
#define CHAOS_SAMPLES_JITTER 1 /* samples_per_pixel seeded uniform offsets */

#define CHAOS_TIER_F32 0         /* escape loop in binary32 */
#define CHAOS_TIER_F64 1         /* escape loop in binary64 */
#define CHAOS_TIER_FLOATFLOAT 2  /* float-float (two binary32 words, ~48 bits), batched viewports */
#define CHAOS_TIER_PERTURB_F32 3 /* perturbation, binary32 differences, rescaled by 2^e below pixel 1e-30 (>= 1e-290) */
#define CHAOS_TIER_PERTURB_F64 4 /* perturbation, binary64 differences (pixel size >= 1e-290) */

/* One frame of the plain escape-time renderer.  Sample s of pixel (px, py)
 * sits at plane point
 *   c = (center_x + ((px + ox) - width/2) * pixel_size,
 *        center_y - ((py + oy) - height/2) * pixel_size)
 * with (ox, oy) = (0.5, 0.5) for CHAOS_SAMPLES_CENTER and a counter-based hash
 * of (seed, pixel, sample) in [0,1)^2 for CHAOS_SAMPLES_JITTER. */
typedef struct chaos_frame_desc {
    uint32_t width, height;
    uint32_t max_iterations;
    uint32_t samples_per_pixel; /* 1..64 */
    uint32_t sample_mode;       /* CHAOS_SAMPLES_* */
    uint32_t tier;              /* CHAOS_TIER_* */
    int32_t arith;              /* CHAOS_ARITH_* */
    uint32_t fractal;           /* 0 mandelbrot, 1 julia */
    uint64_t seed;
    double center_x, center_y;
    double pixel_size;
    double julia_cx, julia_cy;
    /* 0, or a limit on the frame's kernel run time in seconds: past it every
     * warp stops where it is (samples in flight stay unwritten), and the
     * frame completes with CHAOS_ERR_TIMEOUT (chaos_render_frame,
     * chaos_render_frame_host, chaos_render_frame_perturb) or with
     * CHAOS_STATUS_TIMEOUT in *out->status (the _async calls, which need
     * out->status with a limit) */
    double time_limit_s;
} chaos_frame_desc;

/* Outputs (device pointers, each optional):
 *   counts  [height][width][spp] uint32 iterations taken (max_iterations = interior)
 *   smooth  [height][width][spp] float  n + 1 - log2(log2|z_n|), interior = max_iterations
 *   pixels  pitched chaos_pixel_info: value = mean over samples of (smooth, 0 for interior), weight = spp
 *   rgba    [height][width] RGBA8: mean of the sample colours, palette[] sampled with linear
 *           interpolation at smooth mod palette_len, interior samples = interior_rgba
 *   total_iterations: one uint64 the kernel adds the frame's pixel-iterations to. */
typedef struct chaos_frame_out {
    uint32_t *counts;
    float *smooth;
    chaos_pixel_info *pixels;
    long pixels_pitch;
    uint32_t *rgba;
    const uint32_t *palette;
    uint32_t palette_len;
    uint32_t interior_rgba;
    unsigned long long *total_iterations;
    unsigned long long *rebases; /* perturbation tiers: glitch repairs (rebasing events) */
    /* one uint64 the kernel adds the iterations it did not run to: a sample
     * whose state repeats bit for bit is interior (the iteration is
     * deterministic), so it counts max_iterations without running the rest
     * (binary32 and binary64 tiers; total_iterations counts it in full) */
    unsigned long long *cycle_skipped;
    /* one uint32 the kernel ORs CHAOS_STATUS_* bits into (zeroed by the
     * caller; used with desc->time_limit_s) */
    uint32_t *status;
} chaos_frame_out;

#define CHAOS_STATUS_TIMEOUT 1u /* the launch's time limit ran out: outputs incomplete */

/* Enqueue one frame (does not synchronise). */
int chaos_render_frame_async(const chaos_frame_desc *desc, const chaos_frame_out *out, void *stream);
/* Same, then synchronise the stream. */
int chaos_render_frame(const chaos_frame_desc *desc, const chaos_frame_out *out, void *stream);

/* A whole frame through host memory, for callers that hold no device buffers:
 * copies the palette (host array) to the device, renders the RGBA8 image, and
 * copies the image (width*height words, row-major) and the frame's
 * pixel-iteration count back to host memory.  Device buffers are kept per
 * calling thread and grown as needed; the stream is synchronised before return. */
int chaos_render_frame_host(const chaos_frame_desc *desc, const uint32_t *palette, uint32_t palette_len,
                            uint32_t interior_rgba, uint32_t *rgba_host, unsigned long long *total_host,
                            void *stream);

/* ---- batches: many viewports in one CUDA-graph launch -------------------- */

#define CHAOS_TIER_AUTO 255      /* binary32 / float-float / binary64 by pixel size */
#define CHAOS_TIER_AUTO_DEEP 254 /* binary32 / float-float / perturbation where AUTO would pick binary64 */
/* Batched binary64 with every operation rounded as the reference's
 * computeFractal<double> rounds it (no contraction): the escape counts of the
 * FP64 oracle, bit for bit.  The binary64 viewports of one batch are all
 * CHAOS_TIER_F64 (fused) or all CHAOS_TIER_F64_ROUNDED; mixing the two fails
 * with CHAOS_ERR_INVALID_ARGUMENT.  Launch shape: the binary64 entries of
 * chaos_batch_config. */
#define CHAOS_TIER_F64_ROUNDED 5

/* One viewport of a batch.  Samples as in chaos_frame_desc (the plane point is
 * computed in binary64, then rounded to the viewport's tier).  Outputs are
 * device pointers, each optional: counts/smooth [height][width][spp], rgba
 * [height][width] (needs the batch palette). */
typedef struct chaos_viewport {
    uint32_t width, height;
    uint32_t max_iterations;
    uint32_t samples_per_pixel;
    uint32_t sample_mode;
    uint32_t tier; /* CHAOS_TIER_F32, _FLOATFLOAT, _F64, _F64_ROUNDED, _PERTURB_F32, _PERTURB_F64, _AUTO or _AUTO_DEEP */
    uint64_t seed;
    double center_x, center_y, pixel_size;
    uint32_t *counts;
    float *smooth;
    uint32_t *rgba;
} chaos_viewport;

/* Launch shape per tier (index 0 binary32, 1 float-float, 2 binary64); zero
 * keeps the default (256 threads, 16-step escape blocks, chunk 1).  When a
 * batch holds binary64 viewports and binary32 or float-float ones, their
 * kernels share every SM: the binary64 kernel gets fp64_warps_per_sm warps
 * per SM (default 8; its pipe is saturated by few warps) and the others the
 * rest, so the binary64 and binary32 pipes work at the same time. */
typedef struct chaos_batch_config {
    uint32_t block_threads[3]; /* 32..512, multiple of 32 */
    uint32_t escape_block[3];  /* 8, 16 or 32 */
    uint32_t chunk[3];         /* 1..64 consecutive pixels a lane claims per work-counter update */
    uint32_t fp64_warps_per_sm; /* 1..32, 0 = 8 */
    /* 0, or a limit on each launch's kernel run time in seconds: past it every
     * warp stops where it is (samples in flight stay unwritten) and the
     * launch's status word gets CHAOS_STATUS_TIMEOUT (chaos_batch_read_status) */
    double time_limit_s;
} chaos_batch_config;

typedef struct chaos_batch chaos_batch;

/* The tier CHAOS_TIER_AUTO picks: binary32 while the pixel is at least
 * 2^-18 m, float-float down to 2^-42 m, binary64 below (m = max(|cx|, |cy|, 1/256)). */
uint32_t chaos_batch_auto_tier(double center_x, double center_y, double pixel_size);
/* Upload the viewport table and build one CUDA graph: a memset of the work
 * counters, then one persistent kernel per tier present, forked and joined;
 * perturbation viewports get a reference orbit each (computed here, on the
 * host, at -log2(pixel) + 96 bits) and run one after another on a fourth
 * branch of the graph. */
int chaos_batch_create(const chaos_viewport *viewports, uint32_t n, const uint32_t *palette, uint32_t palette_len,
                       uint32_t interior_rgba, const chaos_batch_config *config, chaos_batch **out);
/* Autotuner: for each tier slot present among the viewports (binary32,
 * float-float, binary64; perturbation viewports are not tuned), time every
 * launch shape of threads {128, 256, 512} x escape block {8, 16, 32} x chunk
 * {1, 2, 4} on a sample of that tier's viewports (each cut to its central
 * window of 1/8 of its width and height, at least 32 pixels, same pixel size,
 * samples and iteration limit) and write the
 * fastest into *config (slots without viewports stay 0 = default).  When
 * binary64 shares the batch with another tier, the shared launch is then
 * tuned on a joint sample (1/4 of each side): threads {128, 256} of each
 * tier, 16-step binary64 blocks and fp64_warps_per_sm {8, 12, 16}.  With a
 * cache_path, shapes found before for the same device, SM count, slot and
 * viewport parameters are read from that text file and new ones appended;
 * *from_cache (optional) is 1 when nothing had to be timed.  Synchronous;
 * allocates a scratch buffer for the sample's counts. */
int chaos_batch_autotune(const chaos_viewport *viewports, uint32_t n, const char *cache_path,
                         chaos_batch_config *config, uint32_t *from_cache);
/* One cudaGraphLaunch on `stream` (does not synchronise). */
int chaos_batch_launch(chaos_batch *batch, void *stream);
/* The tier each viewport got (n >= number of viewports). */
int chaos_batch_tiers(const chaos_batch *batch, uint32_t *tiers, uint32_t n);
/* Device address of the batch's pixel-iteration total (reset by every launch). */
int chaos_batch_total(const chaos_batch *batch, unsigned long long **device_total);
/* The same total copied to host memory (synchronises the device). */
int chaos_batch_read_total(const chaos_batch *batch, unsigned long long *total);
/* Iterations of the last launch not run because a sample's state repeated
 * bit for bit (interior; counted in full in the total), copied to the host. */
int chaos_batch_read_cycle_skipped(const chaos_batch *batch, unsigned long long *skipped);
/* CHAOS_STATUS_* bits of the last launch (after it has finished): 0, or
 * CHAOS_STATUS_TIMEOUT when config->time_limit_s ran out. */
int chaos_batch_read_status(const chaos_batch *batch, uint32_t *status);
int chaos_batch_destroy(chaos_batch *batch);

/* ---- serving: concurrent zoom sessions ----------------------------------- */

/* A viewer zooming toward (target_x, target_y): frame 0 shows the plane of
 * width `span` centred on (center_x, center_y); every later frame shrinks the
 * plane by zoom_per_frame about the target, which keeps its place on screen
 * (RenderingController.zoomAt, J/rendering/RenderingController.java:130-150).
 * Frames follow CudaFractalRenderer: renderQuality first, then renderFast
 * (sample reuse from the previous frame, foveation around the target's pixel
 * when CHAOS_FLAG_FOVEATION is set).  The precision of each frame is
 * chaos_select_precision's (binary32 where the reference's renderer would use
 * it), with two changes: a CHAOS_ARITH_FMA session runs the frames the
 * selector puts in binary64 with the escape loop in float-float (sampling
 * geometry in binary64; precision CHAOS_PRECISION_FLOATFLOAT) while the
 * pixel is at least 2^-42 max(|cx|, |cy|, 1/256), and
 * CHAOS_SESSION_FLAG_BINARY64 puts every frame in binary64. */
typedef struct chaos_session_desc {
    uint32_t width, height;
    uint32_t max_iterations;
    float max_super_sampling;
    uint32_t flags; /* CHAOS_FLAG_ADAPTIVE_SS | CHAOS_FLAG_SAMPLE_REUSE | CHAOS_FLAG_FOVEATION | CHAOS_SESSION_FLAG_* */
    uint32_t fractal;
    int32_t arith;
    uint32_t pad_;
    double center_x, center_y, span;
    double target_x, target_y;
    double zoom_per_frame;
    double julia_cx, julia_cy;
} chaos_session_desc;

/* Session flag (beside the kernel flags): every frame in binary64, also
 * where the reference's renderer would pick binary32. */
#define CHAOS_SESSION_FLAG_BINARY64 (1u << 16)

/* One served frame; times in seconds on the server's clock.  start_s is the
 * moment the frame was admitted into a launch (start_s - arrival_s is its
 * queueing delay); gpu_ms is the device time of the launch that rendered it. */
typedef struct chaos_frame_record {
    uint32_t session, frame;
    double arrival_s, start_s, done_s; /* start_s, done_s < 0: not admitted / not finished */
    int32_t precision;                 /* CHAOS_PRECISION_* the frame used */
    int32_t status; /* CHAOS_OK; CHAOS_ERR_TIMEOUT: waited past max_wait_s, or the launch ran past
                       frame_time_limit_s (the frame is incomplete); CHAOS_ERR_STATE: its session was
                       closed first (cancelled); CHAOS_ERR_CUDA: the launch failed */
    double gpu_ms;
} chaos_frame_record;

/* Admission and time limits of a server (chaos_server_configure). */
typedef struct chaos_server_config {
    uint32_t max_frames_in_flight;   /* frames admitted and not finished, over all sessions (default 64, 1..4096) */
    uint32_t max_launches_in_flight; /* launches on the GPU at once, side by side on their own
                                        streams (default 4, 1..6) */
    double max_wait_s;               /* a request not admitted within this time completes with
                                        CHAOS_ERR_TIMEOUT (default 30; 0 = no limit) */
    double frame_time_limit_s;       /* device time a launch may run before its unfinished frames stop
                                        and complete with CHAOS_ERR_TIMEOUT (default 0 = none) */
    double call_timeout_s;           /* longest wait of drain / read / close (default 120) */
} chaos_server_config;

typedef struct chaos_server chaos_server;

/* A server with an HBM budget (bytes) for its sessions' device buffers and
 * one palette (host array, copied).  Its scheduler thread admits frame
 * requests and renders every admitted frame of all sessions in one launch
 * (one persistent kernel per precision / arithmetic / fractal present, each
 * pulling 8x4 tiles of all its frames from one work counter and composing
 * each pixel as it is stored).  A frame completes as soon as its last tile
 * is done (the kernel publishes it to the host), not when its launch ends;
 * a session's next frame is admitted once its previous one has completed,
 * into a new launch that runs beside the ones still on the GPU.  Replaces, per session, the frame loop of
 * CudaFractalRenderer.renderQuality / renderFast
 * (J/cudarenderer/CudaFractalRenderer.java:159-206). */
int chaos_server_create(size_t hbm_budget_bytes, const uint32_t *palette, uint32_t palette_len,
                        chaos_server **out);
int chaos_server_configure(chaos_server *server, const chaos_server_config *config);
int chaos_server_get_config(const chaos_server *server, chaos_server_config *config);
/* Bytes a session of this shape is charged (two reuse buffers + RGBA8 output). */
int chaos_server_session_bytes(const chaos_session_desc *desc, size_t *bytes);
/* Open a session.  Nothing is allocated yet: the session's buffers are
 * allocated when its first frame is admitted, against the HBM budget, and
 * held (with the session's reference orbit, for deep frames) until it is
 * closed.  Fails with CHAOS_ERR_OUT_OF_MEMORY only when the session alone is
 * larger than the whole budget. */
int chaos_server_open(chaos_server *server, const chaos_session_desc *desc, uint32_t *session);
/* Close a session: its queued frames are dropped (status CHAOS_ERR_STATE),
 * its frames on the GPU are cancelled (their kernels stop taking the
 * session's tiles), and its buffers are released, which admits waiting
 * requests.  Returns once that is done, or CHAOS_ERR_TIMEOUT after
 * call_timeout_s. */
int chaos_server_close(chaos_server *server, uint32_t session);
/* Queue the session's next frame and return at once (arrival_s is recorded
 * as the request's arrival time).  The request is admitted when a slot is
 * free (max_frames_in_flight), the session's buffers fit the budget (its
 * first frame; later ones are resident already) and the session's previous
 * frame has been admitted; admitted frames of all sessions go to the GPU
 * together in the next launch.  A Mandelbrot frame past binary64
 * (chaos_select_precision says CHAOS_PRECISION_TOO_BIG, where the
 * reference's renderer stops) is rendered by perturbation around the
 * session's target with binary64 differences, one sample per pixel centre;
 * the target's reference orbit is computed at the first such frame (again
 * when the zoom needs more bits) and held by the session until it closes. */
int chaos_server_submit(chaos_server *server, uint32_t session, double arrival_s);
/* Wait until every queued frame has finished (CHAOS_ERR_TIMEOUT after call_timeout_s). */
int chaos_server_drain(chaos_server *server);
/* Replay a request trace in real time: request k is submitted when the
 * server clock reaches (clock at the call) + arrival_s[k]; then drain. */
int chaos_server_run_trace(chaos_server *server, const uint32_t *sessions, const double *arrival_s, uint32_t n);
/* Records of the most recent frames (at most 65536 are kept, oldest first;
 * *n = their number; at most max are copied). */
int chaos_server_records(chaos_server *server, chaos_frame_record *out, uint32_t max, uint32_t *n);
/* Frames waiting for admission and frames on the GPU. */
int chaos_server_queue(chaos_server *server, uint32_t *waiting, uint32_t *in_flight);
/* The session's latest RGBA8 image (width*height words) and the pixel-iterations
 * its frames have run so far; waits for the session's queued frames. */
int chaos_server_read(chaos_server *server, uint32_t session, uint32_t *host_rgba,
                      unsigned long long *pixel_iterations);

/* The session's latest finished frame, for checking it: its parameters and
 * the device records it wrote (and, for a renderFast frame, the previous
 * frame's records it reused, which stay intact until the session's next
 * frame is admitted). */
typedef struct chaos_served_frame {
    uint32_t frame;
    int32_t precision;  /* CHAOS_PRECISION_* */
    uint32_t advanced;  /* 1: renderFast (fractalRenderAdvanced), 0: renderQuality (fractalRenderMain) */
    uint32_t flags;     /* kernel flags the frame ran with */
    int32_t arith;      /* CHAOS_ARITH_* */
    uint32_t max_iterations;
    float max_super_sampling;
    uint32_t focus_x, focus_y;
    uint32_t pad_;
    double rect[4], rect_reused[4];
    const chaos_pixel_info *pixels;
    long pixels_pitch;
    const chaos_pixel_info *previous;
    long previous_pitch;
} chaos_served_frame;
int chaos_server_frame_state(chaos_server *server, uint32_t session, chaos_served_frame *out);
/* Bytes held by sessions' buffers and the budget. */
int chaos_server_usage(const chaos_server *server, size_t *used, size_t *budget);
/* Seconds since the server was created. */
double chaos_server_clock(const chaos_server *server);
int chaos_server_destroy(chaos_server *server);

/* ---- deep zoom: perturbation against a multi-word reference orbit ------- */

/* The reference orbit Z_n of the frame centre, computed on the host in
 * multi-word fixed point (`bits` of fraction, 64..1536) and kept on the current
 * device.  The centre is given as "[-]I.hex": a decimal integer part and
 * hexadecimal fraction digits (4 bits each), e.g. "-0.8a3f...".  The orbit is
 * stored until the reference escapes or reaches max_iterations. */
typedef struct chaos_orbit chaos_orbit;
int chaos_orbit_create(const char *center_x, const char *center_y, uint32_t bits, uint32_t max_iterations,
                       chaos_orbit **out);
/* Stored entries (Z_0..Z_{stored-1}), the iteration the reference escaped at
 * (max_iterations if it did not) and the precision actually used. */
int chaos_orbit_info(const chaos_orbit *orbit, uint32_t *stored, uint32_t *escaped_at, uint32_t *bits);
int chaos_orbit_destroy(chaos_orbit *orbit);

/* A frame by perturbation (tier CHAOS_TIER_PERTURB_F32 or _F64, Mandelbrot).
 * Sample positions as in chaos_render_frame, with desc->center_x/y read as the
 * frame centre's offset from the orbit's centre in plane units (0, 0: the
 * frame is centred on the orbit): each sample iterates its difference from the
 * reference orbit and restarts from the orbit's start (rebasing) when
 * |z| < |difference| or when the orbit ends.  Outputs as chaos_render_frame. */
int chaos_render_frame_perturb_async(const chaos_frame_desc *desc, const chaos_orbit *orbit,
                                     const chaos_frame_out *out, void *stream);
int chaos_render_frame_perturb(const chaos_frame_desc *desc, const chaos_orbit *orbit, const chaos_frame_out *out,
                               void *stream);

/* chaos_render_frame_host for callers that must not allocate GPU memory (a
 * host whose GPU memory is fixed before it starts serving frames, a JNI/Panama
 * binding without a CUDA allocator).  No counterpart in the reference.  The
 * device-side image, palette, work counter and total live in one 64 MiB array
 * that is part of the library (every GPU that loads it holds the array until
 * exit): frames of at most 16,773,056 pixels (3840x2160 fits), palettes of at
 * most 4096 entries, tiers CHAOS_TIER_F32/F64; larger requests fail with
 * CHAOS_ERR_INVALID_ARGUMENT.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); under lazy module loading
 * (the CUDA default) the array is reserved on that device at the same moment,
 * so make one call during set-up, before the GPU's memory is handed out and
 * before any stream capture.  A failed look-up is retried by the next call.
 * The call synchronises the stream before it returns.  All calls share the
 * array: calls whose GPU work overlaps race.  It takes no time limit
 * (desc->time_limit_s must be 0). */
int chaos_render_frame_host_noalloc(const chaos_frame_desc *desc, const uint32_t *palette, uint32_t palette_len,
                                    uint32_t interior_rgba, uint32_t *rgba_host, unsigned long long *total_host,
                                    void *stream);

/* ---- diagnostics -------------------------------------------------------- */

/* Measured fused-multiply-add throughput of the current device in FLOP/s
 * (an FMA counts 2), binary32 (tier CHAOS_TIER_F32) or binary64
 * (CHAOS_TIER_F64): every thread of a full-occupancy grid runs 8 independent
 * FMA chains.  The roofline denominator of the escape-time kernels. */
int chaos_measure_fma_peak(uint32_t tier, double *flops_per_second);

#ifdef __cplusplus
}
#endif
#endif /* CHAOS_GB300_H */
