// dropin_module.cu -- the CUDA module the Java host loads by file path.
//
// Built once per fractal (-DCHAOS_DROPIN_FRACTAL=0 mandelbrot, 1 julia) and per
// arithmetic (-DCHAOS_DROPIN_ARITH=ARITH_CONTRACTED | ARITH_PARITY | ARITH_FMA)
// into a cubin that
// J/cudarenderer/FractalRenderingModule.java:73-100 opens with cuModuleLoad and
// resolves with cuModuleGetFunction.  It exports the seven entry points
// FractalRenderingModule.initialize requires, with the parameter order and
// sizes the Java marshalling produces (J/cudarenderer/CudaKernel.java:52-121,
// RenderingKernel.java:20-25, KernelMain.java:19-20, KernelAdvanced.java:26-29,
// KernelCompose.java:24-33, KernelUnderSampled.java), and the __constant__
// symbols the host writes by name (cuModuleGetGlobal):
//     VISUALIZE_SAMPLE_COUNT  bool, 1 byte                     gen.cu:14
//     julia_c                 double[2] (julia)                julia.cu:3
//     roots                   Point<double>[3] = double[6]     newton_generic.cu:7, newton_iterations.cu:7
//     coefficients            double[4]                        newton_generic.cu:8, newton_iterations.cu:8
//     colorMagnifier          int (newton iterations)          newton_iterations.cu:9
// Fractal ids: 0 mandelbrot, 1 julia, 2 newton_wired, 3 newton_generic,
// 4 newton_iterations.
//
// Launch shape is the host's: blocks of 32x32 threads, grid ceil(W/32) x
// ceil(H/32) (CudaFractalRenderer.java:36-37, 242-243, 371-378).  Each warp
// renders the 8x4 pixel tile the reference's getImageIndexes gives it
// (gen.cu:43-53), so adaptive super-sampling votes over the same pixels.
//
// Parameter types mirror the reference's: Point<uint> -> UInt2 (4-byte
// aligned), Rectangle<float|double> -> Rect<float|double> (4- or 8-byte
// aligned), pixel_info_t** -> PixelInfo* (only the pointer value is used).
// Byte offsets (CUDA parameter ABI): Main float 0,8,16,24,40,44,48 (52 B);
// Main double 0,8,16,24,56,60,64 (68 B); Advanced float adds rectReused@52,
// in@72, inPitch@80, focus@88 (96 B); Advanced double adds @72,@104,@112,@120
// (128 B); compose 0,8,16,24,32,40,44,48,56,60 (64 B).
#include <cstdio>

#include "chaos_device.cuh"

#ifndef CHAOS_DROPIN_FRACTAL
#error "define CHAOS_DROPIN_FRACTAL (0 mandelbrot, 1 julia, 2-4 newton wired/generic/iterations)"
#endif
#if CHAOS_DROPIN_FRACTAL >= 2
#include "chaos_newton.cuh"
#endif
#ifndef CHAOS_DROPIN_ARITH
#define CHAOS_DROPIN_ARITH chaos::ARITH_FMA
#endif

using chaos::PixelInfo;
using chaos::Rect;
using chaos::UInt2;

__constant__ bool VISUALIZE_SAMPLE_COUNT = false;
#if CHAOS_DROPIN_FRACTAL == 1
__constant__ double julia_c[2];
#endif
#if CHAOS_DROPIN_FRACTAL == 3 || CHAOS_DROPIN_FRACTAL == 4
__constant__ double roots[6];
__constant__ double coefficients[4];
#endif
#if CHAOS_DROPIN_FRACTAL == 4
__constant__ int colorMagnifier;
#endif

namespace {

constexpr int kFractal = CHAOS_DROPIN_FRACTAL;
constexpr int kArith = CHAOS_DROPIN_ARITH;

__device__ __forceinline__ void julia_constant(double &jx, double &jy)
{
#if CHAOS_DROPIN_FRACTAL == 1
    jx = julia_c[0];
    jy = julia_c[1];
#else
    jx = 0.0;
    jy = 0.0;
#endif
}

__device__ __forceinline__ void newton_constants(chaos::NewtonParams &p)
{
#if CHAOS_DROPIN_FRACTAL == 3 || CHAOS_DROPIN_FRACTAL == 4
    for (int k = 0; k < 6; k++) p.roots[k] = roots[k];
    for (int k = 0; k < 4; k++) p.coefficients[k] = coefficients[k];
#endif
#if CHAOS_DROPIN_FRACTAL == 4
    p.color_magnifier = colorMagnifier;
#endif
    (void)p;
}

__device__ __forceinline__ int color_mode()
{
    return kFractal == 2 || kFractal == 3 ? chaos::COLOR_ROOTS : kFractal == 4 ? chaos::COLOR_MAGNIFIED
                                                                               : chaos::COLOR_PALETTE;
}

__device__ __forceinline__ int color_magnifier()
{
#if CHAOS_DROPIN_FRACTAL == 4
    return colorMagnifier;
#else
    return 1;
#endif
}

// Warp tile of this thread: warp k of a 32-wide block covers x in [8(k%4), +8),
// y in [4(k/4), +4) of the block's region (gen.cu:43-53, blockDim.x == 32).
__device__ __forceinline__ void warp_tile(uint32_t &x0, uint32_t &y0, uint32_t &lane)
{
    uint32_t tid = threadIdx.x + threadIdx.y * blockDim.x;
    uint32_t warp = tid >> 5;
    lane = tid & 31u;
    x0 = blockDim.x * blockIdx.x + 8u * (warp & 3u);
    y0 = blockDim.y * blockIdx.y + 4u * (warp >> 2);
}

template <class R>
__device__ __forceinline__ void main_entry(PixelInfo *out, long pitch, UInt2 size, Rect<R> image, uint32_t max_iter,
                                           float max_ss, uint32_t flags)
{
    uint32_t x0, y0, lane;
    warp_tile(x0, y0, lane);
    if (x0 >= size.x || y0 >= size.y) return;  // whole warp outside the image
    double jx, jy;
    julia_constant(jx, jy);
    chaos::SampleGeometry<R> g = chaos::make_geometry(image, size, max_iter, jx, jy);
    newton_constants(g.newton);
    unsigned long long iters = 0;  // the Java host reads no iteration counts
    chaos::render_main_tile<R, kArith, kFractal>(g, out, pitch, size, x0, y0, lane, max_ss, flags, iters);
}

template <class R>
__device__ __forceinline__ void advanced_entry(PixelInfo *out, long pitch, UInt2 size, Rect<R> image,
                                               uint32_t max_iter, float max_ss, uint32_t flags, Rect<R> image_reused,
                                               PixelInfo *in, long in_pitch, UInt2 focus)
{
    uint32_t x0, y0, lane;
    warp_tile(x0, y0, lane);
    if (x0 >= size.x || y0 >= size.y) return;
    double jx, jy;
    julia_constant(jx, jy);
    chaos::SampleGeometry<R> g = chaos::make_geometry(image, size, max_iter, jx, jy);
    newton_constants(g.newton);
    unsigned long long iters = 0;
    chaos::render_advanced_tile<R, kArith, kFractal>(g, image, image_reused, out, pitch, size, in, in_pitch, focus, x0,
                                                     y0, lane, max_ss, flags, iters);
}

}  // namespace

extern "C" __global__ void __launch_bounds__(1024, 1) init() {}

// gen.cu:384-387
extern "C" __global__ void __launch_bounds__(1024, 1)
    fractalRenderMainFloat(PixelInfo *output, long outputPitch, UInt2 outputSize, Rect<float> image,
                           unsigned maxIterations, float maxSuperSampling, unsigned flags)
{
    main_entry<float>(output, outputPitch, outputSize, image, maxIterations, maxSuperSampling, flags);
}

// gen.cu:401-405
extern "C" __global__ void __launch_bounds__(1024, 1)
    fractalRenderMainDouble(PixelInfo *output, long outputPitch, UInt2 outputSize, Rect<double> image,
                            unsigned maxIterations, float maxSuperSampling, unsigned flags)
{
    main_entry<double>(output, outputPitch, outputSize, image, maxIterations, maxSuperSampling, flags);
}

// gen.cu:423-426
extern "C" __global__ void __launch_bounds__(1024, 1)
    fractalRenderAdvancedFloat(PixelInfo *output, long outputPitch, UInt2 outputSize, Rect<float> image,
                               unsigned maxIterations, float maxSuperSampling, unsigned flags,
                               Rect<float> imageReused, PixelInfo *input, long inputPitch, UInt2 focus)
{
    advanced_entry<float>(output, outputPitch, outputSize, image, maxIterations, maxSuperSampling, flags, imageReused,
                          input, inputPitch, focus);
}

// gen.cu:444-448
extern "C" __global__ void __launch_bounds__(1024, 1)
    fractalRenderAdvancedDouble(PixelInfo *output, long outputPitch, UInt2 outputSize, Rect<double> image,
                                unsigned maxIterations, float maxSuperSampling, unsigned flags,
                                Rect<double> imageReused, PixelInfo *input, long inputPitch, UInt2 focus)
{
    advanced_entry<double>(output, outputPitch, outputSize, image, maxIterations, maxSuperSampling, flags,
                           imageReused, input, inputPitch, focus);
}

// gen.cu:455-475.  The output and palette are CUDA surface objects (the GL
// textures of the Java host); the palette is one row of 32-bit words.
extern "C" __global__ void __launch_bounds__(1024, 1)
    compose(PixelInfo *inputMain, long inputMainPitch, PixelInfo *inputBcg, long inputBcgPitch,
            cudaSurfaceObject_t surfaceOutput, unsigned width, unsigned height, cudaSurfaceObject_t colorPalette,
            unsigned paletteLength, float maxSuperSampling)
{
    const uint32_t x = blockDim.x * blockIdx.x + threadIdx.x;
    const uint32_t y = blockDim.y * blockIdx.y + threadIdx.y;
    if (x >= width || y >= height) return;
    PixelInfo p = chaos::load_pixel(chaos::pixel_ptr(inputMain, inputMainPitch, x, y));
    uint32_t color;
    if (VISUALIZE_SAMPLE_COUNT) {
        uint32_t full = (uint32_t)fmax(1.0, (double)maxSuperSampling);
        color = chaos::colorize_sample_count((uint32_t)p.weight, full);
        if (p.is_reused) color = chaos::colorize_sample_count((uint32_t)p.weight_of_new_samples, full);
    } else if (color_mode() == chaos::COLOR_ROOTS) {
        color = chaos::colorize_value(p.value, nullptr, 0, chaos::COLOR_ROOTS, 1);
    } else {
        uint32_t vi = (uint32_t)roundf(p.value);
        uint32_t idx = color_mode() == chaos::COLOR_MAGNIFIED
                           ? paletteLength - (vi * (uint32_t)color_magnifier() % paletteLength) - 1u
                           : chaos::palette_index(p.value, paletteLength);
        surf2Dread(&color, colorPalette, (int)(idx * sizeof(uint32_t)), 0);
    }
    surf2Dwrite(color, surfaceOutput, (int)(x * sizeof(uint32_t)), (int)y);
}

// gen.cu:478-503
extern "C" __global__ void __launch_bounds__(1024, 1)
    fractalRenderUnderSampled(PixelInfo *output, long outputPitch, unsigned width, unsigned height,
                              float left_bottom_x, float left_bottom_y, float right_top_x, float right_top_y,
                              unsigned maxIterations, unsigned underSamplingLevel)
{
    const uint32_t ix = (blockDim.x * blockIdx.x + threadIdx.x) * underSamplingLevel;
    const uint32_t iy = (blockDim.y * blockIdx.y + threadIdx.y) * underSamplingLevel;
    if (ix >= width - underSamplingLevel || iy >= height - underSamplingLevel) return;
    float pw = __fdiv_rn(__fsub_rn(right_top_x, left_bottom_x), (float)width);
    float ph = __fdiv_rn(__fsub_rn(right_top_y, left_bottom_y), (float)height);
    float cx = __fadd_rn(left_bottom_x, __fmul_rn((float)ix, pw));
    float cy = __fsub_rn(right_top_y, __fmul_rn((float)iy, ph));
    double jx, jy;
    julia_constant(jx, jy);
    chaos::SampleGeometry<float> g{};
    g.max_iter = maxIterations;
    g.jcx = (float)jx;
    g.jcy = (float)jy;
    newton_constants(g.newton);
    uint32_t e = chaos::compute_fractal_g<float, kArith, kFractal>(g, cx, cy);
    chaos::store_pixel(chaos::pixel_ptr(output, outputPitch, ix, iy),
                       chaos::make_pixel((float)e, __fdiv_rn(1.f, (float)underSamplingLevel)));
}

// gen.cu:505-512
extern "C" __global__ void debug()
{
    const uint32_t x = blockDim.x * blockIdx.x + threadIdx.x;
    const uint32_t y = blockDim.y * blockIdx.y + threadIdx.y;
    // debugFractal: the escape-time modules greet, the Newton modules' is empty
    if (x == 0 && y == 0 && kFractal <= 1) printf("hello from %s\n", kFractal == 1 ? "julia" : "mandelbrot");
}
