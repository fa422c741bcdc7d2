// chaos_kernels.cuh -- launch interface between the C ABI (chaos_api.cu) and the
// library kernels (chaos_kernels.cu).  Internal; not installed.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "chaos_device.cuh"

namespace chaos {

// Counter-based hash for jittered sample offsets: the SplitMix64 output
// function (Steele, Lea, Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014) applied twice.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t sample_hash(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t axis)
{
    return mix64(seed ^ mix64(((uint64_t)pixel << 7) | ((uint64_t)sample << 1) | axis));
}

enum SampleMode { SAMPLES_CENTER = 0, SAMPLES_JITTER = 1 };

template <class R> struct MainArgs {
    void *out;
    long pitch;
    UInt2 size;
    Rect<R> image;
    uint32_t max_iter;
    float max_ss;
    uint32_t flags;
    double jcx, jcy;
    uint32_t tiles_x, n_tiles;
    uint32_t *counter;
    unsigned long long *total;  // optional: pixel-iterations of the samples taken
    NewtonParams newton;        // Newton modules only
    uint32_t tile_chunk;        // tiles per claim (set by the launcher)
};

template <class R> struct AdvancedArgs {
    MainArgs<R> m;
    Rect<R> image_reused;
    const void *in;
    long in_pitch;
    UInt2 focus;
};

template <class R> struct FrameArgs {
    uint32_t w, h, spp, mode, max_iter, n_pix;
    uint64_t seed;
    R center_x, center_y, ps, half_w, half_h;
    R jcx, jcy;
    uint32_t *counts;
    float *smooth;
    PixelInfo *pixels;
    long pixels_pitch;
    uint32_t *rgba;
    const uint32_t *palette;
    uint32_t palette_len;
    uint32_t interior_rgba;
    unsigned long long *total;
    uint32_t *counter;
    unsigned long long *skipped;  // optional: iterations of interior samples proven by a repeated state, not run
    unsigned long long budget_ns; // 0, or the run time after which warps stop (RUN_STATUS_TIMEOUT into *status)
    uint32_t *status;
};

struct ComposeArgs {
    const void *in;
    long pitch;
    uint32_t *out;
    long out_pitch;
    uint32_t w, h;
    const uint32_t *palette;
    uint32_t palette_len;
    float max_ss;
    bool visualize;
    int color_mode;  // ColorMode of the module
    int magnifier;   // colorMagnifier (COLOR_MAGNIFIED)
};

// Launchers (chaos_kernels.cu).  Return the cudaError_t of the launch.
template <class R>
cudaError_t launch_main(const MainArgs<R> &a, int arith, int fractal, int device_sms, cudaStream_t s);
template <class R>
cudaError_t launch_advanced(const AdvancedArgs<R> &a, int arith, int fractal, int device_sms, cudaStream_t s);
template <class R>
cudaError_t launch_frame(const FrameArgs<R> &a, int arith, int fractal, int device_sms, cudaStream_t s);
cudaError_t launch_compose(const ComposeArgs &a, cudaStream_t s);
cudaError_t launch_under_sampled(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> rect, uint32_t max_iter,
                                 uint32_t level, int fractal, double jcx, double jcy, cudaStream_t s);
cudaError_t launch_debug(int fractal, cudaStream_t s);
// Newton modules (chaos_newton.cu, rounded arithmetic).
template <class R> cudaError_t launch_main_newton(const MainArgs<R> &a, int fractal, int device_sms, cudaStream_t s);
template <class R>
cudaError_t launch_advanced_newton(const AdvancedArgs<R> &a, int fractal, int device_sms, cudaStream_t s);
cudaError_t launch_under_sampled_newton(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> rect,
                                        uint32_t max_iter, uint32_t level, int fractal, const NewtonParams &p,
                                        cudaStream_t s);
// FMA-pipe probe: grid x 256 threads, `iters` rounds of 8 independent FMA chains.
cudaError_t launch_fma_peak(bool dbl, int blocks, uint32_t iters, double *sink, cudaStream_t s);

}  // namespace chaos
