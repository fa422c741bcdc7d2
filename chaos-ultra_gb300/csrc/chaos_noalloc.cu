// chaos_noalloc.cu -- chaos_render_frame_host_noalloc: a frame through host
// memory that allocates no device memory at any point.
//
// Who needs it: callers that may not call cudaMalloc -- a host whose GPU
// memory is budgeted up front and must not grow while it serves frames, or a
// thin JNI/Panama binding that owns no CUDA allocator.  chaos_render_frame_host
// keeps its device buffers per thread and grows them with cudaMalloc; this
// entry point puts the same buffers in one fixed array that is part of the
// library image instead.
//
// The array g_noalloc_scratch (64 MiB, 256-byte aligned) is a file-scope
// __device__ variable: every GPU that loads the library holds it until the
// process exits.  Layout: [0, 256) work counter and pixel-iteration total,
// [256, 256 + 16 KiB) the palette (at most 4096 entries), the rest the RGBA8
// image, so a frame may have at most (64 MiB - 256 B - 16 KiB) / 4 =
// 16,773,056 pixels (3840x2160 fits; 4096x4096 does not).
//
// In host code the name g_noalloc_scratch is only a host-side stand-in, not a
// device address.  The first call on each device (with that device current)
// asks the runtime for the real address with cudaGetSymbolAddress and keeps
// it; under lazy module loading (the CUDA default) that is also when the
// device's copy of the array is reserved, so make one call during set-up,
// before the GPU's memory is handed out and before any stream capture.  A
// failed look-up is not kept: the next call tries again.  All calls share the
// one array and it keeps the last call's contents: each call clears the
// counter and total itself, and calls whose GPU work overlaps (different
// streams or threads at once) race on the array.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/chaos_gb300.h"
#include "chaos_kernels.cuh"

namespace chaos {
int api_fail(int code, const char *fmt, ...);  // chaos_api.cu
}

using namespace chaos;

namespace {
constexpr size_t kScratchBytes = 64u << 20;
}

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr size_t kHeaderBytes = 256;
constexpr uint32_t kMaxPalette = 4096;
constexpr size_t kPaletteBytes = kMaxPalette * sizeof(uint32_t);
constexpr size_t kImageOffset = kHeaderBytes + kPaletteBytes;
constexpr uint64_t kMaxPixels = (kScratchBytes - kImageOffset) / sizeof(uint32_t);

constexpr int kMaxDevices = 64;
struct NoAllocDevice {
    std::mutex mu;
    unsigned char *base = nullptr;  // device address of g_noalloc_scratch, once looked up
    int sms = 0;
};
NoAllocDevice g_noalloc[kMaxDevices];

// The device address of this device's copy of the array (with `dev`
// current).  Only a successful look-up is kept.
cudaError_t scratch_of(int dev, unsigned char **base, int *sms)
{
    NoAllocDevice &nd = g_noalloc[dev];
    std::lock_guard<std::mutex> g(nd.mu);
    if (!nd.base) {
        unsigned char *p = nullptr;
        int n = 0;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        nd.sms = n;
        nd.base = p;
    }
    *base = nd.base;
    *sms = nd.sms;
    return cudaSuccess;
}

template <class R>
cudaError_t launch(const chaos_frame_desc *d, unsigned char *base, uint32_t palette_len, uint32_t interior_rgba,
                   int sms, cudaStream_t s)
{
    FrameArgs<R> a{};
    a.w = d->width;
    a.h = d->height;
    a.spp = d->samples_per_pixel;
    a.mode = d->sample_mode;
    a.max_iter = d->max_iterations;
    a.n_pix = d->width * d->height;
    a.seed = d->seed;
    a.center_x = (R)d->center_x;
    a.center_y = (R)d->center_y;
    a.ps = (R)d->pixel_size;
    a.half_w = (R)(0.5 * d->width);
    a.half_h = (R)(0.5 * d->height);
    a.jcx = (R)d->julia_cx;
    a.jcy = (R)d->julia_cy;
    a.counter = reinterpret_cast<uint32_t *>(base);
    a.total = reinterpret_cast<unsigned long long *>(base + 8);
    a.palette = reinterpret_cast<const uint32_t *>(base + kHeaderBytes);
    a.palette_len = palette_len;
    a.interior_rgba = interior_rgba;
    a.rgba = reinterpret_cast<uint32_t *>(base + kImageOffset);
    int arith = d->arith == CHAOS_ARITH_PARITY ? ARITH_PARITY : ARITH_FMA;
    return launch_frame<R>(a, arith, (int)d->fractal, sms, s);
}

}  // namespace

int chaos_render_frame_host_noalloc(const chaos_frame_desc *desc, const uint32_t *palette, uint32_t palette_len,
                                    uint32_t interior_rgba, uint32_t *rgba_host, unsigned long long *total_host,
                                    void *stream)
{
    if (!desc || !palette || !rgba_host) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "desc, palette and rgba_host are required");
    if (palette_len == 0 || palette_len > kMaxPalette)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "palette must have 1..%u entries (got %u)", kMaxPalette,
                        palette_len);
    const uint64_t pixels = (uint64_t)desc->width * desc->height;
    if (desc->width == 0 || desc->height == 0)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "width and height must be positive");
    if (pixels > kMaxPixels)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT,
                        "frame of %llu pixels exceeds the no-alloc scratch limit of %llu pixels (64 MiB)",
                        (unsigned long long)pixels, (unsigned long long)kMaxPixels);
    if (desc->samples_per_pixel < 1 || desc->samples_per_pixel > 64)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "samples_per_pixel must be 1..64");
    if (desc->sample_mode == CHAOS_SAMPLES_CENTER && desc->samples_per_pixel != 1)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "pixel-centre sampling takes one sample per pixel");
    if (desc->sample_mode > CHAOS_SAMPLES_JITTER) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "unknown sample mode");
    if (desc->fractal > 1) return api_fail(CHAOS_ERR_UNKNOWN_FRACTAL, "unknown fractal id %u", desc->fractal);
    if (desc->tier != CHAOS_TIER_F32 && desc->tier != CHAOS_TIER_F64)
        return api_fail(CHAOS_ERR_UNSUPPORTED, "tier %u has no no-alloc variant", desc->tier);
    if (desc->arith != CHAOS_ARITH_FMA && desc->arith != CHAOS_ARITH_PARITY)
        return api_fail(CHAOS_ERR_UNSUPPORTED, "frames take CHAOS_ARITH_FMA or CHAOS_ARITH_PARITY");
    if (desc->time_limit_s != 0.0)
        return api_fail(CHAOS_ERR_UNSUPPORTED, "the no-alloc frame takes no time limit (time_limit_s = 0)");
    if (!std::isfinite(desc->center_x) || !std::isfinite(desc->center_y) || !(desc->pixel_size > 0) ||
        !std::isfinite(desc->pixel_size))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "centre and pixel size must be finite, pixel size > 0");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return api_fail(CHAOS_ERR_UNSUPPORTED, "device %d out of range", dev);
    unsigned char *base = nullptr;
    int sms = 0;
    e = scratch_of(dev, &base, &sms);
    if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "no-alloc scratch set-up: %s", cudaGetErrorString(e));

    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemsetAsync(base, 0, kHeaderBytes, s);  // work counter and total start at zero
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + kHeaderBytes, palette, palette_len * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = desc->tier == CHAOS_TIER_F64 ? launch<double>(desc, base, palette_len, interior_rgba, sms, s)
                                         : launch<float>(desc, base, palette_len, interior_rgba, sms, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgba_host, base + kImageOffset, pixels * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    unsigned long long total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, base + 8, sizeof total, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        // copies queued before the failure may still target rgba_host and the
        // local total: let the stream finish before returning (its own status
        // is already the error reported)
        cudaStreamSynchronize(s);
        return api_fail(CHAOS_ERR_CUDA, "no-alloc frame: %s", cudaGetErrorString(e));
    }
    if (total_host) *total_host = total;
    return CHAOS_OK;
}
