// chaos_frame.cuh -- pieces shared by the frame-style kernels (independent
// samples): sample offsets, smooth iteration count, palette interpolation.
// (The float-float number type lives in chaos_device.cuh.)
#pragma once

#include <cstdint>

#include "chaos_device.cuh"
#include "chaos_kernels.cuh"

namespace chaos {

template <class R> __device__ __forceinline__ R unit_interval_t(uint64_t h);
template <> __device__ __forceinline__ float unit_interval_t<float>(uint64_t h)
{
    return (float)(uint32_t)(h >> 40) * 0x1p-24f;
}
template <> __device__ __forceinline__ double unit_interval_t<double>(uint64_t h)
{
    return (double)(h >> 11) * 0x1p-53;
}

// n + 1 - log2(log2|z_n|) for an escaped sample, max_iter for an interior one.
__device__ __forceinline__ float frame_smooth(uint32_t i, float r2, uint32_t max_iter)
{
    if (i >= max_iter) return (float)max_iter;
    if (!(r2 < 3.0e38f)) return (float)i;
    float l = __fmul_rn(0.5f, log2f(r2));
    return __fsub_rn((float)(i + 1u), log2f(l));
}

// Palette sampled with linear interpolation at t = nu mod len.
__device__ __forceinline__ void frame_palette_lerp(const uint32_t *pal, uint32_t len, float nu, float ch[4])
{
    float fl = (float)len;
    float t = fmodf(nu, fl);
    if (t < 0.f) t = __fadd_rn(t, fl);
    uint32_t i0 = (uint32_t)t;
    if (i0 >= len) i0 = len - 1u;
    float f = __fsub_rn(t, (float)i0);
    uint32_t i1 = i0 + 1u == len ? 0u : i0 + 1u;
    uint32_t c0 = pal[i0], c1 = pal[i1];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float a0 = (float)((c0 >> (8 * k)) & 255u), a1 = (float)((c1 >> (8 * k)) & 255u);
        ch[k] = __fmaf_rn(__fsub_rn(a1, a0), f, a0);
    }
}

__device__ __forceinline__ uint32_t frame_pack_rgba(const float acc[4], uint32_t spp)
{
    uint32_t out = 0;
    float n = (float)spp;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float v = __fadd_rn(__fdiv_rn(acc[k], n), 0.5f);
        v = v < 255.f ? v : 255.f;
        out |= ((uint32_t)v & 255u) << (8 * k);
    }
    return out;
}

}  // namespace chaos
