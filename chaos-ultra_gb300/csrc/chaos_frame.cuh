// chaos_frame.cuh -- pieces shared by the frame-style kernels (independent
// samples): sample offsets, smooth iteration count, palette interpolation, and
// the float-float number type of the batched tier.
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

// ---------------------------------------------------------------------------
// float-float: a value hi + lo of two binary32 numbers (|lo| <= ulp(hi)/2),
// about 48 significant bits on the binary32 pipe.  Error-free transformations
// after Knuth (TwoSum), Dekker (Fast2Sum) and the fma-based TwoProd; the
// compositions are the usual double-word ones (Hida, Li, Bailey 2001).
// ---------------------------------------------------------------------------
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_fast_two_sum(float a, float b)  // |a| >= |b|
{
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return FF{s, e};
}

__host__ __device__ __forceinline__ FF ff_from_double(double d)
{
    float hi = (float)d;
    float lo = (float)(d - (double)hi);
    return FF{hi, lo};
}

// Knuth's two-sum: s + err == a + b exactly.
__device__ __forceinline__ float ff_two_sum(float a, float b, float &err)
{
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// One z <- z^2 + c step in float-float, 43 binary32 operations.  The three
// products stay unnormalised (leading product + error term by fused
// multiply-add), the leading terms meet in two-sums, all error terms are
// summed in one fixed order, and each coordinate is normalised once at the
// end:
//   x' = fast_two_sum(t, ((ex - ey) + e1) + e2 + cx.lo),
//        s = two_sum(px, -py; e1), t = two_sum(s, cx.hi; e2)
//   y' = fast_two_sum(u, fma(2, exy, e3) + cy.lo),  u = two_sum(2 pxy, cy.hi; e3)
__device__ __forceinline__ void ff_step(FF &x, FF &y, FF cx, FF cy)
{
    const float px = __fmul_rn(x.hi, x.hi);
    float ex = __fmaf_rn(x.hi, x.hi, -px);
    ex = __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, ex);
    const float py = __fmul_rn(y.hi, y.hi);
    float ey = __fmaf_rn(y.hi, y.hi, -py);
    ey = __fmaf_rn(__fadd_rn(y.hi, y.hi), y.lo, ey);
    const float pxy = __fmul_rn(x.hi, y.hi);
    float exy = __fmaf_rn(x.hi, y.hi, -pxy);
    exy = __fmaf_rn(x.hi, y.lo, exy);
    exy = __fmaf_rn(x.lo, y.hi, exy);

    float e1, e2, e3;
    const float s = ff_two_sum(px, -py, e1);
    const float t = ff_two_sum(s, cx.hi, e2);
    float e = __fsub_rn(ex, ey);
    e = __fadd_rn(e, e1);
    e = __fadd_rn(e, e2);
    e = __fadd_rn(e, cx.lo);
    const FF xn = ff_fast_two_sum(t, e);

    const float u = ff_two_sum(__fadd_rn(pxy, pxy), cy.hi, e3);
    const float f = __fadd_rn(__fmaf_rn(2.f, exy, e3), cy.lo);
    y = ff_fast_two_sum(u, f);
    x = xn;
}

__device__ __forceinline__ float ff_radius2(FF x, FF y) { return __fmaf_rn(x.hi, x.hi, __fmul_rn(y.hi, y.hi)); }

}  // namespace chaos
