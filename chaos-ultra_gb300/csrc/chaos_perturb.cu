// chaos_perturb.cu -- deep-zoom tier: perturbation against a reference orbit.
//
// The reference orbit Z_n of the frame centre C is computed on the host in
// multi-word fixed point (bigfix.h) and kept on the device.  Each sample at
// c = C + dc iterates only its difference d_n = z_n - Z_m in binary32 or
// binary64:
//     d_{n+1} = (2 Z_m + d_n) d_n + dc,   m <- m + 1,   z_{n+1} = Z_m + d_{n+1}
// Escape is tested on z (continue while |z|^2 < 4, as the reference loop).
// Glitch test and repair (rebasing): when |z| < |d| the difference has lost
// its precision relative to z, so the sample restarts from the start of the
// orbit with d = z (Z_0 = 0); the same happens when m reaches the end of a
// reference orbit that escaped early.  Rebases are counted.  The squares of
// the glitch test underflow at depth (|d| < 1e-19 in binary32, 1e-154 in
// binary64), so when |z|^2 is that small the test is redone with scaled or
// wider operands.
//
// Binary32 differences below the binary32 range (pixel < 1e-30) are rescaled:
// d = w 2^e, dc = u 2^e with w, u binary32 near 1 and e an integer per sample,
//     w' = (2 Z + 2^e w) w + u
// (the 2^e w term is dropped once 2^e is below the binary32 normal range, where
// it is below binary32 resolution against 2 Z), renormalised by powers of 2^24
// when |w| leaves [2^-24, 2^24].  Once 2^e reaches 2^-100 the sample continues with
// plain binary32 differences d = w 2^e.  While rescaled, |d| < 2^-76, so a
// glitch needs |Z_m| below 2^-50: that rare case is tested on the binary64
// orbit in units of 2^e.  While 2^e is below the normal range the step is
// linear, w' = 2 Z w + u, and the tests of a step depend on the orbit index
// alone (escape only where binary32 |Z|^2 >= 4, the glitch test only where it
// is below 2^-100, the orbit's end), so the orbit carries, per index, the next
// index where one of them can fire, and steps up to it run as a block of
// 4 FFMA each on a stored 2Z; a whole block of 16 runs as one composed map
// w' = P w + Q u.  The same composed map also stands in for 16 full steps of a
// binary32 difference at e >= -126 or a plain one, while the difference stays
// so far below the orbit over the block that the dropped d^2 term is below
// binary32 rounding (a per-index exponent bound, lin_lim, set on the host from
// |Z_j| and the partial products); 64-step maps go first where their bound
// allows.  Binary64 differences have their own 16- and 64-step maps and bounds
// (binary64 rounding); where those do not apply, short linear steps run
// while |d| and |dc| stay below 2^-120 and both components of Z above 2^-20:
// then 2Z + d rounds to 2Z and Z + d' to Z, so d' = 2Z d + dc (4 DFMA) is the
// full step bit for bit, and its tests depend on the orbit index alone.
// A sample past all of these forms for the rest of a round (a plain difference
// too large for the blocks) runs its steps in a tight loop, entered by all the
// warp's stepping lanes together or by none.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "bigfix.h"
#include "chaos_kernels.cuh"
#include "chaos_trace.h"

namespace chaos {

int api_fail(int code, const char *fmt, ...);  // chaos_api.cu
int api_device_counter(cudaStream_t s, uint32_t **counter, int *sms);
int api_device_status(const uint32_t *counter, cudaStream_t s, uint32_t **status);
bool api_budget(double seconds, unsigned long long *ns);
int api_read_status(const uint32_t *status, cudaStream_t s, double seconds);

template <class D> struct Vec2T;
template <> struct Vec2T<float> {
    using type = float2;
};
template <> struct Vec2T<double> {
    using type = double2;
};

template <class D> struct PerturbArgs {
    uint32_t w, h, spp, mode, max_iter, n_pix;
    uint64_t seed;
    double ps, half_w, half_h;
    double off_x, off_y;                   // frame centre - orbit centre (plane units)
    const typename Vec2T<D>::type *orbit;  // Z_0 .. Z_{orbit_last}
    const double2 *orbit64;                // the same orbit in binary64 (rescaled glitch test)
    const float2 *orbit2;                  // 2 Z_m in binary32 (rescaled linear steps)
    const float4 *bla16;                   // the 16 rescaled linear steps from m composed: (P, Q), w' = P w + Q u
    const float4 *bla64;                   // the same for 64 steps
    const char2 *lin_lim;                  // largest e + ilogb(max |w|, |u|) for which bla16[m] (x) and bla64[m] (y)
                                           // stand in for full steps
    const double2 *bla16d, *bla64d;        // the same for binary64 differences: P at [2m], Q at [2m + 1]
    const char2 *lin_limd;                 // their bounds on ilogb(max |d|, |dc|)
    const uint32_t *next_event;            // first index >= m where a rescaled step's test can fire
    const double2 *orbit2_64;              // 2 Z_m in binary64 (binary64 linear steps)
    const uint32_t *next_event64;          // first index >= m where a binary64 linear step may not be exact
    uint32_t orbit_last;
    uint32_t *counts;
    float *smooth;
    PixelInfo *pixels;
    long pixels_pitch;
    uint32_t *rgba;
    const uint32_t *palette;
    uint32_t palette_len;
    uint32_t interior_rgba;
    unsigned long long *total;
    unsigned long long *rebases;
    uint32_t *counter;
    unsigned long long budget_ns;  // 0, or the run time after which warps stop (RUN_STATUS_TIMEOUT into *status)
    uint32_t *status;
    // binary32 set-up of rescaled samples at pixel centres (dc_fast): with
    // t = p - (half - 1/2), exact in binary32, dc 2^-dc_e = t ps' + off' where
    // ps' = ps 2^-dc_e in [1, 2) and off' = off 2^-dc_e are binary32 pairs
    bool dc_fast;
    int dc_e;
    float dc_hw, dc_hh, dc_ps_hi, dc_ps_lo, dc_ox_hi, dc_ox_lo, dc_oy_hi, dc_oy_lo;
};

__device__ __forceinline__ double unit53(uint64_t h) { return (double)(h >> 11) * 0x1p-53; }

// n + 1 - log2(log2|z_n|), as the plain frame path.
__device__ __forceinline__ float perturb_smooth(uint32_t i, float r2, uint32_t max_iter)
{
    if (i >= max_iter) return (float)max_iter;
    if (!(r2 < 3.0e38f)) return (float)i;
    float l = __fmul_rn(0.5f, log2f(r2));
    return __fsub_rn((float)(i + 1u), log2f(l));
}

__device__ __forceinline__ void perturb_palette(const uint32_t *pal, uint32_t len, float nu, float ch[4])
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

// |z| < |d| for the glitch test, exact where the squares would underflow.
__device__ __forceinline__ bool glitch_test(float zx, float zy, float dx, float dy, float r2)
{
    if (r2 >= 0x1p-60f) return r2 < __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
    double z2 = (double)zx * zx + (double)zy * zy, d2 = (double)dx * dx + (double)dy * dy;
    return z2 < d2;
}
__device__ __forceinline__ bool glitch_test(double zx, double zy, double dx, double dy, double r2)
{
    if (r2 >= 0x1p-500) return r2 < __fma_rn(dx, dx, __dmul_rn(dy, dy));
    const double k = 0x1p600;  // exact scaling; an infinite |d|^2 means |d| >> |z|
    zx *= k, zy *= k, dx *= k, dy *= k;
    return zx * zx + zy * zy < dx * dx + dy * dy;
}

// 2^e as a binary32, or 0 below the normal range
__device__ __forceinline__ float pow2f(int e) { return e >= -126 ? __int_as_float((e + 127) << 23) : 0.f; }

// lin_lim[m] where no composed block may start at m
constexpr int LIN_NONE = -128;

// Keep the scaled difference's larger component within [2^-24, 2^24]: w and u
// move by multiples of 2^24 and e the other way.  Past e > -100 the sample leaves the
// rescaled form and holds d = w 2^e, dc = u 2^e directly.
template <class D>
__device__ __forceinline__ void renormalise(D &dx, D &dy, D &dcx, D &dcy, int &e, bool &scaled)
{
    const float mag = fmaxf(fabsf((float)dx), fabsf((float)dy));
    if (mag > 0x1p24f) {
        // by the multiple of 24 that brings |w| below 2^24 (more than one after a
        // 64-step block; |w| < 2^128 so k <= 120)
        const int k = 24 * (((int)((__float_as_uint(mag) >> 23) & 255u) - 127) / 24);
        const float sc = __int_as_float((127 - k) << 23);
        dx *= D(sc), dy *= D(sc), dcx *= D(sc), dcy *= D(sc);
        e += k;
        if (e > -100) {
            const float q = pow2f(e);
            dx *= q, dy *= q, dcx *= q, dcy *= q;
            scaled = false;
        }
    } else if (mag < 0x1p-24f && mag > 0.f && e > -1000) {
        dx *= D(0x1p24f), dy *= D(0x1p24f), dcx *= D(0x1p24f), dcy *= D(0x1p24f);
        e -= 24;
    }
}

// Five blocks of 256 per SM for binary32 differences (48 registers: the
// kernel is issue-bound and a sixth warp per scheduler hides more of the
// orbit loads than extra registers save), four for binary64 (64 registers)
template <class D, int K, bool S> __global__ void __launch_bounds__(256, sizeof(D) == 4 ? 5 : 4) k_perturb(PerturbArgs<D> a)
{
    static_assert(!S || sizeof(D) == 4, "rescaling is for binary32 differences");
    using O = Op<D>;
    constexpr uint32_t FULLM = 0xffffffffu;
    __shared__ uint32_t s_pal[4096];
    const uint32_t *pal = a.palette;
    if (a.rgba && a.palette_len <= 4096u) {
        for (uint32_t k = threadIdx.x; k < a.palette_len; k += blockDim.x) s_pal[k] = a.palette[k];
        pal = s_pal;
    }
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t w_magic = div_magic(a.w);
    uint32_t pix = 0xffffffffu, s = 0, i = 0, m = 0;
    // rescaled samples keep w in (dx, dy) and u in (dcx, dcy), with d = w 2^e
    D dx = D(0), dy = D(0), dcx = D(0), dcy = D(0), Zx = D(0), Zy = D(0);
    int e = 0;
    bool scaled = false;
    bool lin = true;      // composed blocks may still apply to this sample
    uint32_t lin_at = 0;  // the iteration from which to check for them again
    bool need = true, begin = false;
    float acc_v = 0.f, acc[4] = {0.f, 0.f, 0.f, 0.f};
    unsigned long long iters = 0, rebases = 0;
    const unsigned long long t_start = a.budget_ns ? global_ns() : 0ull;

    for (;;) {
        // a time limit: the warp stops where it is (its samples in flight stay unwritten)
        if (out_of_time(a.budget_ns, t_start, a.status, lane)) break;
        uint32_t need_mask = __ballot_sync(FULLM, need);
        if (need_mask) {
            uint32_t leader = __ffs(need_mask) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (uint32_t)__popc(need_mask));
            base = __shfl_sync(FULLM, base, leader);
            if (need) {
                pix = base + (uint32_t)__popc(need_mask & lt_mask);
                need = false;
                begin = true;
                s = 0;
                acc_v = 0.f;
                acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
            }
        }
        const bool active = pix < a.n_pix;
        if (!__any_sync(FULLM, active)) break;

        bool done = false;
        D r2 = D(0);
        if (active) {
            if (begin) {
                begin = false;
                uint32_t px, py;
                divmod_magic(pix, a.w, w_magic, py, px);
                scaled = false;
                bool wide = true;  // the binary64 set-up
                if constexpr (S) if (a.dc_fast) {
                    // on the FP32 pipe: the binary64 one costs each sample a chain of
                    // seven dependent binary64 operations
                    const float tx = __fsub_rn((float)px, a.dc_hw), ty = __fsub_rn(a.dc_hh, (float)py);
                    const float vx =
                        __fmaf_rn(tx, a.dc_ps_hi, __fadd_rn(__fmaf_rn(tx, a.dc_ps_lo, a.dc_ox_lo), a.dc_ox_hi));
                    const float vy =
                        __fmaf_rn(ty, a.dc_ps_hi, __fadd_rn(__fmaf_rn(ty, a.dc_ps_lo, a.dc_oy_lo), a.dc_oy_hi));
                    const float big = fmaxf(fabsf(vx), fabsf(vy));
                    if (big >= 0x1p-100f) {  // |v| < 2^102 by the host's bound on off'
                        const int k = (int)((__float_as_uint(big) >> 23) & 255u) - 127;
                        const float sk = __int_as_float((127 - k) << 23);  // 2^-k, exact
                        const int e0 = a.dc_e + k;
                        dcx = (D)(vx * sk);
                        dcy = (D)(vy * sk);
                        if (e0 < -100) {
                            e = e0;
                            scaled = true;
                        } else {
                            const float s0 = __int_as_float((127 + e0) << 23);  // 2^e0, normal
                            dcx *= D(s0), dcy *= D(s0);
                        }
                        wide = false;
                    }
                }
                if (wide) {
                    double ox = 0.5, oy = 0.5;
                    if (a.mode == SAMPLES_JITTER) {
                        ox = unit53(sample_hash(a.seed, pix, s, 0));
                        oy = unit53(sample_hash(a.seed, pix, s, 1));
                    }
                    double ddx = __fma_rn(__dsub_rn(__dadd_rn((double)px, ox), a.half_w), a.ps, a.off_x);
                    double ddy = __fma_rn(-__dsub_rn(__dadd_rn((double)py, oy), a.half_h), a.ps, a.off_y);
                    dcx = (D)ddx;
                    dcy = (D)ddy;
                    if constexpr (S) {
                        // exponent of the larger component (binary64 field), u = dc 2^-e
                        double big = fmax(fabs(ddx), fabs(ddy));
                        int e0 = (int)((__double_as_longlong(big) >> 52) & 0x7ff) - 1023;
                        if (big != 0.0 && e0 < -100) {
                            double k = __longlong_as_double((long long)(1023 - e0) << 52);
                            dcx = (D)(ddx * k);
                            dcy = (D)(ddy * k);
                            e = e0;
                            scaled = true;
                        }
                    }
                }
                dx = D(0);
                dy = D(0);
                Zx = D(0);
                Zy = D(0);
                m = 0;
                i = 0;
                lin = true;
                lin_at = 0;
                if (a.max_iter == 0) done = true;
            }
            // d' = (2Z + d) d + dc with its tests; true when the sample is done
            auto plain_step = [&]() -> bool {
                D wx = O::fma(D(2), Zx, dx), wy = O::fma(D(2), Zy, dy);
                D ndx = O::fma(wx, dx, O::fma(-wy, dy, dcx));
                D ndy = O::fma(wx, dy, O::fma(wy, dx, dcy));
                ++m;
                ++i;
                typename Vec2T<D>::type Z = a.orbit[m];
                D zx = O::add(Z.x, ndx), zy = O::add(Z.y, ndy);
                r2 = O::fma(zx, zx, O::mul(zy, zy));
                if (!(r2 < D(4)) || i == a.max_iter) return true;
                if (m == a.orbit_last || glitch_test(zx, zy, ndx, ndy, r2)) {
                    dx = zx;
                    dy = zy;
                    Zx = D(0);
                    Zy = D(0);
                    m = 0;
                    ++rebases;
                } else {
                    dx = ndx;
                    dy = ndy;
                    Zx = Z.x;
                    Zy = Z.y;
                }
                return false;
            };
#pragma unroll 1
            for (int k = 0; k < K && !done; k++) {
                // the lanes still stepping this round, together here (k is the same on all)
                if (__all_sync(__activemask(), !scaled && (!lin || lin_at >= i + (uint32_t)(K - k)))) {
                    // every one past the composed and linear forms for this round (a
                    // plain difference too large for them): plain steps for the rest of
                    // the round.  Taken by the whole group only: a lane that entered
                    // alone would run its loop while the others wait, and then they theirs.
#pragma unroll 1
                    for (; k < K; k++)
                        if (plain_step()) {
                            done = true;
                            break;
                        }
                    break;
                }
                if constexpr (sizeof(D) == 4) if (lin && i >= lin_at) {
                    // a difference far below the orbit: over the next 64 (16) steps
                    // (2Z_j + d_j) d_j stays within 2^-25 of 2Z_j d_j, below binary32
                    // rounding, and no escape, glitch or orbit end can come, when
                    // e + ilogb(max |w|, |u|) <= lin_lim[m].y (.x); then the composed
                    // map w' = P w + Q u stands in for those steps
                    const float big = fmaxf(fmaxf(fabsf((float)dx), fabsf((float)dy)),
                                            fmaxf(fabsf((float)dcx), fabsf((float)dcy)));
                    const int eb = (scaled ? e : 0) + (int)((__float_as_uint(big) >> 23) & 255u) - 127;
                    const char2 lim = a.lin_lim[m];
                    const uint32_t left = a.max_iter - i;
                    const bool b64 = lim.y != LIN_NONE && eb <= lim.y && left > 64u;
                    if (b64 || (lim.x != LIN_NONE && eb <= lim.x && left > 16u)) {
                        const float4 pq = (b64 ? a.bla64 : a.bla16)[m];
                        const float wx = (float)dx, wy = (float)dy, ux = (float)dcx, uy = (float)dcy;
                        dx = __fmaf_rn(pq.x, wx, __fmaf_rn(-pq.y, wy, __fmaf_rn(pq.z, ux, -pq.w * uy)));
                        dy = __fmaf_rn(pq.x, wy, __fmaf_rn(pq.y, wx, __fmaf_rn(pq.z, uy, pq.w * ux)));
                        const uint32_t L = b64 ? 64u : 16u;
                        m += L;
                        i += L;
                        const typename Vec2T<D>::type Z = a.orbit[m];
                        Zx = Z.x;
                        Zy = Z.y;
                        if (scaled) renormalise(dx, dy, dcx, dcy, e, scaled);
                        continue;
                    }
                    // lin_lim never exceeds -25: a plain difference that large stays out;
                    // one 8 binades past this index's bound (it grows ~1 binade a step,
                    // and the bound moves by a few between indices) is taken as out too
                    if (!scaled && (eb > -25 || (lim.x != LIN_NONE && eb > lim.x + 8)))
                        lin = false;
                    else if (lim.x != LIN_NONE)
                        lin_at = i + K;  // near the bound: a difference that hovers there
                                         // (interior samples) is checked once a round
                }
                if constexpr (S) if (scaled && e < -126) {
                    // linear steps up to (not onto) the next index whose tests can fire
                    constexpr uint32_t B = 16;  // |w| <= 2^24 grows at most 4^16-fold: below 2^56
                    const uint32_t ev = a.next_event[m + 1];
                    const uint32_t n = min(min(B, ev - (m + 1)), a.max_iter - 1u - i);
                    if (n > 0) {
                        float wx = (float)dx, wy = (float)dy;
                        const float ux = (float)dcx, uy = (float)dcy;
                        const float2 *Z2p = a.orbit2 + m;
                        if (n == B) {
                            // the usual case: a whole block, its 16 steps composed on the host
                            // into w' = P w + Q u (one 16-byte load, eight operations)
                            const float4 pq = a.bla16[m];
                            const float nx =
                                __fmaf_rn(pq.x, wx, __fmaf_rn(-pq.y, wy, __fmaf_rn(pq.z, ux, -pq.w * uy)));
                            const float ny = __fmaf_rn(pq.x, wy, __fmaf_rn(pq.y, wx, __fmaf_rn(pq.z, uy, pq.w * ux)));
                            wx = nx;
                            wy = ny;
                        } else {
                            for (uint32_t j = 0; j < n; j++) {
                                const float2 Z2 = Z2p[j];
                                const float nx = __fmaf_rn(Z2.x, wx, __fmaf_rn(-Z2.y, wy, ux));
                                const float ny = __fmaf_rn(Z2.x, wy, __fmaf_rn(Z2.y, wx, uy));
                                wx = nx;
                                wy = ny;
                            }
                        }
                        m += n;
                        i += n;
                        const typename Vec2T<D>::type Z = a.orbit[m];
                        Zx = Z.x;
                        Zy = Z.y;
                        dx = wx;
                        dy = wy;
                        renormalise(dx, dy, dcx, dcy, e, scaled);
                        continue;
                    }
                }
                if constexpr (S) if (scaled) {
                    // w' = (2Z + 2^e w) w + u
                    const float q = pow2f(e);
                    float ax = __fmaf_rn(q, (float)dx, 2.f * (float)Zx), ay = __fmaf_rn(q, (float)dy, 2.f * (float)Zy);
                    float nwx = __fmaf_rn(ax, (float)dx, __fmaf_rn(-ay, (float)dy, (float)dcx));
                    float nwy = __fmaf_rn(ax, (float)dy, __fmaf_rn(ay, (float)dx, (float)dcy));
                    ++m;
                    ++i;
                    typename Vec2T<D>::type Z = a.orbit[m];
                    float zx = __fmaf_rn(nwx, q, (float)Z.x), zy = __fmaf_rn(nwy, q, (float)Z.y);
                    r2 = O::fma(zx, zx, O::mul(zy, zy));
                    if (!(r2 < D(4)) || i == a.max_iter) {
                        done = true;
                        break;
                    }
                    if (m == a.orbit_last) {
                        // the orbit ends: continue unscaled from z
                        dx = zx;
                        dy = zy;
                        dcx = (D)((float)dcx * q);
                        dcy = (D)((float)dcy * q);
                        scaled = false;
                        Zx = Zy = D(0);
                        m = 0;
                        ++rebases;
                        continue;
                    }
                    if (r2 < 0x1p-100f) {
                        // |Z| < 2^-50: glitch test in units of 2^e on the binary64 orbit
                        const double2 Zd = a.orbit64[m];
                        const double k2 = __longlong_as_double((long long)(1023 - e) << 52);
                        double sx = fma(Zd.x, k2, (double)nwx), sy = fma(Zd.y, k2, (double)nwy);
                        if (sx * sx + sy * sy < (double)nwx * nwx + (double)nwy * nwy) {
                            dx = (D)sx;
                            dy = (D)sy;
                            Zx = Zy = D(0);
                            m = 0;
                            ++rebases;
                            continue;
                        }
                    }
                    dx = nwx;
                    dy = nwy;
                    Zx = Z.x;
                    Zy = Z.y;
                    renormalise(dx, dy, dcx, dcy, e, scaled);
                    continue;
                }
                if constexpr (sizeof(D) == 8) if (lin && i >= lin_at) {
                    // the composed blocks for binary64 differences: over the next 64 (16)
                    // steps the dropped d^2 term stays below binary64 rounding and no
                    // test can fire when ilogb(max |d|, |dc|) <= lin_limd[m].y (.x)
                    const double big = fmax(fmax(fabs((double)dx), fabs((double)dy)),
                                            fmax(fabs((double)dcx), fabs((double)dcy)));
                    const int eb = (int)(((uint32_t)__double2hiint(big) >> 20) & 0x7ffu) - 1023;
                    const char2 lim = a.lin_limd[m];
                    const uint32_t left = a.max_iter - i;
                    const bool b64 = lim.y != LIN_NONE && eb <= lim.y && left > 64u;
                    if (b64 || (lim.x != LIN_NONE && eb <= lim.x && left > 16u)) {
                        const double2 *pq = (b64 ? a.bla64d : a.bla16d) + 2u * m;
                        const double2 P = pq[0], Q = pq[1];
                        const double wx = (double)dx, wy = (double)dy, ux = (double)dcx, uy = (double)dcy;
                        dx = (D)__fma_rn(P.x, wx, __fma_rn(-P.y, wy, __fma_rn(Q.x, ux, -Q.y * uy)));
                        dy = (D)__fma_rn(P.x, wy, __fma_rn(P.y, wx, __fma_rn(Q.x, uy, Q.y * ux)));
                        const uint32_t L = b64 ? 64u : 16u;
                        m += L;
                        i += L;
                        const typename Vec2T<D>::type Z = a.orbit[m];
                        Zx = Z.x;
                        Zy = Z.y;
                        continue;
                    }
                    // lin_limd never exceeds -54: a difference that large stays out (and,
                    // as for binary32, one 8 binades past this index's bound)
                    if (eb > -54 || (lim.x != LIN_NONE && eb > lim.x + 8))
                        lin = false;
                    else if (lim.x != LIN_NONE)
                        lin_at = i + K;
                }
                if constexpr (!S && sizeof(D) == 8) {
                    // binary64 differences far below the orbit (|d|, |dc| < 2^-120 while
                    // both components of Z stay above 2^-20): 2Z + d rounds to 2Z and
                    // Z + d' to Z, so the step is d' = 2Z d + dc bit for bit and its tests
                    // depend on the orbit index alone; run up to 16 such steps, stopping
                    // before the next index where that fails (next_event64)
                    const uint32_t big = max(max((uint32_t)__double2hiint(dx) & 0x7ff00000u,
                                                 (uint32_t)__double2hiint(dy) & 0x7ff00000u),
                                             max((uint32_t)__double2hiint(dcx) & 0x7ff00000u,
                                                 (uint32_t)__double2hiint(dcy) & 0x7ff00000u));
                    if (big < (903u << 20)) {
                        const uint32_t ev = a.next_event64[m];
                        const uint32_t n = min(min(16u, ev > m ? ev - m - 1u : 0u), a.max_iter - 1u - i);
                        if (n > 0) {
                            double wx = dx, wy = dy;
                            const double2 *Z2p = a.orbit2_64 + m;
                            if (n == 16) {
#pragma unroll
                                for (uint32_t j = 0; j < 16; j++) {
                                    const double2 Z2 = Z2p[j];
                                    const double nx = __fma_rn(Z2.x, wx, __fma_rn(-Z2.y, wy, (double)dcx));
                                    const double ny = __fma_rn(Z2.x, wy, __fma_rn(Z2.y, wx, (double)dcy));
                                    wx = nx;
                                    wy = ny;
                                }
                            } else {
                                for (uint32_t j = 0; j < n; j++) {
                                    const double2 Z2 = Z2p[j];
                                    const double nx = __fma_rn(Z2.x, wx, __fma_rn(-Z2.y, wy, (double)dcx));
                                    const double ny = __fma_rn(Z2.x, wy, __fma_rn(Z2.y, wx, (double)dcy));
                                    wx = nx;
                                    wy = ny;
                                }
                            }
                            m += n;
                            i += n;
                            const typename Vec2T<D>::type Z = a.orbit[m];
                            Zx = Z.x;
                            Zy = Z.y;
                            dx = wx;
                            dy = wy;
                            continue;
                        }
                    }
                }
                if (plain_step()) {
                    done = true;
                    break;
                }
            }
        }
        if (done) {
            const bool escaped = i < a.max_iter || !(r2 < D(4));
            const uint32_t cnt = i;
            const float nu = escaped && i < a.max_iter ? perturb_smooth(i, (float)r2, a.max_iter)
                                                       : (float)a.max_iter;
            const size_t sidx = (size_t)pix * a.spp + s;
            if (a.counts) a.counts[sidx] = cnt;
            if (a.smooth) a.smooth[sidx] = nu;
            iters += cnt;
            const bool esc = cnt < a.max_iter;
            acc_v = __fadd_rn(acc_v, esc ? nu : 0.f);
            if (a.rgba) {
                float ch[4];
                if (esc) {
                    perturb_palette(pal, a.palette_len, nu, ch);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) ch[k] = (float)((a.interior_rgba >> (8 * k)) & 255u);
                }
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = __fadd_rn(acc[k], ch[k]);
            }
            ++s;
            if (s == a.spp) {
                uint32_t px, py;
                divmod_magic(pix, a.w, w_magic, py, px);
                if (a.pixels)
                    store_pixel(pixel_ptr(a.pixels, a.pixels_pitch, px, py),
                                make_pixel(a.spp == 1u ? acc_v : __fdiv_rn(acc_v, (float)a.spp), (float)a.spp));
                if (a.rgba) {
                    uint32_t out = 0;
                    float n = (float)a.spp;
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        float v = __fadd_rn(a.spp == 1u ? acc[k] : __fdiv_rn(acc[k], n), 0.5f);
                        v = v < 255.f ? v : 255.f;
                        out |= ((uint32_t)v & 255u) << (8 * k);
                    }
                    a.rgba[pix] = out;
                }
                need = true;
            } else {
                begin = true;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        iters += __shfl_down_sync(FULLM, iters, o);
        rebases += __shfl_down_sync(FULLM, rebases, o);
    }
    if (lane == 0) {
        if (a.total && iters) atomicAdd(a.total, iters);
        if (a.rebases && rebases) atomicAdd(a.rebases, rebases);
    }
}

// K = 64 steps (a linear block counts as one) per round between the warp's
// refill checks: on the C3 frames 16, 32, 64, 128 and 256 gave 1508, 1582,
// 1635, 1661 and 1688 Gpixel-iter/s, but a long round also keeps a lane that
// escaped early idle until its warp's round ends, which costs on views whose
// escape counts vary (batch viewports); 64 gained there too (676 -> 687).
template <class D, bool S> static cudaError_t launch_perturb(const PerturbArgs<D> &a, int sms, cudaStream_t s)
{
    static const int occ = [] {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_perturb<D, 64, S>, 256, 0) != cudaSuccess || n < 1)
            n = 1;
        return n;
    }();
    unsigned long long warps = ((unsigned long long)a.n_pix + 31ull) / 32ull;
    unsigned long long blocks = (warps + 7ull) / 8ull;
    unsigned long long cap = (unsigned long long)occ * (unsigned long long)sms;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_perturb<D, 64, S><<<(unsigned)blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace chaos

using namespace chaos;

// ---- reference orbit ---------------------------------------------------------

struct chaos_orbit {
    int device = -1;
    uint32_t max_iter = 0;
    uint32_t last = 0;        // index of the last stored Z
    uint32_t escaped_at = 0;  // iteration at which the reference escaped, or max_iter
    uint32_t bits = 0;
    double center_x = 0, center_y = 0;  // rounded centre, for reporting
    unsigned char *arena = nullptr;     // the one device allocation that holds every table below
    float2 *z32 = nullptr;
    double2 *z64 = nullptr;
    float2 *z2 = nullptr;              // 2 Z in binary32
    float4 *bla16 = nullptr;           // see the rescaled linear steps of k_perturb
    float4 *bla64 = nullptr;           // see the composed blocks of k_perturb
    char2 *lin_lim = nullptr;          // see the composed blocks of k_perturb
    double2 *bla16d = nullptr;         // the same blocks for binary64 differences ((P, Q) as two double2)
    double2 *bla64d = nullptr;
    char2 *lin_limd = nullptr;
    uint32_t *next_event = nullptr;    // see the rescaled linear steps of k_perturb
    double2 *z2_64 = nullptr;          // 2 Z in binary64
    uint32_t *next_event64 = nullptr;  // see the binary64 linear steps of k_perturb
};

static int orbit_compute(const BigFix &cx, const BigFix &cy, int limbs, uint32_t max_iterations, chaos_orbit **out);

int chaos_orbit_create(const char *center_x, const char *center_y, uint32_t bits, uint32_t max_iterations,
                       chaos_orbit **out)
{
    TraceRange trace_("chaos_orbit_create");
    if (!center_x || !center_y || !out) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (max_iterations < 1) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "maxIterations must be a positive number");
    if (bits < 64 || bits > 64u * BIGFIX_MAX_LIMBS)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "precision must be 64..%d bits", 64 * BIGFIX_MAX_LIMBS);
    const int limbs = (int)((bits + 63) / 64);
    BigFix cx, cy;
    if (!bigfix_parse_hex(center_x, limbs, cx) || !bigfix_parse_hex(center_y, limbs, cy))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "centre must be \"[-]I.hex\" fixed point");
    if (cx.w[limbs] > 4 || cy.w[limbs] > 4) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "centre outside |c| < 4");
    return orbit_compute(cx, cy, limbs, max_iterations, out);
}

namespace chaos {
// The orbit of a binary64 centre (the batch's perturbation viewports).
int api_orbit_create_d(double center_x, double center_y, uint32_t bits, uint32_t max_iterations, chaos_orbit **out)
{
    if (!std::isfinite(center_x) || !std::isfinite(center_y) || std::fabs(center_x) >= 4 || std::fabs(center_y) >= 4)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "centre outside |c| < 4");
    const int limbs = (int)((std::min(std::max(bits, 64u), 64u * BIGFIX_MAX_LIMBS) + 63) / 64);
    return orbit_compute(bigfix_from_double(center_x, limbs), bigfix_from_double(center_y, limbs), limbs,
                         max_iterations, out);
}
}  // namespace chaos

// A composed block: L linear steps w <- a_j w + u (a_j = 2Z_j) from m as
// w <- P w + Q u.
struct BlockMap {
    double px = 0, py = 0, qx = 0, qy = 0;
};

// The 16- and 64-step blocks from every index m, composed in binary64 from
// a2[j] = 2Z_j as the kernel holds it, and where each may stand in for full
// steps (lim[m] = (l16, l64)).  With w_j = P_(m->j) w + Q_(m->j) u the
// difference at step j and M = max(|w|, |u|) componentwise,
//     |2^e w_j| < 2^(e + ilogb(M) + 1.5) (|P_j| + |Q_j|)
//              <= 2^(e + ilogb(M) + 1.5) sqrt(2 (|P_j|^2 + |Q_j|^2)),
// and the quadratic term of step j is below the arithmetic's rounding (2^-p
// relative) when that stays below 2^-p |Z_j| (p = slack - 1.5): for
// j = m..m+L that holds when
//     e + ilogb(M) <= floor(log2(rho) / 2 - slack),
//     rho = min_j |Z_j|^2 / (2 (|P_j|^2 + |Q_j|^2))   (zz[j] = |Z_j|^2).
// No test may fire inside: ev[j] is false for j = m+1..m+L (the caller sets
// it where |Z_j|^2 >= 3.99 or < 2^-98, margins on the escape and glitch tests,
// which then see z_j = Z_j to the arithmetic's precision), the block ends
// before the orbit's last index, and Z_m != 0.  A 64-step block also keeps
// |w| below 2^127 at its end (|w|, |u| <= 2^25 before it):
// 2 (|P|^2 + |Q|^2) <= 2^200.  A bound below -127 is stored as none.
static void compose_blocks(const std::vector<double2> &a2, const std::vector<double> &zz,
                           const std::vector<char> &ev, double slack, std::vector<BlockMap> &b16,
                           std::vector<BlockMap> &b64, std::vector<char2> &lim)
{
    const size_t n = a2.size(), last = n - 1;
    b16.assign(n, BlockMap());
    b64.assign(n, BlockMap());
    lim.assign(n, make_char2((signed char)LIN_NONE, (signed char)LIN_NONE));
    auto lim_of = [slack](double rho) {
        if (!(rho > 0.0) || !std::isfinite(rho)) return (int)LIN_NONE;
        const double l = std::floor(0.5 * std::log2(rho) - slack);
        return l < -127.0 ? (int)LIN_NONE : (int)std::min(127.0, l);
    };
    auto part = [&](size_t m0, size_t m1) {
        for (size_t m = m0; m < m1; m++) {
            double px = 1.0, py = 0.0, qx = 0.0, qy = 0.0;
            bool ok16 = m + 16 < last && zz[m] > 0.0, ok64 = m + 64 < last && zz[m] > 0.0;
            double rho = INFINITY, rho16 = INFINITY;
            for (size_t j = m; j <= m + 64 && j < n; j++) {
                if (j > m && ev[j]) {
                    if (j <= m + 16) ok16 = false;
                    ok64 = false;
                }
                if (!ok64 && j > m + 16) break;
                rho = std::min(rho, zz[j] / (2.0 * (px * px + py * py + qx * qx + qy * qy)));
                if (j == m + 16) {
                    rho16 = rho;
                    b16[m] = BlockMap{px, py, qx, qy};
                    if (!ok64) break;
                }
                if (j == m + 64) {
                    if (!(2.0 * (px * px + py * py + qx * qx + qy * qy) <= 0x1p200)) ok64 = false;
                    b64[m] = BlockMap{px, py, qx, qy};
                    break;
                }
                const double ax = a2[j].x, ay = a2[j].y;
                const double npx = ax * px - ay * py, npy = ax * py + ay * px;
                const double nqx = ax * qx - ay * qy + 1.0, nqy = ax * qy + ay * qx;
                px = npx;
                py = npy;
                qx = nqx;
                qy = nqy;
            }
            lim[m] = make_char2((signed char)(ok16 ? lim_of(rho16) : LIN_NONE), (signed char)(ok64 ? lim_of(rho) : LIN_NONE));
        }
    };
    // the indices are independent: they are split over up to 8 host threads
    // (one per 256 indices); a thread that cannot start leaves its share here
    const size_t count = n >= 16 ? n - 15 : 0;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t parts = std::min<size_t>(std::min(8u, hw), std::max<size_t>(1, count / 256));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < parts; t++) {
        const size_t m0 = count * t / parts, m1 = count * (t + 1) / parts;
        try {
            pool.emplace_back(part, m0, m1);
        } catch (...) {
            part(m0, m1);
        }
    }
    part(0, count / parts);
    for (std::thread &th : pool) th.join();
}

static int orbit_compute(const BigFix &cx, const BigFix &cy, int limbs, uint32_t max_iterations, chaos_orbit **out)
{

    std::vector<double2> z64;
    z64.reserve(std::min<uint32_t>(max_iterations, 1u << 20) + 1);
    z64.push_back(make_double2(0.0, 0.0));
    BigFix zx = bigfix_zero(limbs), zy = bigfix_zero(limbs);
    uint32_t n = 0;
    uint32_t escaped = max_iterations;
    while (n < max_iterations) {
        // x^2 - y^2 as (x + y)(x - y): two products a step instead of three (the
        // binary64 orbit of the deep-zoom centre comes out the same, value for value)
        BigFix d2 = bigfix_mul(bigfix_add(zx, zy), bigfix_sub(zx, zy)), xy = bigfix_mul(zx, zy);
        BigFix nx = bigfix_add(d2, cx);
        BigFix ny = bigfix_add(bigfix_mul2(xy), cy);
        zx = nx;
        zy = ny;
        ++n;
        double dx = bigfix_to_double(zx), dy = bigfix_to_double(zy);
        z64.push_back(make_double2(dx, dy));
        if (!(dx * dx + dy * dy < 4.0)) {
            escaped = n;
            break;
        }
    }
    std::vector<float2> z32(z64.size()), z2(z64.size());
    for (size_t k = 0; k < z64.size(); k++) {
        z32[k] = make_float2((float)z64[k].x, (float)z64[k].y);
        z2[k] = make_float2(2.f * z32[k].x, 2.f * z32[k].y);
    }
    // the composed 16- and 64-step blocks of binary32 differences, from 2Z_j
    // as that kernel holds it (binary32) and its |Z_j|^2 and tests
    std::vector<float4> bla16(z64.size(), make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float4> bla64(z64.size(), make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<char2> lin_lim;
    {
        std::vector<double2> a2(z64.size());
        std::vector<double> zz(z64.size());
        std::vector<char> ev(z64.size());
        for (size_t j = 0; j < z64.size(); j++) {
            a2[j] = make_double2(z2[j].x, z2[j].y);
            zz[j] = (double)z32[j].x * z32[j].x + (double)z32[j].y * z32[j].y;
            const float r2 = std::fmaf(z32[j].x, z32[j].x, z32[j].y * z32[j].y);
            ev[j] = !(r2 < 3.99f) || r2 < 0x1p-98f;
        }
        std::vector<BlockMap> b16, b64;
        compose_blocks(a2, zz, ev, 25.5, b16, b64, lin_lim);
        for (size_t m = 0; m < z64.size(); m++) {
            bla16[m] = make_float4((float)b16[m].px, (float)b16[m].py, (float)b16[m].qx, (float)b16[m].qy);
            bla64[m] = make_float4((float)b64[m].px, (float)b64[m].py, (float)b64[m].qx, (float)b64[m].qy);
        }
    }
    // next_event[m]: first index j >= m where a rescaled step's test can fire,
    // evaluated as the kernel does (binary32 |Z_j|^2 with one fused add)
    std::vector<uint32_t> next_event(z64.size());
    {
        const size_t last = z64.size() - 1;
        uint32_t next = (uint32_t)last;
        for (size_t j = last + 1; j-- > 0;) {
            const float r2 = std::fmaf(z32[j].x, z32[j].x, z32[j].y * z32[j].y);
            if (j == last || !(r2 < 4.f) || r2 < 0x1p-100f) next = (uint32_t)j;
            next_event[j] = next;
        }
    }
    // next_event64[m]: first index j >= m where a binary64 linear step from or to
    // j may differ from the full step: the orbit's end, |Z|^2 >= 4 (as the
    // kernel's escape test computes it), or a component of Z below 2^-20
    std::vector<double2> z2_64(z64.size());
    std::vector<uint32_t> next_event64(z64.size());
    {
        const size_t last = z64.size() - 1;
        uint32_t next = (uint32_t)last;
        for (size_t j = last + 1; j-- > 0;) {
            const double zx = z64[j].x, zy = z64[j].y;
            z2_64[j] = make_double2(2.0 * zx, 2.0 * zy);
            const double r2 = std::fma(zx, zx, zy * zy);
            if (j == last || !(r2 < 4.0) || !(std::fabs(zx) >= 0x1p-20) || !(std::fabs(zy) >= 0x1p-20))
                next = (uint32_t)j;
            next_event64[j] = next;
        }
    }
    // the same blocks for binary64 differences, from the binary64 orbit, with
    // binary64 rounding (2^-53 in place of 2^-24)
    std::vector<double2> bla16d(2 * z64.size()), bla64d(2 * z64.size());
    std::vector<char2> lin_limd;
    {
        std::vector<double> zz(z64.size());
        std::vector<char> ev(z64.size());
        for (size_t j = 0; j < z64.size(); j++) {
            zz[j] = z64[j].x * z64[j].x + z64[j].y * z64[j].y;
            const double r2 = std::fma(z64[j].x, z64[j].x, z64[j].y * z64[j].y);
            ev[j] = !(r2 < 3.99) || r2 < 0x1p-98;
        }
        std::vector<BlockMap> b16, b64;
        compose_blocks(z2_64, zz, ev, 54.5, b16, b64, lin_limd);
        for (size_t m = 0; m < z64.size(); m++) {
            bla16d[2 * m] = make_double2(b16[m].px, b16[m].py);
            bla16d[2 * m + 1] = make_double2(b16[m].qx, b16[m].qy);
            bla64d[2 * m] = make_double2(b64[m].px, b64[m].py);
            bla64d[2 * m + 1] = make_double2(b64[m].qx, b64[m].qy);
        }
    }

    chaos_orbit *o = new (std::nothrow) chaos_orbit();
    if (!o) return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
    cudaGetDevice(&o->device);
    o->max_iter = max_iterations;
    o->last = (uint32_t)(z64.size() - 1);
    o->escaped_at = escaped;
    o->bits = (uint32_t)(64 * limbs);
    o->center_x = bigfix_to_double(cx);
    o->center_y = bigfix_to_double(cy);
    // every table in one device allocation, filled by one copy from one host
    // image (256-byte aligned parts): an orbit is made per zoom step or batch
    std::vector<unsigned char> image;
    image.reserve(z64.size() * 160 + 12 * 256);
    auto stage = [&image](const auto &v) -> size_t {
        const size_t at = image.size(), bytes = v.size() * sizeof(v[0]);
        image.resize((at + bytes + 255) & ~(size_t)255);
        if (bytes) std::memcpy(image.data() + at, v.data(), bytes);
        return at;
    };
    const size_t at_z64 = stage(z64), at_z32 = stage(z32), at_z2 = stage(z2), at_bla16 = stage(bla16),
                 at_bla64 = stage(bla64), at_lim = stage(lin_lim), at_ev = stage(next_event),
                 at_bla16d = stage(bla16d), at_bla64d = stage(bla64d), at_limd = stage(lin_limd),
                 at_z2_64 = stage(z2_64), at_ev64 = stage(next_event64);
    unsigned char *dev = nullptr;
    cudaError_t e = cudaMalloc(&dev, image.size());
    if (e == cudaSuccess) e = cudaMemcpy(dev, image.data(), image.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (dev) cudaFree(dev);
        delete o;
        return api_fail(CHAOS_ERR_CUDA, "reference orbit upload: %s", cudaGetErrorString(e));
    }
    o->arena = dev;
    o->z64 = reinterpret_cast<double2 *>(dev + at_z64);
    o->z32 = reinterpret_cast<float2 *>(dev + at_z32);
    o->z2 = reinterpret_cast<float2 *>(dev + at_z2);
    o->bla16 = reinterpret_cast<float4 *>(dev + at_bla16);
    o->bla64 = reinterpret_cast<float4 *>(dev + at_bla64);
    o->lin_lim = reinterpret_cast<char2 *>(dev + at_lim);
    o->next_event = reinterpret_cast<uint32_t *>(dev + at_ev);
    o->bla16d = reinterpret_cast<double2 *>(dev + at_bla16d);
    o->bla64d = reinterpret_cast<double2 *>(dev + at_bla64d);
    o->lin_limd = reinterpret_cast<char2 *>(dev + at_limd);
    o->z2_64 = reinterpret_cast<double2 *>(dev + at_z2_64);
    o->next_event64 = reinterpret_cast<uint32_t *>(dev + at_ev64);
    *out = o;
    return CHAOS_OK;
}

int chaos_orbit_info(const chaos_orbit *o, uint32_t *stored, uint32_t *escaped_at, uint32_t *bits)
{
    if (!o) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL orbit");
    if (stored) *stored = o->last + 1;
    if (escaped_at) *escaped_at = o->escaped_at;
    if (bits) *bits = o->bits;
    return CHAOS_OK;
}

int chaos_orbit_destroy(chaos_orbit *o)
{
    if (!o) return CHAOS_OK;
    if (o->arena) cudaFree(o->arena);
    delete o;
    return CHAOS_OK;
}

// counter: a zeroed work counter the caller owns (a batch graph), or null to
// take one from the device's ring
template <class D>
static int perturb_impl(const chaos_frame_desc *d, const chaos_orbit *orb, const chaos_frame_out *o, cudaStream_t s,
                        bool sync, uint32_t *counter)
{
    PerturbArgs<D> a{};
    a.w = d->width;
    a.h = d->height;
    a.spp = d->samples_per_pixel;
    a.mode = d->sample_mode;
    a.max_iter = d->max_iterations;
    a.n_pix = d->width * d->height;
    a.seed = d->seed;
    a.ps = d->pixel_size;
    a.half_w = 0.5 * d->width;
    a.off_x = d->center_x;
    a.off_y = d->center_y;
    a.half_h = 0.5 * d->height;
    a.dc_fast = false;
    if (std::is_same<D, float>::value && d->pixel_size < 1e-30 && d->sample_mode == SAMPLES_CENTER &&
        d->width < (1u << 22) && d->height < (1u << 22)) {
        // the binary32 set-up of the rescaled kernel (see PerturbArgs::dc_fast)
        const int E = std::ilogb(d->pixel_size);
        const double psn = std::ldexp(d->pixel_size, -E), oxn = std::ldexp(d->center_x, -E),
                     oyn = std::ldexp(d->center_y, -E);
        if (std::isfinite(oxn) && std::isfinite(oyn) && std::fabs(oxn) < 0x1p100 && std::fabs(oyn) < 0x1p100) {
            a.dc_fast = true;
            a.dc_e = E;
            a.dc_hw = (float)(a.half_w - 0.5);
            a.dc_hh = (float)(a.half_h - 0.5);
            a.dc_ps_hi = (float)psn;
            a.dc_ps_lo = (float)(psn - (double)a.dc_ps_hi);
            a.dc_ox_hi = (float)oxn;
            a.dc_ox_lo = (float)(oxn - (double)a.dc_ox_hi);
            a.dc_oy_hi = (float)oyn;
            a.dc_oy_lo = (float)(oyn - (double)a.dc_oy_hi);
        }
    }
    if (std::is_same<D, float>::value)
        a.orbit = reinterpret_cast<const typename Vec2T<D>::type *>(orb->z32);
    else
        a.orbit = reinterpret_cast<const typename Vec2T<D>::type *>(orb->z64);
    a.orbit_last = orb->last;
    a.orbit64 = orb->z64;
    a.orbit2 = orb->z2;
    a.bla16 = orb->bla16;
    a.bla64 = orb->bla64;
    a.lin_lim = orb->lin_lim;
    a.bla16d = orb->bla16d;
    a.bla64d = orb->bla64d;
    a.lin_limd = orb->lin_limd;
    a.next_event = orb->next_event;
    a.orbit2_64 = orb->z2_64;
    a.next_event64 = orb->next_event64;
    a.counts = o->counts;
    a.smooth = o->smooth;
    a.pixels = reinterpret_cast<PixelInfo *>(o->pixels);
    a.pixels_pitch = o->pixels_pitch;
    a.rgba = o->rgba;
    a.palette = o->palette;
    a.palette_len = o->palette_len;
    a.interior_rgba = o->interior_rgba;
    a.total = o->total_iterations;
    a.rebases = o->rebases;
    a.status = o->status;
    if (!api_budget(d->time_limit_s, &a.budget_ns))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "time_limit_s must be >= 0");
    int sms = 0;
    if (counter) {
        a.counter = counter;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    } else {
        int rc = api_device_counter(s, &a.counter, &sms);
        if (rc) return rc;
    }
    if (a.budget_ns && !a.status) {
        if (!sync || counter)
            return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "a time limit on an unsynchronised frame needs out->status");
        int rc = api_device_status(a.counter, s, &a.status);
        if (rc) return rc;
    }
    // binary32 differences are rescaled below pixel 1e-30 (2^-100)
    cudaError_t e;
    if constexpr (std::is_same<D, float>::value)
        e = d->pixel_size < 1e-30 ? launch_perturb<float, true>(a, sms, s) : launch_perturb<float, false>(a, sms, s);
    else
        e = launch_perturb<D, false>(a, sms, s);
    if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    if (sync) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "cudaStreamSynchronize: %s", cudaGetErrorString(e));
        if (a.budget_ns) return api_read_status(a.status, s, d->time_limit_s);
    }
    return CHAOS_OK;
}

static int perturb_entry(const chaos_frame_desc *d, const chaos_orbit *orb, const chaos_frame_out *o, cudaStream_t s,
                         bool sync, uint32_t *counter = nullptr)
{
    TraceRange trace_("chaos_render_frame_perturb");
    if (!d || !orb || !o) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (d->width == 0 || d->height == 0 || (uint64_t)d->width * d->height > (1ull << 31))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "bad frame size %u x %u", d->width, d->height);
    if (d->samples_per_pixel < 1 || d->samples_per_pixel > 64)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "samples_per_pixel must be 1..64");
    if (d->sample_mode == CHAOS_SAMPLES_CENTER && d->samples_per_pixel != 1)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "pixel-centre sampling takes one sample per pixel");
    if (d->fractal != 0) return api_fail(CHAOS_ERR_UNSUPPORTED, "perturbation is implemented for mandelbrot");
    if (!(d->pixel_size > 0) || !std::isfinite(d->pixel_size))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "pixel size must be finite and > 0");
    if (d->max_iterations > orb->max_iter)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "orbit computed for maxIterations %u < %u", orb->max_iter,
                        d->max_iterations);
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != orb->device) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "orbit lives on device %d", orb->device);
    if (o->rgba && (!o->palette || o->palette_len == 0))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "rgba output needs a palette");
    if (d->tier == CHAOS_TIER_PERTURB_F32) {
        // the differences must stay normal binary32 numbers
        if (d->pixel_size < 1e-290)
            return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "rescaled binary32 differences need pixel size >= 1e-290");
        return perturb_impl<float>(d, orb, o, s, sync, counter);
    }
    if (d->tier == CHAOS_TIER_PERTURB_F64) {
        if (d->pixel_size < 1e-290)
            return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "binary64 differences need pixel size >= 1e-290");
        return perturb_impl<double>(d, orb, o, s, sync, counter);
    }
    return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "tier %u is not a perturbation tier", d->tier);
}

namespace chaos {
// Enqueue a perturbation frame with a work counter the caller zeroes (batch graphs).
int api_perturb_enqueue(const chaos_frame_desc *desc, const chaos_orbit *orbit, const chaos_frame_out *out,
                        cudaStream_t stream, uint32_t *counter)
{
    return perturb_entry(desc, orbit, out, stream, false, counter);
}
}  // namespace chaos

int chaos_render_frame_perturb_async(const chaos_frame_desc *desc, const chaos_orbit *orbit,
                                     const chaos_frame_out *out, void *stream)
{
    return perturb_entry(desc, orbit, out, (cudaStream_t)stream, false);
}

int chaos_render_frame_perturb(const chaos_frame_desc *desc, const chaos_orbit *orbit, const chaos_frame_out *out,
                               void *stream)
{
    return perturb_entry(desc, orbit, out, (cudaStream_t)stream, true);
}
