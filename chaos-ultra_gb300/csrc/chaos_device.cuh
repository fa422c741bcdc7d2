// chaos_device.cuh -- device building blocks of the escape-time path (sm_103a).
//
// Shared by the drop-in module (dropin_module.cu, the seven kernels the Java
// host loads by name) and by the library kernels (chaos_kernels.cu).
//
// Reference behaviour restated here (paths relative to the chaos-ultra root,
// gen.cu = src/main/cuda/fractalRendererGeneric.cu):
//   escape loop ........ src/main/cuda/fractals/mandelbrot.cu:11-25, julia.cu:5-17
//   sample pattern ..... gen.cu:85-155 (sampleTheFractal), gen.cu:24-34 (computeDispersion)
//   warp tile .......... gen.cu:36-53 (getImageIndexes: one warp = one 8x4 pixel tile)
//   sample reuse ....... gen.cu:194-203, 259-302, 307-368
//   foveation .......... gen.cu:209-257
//   compose / colorize . gen.cu:455-475, 67-77, mandelbrot.cu:27-35
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "chaos_intarith.cuh"

namespace chaos {

// 16-byte per-pixel record, identical in layout to pixel_info_t
// (src/main/cuda/helpers.cuh:106-130): value@0, weight@4, isReused@8, weightOfNewSamples@12.
struct PixelInfo {
    float value;
    float weight;
    uint8_t is_reused;
    uint8_t pad[3];
    float weight_of_new_samples;
};
static_assert(sizeof(PixelInfo) == 16, "pixel_info_t is 16 bytes");

// ARITH_CONTRACTED: the reference modules as nvcc builds them by default
// (contraction on).  Established against the reference's own default build:
// every product and sum is rounded except where nvcc fuses a product that has
// no other use into the add after it -- the escape step's y' = fma(2x, y, cy),
// the sample's x coordinate fma(px + dx, psx, lbx), and in the reuse path
// the warp to the old frame, the filter's chain of products and the blend.  The
// squares x*x and y*y feed both the test and x' and stay rounded.
// ARITH_FLOATFLOAT (binary64 frames only): the escape loop in float-float
// (ff_step, about 48 bits on the binary32 pipe) from the binary64 sample
// point; the sampling geometry stays binary64.
enum Arith { ARITH_PARITY = 0, ARITH_FMA = 1, ARITH_CONTRACTED = 2, ARITH_FLOATFLOAT = 3 };
enum FractalKind {
    FRACTAL_MANDELBROT = 0,
    FRACTAL_JULIA = 1,
    FRACTAL_NEWTON_WIRED = 2,      // src/main/cuda/fractals/newton_wired.cu
    FRACTAL_NEWTON_GENERIC = 3,    // newton_generic.cu
    FRACTAL_NEWTON_ITERATIONS = 4  // newton_iterations.cu
};

// The Newton modules' __constant__ symbols (newton_generic.cu:7-8,
// newton_iterations.cu:7-9): roots as (re, im) pairs, polynomial coefficients
// c0..c3 (f = c0 + c1 z + c2 z^2 + c3 z^3), and the palette stride of the
// iteration colouring.
struct NewtonParams {
    double roots[6];
    double coefficients[4];
    int color_magnifier;
    int pad;
};

// Newton-method value of a start point (chaos_newton.cuh; only the
// translation units that render Newton fractals include its definition).
template <class R, int F> __device__ uint32_t newton_compute(uint32_t max_iterations, R zx, R zy, const NewtonParams &p);

// kernel flag bits, gen.cu:157-161 (bit 1 is the Java-side "visualise" flag)
constexpr uint32_t FLAG_ADAPTIVE_SS = 1u << 0;
constexpr uint32_t FLAG_FOVEATION = 1u << 2;
constexpr uint32_t FLAG_SAMPLE_REUSE = 1u << 3;
constexpr uint32_t FLAG_IS_ZOOMING = 1u << 4;
constexpr uint32_t FLAG_ZOOMING_IN = 1u << 5;

constexpr uint32_t MAX_SUPER_SAMPLING = 64;  // gen.cu:12
constexpr uint32_t ADAPTIVE_THRESHOLD = 10;  // gen.cu:93

// Iterations run between two escape tests on the fast path (see escape()).
constexpr int ESCAPE_BLOCK = 16;

// n / d and n % d for a divisor fixed per launch: m = floor(2^32 / d) (2^32 - 1
// for d = 1) gives a quotient at most one short for any 32-bit n, fixed by one
// comparison -- a multiply-high and a few integer operations instead of a
// division.
__host__ __device__ __forceinline__ uint32_t div_magic(uint32_t d)
{
    return d <= 1u ? 0xffffffffu : (uint32_t)(0x100000000ull / d);
}
__device__ __forceinline__ void divmod_magic(uint32_t n, uint32_t d, uint32_t m, uint32_t &q, uint32_t &r)
{
    q = __umulhi(n, m);
    r = n - q * d;
    if (r >= d) {
        ++q;
        r -= d;
    }
}

// The GPU's global nanosecond timer (the clock of the persistent kernels'
// time limits).
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Status bits a persistent kernel ORs into its launch's status word.
constexpr uint32_t RUN_STATUS_TIMEOUT = 1u;  // the launch's time limit ran out: outputs incomplete

// A warp-uniform time-limit check: true (and the status bit set once per
// warp) when `budget_ns` is non-zero and the warp has run longer than it
// since `t0` (lane 0's clock).
__device__ __forceinline__ bool out_of_time(unsigned long long budget_ns, unsigned long long t0, uint32_t *status,
                                            uint32_t lane)
{
    if (!budget_ns) return false;
    uint32_t late = 0;
    if (lane == 0) late = global_ns() - t0 > budget_ns ? 1u : 0u;
    late = __shfl_sync(0xffffffffu, late, 0);
    if (late && lane == 0 && status) atomicOr(status, RUN_STATUS_TIMEOUT);
    return late != 0;
}

// ---------------------------------------------------------------------------
// Correctly rounded scalar operations.  Every product and sum is rounded on its
// own unless an fma is written out, so the compiler cannot contract (the
// parity arithmetic matches the reference built with --fmad=false).
// ---------------------------------------------------------------------------
template <class R> struct Op;
template <> struct Op<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};
template <> struct Op<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
};

// |z|^2 as the escape test computes it.
template <class R, int A> __device__ __forceinline__ R radius2(R x, R y)
{
    using O = Op<R>;
    if (A == ARITH_PARITY || A == ARITH_CONTRACTED) return O::add(O::mul(x, x), O::mul(y, y));
    return O::fma(x, x, O::mul(y, y));
}

// One step of z <- z^2 + c.
//   parity:     x' = (x*x - y*y) + cx, y' = (2*x)*y + cy  (mandelbrot.cu:17-18 order)
//   contracted: x' as parity, y' = fma(x + x, y, cy)
//   fma:        x' = fma(x, x, fma(-y, y, cx)), y' = fma(x + x, y, cy)  (4 FP32-pipe ops)
template <class R, int A> __device__ __forceinline__ void step(R &x, R &y, R cx, R cy)
{
    using O = Op<R>;
    if (A == ARITH_PARITY) {
        R xx = O::mul(x, x), yy = O::mul(y, y);
        R xn = O::add(O::sub(xx, yy), cx);
        y = O::add(O::mul(O::mul(R(2), x), y), cy);
        x = xn;
    } else if (A == ARITH_CONTRACTED) {
        R xx = O::mul(x, x), yy = O::mul(y, y);
        R xn = O::add(O::sub(xx, yy), cx);
        y = O::fma(O::add(x, x), y, cy);
        x = xn;
    } else {
        R t = O::fma(-y, y, cx);
        R xn = O::fma(x, x, t);
        y = O::fma(O::add(x, x), y, cy);
        x = xn;
    }
}

// The rounded step in 6 operations instead of 7: y' = fma(2, round(x*y), cy).
// Doubling is exact, so round((2x)*y) = 2 round(x*y) whenever round(x*y) is at
// least twice the smallest normal number, and the fused add rounds 2p + cy
// once, as the reference's add does.  emin collects the exponent field of
// every product (integer ops, off the floating-point pipe and off the step's
// dependency chain); a block whose emin is below 2 (a product that small) is
// redone with step<R, ARITH_PARITY>.
__device__ __forceinline__ uint32_t exponent_bits(float p) { return __float_as_uint(p) & 0x7f800000u; }
__device__ __forceinline__ uint32_t exponent_bits(double p) { return (uint32_t)__double2hiint(p) & 0x7ff00000u; }
template <class R> __device__ __forceinline__ uint32_t exponent_bits_two();
template <> __device__ __forceinline__ uint32_t exponent_bits_two<float>() { return 2u << 23; }
template <> __device__ __forceinline__ uint32_t exponent_bits_two<double>() { return 2u << 20; }

template <class R> __device__ __forceinline__ void step_rounded6(R &x, R &y, R cx, R cy, uint32_t &emin)
{
    using O = Op<R>;
    R xx = O::mul(x, x), yy = O::mul(y, y);
    R xn = O::add(O::sub(xx, yy), cx);
    R p = O::mul(x, y);
    y = O::fma(R(2), p, cy);
    x = xn;
    emin = min(emin, exponent_bits(p));
}

// Binary64: the same step with x*x - y*y formed on the integer units
// (sub_nonneg_bits, exactly the rounded difference), which leaves five
// operations per step on the binary64 pipe.  A difference the integer
// routine hands back (a subnormal operand or result) sets emin to 0, so the
// block is redone with step<double, ARITH_PARITY> like a small product.
template <> __device__ __forceinline__ void step_rounded6<double>(double &x, double &y, double cx, double cy,
                                                                  uint32_t &emin)
{
    const double xx = __dmul_rn(x, x), yy = __dmul_rn(y, y);
    bool exact;
    const double t = __longlong_as_double((long long)sub_nonneg_bits((uint64_t)__double_as_longlong(xx),
                                                                     (uint64_t)__double_as_longlong(yy), exact));
    const double xn = __dadd_rn(t, cx);
    const double p = __dmul_rn(x, y);
    y = __fma_rn(2.0, p, cy);
    x = xn;
    emin = min(emin, exact ? exponent_bits(p) : 0u);
}

// The binary64 fused step with 2x formed on the integer pipe: adding 1 to the
// exponent field doubles a normal number exactly, and x + x is the binary64
// pipe's fourth operation per step.  emin collects the exponent field of
// every x; a block that met x = 0 or a subnormal x (field 0) is redone with
// step<double, ARITH_FMA>.  At the top of the range the integer doubling
// gives inf or NaN where 2x overflows (a NaN where x + x gives inf): both
// only arise after an escape and never test below 4, which is all the
// blocked escape loop asks of the steps past an escape.  Everything else is
// step<double, ARITH_FMA> bit for bit.
__device__ __forceinline__ double twice_on_int(double x, uint32_t &emin)
{
    const int hi = __double2hiint(x), lo = __double2loint(x);
    emin = min(emin, (uint32_t)hi & 0x7ff00000u);
    return __hiloint2double(hi + 0x00100000, lo);
}
__device__ __forceinline__ void step_fma3(double &x, double &y, double cx, double cy, uint32_t &emin)
{
    double t = __fma_rn(-y, y, cx);
    double xn = __fma_rn(x, x, t);
    y = __fma_rn(twice_on_int(x, emin), y, cy);
    x = xn;
}

// step<double, ARITH_CONTRACTED> in four binary64 operations: x*x - y*y on the
// integer units (sub_nonneg_bits) and 2x by the exponent field.  A block that
// met x = 0, a subnormal x or a difference the integer routine hands back
// (emin = 0) is redone with the literal step.
__device__ __forceinline__ void step_contracted4(double &x, double &y, double cx, double cy, uint32_t &emin)
{
    const double xx = __dmul_rn(x, x), yy = __dmul_rn(y, y);
    bool exact;
    const double t = __longlong_as_double((long long)sub_nonneg_bits((uint64_t)__double_as_longlong(xx),
                                                                     (uint64_t)__double_as_longlong(yy), exact));
    const double xn = __dadd_rn(t, cx);
    y = __fma_rn(twice_on_int(x, emin), y, cy);
    x = xn;
    emin = exact ? emin : 0u;
}

// Exact cycle detection (Brent's method on checkpoints).  The rounded
// iteration is deterministic, so once a state repeats bit for bit the orbit
// cycles through states that all tested below 4 and never escapes: the
// sample is interior, with the reference's answer (maxIterations), however
// many steps remain.  A checkpoint comes at the end of every full block of a
// sample (a fixed number of steps); the state there is compared with the one
// saved at the last power-of-two checkpoint (the saved state moves at
// checkpoints 1, 2, 4, 8, ...).  Equal states prove the cycle: binary64
// states are compared as bit patterns (on the integer units, beside the
// binary64 pipe's step), binary32 ones under == (where only a zero's sign
// can differ between equal values, and it changes no later magnitude).
constexpr uint32_t CYCLE_SPAN = 16;  // steps between checkpoints in the tested binary32 blocks

__device__ __forceinline__ bool same_state(float a, float b) { return a == b; }
__device__ __forceinline__ bool same_state(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}

template <class T> struct CycleWatch {
    T sx, sy;
    uint32_t ck, save_at, tick;
    __device__ __forceinline__ void reset(T x, T y)
    {
        sx = x;
        sy = y;
        ck = 0;
        save_at = 1;
        tick = 0;
    }
    // At a checkpoint: true when the state repeats the saved one.
    __device__ __forceinline__ bool check(T x, T y)
    {
        if (same_state(x, sx) && same_state(y, sy)) return true;
        if (++ck == save_at) {
            sx = x;
            sy = y;
            save_at <<= 1;
        }
        return false;
    }
    // Called at every full block; a checkpoint at every N-th one.  Binary64
    // loops take N = 8: there repeats are rare at the depths binary64 serves
    // and every instruction beside the step costs, so checkpoints every 128
    // steps cost little (0.4 % of a deep frame without cycles) and find most
    // cycles a little later.
    template <int N> __device__ __forceinline__ bool check_every(T x, T y)
    {
        if (N > 1 && ((++tick) & (uint32_t)(N - 1)) != 0u) return false;
        return check(x, y);
    }
};
template <class T> constexpr int cycle_blocks() { return sizeof(T) == 8 ? 8 : 1; }

// Up to K steps of the reference loop, each with its own test (binary32
// frames): stops at a state that tests >= 4 (esc, r2 = its test value) or
// after `lim` steps when BOUNDED.  Returns the steps taken.  In rounded
// arithmetic the test's products are the step's own, so a test costs one add,
// a compare and a branch; a lane that stops waits for its warp at the end of
// the block.  Exact for every c, with no roll-back or search.
// With a CycleWatch (unbounded blocks only, K a multiple of CYCLE_SPAN), a
// checkpoint comes after every CYCLE_SPAN steps; `cyc` reports a repeat.
template <class R, int A, int K, bool BOUNDED>
__device__ __forceinline__ uint32_t tested_block(R &x, R &y, R cx, R cy, uint32_t lim, R &r2, bool &esc,
                                                 CycleWatch<R> *cw = nullptr, bool *cyc = nullptr)
{
#pragma unroll
    for (int k = 0; k < K; k++) {
        if (BOUNDED && (uint32_t)k == lim) return lim;
        r2 = radius2<R, A>(x, y);
        if (!(r2 < R(4))) {
            esc = true;
            return (uint32_t)k;
        }
        step<R, A>(x, y, cx, cy);
        if (!BOUNDED && cw && ((k + 1) % (int)CYCLE_SPAN) == 0 && cw->check(x, y)) {
            *cyc = true;
            return (uint32_t)(k + 1);
        }
    }
    return (uint32_t)K;
}

// Escape loop with the reference's semantics:
//     i = 0; while (i < max_iter && r2(z) < 4) { z = z^2 + c; ++i; }  return i
// run as blocks of ESCAPE_BLOCK untested steps.  A block is kept when its last
// state still tests below 4; otherwise the state rolls back to the block start
// and the steps are redone one test at a time.  This is exact when
// |c|^2 <= 3.99 (|c| <= 1.9975): once a computed |z|^2 reaches 4,
// |z'| >= 4 - 1.9975 > 2.002 (rounding moves these by ~1e-6 at most in
// binary32), and |z| keeps growing until it overflows to inf/NaN; neither
// tests below 4, so a block whose last state tests below 4 contains no
// escape.  Otherwise `blockable` is false and every step is tested.
// Every kept block ends at a checkpoint of the exact cycle detection
// (CycleWatch): a state that repeats proves the sample interior.
// r2_exit is r2 of the final state.  (Tested blocks, which the binary32
// frame kernel uses, were slower here: a tile's lanes run in lock step, so
// every lane pays the per-step test for as long as the tile's slowest lane
// runs, while a roll-back costs only the lane that escaped.)
// Binary64 blocks run step_rounded6 / step_fma3 (the same values as step<>)
// and are redone with step<> when the integer checks ask for it.  i0 is the
// iteration count of the state passed in (1 when a Mandelbrot caller starts
// at z1 = c).
template <class R, int A>
__device__ __forceinline__ uint32_t escape(uint32_t max_iter, R x, R y, R cx, R cy, bool blockable, R &r2_exit,
                                           uint32_t i0 = 0)
{
    R r2 = radius2<R, A>(x, y);
    if (i0 >= max_iter || !(r2 < R(4))) {
        r2_exit = r2;
        return i0 < max_iter ? i0 : max_iter;
    }
    uint32_t i = i0;
    if (blockable) {
        CycleWatch<R> cw;
        cw.reset(x, y);
        while (max_iter - i >= (uint32_t)ESCAPE_BLOCK) {
            R sx = x, sy = y;
            bool redo = false;
            if constexpr (sizeof(R) == 8 && A == ARITH_PARITY) {
                uint32_t emin = 0xffffffffu;
#pragma unroll
                for (int k = 0; k < ESCAPE_BLOCK; k++) step_rounded6<R>(x, y, cx, cy, emin);
                redo = emin < exponent_bits_two<R>();
            } else if constexpr (sizeof(R) == 8 && A == ARITH_CONTRACTED) {
                uint32_t emin = 0xffffffffu;
#pragma unroll
                for (int k = 0; k < ESCAPE_BLOCK; k++) step_contracted4(x, y, cx, cy, emin);
                redo = emin == 0u;
            } else if constexpr (sizeof(R) == 8) {
                uint32_t emin = 0xffffffffu;
#pragma unroll
                for (int k = 0; k < ESCAPE_BLOCK; k++) step_fma3(x, y, cx, cy, emin);
                redo = emin == 0u;
            } else {
#pragma unroll
                for (int k = 0; k < ESCAPE_BLOCK; k++) step<R, A>(x, y, cx, cy);
            }
            if (redo) {
                x = sx;
                y = sy;
#pragma unroll
                for (int k = 0; k < ESCAPE_BLOCK; k++) step<R, A>(x, y, cx, cy);
            }
            if (!(radius2<R, A>(x, y) < R(4))) {
                x = sx;
                y = sy;
                break;
            }
            i += ESCAPE_BLOCK;
            if (cw.template check_every<cycle_blocks<R>()>(x, y)) {  // a repeated state: interior
                r2_exit = radius2<R, A>(x, y);
                return max_iter;
            }
        }
    }
    while (i < max_iter) {
        step<R, A>(x, y, cx, cy);
        ++i;
        r2 = radius2<R, A>(x, y);
        if (!(r2 < R(4))) break;
    }
    r2_exit = r2;
    return i;
}

template <class R> __device__ __forceinline__ bool blockable_c(R cx, R cy)
{
    return radius2<R, ARITH_PARITY>(cx, cy) <= R(3.99);
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

__device__ __forceinline__ bool same_state(FF a, FF b) { return same_state(a.hi, b.hi) && same_state(a.lo, b.lo); }

// The escape loop of escape() in float-float: blocks of ESCAPE_BLOCK untested
// steps while |c| <= 1.9975 (after an escape the leading words grow until
// they overflow, so a block whose last state tests below 4 holds no escape),
// the rest one tested step at a time.  The test reads the leading words, as
// the batched float-float tier's does; the count is the first step index
// whose state tests >= 4, so both give the same count for the same c.
__device__ __forceinline__ uint32_t escape_ff(uint32_t max_iter, FF x, FF y, FF cx, FF cy, bool blockable)
{
    if (max_iter == 0u || !(ff_radius2(x, y) < 4.f)) return 0u;
    uint32_t i = 0;
    if (blockable) {
        CycleWatch<FF> cw;
        cw.reset(x, y);
        while (max_iter - i >= (uint32_t)ESCAPE_BLOCK) {
            const FF sx = x, sy = y;
#pragma unroll
            for (int k = 0; k < ESCAPE_BLOCK; k++) ff_step(x, y, cx, cy);
            if (!(ff_radius2(x, y) < 4.f)) {
                x = sx;
                y = sy;
                break;
            }
            i += ESCAPE_BLOCK;
            if (cw.check(x, y)) return max_iter;  // a repeated state: interior
        }
    }
    while (i < max_iter) {
        ff_step(x, y, cx, cy);
        ++i;
        if (!(ff_radius2(x, y) < 4.f)) break;
    }
    return i;
}


// computeFractal (mandelbrot.cu:11-25, julia.cu:5-17) as an unsigned escape
// value: Mandelbrot maps an interior point (i == maxIterations) to 0, Julia
// returns i.  `jc` is julia_c already converted to Real.
template <class R, int A, int F> __device__ __forceinline__ uint32_t compute_fractal(uint32_t max_iter, R px, R py, R jcx, R jcy)
{
    if constexpr (A == ARITH_FLOATFLOAT) {
        static_assert(sizeof(R) == 8, "float-float escape loops start from binary64 points");
        const FF fx = ff_from_double(px), fy = ff_from_double(py);
        if (F == FRACTAL_MANDELBROT) {
            const uint32_t i = escape_ff(max_iter, FF{0.f, 0.f}, FF{0.f, 0.f}, fx, fy, blockable_c(fx.hi, fy.hi));
            return i == max_iter ? 0u : i;
        }
        const FF jx = ff_from_double(jcx), jy = ff_from_double(jcy);
        return escape_ff(max_iter, fx, fy, jx, jy, blockable_c(jx.hi, jy.hi));
    }
    R r2;
    if (F == FRACTAL_MANDELBROT) {
        // from z1 = c, the first step's exact result (+0 in place of -0)
        uint32_t i = max_iter == 0 ? 0u
                                   : escape<R, A>(max_iter, Op<R>::add(px, R(0)), Op<R>::add(py, R(0)), px, py,
                                                  blockable_c(px, py), r2, 1u);
        return i == max_iter ? 0u : i;
    }
    return escape<R, A>(max_iter, px, py, jcx, jcy, blockable_c(jcx, jcy), r2);
}

// ---------------------------------------------------------------------------
// Reference-mode sampling (sampleTheFractal, gen.cu:85-155)
// ---------------------------------------------------------------------------

// Plane rectangle as the kernel receives it (Rectangle<Real>): left-bottom and
// right-top corners.  4-byte (float) or 8-byte (double) aligned, as in the
// reference's parameter layout.
template <class R> struct Rect {
    R lbx, lby, rtx, rty;
};

struct UInt2 {
    uint32_t x, y;
};

template <class R> struct SampleGeometry {
    R lbx, rty;  // image left-top corner
    R psx, psy;  // pixel size, image.size() / gridSize (gen.cu:97)
    uint32_t max_iter;
    R jcx, jcy;
    NewtonParams newton;  // Newton modules only
};

// computeFractal of the module F at plane point (cx, cy).
template <class R, int A, int F> __device__ __forceinline__ uint32_t compute_fractal_g(const SampleGeometry<R> &g, R cx, R cy)
{
    if constexpr (F >= FRACTAL_NEWTON_WIRED)
        return newton_compute<R, F>(g.max_iter, cx, cy, g.newton);
    else
        return compute_fractal<R, A, F>(g.max_iter, cx, cy, g.jcx, g.jcy);
}

template <class R>
__device__ __forceinline__ SampleGeometry<R> make_geometry(const Rect<R> &r, UInt2 size, uint32_t max_iter, double jcx,
                                                            double jcy)
{
    using O = Op<R>;
    SampleGeometry<R> g;
    g.lbx = r.lbx;
    g.rty = r.rty;
    g.psx = O::div(O::sub(r.rtx, r.lbx), (R)size.x);
    g.psy = O::div(O::sub(r.rty, r.lby), (R)size.y);
    g.max_iter = max_iter;
    g.jcx = (R)jcx;
    g.jcy = (R)jcy;
    return g;
}

// Sample offset i (gen.cu:104-117) and plane point (gen.cu:119-124).  The
// contracted build fuses the x coordinate's product into its add; in the
// Newton modules it fuses the y coordinate's too (established, like the rest
// of the contracted arithmetic, against outputs of the reference's own
// default-build modules: with y fused every record of 24 seeded views of each
// Newton module matches, without it some do not).
template <class R, int A = ARITH_PARITY, int F = FRACTAL_MANDELBROT>
__device__ __forceinline__ void sample_point(const SampleGeometry<R> &g, uint32_t px, uint32_t py, uint32_t i,
                                             float sample_count_f, R &cx, R &cy)
{
    using O = Op<R>;
    const uint32_t skip_first = 2;
    R dx, dy;
    if (i <= skip_first) {
        dx = dy = O::div((R)i, (R)(skip_first + 1));
    } else {
        float spr_f = __fsqrt_rn(__fsub_rn(sample_count_f, (float)skip_first));
        uint32_t spr = (uint32_t)roundf(spr_f);
        dx = (R)__fdiv_rn((float)((i - skip_first) % spr), spr_f);
        dy = (R)__fdiv_rn((float)((i - skip_first) / spr), spr_f);
    }
    if (A == ARITH_CONTRACTED)
        cx = O::fma(O::add((R)px, dx), g.psx, g.lbx);
    else
        cx = O::add(g.lbx, O::mul(O::add((R)px, dx), g.psx));
    if (A == ARITH_CONTRACTED && F >= FRACTAL_NEWTON_WIRED)
        cy = O::fma(-O::add((R)py, dy), g.psy, g.rty);
    else
        cy = O::add(g.rty, O::mul(-O::add((R)py, dy), g.psy));
}

// computeDispersion (gen.cu:24-34) over the first data_length stored samples.
// The reference stores 10 samples and reads past them when data_length > 10;
// those reads are skipped here.
__device__ __forceinline__ float dispersion(const float *data, uint32_t data_length, float mean)
{
    float variance = 0.f;
    uint32_t m = data_length < ADAPTIVE_THRESHOLD ? data_length : ADAPTIVE_THRESHOLD;
    for (uint32_t k = 0; k < m; k++) {
        float d = __fsub_rn(data[k], mean);
        variance = __fadd_rn(variance, __fmul_rn(d, d));
    }
    variance = __fdiv_rn(variance, (float)(uint32_t)(data_length - 1u));
    return __fdiv_rn(variance, mean);
}

// sampleTheFractal for the lanes of `mask`, which call it together with the
// same sample_count_f.  Lanes with valid == false (pixels outside the image)
// take part in the votes as "yes" and compute nothing, which is how the
// reference's exited lanes drop out of __activemask().  `iters` accumulates the
// pixel-iterations of the samples taken (an interior sample counts max_iter).
template <class R, int A, int F>
__device__ uint32_t sample_the_fractal(const SampleGeometry<R> &g, uint32_t px, uint32_t py, float &sample_count_f,
                                       bool adaptive, bool valid, uint32_t mask, unsigned long long &iters)
{
    if (sample_count_f < 1.f) {  // gen.cu:87-90
        sample_count_f = 0.f;
        return 0;
    }
    uint32_t sc = (uint32_t)roundf(sample_count_f);
    sc = sc < MAX_SUPER_SAMPLING ? sc : MAX_SUPER_SAMPLING;
    float samples[ADAPTIVE_THRESHOLD];
    uint32_t sum = 0;
    for (uint32_t i = 0; i < sc; i++) {
        uint32_t e = 0;
        if (valid) {
            R cx, cy;
            sample_point<R, A, F>(g, px, py, i, sample_count_f, cx, cy);
            e = compute_fractal_g<R, A, F>(g, cx, cy);
            // pixel-iterations (escape-time modules; the Newton modules return a root index)
            if (F < FRACTAL_NEWTON_WIRED) iters += (F == FRACTAL_MANDELBROT && e == 0u) ? g.max_iter : e;
        }
        sum += e;
        if (i < ADAPTIVE_THRESHOLD) samples[i] = (float)e;
        if ((adaptive && (i > 0 && i < ADAPTIVE_THRESHOLD)) || (i == sc / 2)) {
            float mean = (float)(sum / (i + 1));
            float disp = dispersion(samples, i, mean);
            if (i == 1 && __all_sync(mask, !valid || fabsf(__fsub_rn(samples[0], samples[1])) < 1.19209290e-7f))
                sc = i + 1;
            else if (__all_sync(mask, !valid || disp < 0.01f))
                sc = i + 1;
            else if (__all_sync(mask, !valid || disp <= 1.f) && i >= sc / 2)
                sc = i + 1;
        }
    }
    sample_count_f = (float)sc;
    return sum / sc;
}

// Pixel of lane `lane` in the 8x4 warp tile whose top-left pixel is (x0, y0):
// the lane order of getImageIndexes (gen.cu:43-53) with blockDim.x == 32.
__device__ __forceinline__ UInt2 tile_pixel(uint32_t x0, uint32_t y0, uint32_t lane)
{
    UInt2 p;
    p.x = x0 + 4 * (lane >> 4) + (lane & 3);
    p.y = y0 + ((lane >> 2) & 3);
    return p;
}

__device__ __forceinline__ PixelInfo *pixel_ptr(void *base, long pitch, uint32_t x, uint32_t y)
{
    return reinterpret_cast<PixelInfo *>(static_cast<char *>(base) + (size_t)y * (size_t)pitch) + x;
}
__device__ __forceinline__ const PixelInfo *pixel_ptr(const void *base, long pitch, uint32_t x, uint32_t y)
{
    return reinterpret_cast<const PixelInfo *>(static_cast<const char *>(base) + (size_t)y * (size_t)pitch) + x;
}

// Store a whole 16-byte record (padding bytes zero) with one vector store when
// the address allows it.
__device__ __forceinline__ void store_pixel(PixelInfo *p, const PixelInfo &v)
{
    uint32_t w2 = (uint32_t)v.is_reused;
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
        uint4 u = make_uint4(__float_as_uint(v.value), __float_as_uint(v.weight), w2,
                             __float_as_uint(v.weight_of_new_samples));
        *reinterpret_cast<uint4 *>(p) = u;
    } else {
        uint32_t *q = reinterpret_cast<uint32_t *>(p);
        q[0] = __float_as_uint(v.value);
        q[1] = __float_as_uint(v.weight);
        q[2] = w2;
        q[3] = __float_as_uint(v.weight_of_new_samples);
    }
}

__device__ __forceinline__ PixelInfo load_pixel(const PixelInfo *p)
{
    PixelInfo v;
    uint4 u;
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
        u = __ldg(reinterpret_cast<const uint4 *>(p));
    } else {
        const uint32_t *q = reinterpret_cast<const uint32_t *>(p);
        u = make_uint4(q[0], q[1], q[2], q[3]);
    }
    v.value = __uint_as_float(u.x);
    v.weight = __uint_as_float(u.y);
    v.is_reused = (uint8_t)(u.z & 0xffu);
    v.pad[0] = v.pad[1] = v.pad[2] = 0;
    v.weight_of_new_samples = __uint_as_float(u.w);
    return v;
}

__device__ __forceinline__ PixelInfo make_pixel(float value, float weight)
{
    PixelInfo p;
    p.value = value;
    p.weight = weight;
    p.is_reused = 0;
    p.pad[0] = p.pad[1] = p.pad[2] = 0;
    p.weight_of_new_samples = 0.f;
    return p;
}

// fractalRenderMain for one lane of an 8x4 warp tile (gen.cu:168-181).
// Returns the record stored for the lane's pixel (meaningful where the pixel
// lies in the image).
template <class R, int A, int F>
__device__ __forceinline__ PixelInfo render_main_tile(const SampleGeometry<R> &g, void *out, long pitch, UInt2 size,
                                                      uint32_t x0, uint32_t y0, uint32_t lane, float max_ss,
                                                      uint32_t flags, unsigned long long &iters)
{
    UInt2 p = tile_pixel(x0, y0, lane);
    bool valid = p.x < size.x && p.y < size.y;
    float sc = max_ss;
    uint32_t result =
        sample_the_fractal<R, A, F>(g, p.x, p.y, sc, (flags & FLAG_ADAPTIVE_SS) != 0, valid, 0xffffffffu, iters);
    const PixelInfo rec = make_pixel((float)result, sc);
    if (valid) store_pixel(pixel_ptr(out, pitch, p.x, p.y), rec);
    return rec;
}

// ---------------------------------------------------------------------------
// Sample reuse and foveation (fractalRenderAdvanced, gen.cu:194-368)
// ---------------------------------------------------------------------------

// getWarpingOriginOfSampleReuse, gen.cu:194-203 (contracted: the pixel's
// position in the plane and the y flip are fused multiply-adds).  The origin
// is separable: its x depends on the pixel's column only, its y on the
// pixel's row only, so a warp can compute each once per column and row.
template <class R, int A = ARITH_PARITY>
__device__ __forceinline__ float warping_origin_x(uint32_t px, UInt2 grid, const Rect<R> &cur, const Rect<R> &old)
{
    using O = Op<R>;
    R ppx;
    if (A == ARITH_CONTRACTED)
        ppx = O::fma(O::div((R)px, (R)grid.x), O::sub(cur.rtx, cur.lbx), cur.lbx);
    else
        ppx = O::add(O::mul(O::div((R)px, (R)grid.x), O::sub(cur.rtx, cur.lbx)), cur.lbx);
    R rx = O::div(O::sub(ppx, old.lbx), O::sub(old.rtx, old.lbx));
    return __fmul_rn((float)rx, (float)grid.x);
}

template <class R, int A = ARITH_PARITY>
__device__ __forceinline__ float warping_origin_y(uint32_t py, UInt2 grid, const Rect<R> &cur, const Rect<R> &old)
{
    using O = Op<R>;
    uint32_t qy = grid.y - py;
    R ppy;
    if (A == ARITH_CONTRACTED)
        ppy = O::fma(O::div((R)qy, (R)grid.y), O::sub(cur.rty, cur.lby), cur.lby);
    else
        ppy = O::add(O::mul(O::div((R)qy, (R)grid.y), O::sub(cur.rty, cur.lby)), cur.lby);
    R ry = O::div(O::sub(ppy, old.lby), O::sub(old.rty, old.lby));
    if (A == ARITH_CONTRACTED) return __fmaf_rn(-(float)ry, (float)grid.y, (float)grid.y);
    return __fsub_rn((float)grid.y, __fmul_rn((float)ry, (float)grid.y));
}

// One coordinate of the reuse read (gen.cu:320-331): the range test of the
// rounded origin (>= 2 and < n - 2) and the filter's corner and weight
// (floor, fraction).  `at` holds the corner with bit 31 set when the
// coordinate is in range.  Frames narrower than 5 pixels reuse nothing:
// there the reference's test (an unsigned n - 2) can pass for a corner
// outside the frame.
struct ReuseAxis {
    uint32_t at;
    float frac;
};

__device__ __forceinline__ ReuseAxis reuse_axis(float o, uint32_t n)
{
    const int oi = (int)roundf(o);
    const bool ok = n >= 5u && !(oi < 2 || (uint32_t)oi >= n - 2u);
    const uint32_t f = (uint32_t)floorf(o);
    ReuseAxis r;
    r.frac = __fsub_rn(o, (float)f);
    r.at = ok ? (f | 0x80000000u) : 0u;
    return r;
}

// The filter of readFromArrayUsingFiltering<float> (gen.cu:259-302) on the
// four neighbours (value, weight) a = (i, j), b = (i+1, j), c = (i, j+1),
// d = (i+1, j+1) (contracted: each term after the first is a fused
// multiply-add onto the sum so far, the first two as fma(w00, T00, w10*T10)).
template <int A = ARITH_PARITY>
__device__ __forceinline__ void filter_bilinear(float alpha, float beta, float2 a2, float2 b2, float2 c2, float2 d2,
                                                float &value, float &weight)
{
    struct VW {
        float value, weight;
    };
    const VW a{a2.x, a2.y}, b{b2.x, b2.y}, c{c2.x, c2.y}, d{d2.x, d2.y};
    float oa = __fsub_rn(1.f, alpha), ob = __fsub_rn(1.f, beta);
    float w00 = __fmul_rn(oa, ob), w10 = __fmul_rn(alpha, ob), w01 = __fmul_rn(oa, beta), w11 = __fmul_rn(alpha, beta);
    float r, w;
    if (A == ARITH_CONTRACTED) {
        r = __fmaf_rn(w00, a.value, __fmul_rn(w10, b.value));
        r = __fmaf_rn(w01, c.value, r);
        r = __fmaf_rn(w11, d.value, r);
        w = __fmaf_rn(w00, a.weight, __fmul_rn(w10, b.weight));
        w = __fmaf_rn(w01, c.weight, w);
        w = __fmaf_rn(w11, d.weight, w);
    } else {
        r = __fadd_rn(__fmul_rn(w00, a.value), __fmul_rn(w10, b.value));
        r = __fadd_rn(r, __fmul_rn(w01, c.value));
        r = __fadd_rn(r, __fmul_rn(w11, d.value));
        w = __fadd_rn(__fmul_rn(w00, a.weight), __fmul_rn(w10, b.weight));
        w = __fadd_rn(w, __fmul_rn(w01, c.weight));
        w = __fadd_rn(w, __fmul_rn(w11, d.weight));
    }
    value = r;
    weight = w;
}

// getFoveationAdvisedSampleCount + linearMapping<float>, gen.cu:209-257.
// Uniform over the 8x4 warp tile (the pixel is snapped to the tile corner).
// Contracted: the distance's sum of squares and k*x + q are fused.
template <int A = ARITH_PARITY>
__device__ __forceinline__ void foveation(UInt2 p, UInt2 focus, float max_ss, float &advised, bool &inside)
{
    const float pi_f = 3.14159265358979f;
    const float screen_distance = 60.f, pixel_cm = 0.02652f;
    uint32_t nx = p.x - p.x % 8u, ny = p.y - p.y % 4u;
    float foveal = max_ss >= 1.f ? 5.5f : (float)__dmul_rn(5.5, (double)max_ss);
    float peripheral = 60.f;
    float ddx = __fsub_rn((float)focus.x, (float)nx), ddy = __fsub_rn((float)focus.y, (float)ny);
    float sq = A == ARITH_CONTRACTED ? __fmaf_rn(ddx, ddx, __fmul_rn(ddy, ddy))
                                     : __fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(ddy, ddy));
    float dist = __fmul_rn(__fsqrt_rn(sq), pixel_cm);
    float angle = __fdiv_rn(__fmul_rn(atanf(__fdiv_rn(dist, screen_distance)), 180.f), pi_f);
    float k = __fdiv_rn(__fsub_rn(0.f, 1.f), __fsub_rn(peripheral, foveal));
    float q = __fdiv_rn(__fsub_rn(__fmul_rn(peripheral, 1.f), __fmul_rn(0.f, foveal)), __fsub_rn(peripheral, foveal));
    float lin = A == ARITH_CONTRACTED ? __fmaf_rn(k, angle, q) : __fadd_rn(__fmul_rn(k, angle), q);
    float rel = (float)fmin(1.0, (double)lin);
    float adv = __fmul_rn(max_ss, rel);
    inside = false;
    if (angle <= foveal) {
        adv = (float)fmax(1.0, (double)adv);
        inside = true;
    }
    advised = adv;
}

// The previous-frame read of sample reuse for one lane (gen.cu:320-331:
// getWarpingOriginOfSampleReuse, the range test, readFromArrayUsingFiltering),
// in two halves so that a warp can put the reads of several tiles in flight
// before it filters any of them: reuse_fetch issues the four neighbours'
// (value, weight) loads for the column and row terms of the lane's pixel,
// reuse_filter combines them.  An origin outside the reusable range reads the
// frame's top-left 2x2 records (values not used), so the loads need no
// branch; callers fetch only for frames of at least 5x5 pixels (smaller ones
// reuse nothing).  AL8: the previous frame's base and pitch are multiples of
// 8 bytes, and each pair is one 8-byte load.
struct ReuseFetch {
    float2 a, b, c, d;
    float alpha, beta;
    bool in_range;
};

template <bool AL8> __device__ __forceinline__ float2 load_value_weight(const char *p)
{
    if (AL8) return __ldg(reinterpret_cast<const float2 *>(p));
    const float *q = reinterpret_cast<const float *>(p);
    return make_float2(__ldg(q), __ldg(q + 1));
}

template <bool AL8>
__device__ __forceinline__ ReuseFetch reuse_fetch(ReuseAxis ax, ReuseAxis ay, const void *in, long in_pitch)
{
    ReuseFetch f;
    f.in_range = ((ax.at & ay.at) >> 31) != 0u;
    f.alpha = ax.frac;
    f.beta = ay.frac;
    const uint32_t i = f.in_range ? ax.at & 0x7fffffffu : 0u, j = f.in_range ? ay.at & 0x7fffffffu : 0u;
    const char *q = reinterpret_cast<const char *>(pixel_ptr(in, in_pitch, i, j));
    const char *q1 = q + in_pitch;
    f.a = load_value_weight<AL8>(q);
    f.b = load_value_weight<AL8>(q + sizeof(PixelInfo));
    f.c = load_value_weight<AL8>(q1);
    f.d = load_value_weight<AL8>(q1 + sizeof(PixelInfo));
    return f;
}

template <int A> __device__ __forceinline__ void reuse_filter(const ReuseFetch &f, float &value, float &weight)
{
    filter_bilinear<A>(f.alpha, f.beta, f.a, f.b, f.c, f.d, value, weight);
}

// The rest of fractalRenderAdvanced for one lane of an 8x4 warp tile
// (gen.cu:332-368), given the lane's reuse result: foveation, the vote
// groups (lanes that reach the same sampleTheFractal call site vote
// together), the samples, the record.  `reusing` is false for lanes outside
// the image and without the sample-reuse flag.  Returns the record stored.
template <class R, int A, int F>
__device__ __forceinline__ PixelInfo finish_advanced_tile(const SampleGeometry<R> &g, void *out, long pitch, UInt2 size,
                                                          UInt2 focus, uint32_t x0, uint32_t y0, uint32_t lane,
                                                          float max_ss, uint32_t flags, bool reusing, float reused_v,
                                                          float reused_w, unsigned long long &iters)
{
    UInt2 p = tile_pixel(x0, y0, lane);
    bool valid = p.x < size.x && p.y < size.y;
    float advised = max_ss;
    bool inside = false;
    if (valid && (flags & FLAG_FOVEATION) && (flags & FLAG_IS_ZOOMING) && (flags & FLAG_ZOOMING_IN))
        foveation<A>(p, focus, max_ss, advised, inside);
    bool group_a = valid && reusing && (flags & FLAG_ZOOMING_IN) && inside;
    bool group_b = valid && !reusing;
    uint32_t mask_a = __ballot_sync(0xffffffffu, group_a);
    uint32_t mask_b = __ballot_sync(0xffffffffu, group_b);
    bool adaptive = (flags & FLAG_ADAPTIVE_SS) != 0;
    PixelInfo res = make_pixel(0.f, 0.f);
    if (reusing) {
        res.value = reused_v;
        res.weight = reused_w;
        res.is_reused = 1;
    }
    if (group_a) {
        float sc = advised;
        float samples = (float)sample_the_fractal<R, A, F>(g, p.x, p.y, sc, adaptive, true, mask_a, iters);
        float rw = __fmul_rn(reused_w, 0.75f);
        res.weight_of_new_samples = sc;
        res.weight = __fadd_rn(rw, sc);
        const float num = A == ARITH_CONTRACTED ? __fmaf_rn(reused_v, rw, __fmul_rn(samples, sc))
                                                : __fadd_rn(__fmul_rn(reused_v, rw), __fmul_rn(samples, sc));
        res.value = __fdiv_rn(num, res.weight);
    }
    if (group_b) {
        float sc = advised < 1.f ? 1.f : advised;
        res.value = (float)sample_the_fractal<R, A, F>(g, p.x, p.y, sc, adaptive, true, mask_b, iters);
        res.weight = sc;
    }
    if (valid) store_pixel(pixel_ptr(out, pitch, p.x, p.y), res);
    return res;
}

// fractalRenderAdvanced for one lane of an 8x4 warp tile (gen.cu:307-368).
// Returns the record stored for the lane's pixel.
template <class R, int A, int F>
__device__ __forceinline__ PixelInfo render_advanced_tile(const SampleGeometry<R> &g, const Rect<R> &image,
                                                          const Rect<R> &image_reused, void *out, long pitch,
                                                          UInt2 size, const void *in, long in_pitch, UInt2 focus,
                                                          uint32_t x0, uint32_t y0, uint32_t lane, float max_ss,
                                                          uint32_t flags, unsigned long long &iters)
{
    UInt2 p = tile_pixel(x0, y0, lane);
    bool valid = p.x < size.x && p.y < size.y;
    bool reusing = false;
    float reused_v = 0.f, reused_w = 0.f;
    if (valid && (flags & FLAG_SAMPLE_REUSE) && size.x >= 5u && size.y >= 5u) {
        const ReuseAxis ax = reuse_axis(warping_origin_x<R, A>(p.x, size, image, image_reused), size.x);
        const ReuseAxis ay = reuse_axis(warping_origin_y<R, A>(p.y, size, image, image_reused), size.y);
        const ReuseFetch f = ((reinterpret_cast<uintptr_t>(in) | (uintptr_t)in_pitch) & 7u) == 0
                                 ? reuse_fetch<true>(ax, ay, in, in_pitch)
                                 : reuse_fetch<false>(ax, ay, in, in_pitch);
        if (f.in_range) {
            reuse_filter<A>(f, reused_v, reused_w);
            reusing = !(reused_w < 0.1f);
        }
    }
    // a tile whose pixels all reuse and take no new samples (outside the
    // foveal region, which is uniform over a tile, when zooming in with
    // foveation) stores (value, weight, isReused = 1, 0) without the vote code
    if (__all_sync(0xffffffffu, reusing || !valid)) {
        bool sample = false;
        if ((flags & FLAG_FOVEATION) && (flags & FLAG_IS_ZOOMING) && (flags & FLAG_ZOOMING_IN)) {
            float advised;
            foveation<A>(p, focus, max_ss, advised, sample);
        }
        if (!sample) {
            PixelInfo rec = make_pixel(reused_v, reused_w);
            rec.is_reused = 1;
            if (valid) store_pixel(pixel_ptr(out, pitch, p.x, p.y), rec);
            return rec;
        }
    }
    return finish_advanced_tile<R, A, F>(g, out, pitch, size, focus, x0, y0, lane, max_ss, flags, reusing, reused_v,
                                         reused_w, iters);
}

// ---------------------------------------------------------------------------
// Compose (gen.cu:455-475)
// ---------------------------------------------------------------------------

// colorizeSampleCount, gen.cu:67-77.  The channels are `char`: built with the
// reference's x86-64 toolchain (signed char) the float-to-char conversion
// saturates at 127, which is what this reproduces.
__device__ __forceinline__ uint32_t colorize_sample_count(uint32_t sample_count, uint32_t full)
{
    sample_count = sample_count < full ? sample_count : full;
    float rel = __fdiv_rn((float)sample_count, (float)full);
    float f = __fmul_rn(255.f, rel);
    int c = (int)f;
    c = c > 127 ? 127 : c;
    uint32_t b = (uint32_t)(uint8_t)(int8_t)c;
    return b | (b << 8) | (b << 16) | 0xff000000u;
}

// colorize, mandelbrot.cu:27-35 / julia.cu:19-27
__device__ __forceinline__ uint32_t palette_index(float value, uint32_t palette_len)
{
    uint32_t vi = (uint32_t)roundf(value);
    return palette_len - (vi % palette_len) - 1u;
}

// Colouring modes of the modules' colorize().
enum ColorMode {
    COLOR_PALETTE = 0,     // mandelbrot.cu:27-35, julia.cu:19-27
    COLOR_ROOTS = 1,       // newton_wired.cu:67-80, newton_generic.cu:75-88: red/green/blue per root, black
    COLOR_MAGNIFIED = 2    // newton_iterations.cu:70-78: palette stride colorMagnifier
};

__device__ __forceinline__ uint32_t colorize_value(float value, const uint32_t *palette, uint32_t palette_len,
                                                   int mode, int magnifier)
{
    if (mode == COLOR_ROOTS) {
        uint32_t r = (uint32_t)roundf(value);
        return r == 1u ? 0xff0000ffu : r == 2u ? 0xff00ff00u : r == 3u ? 0xffff0000u : 0xff000000u;
    }
    if (mode == COLOR_MAGNIFIED) {
        uint32_t vi = (uint32_t)roundf(value);
        return palette[palette_len - (vi * (uint32_t)magnifier % palette_len) - 1u];
    }
    return palette[palette_index(value, palette_len)];
}

__device__ __forceinline__ uint32_t compose_pixel(const PixelInfo &p, const uint32_t *palette, uint32_t palette_len,
                                                  float max_ss, bool visualize, int mode = COLOR_PALETTE,
                                                  int magnifier = 1)
{
    if (visualize) {
        uint32_t full = (uint32_t)fmax(1.0, (double)max_ss);
        uint32_t c = colorize_sample_count((uint32_t)p.weight, full);
        if (p.is_reused) c = colorize_sample_count((uint32_t)p.weight_of_new_samples, full);
        return c;
    }
    return colorize_value(p.value, palette, palette_len, mode, magnifier);
}

}  // namespace chaos
