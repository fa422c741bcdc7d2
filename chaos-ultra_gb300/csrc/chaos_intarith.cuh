// chaos_intarith.cuh -- binary64 subtraction of two non-negative numbers on
// 64-bit integer arithmetic, rounded to nearest (ties to even) exactly as the
// floating-point unit rounds it.
//
// The rounded binary64 escape step spends six operations per iteration on the
// binary64 pipe, which is the kernel's bound, while the integer units sit
// mostly idle.  Moving x*x - y*y (both operands are squares, so never
// negative) to the integer units leaves five binary64 operations per step.
//
// Method (the textbook guard/round/sticky adder): the two non-negative bit
// patterns order like the values they encode, so one unsigned compare picks
// the larger operand and the sign of the result.  Both significands get their
// hidden bit and three extra low bits; the smaller one is shifted right by
// the exponent difference, and every bit shifted out is ORed into the lowest
// bit (sticky).  After the subtraction a count of leading zeros normalises
// the difference (at most one place when the exponents differ by two or
// more, any number of places otherwise, where the difference is exact).  The
// three extra bits then decide the rounding, and the exponent is added to the
// rounded significand, whose carry past 2^53 moves into the exponent field by
// itself.
//
// Special inputs: equal operands give +0, a zero smaller operand gives the
// other operand (negated if it was the subtrahend), and an infinite or NaN
// operand gives NaN (the escape loop only needs such a value never to test
// below 4).  A subnormal smaller operand or a subnormal result clears
// `exact`: the caller computes those on the floating-point unit instead.
//
// Written for host and device alike, so that host tests can check it
// against the host's own subtraction.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CHAOS_HD __host__ __device__ __forceinline__
#else
#define CHAOS_HD static inline
#endif

namespace chaos {

CHAOS_HD int clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// Bits of a - b from the bits A, B of a, b >= +0 (sign bits clear; a NaN with
// its sign bit set is also accepted).
CHAOS_HD uint64_t sub_nonneg_bits(uint64_t A, uint64_t B, bool &exact)
{
    const uint64_t SIGN = 1ull << 63, FRAC = (1ull << 52) - 1, HIDDEN = 1ull << 52;
    const bool neg = A < B;
    const uint64_t hi = neg ? B : A, lo = neg ? A : B;
    const int ea = (int)(hi >> 52), eb = (int)(lo >> 52);  // > 2047 only for a signed NaN
    const uint64_t ma = ((hi & FRAC) | HIDDEN) << 3, mb = ((lo & FRAC) | HIDDEN) << 3;
    const int d = ea - eb;
    const int ds = d < 63 ? d : 63;
    const uint64_t lost = (mb << ((64 - ds) & 63)) != 0 && ds != 0;
    const uint64_t aligned = d >= 58 ? 1ull : ((mb >> ds) | lost);
    uint64_t diff = ma - aligned;
    const int lz = clz64(diff) - 8;  // ma < 2^56, so lz >= 0; 56 when diff == 0
    diff <<= (lz & 63);
    const int e = ea - lz;
    const uint32_t rnd = (uint32_t)diff & 7u;
    uint64_t m = diff >> 3;
    m += (rnd > 4u || (rnd == 4u && (m & 1u))) ? 1u : 0u;
    uint64_t r = (neg ? SIGN : 0ull) | (((uint64_t)(e - 1) << 52) + m);
    r = diff == 0 ? 0ull : r;
    r = ea >= 2047 ? 0x7ff8000000000000ull : r;
    r = lo == 0 ? (neg ? (hi | SIGN) : hi) : r;
    exact = (eb >= 1 || lo == 0) && (e >= 1 || diff == 0 || ea >= 2047);
    return r;
}

}  // namespace chaos
