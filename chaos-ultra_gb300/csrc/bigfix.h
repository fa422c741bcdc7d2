// bigfix.h -- multi-word signed fixed-point numbers for reference orbits (host).
//
// A value is sign * (limb[L] + sum_{k<L} limb[k] * 2^(64(k-L))): limb[L] is the
// integer part, limbs 0..L-1 the fraction, least significant first.  |value|
// stays below 2^63 (orbit values are below 16 before they escape).  Products
// are truncated to L fraction limbs (error below 2^(-64L+1) per product).
// Nothing here depends on the CPU: 64x64->128-bit products use unsigned
// __int128, which gcc provides on x86-64 and aarch64 alike.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

namespace chaos {

constexpr int BIGFIX_MAX_LIMBS = 24;  // 1536 fraction bits

struct BigFix {
    int limbs = 2;  // fraction limbs in use
    bool neg = false;
    uint64_t w[BIGFIX_MAX_LIMBS + 1] = {};

    bool is_zero() const
    {
        for (int k = 0; k <= limbs; k++)
            if (w[k]) return false;
        return true;
    }
};

inline BigFix bigfix_zero(int limbs)
{
    BigFix r;
    r.limbs = limbs;
    return r;
}

// |a| vs |b|
inline int bigfix_cmp_mag(const BigFix &a, const BigFix &b)
{
    for (int k = a.limbs; k >= 0; k--) {
        if (a.w[k] != b.w[k]) return a.w[k] < b.w[k] ? -1 : 1;
    }
    return 0;
}

inline void bigfix_add_mag(const BigFix &a, const BigFix &b, BigFix &r)
{
    unsigned __int128 c = 0;
    for (int k = 0; k <= a.limbs; k++) {
        c += (unsigned __int128)a.w[k] + b.w[k];
        r.w[k] = (uint64_t)c;
        c >>= 64;
    }
}

// |a| - |b| with |a| >= |b|
inline void bigfix_sub_mag(const BigFix &a, const BigFix &b, BigFix &r)
{
    uint64_t borrow = 0;
    for (int k = 0; k <= a.limbs; k++) {
        uint64_t x = a.w[k], y = b.w[k];
        uint64_t d = x - y - borrow;
        borrow = (x < y) || (x == y && borrow) ? 1 : 0;
        r.w[k] = d;
    }
}

inline BigFix bigfix_add(const BigFix &a, const BigFix &b)
{
    BigFix r;
    r.limbs = a.limbs;
    if (a.neg == b.neg) {
        bigfix_add_mag(a, b, r);
        r.neg = a.neg;
    } else if (bigfix_cmp_mag(a, b) >= 0) {
        bigfix_sub_mag(a, b, r);
        r.neg = a.neg;
    } else {
        bigfix_sub_mag(b, a, r);
        r.neg = b.neg;
    }
    if (r.is_zero()) r.neg = false;
    return r;
}

inline BigFix bigfix_neg(BigFix a)
{
    if (!a.is_zero()) a.neg = !a.neg;
    return a;
}

inline BigFix bigfix_sub(const BigFix &a, const BigFix &b) { return bigfix_add(a, bigfix_neg(b)); }

// a * b, truncated to L fraction limbs.
inline BigFix bigfix_mul(const BigFix &a, const BigFix &b)
{
    const int L = a.limbs;
    uint64_t p[2 * BIGFIX_MAX_LIMBS + 3] = {};
    for (int i = 0; i <= L; i++) {
        if (!a.w[i]) continue;
        unsigned __int128 carry = 0;
        for (int j = 0; j <= L; j++) {
            unsigned __int128 t = (unsigned __int128)a.w[i] * b.w[j] + p[i + j] + carry;
            p[i + j] = (uint64_t)t;
            carry = t >> 64;
        }
        int k = i + L + 1;
        while (carry) {
            unsigned __int128 t = (unsigned __int128)p[k] + carry;
            p[k] = (uint64_t)t;
            carry = t >> 64;
            k++;
        }
    }
    BigFix r;
    r.limbs = L;
    for (int k = 0; k <= L; k++) r.w[k] = p[k + L];
    r.neg = (a.neg != b.neg) && !r.is_zero();
    return r;
}

inline BigFix bigfix_mul2(BigFix a)  // exact doubling
{
    uint64_t carry = 0;
    for (int k = 0; k <= a.limbs; k++) {
        uint64_t x = a.w[k];
        a.w[k] = (x << 1) | carry;
        carry = x >> 63;
    }
    return a;
}

inline BigFix bigfix_from_double(double d, int limbs)
{
    BigFix r = bigfix_zero(limbs);
    if (d == 0.0 || !std::isfinite(d)) return r;
    r.neg = d < 0;
    d = std::fabs(d);
    int e;
    double m = std::frexp(d, &e);                // d = m * 2^e, m in [0.5, 1)
    uint64_t mant = (uint64_t)std::ldexp(m, 53);  // exact 53-bit integer
    // d = mant * 2^(e-53); bit position of mant's lsb relative to 2^(-64L)
    int shift = e - 53 + 64 * limbs;
    if (shift < 0) {
        if (shift <= -64) return r;  // below the precision
        mant >>= -shift;
        shift = 0;
    }
    int limb = shift / 64, off = shift % 64;
    if (limb <= limbs) r.w[limb] |= mant << off;
    if (off && limb + 1 <= limbs) r.w[limb + 1] |= mant >> (64 - off);
    if (r.is_zero()) r.neg = false;
    return r;
}

// Correctly rounded? No: truncated to the nearest double below in magnitude,
// plus round-to-nearest of the top 64 bits; accurate to 1 ulp.
inline double bigfix_to_double(const BigFix &a)
{
    int top = -1;
    for (int k = a.limbs; k >= 0; k--)
        if (a.w[k]) {
            top = k;
            break;
        }
    if (top < 0) return 0.0;
    // take up to 128 bits from the top two limbs
    double hi = std::ldexp((double)a.w[top], 64 * (top - a.limbs));
    double lo = top > 0 ? std::ldexp((double)a.w[top - 1], 64 * (top - 1 - a.limbs)) : 0.0;
    double v = hi + lo;
    return a.neg ? -v : v;
}

// Parse "[-]I.HHHH...": decimal integer part I (|I| < 2^63), then hexadecimal
// fraction digits (4 bits each).  Digits past the precision are dropped.
inline bool bigfix_parse_hex(const char *s, int limbs, BigFix &out)
{
    out = bigfix_zero(limbs);
    if (!s) return false;
    bool neg = false;
    if (*s == '-') {
        neg = true;
        s++;
    } else if (*s == '+') {
        s++;
    }
    uint64_t ip = 0;
    bool any = false;
    while (*s >= '0' && *s <= '9') {
        ip = ip * 10 + (uint64_t)(*s - '0');
        s++;
        any = true;
    }
    out.w[limbs] = ip;
    if (*s == '.') {
        s++;
        int bit = 64 * limbs;  // position below the binary point, counting down
        while (*s) {
            int v;
            char c = *s;
            if (c >= '0' && c <= '9')
                v = c - '0';
            else if (c >= 'a' && c <= 'f')
                v = c - 'a' + 10;
            else if (c >= 'A' && c <= 'F')
                v = c - 'A' + 10;
            else
                return false;
            bit -= 4;
            if (bit >= 0) out.w[bit / 64] |= (uint64_t)v << (bit % 64);
            s++;
            any = true;
        }
    }
    if (*s != '\0' || !any) return false;
    out.neg = neg && !out.is_zero();
    return true;
}

}  // namespace chaos
