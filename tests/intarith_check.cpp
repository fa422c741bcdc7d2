// Host check of chaos::sub_nonneg_bits against the host's own binary64
// subtraction (IEEE round to nearest even), over seeded operand classes:
// equal exponents, exponents 1-2 apart, far apart, near-cancellation, the top
// and bottom of the normal range, zeros, subnormals, infinities and NaNs.
// Prints "pairs flagged wrong" and exits 1 on any wrong result.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "chaos_intarith.cuh"

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next()
{
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double from_bits(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static uint64_t to_bits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 4000000;
    const uint64_t FRAC = (1ull << 52) - 1;
    long flagged = 0, wrong = 0;
    for (long i = 0; i < n; i++) {
        const int kind = (int)(i % 9);
        uint64_t ea = 1 + next() % 2046, ma = next() & FRAC, mb = next() & FRAC, eb = ea;
        switch (kind) {
        case 0: break;                                                   // same exponent
        case 1: eb = ea > 2 ? ea - next() % 3 : ea; break;               // 0-2 apart
        case 2: eb = ea > 70 ? ea - next() % 70 : 1 + next() % ea; break;  // far apart
        case 3: mb = ma ^ (next() & ((1ull << (next() % 53)) - 1)); break;  // near-cancellation
        case 4: ea = 2040 + next() % 7; eb = ea - next() % 4; break;     // top of the range
        case 5: ea = 1 + next() % 6; eb = 1 + next() % ea; break;        // bottom of the range
        case 6: ea = 1000 + next() % 50; eb = next() % 2 ? 0 : ea; if (eb == 0) mb = next() % 4 ? 0 : mb; break;  // zeros, subnormals
        case 7: ea = 2047; ma = next() % 2 ? 0 : ma; eb = next() % 2048; break;  // inf / NaN
        default: ea = 1023 + next() % 8 - 4; eb = ea + next() % 3 - 1; ma = FRAC - (next() & 7); mb = FRAC - (next() & 7); break;
        }
        uint64_t A = (ea << 52) | ma, B = (eb << 52) | mb;
        if (next() & 1) { uint64_t t = A; A = B; B = t; }
        bool exact = false;
        const uint64_t got = chaos::sub_nonneg_bits(A, B, exact);
        const double a = from_bits(A), b = from_bits(B);
        if (!exact) { flagged++; continue; }
        if (std::isnan(a) || std::isnan(b) || std::isinf(a) || std::isinf(b)) {
            // only "never a small value" is asked for: NaN, or the IEEE result
            const double g = from_bits(got);
            if (!(std::isnan(g) || got == to_bits(a - b))) wrong++;
            continue;
        }
        if (got != to_bits(a - b)) {
            if (wrong < 5) std::printf("a=%a b=%a got=%a want=%a\n", a, b, from_bits(got), a - b);
            wrong++;
        }
    }
    std::printf("%ld %ld %ld\n", n, flagged, wrong);
    return wrong ? 1 : 0;
}
