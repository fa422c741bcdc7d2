// Device check of chaos::sub_nonneg_bits against the GPU's own binary64
// subtraction (__dsub_rn), on seeded operand classes like the host check
// (tests/intarith_check.cpp): equal, near and far exponents,
// near-cancellation, both ends of the normal range, zeros and subnormals.
// Prints "pairs flagged wrong" and exits 1 on any wrong result or CUDA error.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "chaos_intarith.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void k_check(uint64_t n, unsigned long long *flagged, unsigned long long *wrong)
{
    const uint64_t FRAC = (1ull << 52) - 1;
    unsigned long long f = 0, w = 0;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < n; q += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t r = 0x9e3779b97f4a7c15ull * (q + 1);
        auto next = [&]() { r += 0x9e3779b97f4a7c15ull; return mix(r); };
        const int kind = (int)(q % 7);
        uint64_t ea = 1 + next() % 2046, ma = next() & FRAC, mb = next() & FRAC, eb = ea;
        switch (kind) {
        case 0: break;
        case 1: eb = ea > 2 ? ea - next() % 3 : ea; break;
        case 2: eb = ea > 70 ? ea - next() % 70 : 1 + next() % ea; break;
        case 3: mb = ma ^ (next() & ((1ull << (next() % 53)) - 1)); break;
        case 4: ea = 2040 + next() % 7; eb = ea - next() % 4; break;
        case 5: ea = 1 + next() % 6; eb = 1 + next() % ea; break;
        default: ea = 1000 + next() % 50; eb = next() % 2 ? 0 : ea; if (eb == 0) mb = next() % 4 ? 0 : mb; break;
        }
        uint64_t A = (ea << 52) | ma, B = (eb << 52) | mb;
        if (next() & 1) { uint64_t t = A; A = B; B = t; }
        bool exact = false;
        const uint64_t got = chaos::sub_nonneg_bits(A, B, exact);
        if (!exact) { ++f; continue; }
        const double want = __dsub_rn(__longlong_as_double((long long)A), __longlong_as_double((long long)B));
        if (got != (uint64_t)__double_as_longlong(want)) ++w;
    }
    atomicAdd(flagged, f);
    atomicAdd(wrong, w);
}

int main(int argc, char **argv)
{
    const uint64_t n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ull << 26);
    unsigned long long *d = nullptr, h[2] = {0, 0};
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check<<<1024, 256>>>(n, d, d + 1);
    cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        std::printf("cuda error %s\n", cudaGetErrorString(e));
        return 2;
    }
    std::printf("%llu %llu %llu\n", (unsigned long long)n, h[0], h[1]);
    return h[1] ? 1 : 0;
}
