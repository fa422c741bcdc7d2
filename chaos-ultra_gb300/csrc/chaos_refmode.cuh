// chaos_refmode.cuh -- the reference-mode persistent kernels (fractalRenderMain
// and fractalRenderAdvanced semantics, gen.cu:168-181, 307-368): persistent
// warps take 8x4 pixel tiles from a work counter; one tile is one vote group
// of the adaptive super-sampling.  Included by chaos_kernels.cu (escape-time
// modules) and chaos_newton.cu (Newton modules, built without contraction).
#pragma once

#include "chaos_kernels.cuh"

namespace chaos {

constexpr uint32_t FULL = 0xffffffffu;
constexpr int PERSIST_THREADS = 256;


__device__ __forceinline__ uint32_t next_tile(uint32_t *counter, uint32_t lane)
{
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    return __shfl_sync(FULL, t, 0);
}

__device__ __forceinline__ void add_total(unsigned long long *total, unsigned long long iters, uint32_t lane)
{
    if (!total) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) iters += __shfl_down_sync(FULL, iters, o);
    if (lane == 0 && iters) atomicAdd(total, iters);
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_main(MainArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.image, a.size, a.max_iter, a.jcx, a.jcy);
    g.newton = a.newton;
    unsigned long long iters = 0;
    for (;;) {
        uint32_t t = next_tile(a.counter, lane);
        if (t >= a.n_tiles) break;
        uint32_t x0 = 8u * (t % a.tiles_x), y0 = 4u * (t / a.tiles_x);
        render_main_tile<R, A, F>(g, a.out, a.pitch, a.size, x0, y0, lane, a.max_ss, a.flags, iters);
    }
    add_total(a.total, iters, lane);
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_advanced(AdvancedArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.m.image, a.m.size, a.m.max_iter, a.m.jcx, a.m.jcy);
    g.newton = a.m.newton;
    unsigned long long iters = 0;
    for (;;) {
        uint32_t t = next_tile(a.m.counter, lane);
        if (t >= a.m.n_tiles) break;
        uint32_t x0 = 8u * (t % a.m.tiles_x), y0 = 4u * (t / a.m.tiles_x);
        render_advanced_tile<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size, a.in, a.in_pitch,
                                      a.focus, x0, y0, lane, a.m.max_ss, a.m.flags, iters);
    }
    add_total(a.m.total, iters, lane);
}

template <class KernelPtr> static int occupancy(KernelPtr k, int threads)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, threads, 0) != cudaSuccess || n < 1) n = 1;
    return n;
}

static inline unsigned grid_for(unsigned long long work_warps, int occ, int sms)
{
    unsigned long long blocks = (work_warps + (PERSIST_THREADS / 32) - 1) / (PERSIST_THREADS / 32);
    unsigned long long cap = (unsigned long long)occ * (unsigned long long)sms;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (unsigned)blocks;
}

template <class R, int A, int F> static cudaError_t launch_main_t(const MainArgs<R> &a, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_main<R, A, F>, PERSIST_THREADS);
    k_main<R, A, F><<<grid_for(a.n_tiles, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

template <class R, int A, int F> static cudaError_t launch_advanced_t(const AdvancedArgs<R> &a, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_advanced<R, A, F>, PERSIST_THREADS);
    k_advanced<R, A, F><<<grid_for(a.m.n_tiles, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace chaos
