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


__device__ __forceinline__ void add_total(unsigned long long *total, unsigned long long iters, uint32_t lane)
{
    if (!total) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) iters += __shfl_down_sync(FULL, iters, o);
    if (lane == 0 && iters) atomicAdd(total, iters);
}

// Tiles are claimed `chunk` at a time (consecutive, so a claim is a strip of one
// tile row), and the next claim is issued before the current strip is
// rendered.  With one counter for the whole frame, a claim per tile made the
// counter the bottleneck of large reuse-dominated frames, whose tiles take a
// few loads each; small frames keep claims of one tile made when needed, the
// finest balance (serving latency).
template <class Body>
__device__ __forceinline__ void for_each_tile(uint32_t *counter, uint32_t n_tiles, uint32_t chunk, uint32_t lane,
                                              Body body)
{
    uint32_t claim = 0;
    if (lane == 0) claim = atomicAdd(counter, chunk);
    uint32_t t0 = __shfl_sync(FULL, claim, 0);
    while (t0 < n_tiles) {
        // with strips, the next strip is claimed while this one is rendered;
        // single tiles (small frames) are claimed when needed, which keeps the
        // end of the frame balanced
        if (chunk > 1 && lane == 0) claim = atomicAdd(counter, chunk);
        const uint32_t t1 = min(t0 + chunk, n_tiles);
        for (uint32_t t = t0; t < t1; t++) body(t);
        if (chunk == 1 && lane == 0) claim = atomicAdd(counter, 1u);
        t0 = __shfl_sync(FULL, claim, 0);
    }
}

// Tiles per claim: up to 4, while every resident warp still gets 8 claims.
static inline uint32_t tile_chunk_for(uint32_t n_tiles, int occ, int sms)
{
    const unsigned long long warps = (unsigned long long)occ * sms * (PERSIST_THREADS / 32);
    unsigned long long c = n_tiles / (warps * 8ull);
    return (uint32_t)(c < 1 ? 1 : c > 4 ? 4 : c);
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_main(MainArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.image, a.size, a.max_iter, a.jcx, a.jcy);
    g.newton = a.newton;
    unsigned long long iters = 0;
    for_each_tile(a.counter, a.n_tiles, a.tile_chunk, lane, [&](uint32_t t) {
        uint32_t x0 = 8u * (t % a.tiles_x), y0 = 4u * (t / a.tiles_x);
        render_main_tile<R, A, F>(g, a.out, a.pitch, a.size, x0, y0, lane, a.max_ss, a.flags, iters);
    });
    add_total(a.total, iters, lane);
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_advanced(AdvancedArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.m.image, a.m.size, a.m.max_iter, a.m.jcx, a.m.jcy);
    g.newton = a.m.newton;
    unsigned long long iters = 0;
    for_each_tile(a.m.counter, a.m.n_tiles, a.m.tile_chunk, lane, [&](uint32_t t) {
        uint32_t x0 = 8u * (t % a.m.tiles_x), y0 = 4u * (t / a.m.tiles_x);
        render_advanced_tile<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size, a.in, a.in_pitch,
                                      a.focus, x0, y0, lane, a.m.max_ss, a.m.flags, iters);
    });
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

template <class R, int A, int F> static cudaError_t launch_main_t(const MainArgs<R> &args, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_main<R, A, F>, PERSIST_THREADS);
    MainArgs<R> a = args;
    a.tile_chunk = tile_chunk_for(a.n_tiles, occ, sms);
    k_main<R, A, F><<<grid_for((a.n_tiles + a.tile_chunk - 1) / a.tile_chunk, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

template <class R, int A, int F>
static cudaError_t launch_advanced_t(const AdvancedArgs<R> &args, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_advanced<R, A, F>, PERSIST_THREADS);
    AdvancedArgs<R> a = args;
    a.m.tile_chunk = tile_chunk_for(a.m.n_tiles, occ, sms);
    k_advanced<R, A, F><<<grid_for((a.m.n_tiles + a.m.tile_chunk - 1) / a.m.tile_chunk, occ, sms), PERSIST_THREADS, 0,
                          s>>>(a);
    return cudaGetLastError();
}

}  // namespace chaos
