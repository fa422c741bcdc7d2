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

// Tiles are claimed in strips of consecutive tiles, the next claim issued
// before the current strip is rendered.  With one counter for the whole
// frame, a claim per tile made the counter the bottleneck of large
// reuse-dominated frames, whose tiles take a few loads each.  Claims are
// guided: a quarter of an even share of the tiles left after the warp's
// previous strip, between 1 and `max_chunk`, so long strips early keep the
// counter quiet and short ones late keep the end of the frame balanced;
// single tiles are claimed when needed (the finest balance, small frames).
template <class Body>
__device__ __forceinline__ void for_each_strip(uint32_t *counter, uint32_t n_tiles, uint32_t max_chunk, uint32_t lane,
                                               Body body)
{
    const uint32_t share = 4u * gridDim.x * (blockDim.x >> 5);
    auto size_after = [&](uint32_t at) -> uint32_t {
        const uint32_t c = (at < n_tiles ? n_tiles - at : 0u) / share;
        return c < 1u ? 1u : c > max_chunk ? max_chunk : c;
    };
    uint32_t size = size_after(0u), claim = 0;
    if (lane == 0) claim = atomicAdd(counter, size);
    uint32_t t0 = __shfl_sync(FULL, claim, 0);
    while (t0 < n_tiles) {
        const uint32_t t1 = min(t0 + size, n_tiles), next = size_after(t1);
        if (size > 1u && lane == 0) claim = atomicAdd(counter, next);
        body(t0, t1);
        if (size == 1u && lane == 0) claim = atomicAdd(counter, next);
        t0 = __shfl_sync(FULL, claim, 0);
        size = next;
    }
}

// A tile's column and row in a frame `tiles_x` tiles wide, stepped tile by
// tile: one division per strip instead of two per tile (a reuse tile is ~90
// instructions; the divisions were another ~100).
struct TileCursor {
    uint32_t tx, ty;
    __device__ __forceinline__ TileCursor(uint32_t t, uint32_t tiles_x) : tx(t % tiles_x), ty(t / tiles_x) {}
    __device__ __forceinline__ void next(uint32_t tiles_x)
    {
        if (++tx == tiles_x) {
            tx = 0;
            ++ty;
        }
    }
    // the cursor k tiles further on
    __device__ __forceinline__ TileCursor plus(uint32_t k, uint32_t tiles_x) const
    {
        TileCursor c = *this;
        c.tx += k;
        while (c.tx >= tiles_x) {
            c.tx -= tiles_x;
            ++c.ty;
        }
        return c;
    }
    __device__ __forceinline__ uint32_t x0() const { return 8u * tx; }
    __device__ __forceinline__ uint32_t y0() const { return 4u * ty; }
};

// body(x0, y0) for every tile claimed, (x0, y0) its top-left pixel
template <class Body>
__device__ __forceinline__ void for_each_tile(uint32_t *counter, uint32_t n_tiles, uint32_t tiles_x, uint32_t chunk,
                                              uint32_t lane, Body body)
{
    for_each_strip(counter, n_tiles, chunk, lane, [&](uint32_t t0, uint32_t t1) {
        TileCursor c(t0, tiles_x);
        for (uint32_t t = t0; t < t1; t++, c.next(tiles_x)) body(c.x0(), c.y0());
    });
}

// The longest strip a warp claims: up to `cap` tiles, while every resident
// warp still gets 8 claims.  (An 8K reuse frame is a million tiles: at 4 per
// claim its single work counter took a quarter of a million atomics in
// ~0.3 ms.)
static inline uint32_t tile_chunk_for(uint32_t n_tiles, int occ, int sms, uint32_t cap = 16)
{
    const unsigned long long warps = (unsigned long long)occ * sms * (PERSIST_THREADS / 32);
    unsigned long long c = n_tiles / (warps * 8ull);
    return (uint32_t)(c < 1 ? 1 : c > cap ? cap : c);
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_main(MainArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.image, a.size, a.max_iter, a.jcx, a.jcy);
    g.newton = a.newton;
    unsigned long long iters = 0;
    for_each_tile(a.counter, a.n_tiles, a.tiles_x, a.tile_chunk, lane, [&](uint32_t x0, uint32_t y0) {
        render_main_tile<R, A, F>(g, a.out, a.pitch, a.size, x0, y0, lane, a.max_ss, a.flags, iters);
    });
    add_total(a.total, iters, lane);
}

// Tiles whose previous-frame reads are in flight together.  A reuse-dominated
// frame is a stream of small dependent steps per tile (origin -> four loads
// -> filter -> store); with one tile's loads in flight per warp and the
// origin's four divisions computed per pixel it ran at about half the copy
// rate, bound by the loads' latency and the issue of the divisions.  Two
// tiles (eight 8-byte loads per lane) measured best: four need registers
// that cost a fifth of the warps.
// The strip [t0, t1) of a fractalRenderAdvanced frame, in groups of four
// tiles (32x4 pixels).  The reuse reads of a group run in row order: lane l
// takes column l & 7 of the group's tile l >> 3 and walks its four rows, so
// that a warp's read of one row covers 32 consecutive pixels (contiguous
// records under a near-identity warp), and the reads of all four rows are in
// flight before the first is filtered.  The origin's column term is the
// lane's own; its row terms are computed once per row (lane l: row l & 3 of
// tile (l >> 2) & 3) and taken by shuffles.  The filtered (value, weight)
// pairs (the weight -1 where the origin is out of range) go to the warp's
// `stage` (4 x 32 pairs of shared memory), from which each tile is finished
// in its own 8x4 lane layout (votes, samples, record).
template <class R, int A, int F, bool AL8>
__device__ __forceinline__ void advanced_strip(const AdvancedArgs<R> &a, const SampleGeometry<R> &g, uint32_t lane,
                                               float2 *stage, uint32_t t0, uint32_t t1, unsigned long long &iters)
{
    // (frames smaller than 5x5 pixels reuse nothing, see reuse_axis)
    const bool reuse = (a.m.flags & FLAG_SAMPLE_REUSE) != 0 && a.m.size.x >= 5u && a.m.size.y >= 5u;
    // zooming in with foveation, a reusing pixel in the foveal region takes new samples
    const bool fov =
        (a.m.flags & FLAG_FOVEATION) && (a.m.flags & FLAG_IS_ZOOMING) && (a.m.flags & FLAG_ZOOMING_IN);
    const uint32_t col = 4u * (lane >> 4) + (lane & 3u), row = (lane >> 2) & 3u;  // the 8x4 tile layout
    const uint32_t tiles_x = a.m.tiles_x;
    TileCursor cur(t0, tiles_x);  // the next tile to finish
    for (uint32_t tg = t0; tg < t1; tg += 4u) {
        const uint32_t ng = min(4u, t1 - tg);
        if (reuse) {
            // this lane's column (of its tile k; lanes past the group's end repeat its last tile)
            const uint32_t k = min(lane >> 3, ng - 1u);
            const TileCursor tc = cur.plus(k, tiles_x);
            const TileCursor tr = cur.plus(min((lane >> 2) & 3u, ng - 1u), tiles_x);
            const uint32_t x = tc.x0() + (lane & 7u);
            const ReuseAxis mx = reuse_axis(warping_origin_x<R, A>(x, a.m.size, a.m.image, a.image_reused), a.m.size.x);
            const ReuseAxis my = reuse_axis(
                warping_origin_y<R, A>(tr.y0() + (lane & 3u), a.m.size, a.m.image, a.image_reused), a.m.size.y);
            ReuseFetch f[4];
#pragma unroll
            for (uint32_t r = 0; r < 4u; r++) {
                ReuseAxis ay;
                ay.at = __shfl_sync(FULL, my.at, 4u * k + r);
                ay.frac = __shfl_sync(FULL, my.frac, 4u * k + r);
                f[r] = reuse_fetch<AL8>(mx, ay, a.in, a.in_pitch);
            }
#pragma unroll
            for (uint32_t r = 0; r < 4u; r++) {
                float vv, ww;
                reuse_filter<A>(f[r], vv, ww);
                stage[32u * r + lane] = make_float2(vv, f[r].in_range ? ww : -1.f);
            }
            __syncwarp();
        }
        for (uint32_t k = 0; k < ng; k++, cur.next(tiles_x)) {
            const uint32_t x0 = cur.x0(), y0 = cur.y0();
            const UInt2 p = tile_pixel(x0, y0, lane);
            const bool valid = p.x < a.m.size.x && p.y < a.m.size.y;
            const float2 vw = reuse ? stage[32u * row + 8u * k + col] : make_float2(0.f, 0.f);
            const bool reusing = valid && reuse && !(vw.y < 0.1f);
            if (!fov && __all_sync(FULL, reusing || !valid)) {
                // every pixel reuses and none takes new samples: the record is
                // (value, weight, isReused = 1, 0), as the full path stores it
                if (valid) {
                    PixelInfo rec = make_pixel(vw.x, vw.y);
                    rec.is_reused = 1;
                    store_pixel(pixel_ptr(a.m.out, a.m.pitch, p.x, p.y), rec);
                }
                continue;
            }
            finish_advanced_tile<R, A, F>(g, a.m.out, a.m.pitch, a.m.size, a.focus, x0, y0, lane, a.m.max_ss,
                                          a.m.flags, reusing, vw.x, vw.y, iters);
        }
        __syncwarp();
    }
}

template <class R, int A, int F> __global__ void __launch_bounds__(PERSIST_THREADS) k_advanced(AdvancedArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.m.image, a.m.size, a.m.max_iter, a.m.jcx, a.m.jcy);
    g.newton = a.m.newton;
    unsigned long long iters = 0;
    __shared__ float2 s_stage[PERSIST_THREADS / 32][4 * 32];
    float2 *stage = s_stage[threadIdx.x >> 5];
    const bool al8 = ((reinterpret_cast<uintptr_t>(a.in) | (uintptr_t)a.in_pitch) & 7u) == 0;
    if (al8)
        for_each_strip(a.m.counter, a.m.n_tiles, a.m.tile_chunk, lane, [&](uint32_t t0, uint32_t t1) {
            advanced_strip<R, A, F, true>(a, g, lane, stage, t0, t1, iters);
        });
    else
        for_each_strip(a.m.counter, a.m.n_tiles, a.m.tile_chunk, lane, [&](uint32_t t0, uint32_t t1) {
            advanced_strip<R, A, F, false>(a, g, lane, stage, t0, t1, iters);
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
