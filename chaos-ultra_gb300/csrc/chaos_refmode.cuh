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

// ---------------------------------------------------------------------------
// Staged sample reuse.  The previous frame's records a strip of tiles reads
// lie in a small rectangle of the old frame (the warp to the old frame is
// monotone in x and in y, so the strip's corner pixels bound it).  A warp
// copies that rectangle's (value, weight) pairs into shared memory with
// cp.async -- every lane has several independent 8-byte copies in flight and
// holds no registers for them -- and the filter then reads shared memory.
// The next strip's copies are issued before this strip is rendered.
// ---------------------------------------------------------------------------

constexpr int STAGE_PAIRS = 256;  // (value, weight) pairs per warp buffer

struct Footprint {
    int x0, y0, cols, rows;
    bool ok;
};

// The old-frame rectangle read by tiles [t_first, t_end) of one tile row
// (ok = false when the strip wraps to the next row, reuse is off, or the
// rectangle does not fit a buffer: the strip then reads global memory).
template <class R, int A>
__device__ __forceinline__ Footprint strip_footprint(UInt2 size, const Rect<R> &image, const Rect<R> &reused,
                                                     uint32_t tiles_x, uint32_t t_first, uint32_t t_end,
                                                     uint32_t flags)
{
    Footprint fp{0, 0, 0, 0, false};
    if (!(flags & FLAG_SAMPLE_REUSE) || t_end <= t_first) return fp;
    const uint32_t row = t_first / tiles_x;
    if ((t_end - 1u) / tiles_x != row) return fp;
    const uint32_t px0 = 8u * (t_first % tiles_x), py0 = 4u * row;
    const uint32_t px1 = min(8u * ((t_end - 1u) % tiles_x) + 7u, size.x - 1u), py1 = min(py0 + 3u, size.y - 1u);
    float ax, ay, bx, by;
    warping_origin<R, A>(UInt2{px0, py0}, size, image, reused, ax, ay);
    warping_origin<R, A>(UInt2{px1, py1}, size, image, reused, bx, by);
    const float lim = 1.0e7f;  // also false for NaN
    if (!(fabsf(ax) < lim && fabsf(ay) < lim && fabsf(bx) < lim && fabsf(by) < lim)) return fp;
    int x0 = (int)floorf(fminf(ax, bx)), x1 = (int)floorf(fmaxf(ax, bx)) + 1;
    int y0 = (int)floorf(fminf(ay, by)), y1 = (int)floorf(fmaxf(ay, by)) + 1;
    x0 = max(x0, 0);
    y0 = max(y0, 0);
    x1 = min(x1, (int)size.x - 1);
    y1 = min(y1, (int)size.y - 1);
    const int cols = x1 - x0 + 1, rows = y1 - y0 + 1;
    if (cols <= 0 || rows <= 0 || cols * rows > STAGE_PAIRS) return fp;
    fp = Footprint{x0, y0, cols, rows, true};
    return fp;
}

// Issue the copies of a footprint into buf (one cp.async group).  The
// previous frame's base address and pitch are multiples of 8 bytes (checked
// by the launcher), so every 8-byte copy is aligned.
__device__ __forceinline__ void stage_footprint(float2 *buf, const void *in, long pitch, const Footprint &fp,
                                                uint32_t lane)
{
    if (fp.ok) {
        const int n = fp.cols * fp.rows;
        int r = (int)lane / fp.cols, c = (int)lane - r * fp.cols;
        const int dr = 32 / fp.cols, dc = 32 - dr * fp.cols;
        for (int k = (int)lane; k < n; k += 32) {
            const char *src = static_cast<const char *>(in) + (size_t)(fp.y0 + r) * (size_t)pitch +
                              (size_t)(fp.x0 + c) * sizeof(PixelInfo);
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(buf + k);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
            r += dr;
            c += dc;
            if (c >= fp.cols) {
                c -= fp.cols;
                r++;
            }
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <class R, int A, int F, bool STAGED>
__global__ void __launch_bounds__(PERSIST_THREADS) k_advanced(AdvancedArgs<R> a)
{
    const uint32_t lane = threadIdx.x & 31u;
    SampleGeometry<R> g = make_geometry(a.m.image, a.m.size, a.m.max_iter, a.m.jcx, a.m.jcy);
    g.newton = a.m.newton;
    unsigned long long iters = 0;
    if constexpr (!STAGED) {
        for_each_tile(a.m.counter, a.m.n_tiles, a.m.tile_chunk, lane, [&](uint32_t t) {
            uint32_t x0 = 8u * (t % a.m.tiles_x), y0 = 4u * (t / a.m.tiles_x);
            render_advanced_tile<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size, a.in,
                                          a.in_pitch, a.focus, x0, y0, lane, a.m.max_ss, a.m.flags, iters);
        });
    } else {
        __shared__ float2 s_stage[PERSIST_THREADS / 32][2][STAGE_PAIRS];
        float2(*bufs)[STAGE_PAIRS] = s_stage[threadIdx.x >> 5];
        const uint32_t chunk = a.m.tile_chunk;
        auto footprint_of = [&](uint32_t t0) {
            return strip_footprint<R, A>(a.m.size, a.m.image, a.image_reused, a.m.tiles_x, t0,
                                         min(t0 + chunk, a.m.n_tiles), a.m.flags);
        };
        // claims run two strips ahead: this strip's copies are in shared memory,
        // the next strip's are in flight, the one after is being claimed
        uint32_t c0 = 0, c1 = 0, c2 = 0;
        if (lane == 0) {
            c0 = atomicAdd(a.m.counter, chunk);
            c1 = atomicAdd(a.m.counter, chunk);
        }
        uint32_t t0 = __shfl_sync(FULL, c0, 0), t1 = __shfl_sync(FULL, c1, 0);
        int cur = 0;
        Footprint f0 = t0 < a.m.n_tiles ? footprint_of(t0) : Footprint{0, 0, 0, 0, false};
        stage_footprint(bufs[cur], a.in, a.in_pitch, f0, lane);
        while (t0 < a.m.n_tiles) {
            const Footprint f1 = t1 < a.m.n_tiles ? footprint_of(t1) : Footprint{0, 0, 0, 0, false};
            stage_footprint(bufs[cur ^ 1], a.in, a.in_pitch, f1, lane);
            if (lane == 0) c2 = atomicAdd(a.m.counter, chunk);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
            __syncwarp();
            const uint32_t t_end = min(t0 + chunk, a.m.n_tiles);
            for (uint32_t t = t0; t < t_end; t++) {
                const uint32_t x0 = 8u * (t % a.m.tiles_x), y0 = 4u * (t / a.m.tiles_x);
                if (f0.ok)
                    render_advanced_tile_g<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size,
                                                    StagedGather<A>{bufs[cur], f0.x0, f0.y0, f0.cols}, a.focus, x0,
                                                    y0, lane, a.m.max_ss, a.m.flags, iters);
                else
                    render_advanced_tile<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size, a.in,
                                                  a.in_pitch, a.focus, x0, y0, lane, a.m.max_ss, a.m.flags, iters);
            }
            __syncwarp();  // every lane is done with this buffer before it is refilled
            cur ^= 1;
            t0 = t1;
            f0 = f1;
            t1 = __shfl_sync(FULL, c2, 0);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
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

template <class R, int A, int F> static cudaError_t launch_main_t(const MainArgs<R> &args, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_main<R, A, F>, PERSIST_THREADS);
    MainArgs<R> a = args;
    a.tile_chunk = tile_chunk_for(a.n_tiles, occ, sms);
    k_main<R, A, F><<<grid_for((a.n_tiles + a.tile_chunk - 1) / a.tile_chunk, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

// Large frames that reuse samples stage each strip's source footprint (when
// the previous frame's address and pitch allow 8-byte copies).
template <class R, int A, int F>
static cudaError_t launch_advanced_t(const AdvancedArgs<R> &args, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_advanced<R, A, F, false>, PERSIST_THREADS);
    static const int occ_staged = occupancy(k_advanced<R, A, F, true>, PERSIST_THREADS);
    AdvancedArgs<R> a = args;
    a.m.tile_chunk = tile_chunk_for(a.m.n_tiles, occ, sms);
    const bool staged = a.m.tile_chunk > 1 && (a.m.flags & FLAG_SAMPLE_REUSE) &&
                        (reinterpret_cast<uintptr_t>(a.in) & 7u) == 0 && (a.in_pitch & 7) == 0;
    const unsigned jobs = (a.m.n_tiles + a.m.tile_chunk - 1) / a.m.tile_chunk;
    if (staged)
        k_advanced<R, A, F, true><<<grid_for(jobs, occ_staged, sms), PERSIST_THREADS, 0, s>>>(a);
    else
        k_advanced<R, A, F, false><<<grid_for(jobs, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace chaos
