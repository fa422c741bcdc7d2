// chaos_refmode.cuh -- the reference-mode persistent kernels (fractalRenderMain
// and fractalRenderAdvanced semantics, gen.cu:168-181, 307-368): persistent
// warps take 8x4 pixel tiles from a work counter; one tile is one vote group
// of the adaptive super-sampling.  Included by chaos_kernels.cu (escape-time
// modules) and chaos_newton.cu (Newton modules, built without contraction).
#pragma once

#include <cmath>
#include <cstring>

#include <cuda.h>  // CUtensorMap (tensor maps are encoded through the runtime's driver entry point)

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
// lie in a small rectangle of the old frame.  Lane 0 of the warp copies that
// rectangle's (value, weight) pairs into shared memory with one TMA tile load
// (cp.async.bulk.tensor; the tensor map walks the old frame as 8-byte
// elements with a stride of two, so only the first 8 bytes of each 16-byte
// record travel) completing on an mbarrier; the filter then reads shared
// memory.  The next strip's load is issued before this strip is rendered.
// The rectangle comes from an affine bound of the warp (host-computed, one
// pixel of margin); a pixel whose neighbours still fall outside the copy
// reads global memory, so the bound only has to be good, not exact.
// ---------------------------------------------------------------------------

// Off until the tile load's shared-memory layout is pinned on the GPU.
constexpr bool kStageReuse = false;
constexpr int STAGE_COLS = 36, STAGE_ROWS = 7;           // records per copy
constexpr int STAGE_PAIRS = 256;                         // >= STAGE_COLS * STAGE_ROWS, 2 KiB per buffer
constexpr uint32_t STAGE_BYTES = STAGE_COLS * STAGE_ROWS * 8u;
constexpr uint32_t STAGE_WAIT_LIMIT = 1u << 22;          // mbarrier polls before a copy is given up

struct StageParams {
    CUtensorMap map;           // the previous frame as uint64 elements, box 2*STAGE_COLS x STAGE_ROWS, stride 2
    float ax, bx, ay, by;      // old-frame position ~ a * pixel + b
    uint32_t *error;           // optional: set to 1 when a copy did not complete in time
};

struct Footprint {
    int x0, y0;
    bool ok;
};

// The copy for tiles [t_first, t_end) of one tile row (ok = false when the
// strip wraps to the next row or the bound does not fit a copy).
__device__ __forceinline__ Footprint strip_footprint(const StageParams &sp, UInt2 size, uint32_t tiles_x,
                                                     uint32_t t_first, uint32_t t_end)
{
    Footprint fp{0, 0, false};
    if (t_end <= t_first) return fp;
    const uint32_t row = t_first / tiles_x;
    if ((t_end - 1u) / tiles_x != row) return fp;
    const float px0 = (float)(8u * (t_first % tiles_x)), px1 = (float)min(8u * ((t_end - 1u) % tiles_x) + 7u, size.x - 1u);
    const float py0 = (float)(4u * row), py1 = (float)min(4u * row + 3u, size.y - 1u);
    const float xa = __fmaf_rn(sp.ax, px0, sp.bx), xb = __fmaf_rn(sp.ax, px1, sp.bx);
    const float ya = __fmaf_rn(sp.ay, py0, sp.by), yb = __fmaf_rn(sp.ay, py1, sp.by);
    const float lim = 1.0e7f;  // also false for NaN
    if (!(fabsf(xa) < lim && fabsf(xb) < lim && fabsf(ya) < lim && fabsf(yb) < lim)) return fp;
    const int x0 = max((int)floorf(fminf(xa, xb)) - 1, 0), x1 = (int)floorf(fmaxf(xa, xb)) + 2;
    const int y0 = max((int)floorf(fminf(ya, yb)) - 1, 0), y1 = (int)floorf(fmaxf(ya, yb)) + 2;
    if (x1 - x0 + 1 > STAGE_COLS || y1 - y0 + 1 > STAGE_ROWS || x0 >= (int)size.x || y0 >= (int)size.y) return fp;
    fp = Footprint{x0, y0, true};
    return fp;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Lane 0: one TMA tile load of the footprint into buf, completing on bar.
__device__ __forceinline__ void stage_issue(const CUtensorMap *map, float2 *buf, uint64_t *bar, const Footprint &fp)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(STAGE_BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(buf)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(2 * fp.x0), "r"(fp.y0), "r"(smem_addr(bar))
        : "memory");
}

// Every lane: wait (bounded) for the copy on bar with the given phase.
__device__ __forceinline__ bool stage_wait(uint64_t *bar, uint32_t phase)
{
    for (uint32_t k = 0; k < STAGE_WAIT_LIMIT; k++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <class R, int A, int F, bool STAGED>
__global__ void __launch_bounds__(PERSIST_THREADS) k_advanced(AdvancedArgs<R> a, const __grid_constant__ StageParams sp)
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
        // two buffers per warp, then two spare ones: a copy is never larger than
        // a buffer, and the spares keep even a copy of twice that size inside
        // the block's shared memory
        __shared__ __align__(128) float2 s_stage[2 * (PERSIST_THREADS / 32) + 2][STAGE_PAIRS];
        __shared__ __align__(8) uint64_t s_bar[PERSIST_THREADS / 32][2];
        const uint32_t w = threadIdx.x >> 5;
        float2(*bufs)[STAGE_PAIRS] = &s_stage[2 * w];
        uint64_t *bars = s_bar[w];
        if (lane == 0) {
            for (int k = 0; k < 2; k++)
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[k])) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
        uint32_t phase[2] = {0u, 0u};
        bool pending[2] = {false, false};  // a copy issued into the buffer and not yet waited for
        bool staging = true;               // off for good once a copy timed out
        const uint32_t chunk = a.m.tile_chunk;
        auto footprint_of = [&](uint32_t t0) {
            return t0 < a.m.n_tiles ? strip_footprint(sp, a.m.size, a.m.tiles_x, t0, min(t0 + chunk, a.m.n_tiles))
                                    : Footprint{0, 0, false};
        };
        auto issue = [&](int b, const Footprint &fp) {
            if (staging && fp.ok) {
                if (lane == 0) stage_issue(&sp.map, bufs[b], &bars[b], fp);
                pending[b] = true;
            }
        };
        // claims run two strips ahead: this strip's copy has landed (or is
        // awaited), the next strip's is in flight, the one after is being claimed
        uint32_t c0 = 0, c1 = 0, c2 = 0;
        if (lane == 0) {
            c0 = atomicAdd(a.m.counter, chunk);
            c1 = atomicAdd(a.m.counter, chunk);
        }
        uint32_t t0 = __shfl_sync(FULL, c0, 0), t1 = __shfl_sync(FULL, c1, 0);
        int cur = 0;
        Footprint f0 = footprint_of(t0);
        issue(cur, f0);
        while (t0 < a.m.n_tiles) {
            const Footprint f1 = footprint_of(t1);
            issue(cur ^ 1, f1);
            if (lane == 0) c2 = atomicAdd(a.m.counter, chunk);
            bool have = false;
            if (pending[cur]) {
                have = stage_wait(&bars[cur], phase[cur]);
                pending[cur] = !have;  // a copy that timed out is still outstanding
                if (have) {
                    phase[cur] ^= 1u;
                } else if (staging) {
                    staging = false;
                    if (sp.error && lane == 0) atomicExch(sp.error, 1u);
                }
            }
            const uint32_t t_end = min(t0 + chunk, a.m.n_tiles);
            for (uint32_t t = t0; t < t_end; t++) {
                const uint32_t x0 = 8u * (t % a.m.tiles_x), y0 = 4u * (t / a.m.tiles_x);
                if (have && staging)
                    render_advanced_tile_g<R, A, F>(
                        g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size,
                        StagedGather<A>{bufs[cur], f0.x0, f0.y0, STAGE_COLS, STAGE_ROWS, a.in, a.in_pitch}, a.focus,
                        x0, y0, lane, a.m.max_ss, a.m.flags, iters);
                else
                    render_advanced_tile<R, A, F>(g, a.m.image, a.image_reused, a.m.out, a.m.pitch, a.m.size, a.in,
                                                  a.in_pitch, a.focus, x0, y0, lane, a.m.max_ss, a.m.flags, iters);
            }
            __syncwarp();  // every lane is done with this buffer before a copy refills it
            cur ^= 1;
            t0 = t1;
            f0 = f1;
            t1 = __shfl_sync(FULL, c2, 0);
        }
        // copies still outstanding (only after a time-out): wait for them, bounded, before leaving
        for (int k = 0; k < 2; k++)
            if (pending[k]) stage_wait(&bars[k], phase[k]);
    }
    add_total(a.m.total, iters, lane);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda).
using TensorMapEncoder = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                      const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                      CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static inline TensorMapEncoder tensor_map_encoder()
{
    static const TensorMapEncoder fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<TensorMapEncoder>(p);
    }();
    return fn;
}

// Staging parameters of a reuse frame: the tensor map of the previous frame
// and the affine bound of the warp, from the plane rectangles (binary64).
template <class R>
static bool stage_params(const AdvancedArgs<R> &a, StageParams &sp)
{
    TensorMapEncoder enc = tensor_map_encoder();
    if (!enc) return false;
    const double w = a.m.size.x, h = a.m.size.y;
    const double cw = (double)a.m.image.rtx - (double)a.m.image.lbx, ch = (double)a.m.image.rty - (double)a.m.image.lby;
    const double ow = (double)a.image_reused.rtx - (double)a.image_reused.lbx;
    const double oh = (double)a.image_reused.rty - (double)a.image_reused.lby;
    if (!(ow != 0.0 && oh != 0.0 && std::isfinite(cw / ow) && std::isfinite(ch / oh))) return false;
    sp.ax = (float)(cw / ow);
    sp.bx = (float)(((double)a.m.image.lbx - (double)a.image_reused.lbx) / ow * w);
    sp.ay = (float)(ch / oh);
    sp.by = (float)(h * (1.0 - ch / oh) - ((double)a.m.image.lby - (double)a.image_reused.lby) / oh * h);
    sp.error = nullptr;
    const cuuint64_t dims[2] = {2ull * a.m.size.x, (cuuint64_t)a.m.size.y};
    const cuuint64_t strides[1] = {(cuuint64_t)a.in_pitch};
    const cuuint32_t box[2] = {2u * STAGE_COLS, (cuuint32_t)STAGE_ROWS};
    const cuuint32_t elem[2] = {2u, 1u};
    return enc(&sp.map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void *>(a.in), dims, strides, box, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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
// the previous frame's address and pitch are multiples of 16 bytes, as a
// tensor map needs).
template <class R, int A, int F>
static cudaError_t launch_advanced_t(const AdvancedArgs<R> &args, int sms, cudaStream_t s)
{
    static const int occ = occupancy(k_advanced<R, A, F, false>, PERSIST_THREADS);
    static const int occ_staged = occupancy(k_advanced<R, A, F, true>, PERSIST_THREADS);
    AdvancedArgs<R> a = args;
    a.m.tile_chunk = tile_chunk_for(a.m.n_tiles, occ, sms);
    StageParams sp;
    std::memset(&sp, 0, sizeof sp);
    const bool staged = kStageReuse && a.m.tile_chunk > 1 && (a.m.flags & FLAG_SAMPLE_REUSE) &&
                        (reinterpret_cast<uintptr_t>(a.in) & 15u) == 0 && (a.in_pitch & 15) == 0 &&
                        stage_params(a, sp);
    const unsigned jobs = (a.m.n_tiles + a.m.tile_chunk - 1) / a.m.tile_chunk;
    if (staged)
        k_advanced<R, A, F, true><<<grid_for(jobs, occ_staged, sms), PERSIST_THREADS, 0, s>>>(a, sp);
    else
        k_advanced<R, A, F, false><<<grid_for(jobs, occ, sms), PERSIST_THREADS, 0, s>>>(a, sp);
    return cudaGetLastError();
}

}  // namespace chaos
