// chaos_kernels.cu -- library kernels of the escape-time path (sm_103a).
//
//   k_main / k_advanced   reference-mode frames (fractalRenderMain/Advanced,
//                         gen.cu:168-181, 307-368): persistent warps take 8x4
//                         tiles from a work counter, one tile = one vote group
//   k_frame               independent samples (pixel centres or jittered):
//                         persistent warps with per-lane refill, so a lane whose
//                         sample escaped takes the next one without waiting for
//                         the slowest lane of its warp; binary32 samples run
//                         tested blocks (each step with its own test), binary64
//                         ones untested blocks with an in-warp search of an
//                         overshot block
//   k_compose             palette compose (gen.cu:455-475), HBM-bound
//   k_under_sampled       fractalRenderUnderSampled (gen.cu:478-503)
#include <cstdio>

#include "chaos_frame.cuh"
#include "chaos_kernels.cuh"
#include "chaos_refmode.cuh"

namespace chaos {

constexpr uint32_t PALETTE_SMEM = 4096;

// ---------------------------------------------------------------------------
// Independent-sample frames with per-lane refill
// ---------------------------------------------------------------------------

template <class R>
__device__ __forceinline__ void frame_point(const FrameArgs<R> &a, uint32_t w_magic, uint32_t pix, uint32_t s, R &cx,
                                            R &cy)
{
    using O = Op<R>;
    uint32_t px, py;
    divmod_magic(pix, a.w, w_magic, py, px);
    R ox = R(0.5), oy = R(0.5);
    if (a.mode == SAMPLES_JITTER) {
        ox = unit_interval_t<R>(sample_hash(a.seed, pix, s, 0));
        oy = unit_interval_t<R>(sample_hash(a.seed, pix, s, 1));
    }
    R dxp = O::sub(O::add((R)px, ox), a.half_w);
    R dyp = O::sub(O::add((R)py, oy), a.half_h);
    cx = O::fma(dxp, a.ps, a.center_x);
    cy = O::fma(-dyp, a.ps, a.center_y);
}

template <class R, int A, int F, int K> __global__ void __launch_bounds__(PERSIST_THREADS) k_frame(FrameArgs<R> a)
{
    static_assert(sizeof(R) == 4 ? K % CYCLE_SPAN == 0 : K == ESCAPE_BLOCK, "cycle checkpoints at block ends");
    __shared__ uint32_t s_pal[PALETTE_SMEM];
    const uint32_t *pal = a.palette;
    if (a.rgba && a.palette_len <= PALETTE_SMEM) {
        for (uint32_t k = threadIdx.x; k < a.palette_len; k += blockDim.x) s_pal[k] = a.palette[k];
        pal = s_pal;
    }
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t w_magic = div_magic(a.w);
    uint32_t pix = 0xffffffffu, s = 0, i = 0;
    R x = R(0), y = R(0), cx = R(0), cy = R(0);
    bool blk = false, need = true, begin = false;
    uint32_t window = 0;  // > 0: the escape lies within the next `window` steps
    float acc_v = 0.f, acc[4] = {0.f, 0.f, 0.f, 0.f};
    unsigned long long iters = 0, skipped = 0;
    CycleWatch<R> cw;  // exact cycle detection (see CycleWatch)
    const unsigned long long t_start = a.budget_ns ? global_ns() : 0ull;

    // the grid's first pixels go out without a claim (warp w takes 32w..32w+31),
    // so the launch does not start with every warp's atomic on one counter;
    // claims then count from there
    const uint32_t n_warps = gridDim.x * (blockDim.x >> 5);
    bool first = true;

    for (;;) {
        // a time limit: the warp stops where it is (its samples in flight stay unwritten)
        if (out_of_time(a.budget_ns, t_start, a.status, lane)) break;
        uint32_t need_mask = __ballot_sync(FULL, need);
        if (need_mask) {
            uint32_t base = 0;
            if (first) {
                base = 32u * (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
                first = false;
            } else {
                const uint32_t leader = __ffs(need_mask) - 1u;
                if (lane == leader) base = 32u * n_warps + atomicAdd(a.counter, (uint32_t)__popc(need_mask));
                base = __shfl_sync(FULL, base, leader);
            }
            if (need) {
                pix = base + (uint32_t)__popc(need_mask & lt_mask);
                need = false;
                begin = true;
                s = 0;
                acc_v = 0.f;
                acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
            }
        }
        const bool active = pix < a.n_pix;
        if (!__any_sync(FULL, active)) break;

        bool done = false;
        R r2 = R(0);
        uint32_t lim = 0;  // steps this lane takes this round: a power of two <= K
        if (active) {
            if (begin) {
                begin = false;
                R px, py;
                frame_point(a, w_magic, pix, s, px, py);
                i = 0;
                if (F == FRACTAL_MANDELBROT) {
                    cx = px;
                    cy = py;
                    // the first step from z = 0 gives z = c (+0 in place of -0, as the
                    // step's own additions do); starting there spares every sample a
                    // step whose products are 0
                    x = R(0);
                    y = R(0);
                    if (a.max_iter > 0) {
                        x = Op<R>::add(cx, R(0));
                        y = Op<R>::add(cy, R(0));
                        i = 1;
                    }
                } else {
                    x = px;
                    y = py;
                    cx = a.jcx;
                    cy = a.jcy;
                }
                blk = blockable_c(cx, cy);
                window = 0;
                cw.reset(x, y);
                r2 = radius2<R, A>(x, y);
                if (i == a.max_iter || !(r2 < R(4))) done = true;
            }
            if (!done && sizeof(R) == 8) {
                if (!blk) {
                    lim = 1;
                } else if (window) {
                    lim = window > 1u ? window >> 1 : 1u;
                } else {
                    uint32_t rest = a.max_iter - i;
                    lim = rest >= (uint32_t)K ? (uint32_t)K : 1u << (31 - __clz(rest));
                }
            }
        }
        // Every stepping lane runs the same K unrolled steps.  A lane with
        // lim < K keeps the state it had after lim steps (captured after steps
        // 1, 2, 4, ...): that is how a lane whose block overshot an escape
        // halves its search window each round without holding up the others.
        const bool stepping = active && !done;
        const bool partial = stepping && lim < (uint32_t)K;
        const bool any_partial = sizeof(R) == 8 && __any_sync(FULL, partial);
        // K steps of `stepper`, keeping the state after lim steps on partial lanes
        auto run_block = [&](auto stepper) {
            if (any_partial) {
                R kx = x, ky = y;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    stepper(x, y);
                    if (((k + 1) & k) == 0 && k + 1 < K && (uint32_t)(k + 1) == lim) {
                        kx = x;
                        ky = y;
                    }
                }
                if (partial) {
                    x = kx;
                    y = ky;
                }
            } else {
#pragma unroll
                for (int k = 0; k < K; k++) stepper(x, y);
            }
        };
        if constexpr (sizeof(R) == 4) {
            // binary32: tested steps (see tested_block)
            if (stepping) {
                const uint32_t rest = a.max_iter - i;
                bool esc = false, cyc = false;
                const uint32_t n = rest >= (uint32_t)K
                                       ? tested_block<R, A, K, false>(x, y, cx, cy, K, r2, esc, &cw, &cyc)
                                       : tested_block<R, A, K, true>(x, y, cx, cy, rest, r2, esc);
                i += n;
                if (cyc) {  // a repeated state: interior
                    skipped += a.max_iter - i;
                    i = a.max_iter;
                }
                if (esc || i == a.max_iter) done = true;
            }
        } else if (stepping) {
            const R sx = x, sy = y;
            if constexpr (A == ARITH_PARITY && sizeof(R) == 8) {
                // binary64: one binary64 operation fewer per step for two integer ones
                // (binary32 keeps the literal step: there the integer pipe is the busier one)
                uint32_t emin = 0xffffffffu;
                run_block([&](R &u, R &v) { step_rounded6<R>(u, v, cx, cy, emin); });
                if (emin < exponent_bits_two<R>()) {
                    // a product below twice the smallest normal: redo the block literally
                    x = sx;
                    y = sy;
                    run_block([&](R &u, R &v) { step<R, A>(u, v, cx, cy); });
                }
            } else if constexpr (sizeof(R) == 8) {
                uint32_t emin = 0xffffffffu;
                run_block([&](R &u, R &v) { step_fma3(u, v, cx, cy, emin); });
                if (emin == 0u) {
                    // x = 0 or subnormal: redo the block with x + x
                    x = sx;
                    y = sy;
                    run_block([&](R &u, R &v) { step<R, A>(u, v, cx, cy); });
                }
            } else {
                run_block([&](R &u, R &v) { step<R, A>(u, v, cx, cy); });
            }
            r2 = radius2<R, A>(x, y);
            if (r2 < R(4)) {
                const bool full = window == 0u && lim == (uint32_t)K;  // a checkpoint every K steps
                i += lim;
                window = window > 1u ? window - lim : 0u;
                if (full && cw.template check_every<cycle_blocks<R>()>(x, y)) {  // a repeated state: interior
                    skipped += a.max_iter - i;
                    i = a.max_iter;
                }
                if (i == a.max_iter) done = true;
            } else if (lim == 1u) {
                i += 1u;  // the escape step
                done = true;
            } else {
                // the escape lies within these lim steps: search them
                x = sx;
                y = sy;
                window = lim;
            }
        }
        if (done) {
            const bool escaped = i < a.max_iter;
            const float nu = (a.smooth || a.pixels || a.rgba) ? frame_smooth(i, (float)r2, a.max_iter) : 0.f;
            const size_t sidx = (size_t)pix * a.spp + s;
            if (a.counts) a.counts[sidx] = i;
            if (a.smooth) a.smooth[sidx] = nu;
            iters += i;
            float v = escaped ? nu : (F == FRACTAL_MANDELBROT ? 0.f : (float)a.max_iter);
            acc_v = __fadd_rn(acc_v, v);
            if (a.rgba) {
                float ch[4];
                if (escaped) {
                    frame_palette_lerp(pal, a.palette_len, nu, ch);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) ch[k] = (float)((a.interior_rgba >> (8 * k)) & 255u);
                }
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = __fadd_rn(acc[k], ch[k]);
            }
            ++s;
            if (s == a.spp) {
                uint32_t px, py;
                divmod_magic(pix, a.w, w_magic, py, px);
                if (a.pixels)
                    store_pixel(pixel_ptr(a.pixels, a.pixels_pitch, px, py),
                                make_pixel(__fdiv_rn(acc_v, (float)a.spp), (float)a.spp));
                if (a.rgba) a.rgba[pix] = frame_pack_rgba(acc, a.spp);
                need = true;
            } else {
                begin = true;
            }
        }
    }
    if (a.total) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) iters += __shfl_down_sync(FULL, iters, o);
        if (lane == 0 && iters) atomicAdd(a.total, iters);
    }
    if (a.skipped) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) skipped += __shfl_down_sync(FULL, skipped, o);
        if (lane == 0 && skipped) atomicAdd(a.skipped, skipped);
    }
}

// ---------------------------------------------------------------------------
// Compose, under-sampled preview, debug
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_compose(ComposeArgs a)
{
    __shared__ uint32_t s_pal[PALETTE_SMEM];
    const uint32_t *pal = a.palette;
    if (!a.visualize && a.palette && a.palette_len <= PALETTE_SMEM) {
        for (uint32_t k = threadIdx.x; k < a.palette_len; k += blockDim.x) s_pal[k] = a.palette[k];
        pal = s_pal;
    }
    __syncthreads();
    // A warp takes a run of 128 pixels of one row; lane l handles pixels
    // x0 + 32k + l (k = 0..3), so every load instruction reads 32 consecutive
    // 16-byte records (512 B) and every store writes 32 consecutive words.  The
    // four records are loaded before any is composed, four loads in flight
    // (eight measured the same and cost 57 registers instead of 32).
    constexpr int R = 4;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t runs = (a.w + 32u * R - 1u) / (32u * R);
    const size_t n = (size_t)runs * a.h;
    const size_t warps = (size_t)gridDim.x * (blockDim.x / 32u);
    for (size_t c = (size_t)blockIdx.x * (blockDim.x / 32u) + (threadIdx.x >> 5); c < n; c += warps) {
        const uint32_t y = (uint32_t)(c / runs), x0 = 32u * R * (uint32_t)(c % runs);
        PixelInfo p[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            const uint32_t x = x0 + 32u * k + lane;
            if (x < a.w) p[k] = load_pixel(pixel_ptr(a.in, a.pitch, x, y));
        }
        uint32_t *row = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(a.out) + (size_t)y * (size_t)a.out_pitch);
#pragma unroll
        for (int k = 0; k < R; k++) {
            const uint32_t x = x0 + 32u * k + lane;
            if (x < a.w)
                row[x] = compose_pixel(p[k], pal, a.palette_len, a.max_ss, a.visualize, a.color_mode, a.magnifier);
        }
    }
}

template <int F>
__global__ void k_under_sampled(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> r, uint32_t max_iter,
                                uint32_t level, float jcx, float jcy)
{
    const uint32_t ix = (blockDim.x * blockIdx.x + threadIdx.x) * level;
    const uint32_t iy = (blockDim.y * blockIdx.y + threadIdx.y) * level;
    if (ix >= w - level || iy >= h - level) return;
    float pw = __fdiv_rn(__fsub_rn(r.rtx, r.lbx), (float)w);
    float ph = __fdiv_rn(__fsub_rn(r.rty, r.lby), (float)h);
    float cx = __fadd_rn(r.lbx, __fmul_rn((float)ix, pw));
    float cy = __fsub_rn(r.rty, __fmul_rn((float)iy, ph));
    uint32_t e = compute_fractal<float, ARITH_PARITY, F>(max_iter, cx, cy, jcx, jcy);
    store_pixel(pixel_ptr(out, pitch, ix, iy), make_pixel((float)e, __fdiv_rn(1.f, (float)level)));
}

template <int F> __global__ void k_debug()
{
    if (blockIdx.x == 0 && threadIdx.x == 0) printf("hello from %s\n", F == FRACTAL_MANDELBROT ? "mandelbrot" : "julia");
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------


template <class R>
cudaError_t launch_main(const MainArgs<R> &a, int arith, int fractal, int sms, cudaStream_t s)
{
    if (fractal >= FRACTAL_NEWTON_WIRED) return launch_main_newton<R>(a, fractal, sms, s);
    if (arith == ARITH_PARITY)
        return fractal == FRACTAL_JULIA ? launch_main_t<R, ARITH_PARITY, FRACTAL_JULIA>(a, sms, s)
                                        : launch_main_t<R, ARITH_PARITY, FRACTAL_MANDELBROT>(a, sms, s);
    if (arith == ARITH_CONTRACTED)
        return fractal == FRACTAL_JULIA ? launch_main_t<R, ARITH_CONTRACTED, FRACTAL_JULIA>(a, sms, s)
                                        : launch_main_t<R, ARITH_CONTRACTED, FRACTAL_MANDELBROT>(a, sms, s);
    return fractal == FRACTAL_JULIA ? launch_main_t<R, ARITH_FMA, FRACTAL_JULIA>(a, sms, s)
                                    : launch_main_t<R, ARITH_FMA, FRACTAL_MANDELBROT>(a, sms, s);
}


template <class R>
cudaError_t launch_advanced(const AdvancedArgs<R> &a, int arith, int fractal, int sms, cudaStream_t s)
{
    if (fractal >= FRACTAL_NEWTON_WIRED) return launch_advanced_newton<R>(a, fractal, sms, s);
    if (arith == ARITH_PARITY)
        return fractal == FRACTAL_JULIA ? launch_advanced_t<R, ARITH_PARITY, FRACTAL_JULIA>(a, sms, s)
                                        : launch_advanced_t<R, ARITH_PARITY, FRACTAL_MANDELBROT>(a, sms, s);
    if (arith == ARITH_CONTRACTED)
        return fractal == FRACTAL_JULIA ? launch_advanced_t<R, ARITH_CONTRACTED, FRACTAL_JULIA>(a, sms, s)
                                        : launch_advanced_t<R, ARITH_CONTRACTED, FRACTAL_MANDELBROT>(a, sms, s);
    return fractal == FRACTAL_JULIA ? launch_advanced_t<R, ARITH_FMA, FRACTAL_JULIA>(a, sms, s)
                                    : launch_advanced_t<R, ARITH_FMA, FRACTAL_MANDELBROT>(a, sms, s);
}

// Block length per arithmetic width: binary32 frames run tested blocks of 64
// steps (on the 1024x1024 frame with a mean escape of 173 iterations, 16, 32,
// 64 and 128 steps gave 1499, 1669, 1746 and 1620 Gpixel-iter/s); binary64
// runs untested blocks of 16.
template <class R> constexpr int frame_block() { return sizeof(R) == 4 ? 64 : ESCAPE_BLOCK; }

template <class R, int A, int F> static cudaError_t launch_frame_t(const FrameArgs<R> &a, int sms, cudaStream_t s)
{
    constexpr int K = frame_block<R>();
    static const int occ = occupancy(k_frame<R, A, F, K>, PERSIST_THREADS);
    unsigned long long warps = ((unsigned long long)a.n_pix + 31ull) / 32ull;
    k_frame<R, A, F, K><<<grid_for(warps, occ, sms), PERSIST_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_frame(const FrameArgs<R> &a, int arith, int fractal, int sms, cudaStream_t s)
{
    if (arith == ARITH_PARITY)
        return fractal == FRACTAL_JULIA ? launch_frame_t<R, ARITH_PARITY, FRACTAL_JULIA>(a, sms, s)
                                        : launch_frame_t<R, ARITH_PARITY, FRACTAL_MANDELBROT>(a, sms, s);
    return fractal == FRACTAL_JULIA ? launch_frame_t<R, ARITH_FMA, FRACTAL_JULIA>(a, sms, s)
                                    : launch_frame_t<R, ARITH_FMA, FRACTAL_MANDELBROT>(a, sms, s);
}

cudaError_t launch_compose(const ComposeArgs &a, cudaStream_t s)
{
    unsigned long long runs = (unsigned long long)((a.w + 127u) / 128u) * a.h;  // one warp each
    unsigned long long blocks = (runs + 7ull) / 8ull;
    if (blocks > 152ull * 16ull) blocks = 152ull * 16ull;
    if (blocks < 1) blocks = 1;
    k_compose<<<(unsigned)blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_under_sampled(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> rect, uint32_t max_iter,
                                 uint32_t level, int fractal, double jcx, double jcy, cudaStream_t s)
{
    dim3 block(32, 32);
    dim3 grid((w + 31u) / 32u, (h + 31u) / 32u);
    if (fractal == FRACTAL_JULIA)
        k_under_sampled<FRACTAL_JULIA><<<grid, block, 0, s>>>(out, pitch, w, h, rect, max_iter, level, (float)jcx,
                                                              (float)jcy);
    else
        k_under_sampled<FRACTAL_MANDELBROT><<<grid, block, 0, s>>>(out, pitch, w, h, rect, max_iter, level, 0.f, 0.f);
    return cudaGetLastError();
}

cudaError_t launch_debug(int fractal, cudaStream_t s)
{
    if (fractal >= FRACTAL_NEWTON_WIRED) return cudaSuccess;  // the Newton modules' debugFractal is empty
    if (fractal == FRACTAL_JULIA)
        k_debug<FRACTAL_JULIA><<<1, 1, 0, s>>>();
    else
        k_debug<FRACTAL_MANDELBROT><<<1, 1, 0, s>>>();
    return cudaGetLastError();
}

template <class R> __global__ void __launch_bounds__(256) k_fma_peak(uint32_t iters, double *sink)
{
    R a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = R(threadIdx.x + k) * R(1e-3);
    const R m = R(0.999999), c = R(1e-7);
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = Op<R>::fma(a[k], m, c);
    }
    R t = R(0);
#pragma unroll
    for (int k = 0; k < 8; k++) t += a[k];
    if (t == R(-1)) sink[0] = (double)t;  // never true; keeps the chains live
}

cudaError_t launch_fma_peak(bool dbl, int blocks, uint32_t iters, double *sink, cudaStream_t s)
{
    if (dbl)
        k_fma_peak<double><<<blocks, 256, 0, s>>>(iters, sink);
    else
        k_fma_peak<float><<<blocks, 256, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

template cudaError_t launch_main<float>(const MainArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_main<double>(const MainArgs<double> &, int, int, int, cudaStream_t);
template cudaError_t launch_advanced<float>(const AdvancedArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_advanced<double>(const AdvancedArgs<double> &, int, int, int, cudaStream_t);
template cudaError_t launch_frame<float>(const FrameArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_frame<double>(const FrameArgs<double> &, int, int, int, cudaStream_t);

}  // namespace chaos
