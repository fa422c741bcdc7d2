// chaos_newton.cu -- reference-mode kernels of the Newton modules.
//
// Built with --fmad=false: the thrust::complex arithmetic is then rounded
// operation by operation, like the reference module built the same way and
// like the host restatement in the oracle.
#include "chaos_newton.cuh"
#include "chaos_refmode.cuh"

namespace chaos {

template <class R, int F>
__global__ void k_under_sampled_newton(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> r, uint32_t max_iter,
                                       uint32_t level, NewtonParams p)
{
    const uint32_t ix = (blockDim.x * blockIdx.x + threadIdx.x) * level;
    const uint32_t iy = (blockDim.y * blockIdx.y + threadIdx.y) * level;
    if (ix >= w - level || iy >= h - level) return;
    float pw = __fdiv_rn(__fsub_rn(r.rtx, r.lbx), (float)w);
    float ph = __fdiv_rn(__fsub_rn(r.rty, r.lby), (float)h);
    float cx = __fadd_rn(r.lbx, __fmul_rn((float)ix, pw));
    float cy = __fsub_rn(r.rty, __fmul_rn((float)iy, ph));
    uint32_t e = newton_compute<float, F>(max_iter, cx, cy, p);
    store_pixel(pixel_ptr(out, pitch, ix, iy), make_pixel((float)e, __fdiv_rn(1.f, (float)level)));
}

template <class R> cudaError_t launch_main_newton(const MainArgs<R> &a, int fractal, int sms, cudaStream_t s)
{
    if (fractal == FRACTAL_NEWTON_WIRED) return launch_main_t<R, ARITH_PARITY, FRACTAL_NEWTON_WIRED>(a, sms, s);
    if (fractal == FRACTAL_NEWTON_GENERIC) return launch_main_t<R, ARITH_PARITY, FRACTAL_NEWTON_GENERIC>(a, sms, s);
    return launch_main_t<R, ARITH_PARITY, FRACTAL_NEWTON_ITERATIONS>(a, sms, s);
}

template <class R> cudaError_t launch_advanced_newton(const AdvancedArgs<R> &a, int fractal, int sms, cudaStream_t s)
{
    if (fractal == FRACTAL_NEWTON_WIRED) return launch_advanced_t<R, ARITH_PARITY, FRACTAL_NEWTON_WIRED>(a, sms, s);
    if (fractal == FRACTAL_NEWTON_GENERIC)
        return launch_advanced_t<R, ARITH_PARITY, FRACTAL_NEWTON_GENERIC>(a, sms, s);
    return launch_advanced_t<R, ARITH_PARITY, FRACTAL_NEWTON_ITERATIONS>(a, sms, s);
}

cudaError_t launch_under_sampled_newton(void *out, long pitch, uint32_t w, uint32_t h, Rect<float> rect,
                                        uint32_t max_iter, uint32_t level, int fractal, const NewtonParams &p,
                                        cudaStream_t s)
{
    dim3 block(32, 32);
    dim3 grid((w + 31u) / 32u, (h + 31u) / 32u);
    if (fractal == FRACTAL_NEWTON_WIRED)
        k_under_sampled_newton<float, FRACTAL_NEWTON_WIRED><<<grid, block, 0, s>>>(out, pitch, w, h, rect, max_iter,
                                                                                   level, p);
    else if (fractal == FRACTAL_NEWTON_GENERIC)
        k_under_sampled_newton<float, FRACTAL_NEWTON_GENERIC><<<grid, block, 0, s>>>(out, pitch, w, h, rect, max_iter,
                                                                                     level, p);
    else
        k_under_sampled_newton<float, FRACTAL_NEWTON_ITERATIONS><<<grid, block, 0, s>>>(out, pitch, w, h, rect,
                                                                                        max_iter, level, p);
    return cudaGetLastError();
}

template cudaError_t launch_main_newton<float>(const MainArgs<float> &, int, int, cudaStream_t);
template cudaError_t launch_main_newton<double>(const MainArgs<double> &, int, int, cudaStream_t);
template cudaError_t launch_advanced_newton<float>(const AdvancedArgs<float> &, int, int, cudaStream_t);
template cudaError_t launch_advanced_newton<double>(const AdvancedArgs<double> &, int, int, cudaStream_t);

}  // namespace chaos
