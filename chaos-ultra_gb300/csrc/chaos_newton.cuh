// chaos_newton.cuh -- the Newton-method fractals (newton wired / generic /
// colored by iterations): Newton's method on a cubic, coloured by the root a
// start point converges to, or by the iteration it converged at.
//
// Reference: src/main/cuda/fractals/newton_wired.cu:7-64,
// newton_generic.cu:11-72, newton_iterations.cu:12-67.  The complex arithmetic
// is thrust::complex, as in the reference, and the expressions keep the
// reference's operand types and order: with Real = float, a term like
// coefficients[1] * x is a double times a complex<float> and is evaluated as
// complex<double> before the assignment rounds it back, so the same
// expression forms are what reproduce the reference's results.  Built with
// --fmad=false it matches the reference built the same way; built with nvcc's
// default contraction (the default-build drop-in modules) nvcc fuses these
// expressions as it fuses the reference's own.
#pragma once

#include <thrust/complex.h>

#include "chaos_device.cuh"

namespace chaos {

// newton_wired.cu:18-41 (the roots of z^3 - 1 as literals)
__device__ __constant__ static const double kWiredRoots[6] = {1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378};

template <class R> __device__ __forceinline__ thrust::complex<R> newton_step_wired(thrust::complex<R> x)
{
    thrust::complex<R> x_pow_2 = x * x;
    thrust::complex<R> x_pow_3 = x_pow_2 * x;
    thrust::complex<R> f_eval_x = x_pow_3 - 1;
    thrust::complex<R> f_derivative_eval_x = 3 * x_pow_2;
    return x - (f_eval_x / f_derivative_eval_x);
}

// newton_generic.cu:11-25: f = c0 + c1 x + c2 x^2 + c3 x^3
template <class R>
__device__ __forceinline__ thrust::complex<R> newton_step_generic(thrust::complex<R> x, const double *coefficients)
{
    thrust::complex<R> x_pow_2 = x * x;
    thrust::complex<R> x_pow_3 = x_pow_2 * x;
    thrust::complex<R> f_eval_x =
        coefficients[0] + coefficients[1] * x + coefficients[2] * x_pow_2 + coefficients[3] * x_pow_3;
    thrust::complex<R> f_derivative_eval_x = coefficients[1] + coefficients[2] * 2 * x + coefficients[3] * 3 * x_pow_2;
    return x - (f_eval_x / f_derivative_eval_x);
}

// convergenceRoot: 1-based index of the root within 1e-4 on both axes, else 0
template <class R> __device__ __forceinline__ uint32_t newton_root(thrust::complex<R> x, const double *roots)
{
    const R tolerance = 0.0001;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const thrust::complex<R> root(roots[2 * k], roots[2 * k + 1]);
        thrust::complex<R> difference = x - root;
        if (abs(difference.real()) < tolerance && abs(difference.imag()) < tolerance) return (uint32_t)(k + 1);
    }
    return 0;
}

// computeFractal of the three modules, as an unsigned value (the float the
// reference returns is an integer): the root index (wired, generic) or the
// iteration count (iterations).
// (declared __forceinline__ in chaos_device.cuh; the attribute is not repeated here)
template <class R, int F> __device__ uint32_t newton_compute(uint32_t max_iterations, R zx, R zy, const NewtonParams &p)
{
    thrust::complex<R> x(zx, zy);
    const double *roots = F == FRACTAL_NEWTON_WIRED ? kWiredRoots : p.roots;
    uint32_t i = 0;
    if (F == FRACTAL_NEWTON_ITERATIONS) {  // newton_iterations.cu:54-67
        while (i < max_iterations) {
            x = newton_step_generic<R>(x, p.coefficients);
            ++i;
            if (newton_root<R>(x, roots) != 0) return i;
        }
        return i;
    }
    // newton_wired.cu:45-64, newton_generic.cu:53-72: test every maxIterations/10 steps after the 10th
    uint32_t check = 10;
    while (i < max_iterations) {
        x = F == FRACTAL_NEWTON_WIRED ? newton_step_wired<R>(x) : newton_step_generic<R>(x, p.coefficients);
        ++i;
        if (i == check) {
            uint32_t root = newton_root<R>(x, roots);
            if (root != 0) return root;
            check += max_iterations / 10;
        }
    }
    return newton_root<R>(x, roots);
}

}  // namespace chaos
