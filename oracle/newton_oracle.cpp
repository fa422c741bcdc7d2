/*
 * newton_oracle.cpp -- the Newton modules' computeFractal on the host.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle library).  Restates
 * src/main/cuda/fractals/newton_wired.cu:7-64, newton_generic.cu:11-72 and
 * newton_iterations.cu:12-67 with thrust::complex on the host (the same
 * library the reference uses), expressions in the reference's operand types
 * and order.  Built with -ffp-contract=off.
 */
#include <cstdint>
#include <thrust/complex.h>

namespace {

template <class R> thrust::complex<R> step_wired(thrust::complex<R> x)
{
    thrust::complex<R> x_pow_2 = x * x;
    thrust::complex<R> x_pow_3 = x_pow_2 * x;
    thrust::complex<R> f_eval_x = x_pow_3 - 1;
    thrust::complex<R> f_derivative_eval_x = 3 * x_pow_2;
    return x - (f_eval_x / f_derivative_eval_x);
}

template <class R> thrust::complex<R> step_generic(thrust::complex<R> x, const double *coefficients)
{
    thrust::complex<R> x_pow_2 = x * x;
    thrust::complex<R> x_pow_3 = x_pow_2 * x;
    thrust::complex<R> f_eval_x =
        coefficients[0] + coefficients[1] * x + coefficients[2] * x_pow_2 + coefficients[3] * x_pow_3;
    thrust::complex<R> f_derivative_eval_x = coefficients[1] + coefficients[2] * 2 * x + coefficients[3] * 3 * x_pow_2;
    return x - (f_eval_x / f_derivative_eval_x);
}

template <class R> uint32_t root_of(thrust::complex<R> x, const double *roots)
{
    const R tolerance = 0.0001;
    for (int k = 0; k < 3; k++) {
        const thrust::complex<R> root(roots[2 * k], roots[2 * k + 1]);
        thrust::complex<R> d = x - root;
        if ((d.real() < 0 ? -d.real() : d.real()) < tolerance && (d.imag() < 0 ? -d.imag() : d.imag()) < tolerance)
            return (uint32_t)(k + 1);
    }
    return 0;
}

const double kWired[6] = {1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378};

/* fractal: 2 wired, 3 generic, 4 iterations (the library's numbering) */
template <class R> float compute(int fractal, uint32_t max_iter, R zx, R zy, const double *roots, const double *coeffs)
{
    thrust::complex<R> x(zx, zy);
    uint32_t i = 0;
    if (fractal == 4) {
        while (i < max_iter) {
            x = step_generic<R>(x, coeffs);
            ++i;
            if (root_of<R>(x, roots) != 0) return (float)i;
        }
        return (float)i;
    }
    const double *rr = fractal == 2 ? kWired : roots;
    uint32_t check = 10;
    while (i < max_iter) {
        x = fractal == 2 ? step_wired<R>(x) : step_generic<R>(x, coeffs);
        ++i;
        if (i == check) {
            uint32_t r = root_of<R>(x, rr);
            if (r != 0) return (float)r;
            check += max_iter / 10;
        }
    }
    return (float)root_of<R>(x, rr);
}

}  // namespace

extern "C" float orc_newton_compute_f(int fractal, uint32_t max_iter, float x, float y, const double *roots,
                                      const double *coeffs)
{
    return compute<float>(fractal, max_iter, x, y, roots, coeffs);
}

extern "C" float orc_newton_compute_d(int fractal, uint32_t max_iter, double x, double y, const double *roots,
                                      const double *coeffs)
{
    return compute<double>(fractal, max_iter, x, y, roots, coeffs);
}
