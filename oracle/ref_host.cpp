/*
 * ref_host.cpp -- host build of the reference's own per-pixel fractal code.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file with
 * -I <reference>/src/main/cuda, so the #includes below pull in the reference's
 * unmodified src/main/cuda/fractals/mandelbrot.cu and julia.cu (each inside its
 * own namespace, because both define computeFractal/colorize).  The exported
 * C functions are what the tests use to pin the CPU restatement
 * (oracle/chaos_oracle.c) and what bench.py's reference arm times.
 */
#include "ref_prelude.h"

#include <omp.h>
// The Newton modules include thrust/complex.h themselves; included here first,
// at global scope, their include is a no-op inside the namespaces below.
#include <thrust/complex.h>

namespace ref_mandelbrot {
#include "fractals/mandelbrot.cu"
}
/* helpers.cuh is guarded by HELPERS; clear the guard so each following
 * namespace gets its own copy of Point/Rectangle. */
#undef HELPERS
namespace ref_julia {
#include "fractals/julia.cu"
}
#undef HELPERS
namespace ref_newton_wired {
#include "fractals/newton_wired.cu"
}
#undef HELPERS
namespace ref_newton_generic {
#include "fractals/newton_generic.cu"
}
#undef HELPERS
namespace ref_newton_iterations {
#include "fractals/newton_iterations.cu"
}

extern "C" {

float ref_mandelbrot_f(unsigned max_iter, float cx, float cy)
{
    return ref_mandelbrot::computeFractal<float>(max_iter, ref_mandelbrot::Point<float>(cx, cy));
}

float ref_mandelbrot_d(unsigned max_iter, double cx, double cy)
{
    return ref_mandelbrot::computeFractal<double>(max_iter, ref_mandelbrot::Point<double>(cx, cy));
}

/* julia.cu reads the __constant__ double julia_c[2] that the Java host writes. */
void ref_julia_set_c(double cx, double cy)
{
    ref_julia::julia_c[0] = cx;
    ref_julia::julia_c[1] = cy;
}

float ref_julia_f(unsigned max_iter, float zx, float zy)
{
    return ref_julia::computeFractal<float>(max_iter, ref_julia::Point<float>(zx, zy));
}

float ref_julia_d(unsigned max_iter, double zx, double zy)
{
    return ref_julia::computeFractal<double>(max_iter, ref_julia::Point<double>(zx, zy));
}

unsigned ref_mandelbrot_colorize(const unsigned *palette, unsigned len, float value)
{
    return ref_mandelbrot::colorize((cudaSurfaceObject_t)(uintptr_t)palette, len, value);
}

/* Escape counts of a w x h grid of points c = (x0 + px*dx, y0 - py*dy) through
 * the reference's computeFractal<Real>, one OpenMP thread per row
 * (schedule(dynamic)), threads = n_threads (0: the OpenMP default).  The count
 * of a pixel is what computeFractal returns, except that Mandelbrot's interior
 * value 0 is counted as max_iter (the pixel-iteration metric).  Returns the sum
 * of the counts; counts may be NULL. */
unsigned long long ref_mandelbrot_grid(int dbl, unsigned w, unsigned h, double x0, double y0, double dx, double dy,
                                       unsigned max_iter, int n_threads, unsigned *counts)
{
    unsigned long long total = 0;
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic) reduction(+ : total)
    for (long y = 0; y < (long)h; y++) {
        for (unsigned x = 0; x < w; x++) {
            unsigned e;
            if (dbl) {
                double cx = x0 + (double)x * dx, cy = y0 - (double)y * dy;
                e = (unsigned)ref_mandelbrot_d(max_iter, cx, cy);
            } else {
                float cx = (float)x0 + (float)x * (float)dx, cy = (float)y0 - (float)y * (float)dy;
                e = (unsigned)ref_mandelbrot_f(max_iter, cx, cy);
            }
            if (e == 0) e = max_iter;
            if (counts) counts[(size_t)y * w + x] = e;
            total += e;
        }
    }
    return total;
}

/* Same for an explicit list of sample points (x[k], y[k]) in double. */
unsigned long long ref_mandelbrot_points_d(size_t n, const double *x, const double *y, unsigned max_iter,
                                           int n_threads, unsigned *counts)
{
    unsigned long long total = 0;
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : total)
    for (long k = 0; k < (long)n; k++) {
        unsigned e = (unsigned)ref_mandelbrot_d(max_iter, x[k], y[k]);
        if (e == 0) e = max_iter;
        if (counts) counts[k] = e;
        total += e;
    }
    return total;
}

int ref_max_threads(void) { return omp_get_max_threads(); }

/* The Newton modules' constants (roots as (re, im) x3, coefficients c0..c3,
 * colorMagnifier), as writeToConstantMemory would set them. */
void ref_newton_set(const double *roots, const double *coeffs, int magnifier)
{
    for (int k = 0; k < 3; k++) {
        ref_newton_generic::roots[k] = ref_newton_generic::Point<double>(roots[2 * k], roots[2 * k + 1]);
        ref_newton_iterations::roots[k] = ref_newton_iterations::Point<double>(roots[2 * k], roots[2 * k + 1]);
    }
    for (int k = 0; k < 4; k++) {
        ref_newton_generic::coefficients[k] = coeffs[k];
        ref_newton_iterations::coefficients[k] = coeffs[k];
    }
    ref_newton_iterations::colorMagnifier = magnifier;
}

/* kind: 2 wired, 3 generic, 4 iterations */
float ref_newton_f(int kind, unsigned max_iter, float x, float y)
{
    if (kind == 2) return ref_newton_wired::computeFractal<float>(max_iter, ref_newton_wired::Point<float>(x, y));
    if (kind == 3) return ref_newton_generic::computeFractal<float>(max_iter, ref_newton_generic::Point<float>(x, y));
    return ref_newton_iterations::computeFractal<float>(max_iter, ref_newton_iterations::Point<float>(x, y));
}

float ref_newton_d(int kind, unsigned max_iter, double x, double y)
{
    if (kind == 2) return ref_newton_wired::computeFractal<double>(max_iter, ref_newton_wired::Point<double>(x, y));
    if (kind == 3)
        return ref_newton_generic::computeFractal<double>(max_iter, ref_newton_generic::Point<double>(x, y));
    return ref_newton_iterations::computeFractal<double>(max_iter, ref_newton_iterations::Point<double>(x, y));
}

unsigned ref_newton_colorize(int kind, const unsigned *palette, unsigned len, float value)
{
    cudaSurfaceObject_t s = (cudaSurfaceObject_t)(uintptr_t)palette;
    if (kind == 2) return ref_newton_wired::colorize(s, len, value);
    if (kind == 3) return ref_newton_generic::colorize(s, len, value);
    return ref_newton_iterations::colorize(s, len, value);
}
}
