/*
 * ref_prelude.h -- lets the reference's own device source compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY (oracle side).  Included ahead of the reference's
 * src/main/cuda/fractals/<fractal>.cu when oracle/build_ref.sh builds
 * oracle/_ref/libchaos_ref.so.  It maps the CUDA qualifiers to nothing, gives
 * helpers.cuh the CUDART_VERSION it checks, and stands a plain host array in for
 * the palette surface read by colorize().
 */
#pragma once
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>

#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#ifndef CUDART_VERSION
#define CUDART_VERSION 13000
#endif

typedef unsigned long long cudaSurfaceObject_t;

/* surf2Dread on a one-row palette: the "surface object" is the address of a
 * host uint32 array and x is a byte offset, as in colorize(). */
template <class T>
inline void surf2Dread(T *out, cudaSurfaceObject_t surf, int x, int /*y*/)
{
    *out = *reinterpret_cast<const T *>(reinterpret_cast<const char *>(surf) + x);
}

using std::abs;
using std::round;
using std::sqrt;
