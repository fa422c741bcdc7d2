"""ctypes access to the oracle (test infrastructure only).

`Oracle` wraps oracle/_build/libchaos_oracle.so, the CPU restatement of the
reference's fractal-kernel path (oracle/chaos_oracle.c).  `Reference` wraps
oracle/_ref/libchaos_ref.so, the reference's own computeFractal/colorize built
for the host by oracle/build_ref.sh.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs use this module, as the oracle.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libchaos_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libchaos_ref.so")

MANDELBROT, JULIA = 0, 1
ARITH_FMA, ARITH_PARITY, ARITH_CONTRACTED = 0, 1, 2  # same numbering as CHAOS_ARITH_* in include/chaos_gb300.h
ARITH_FLOATFLOAT = 3  # reference-mode binary64 frames with the float-float escape loop (served frames)

PIXEL_DTYPE = np.dtype([("value", "<f4"), ("weight", "<f4"), ("is_reused", "u1"), ("pad", "u1", 3),
                        ("weight_of_new_samples", "<f4")])
assert PIXEL_DTYPE.itemsize == 16

class FrameDesc(C.Structure):
    """orc_frame_desc (oracle/chaos_oracle.c)."""
    _fields_ = [("w", C.c_uint32), ("h", C.c_uint32), ("max_iter", C.c_uint32), ("spp", C.c_uint32),
                ("mode", C.c_uint32), ("dbl", C.c_uint32), ("arith", C.c_uint32), ("fractal", C.c_uint32),
                ("seed", C.c_uint64), ("center_x", C.c_double), ("center_y", C.c_double),
                ("pixel_size", C.c_double), ("jcx", C.c_double), ("jcy", C.c_double)]


class Viewport(C.Structure):
    """orc_viewport (oracle/chaos_oracle.c); tier 0 binary32, 1 binary64, 2 float-float."""
    _fields_ = [("w", C.c_uint32), ("h", C.c_uint32), ("spp", C.c_uint32), ("mode", C.c_uint32),
                ("max_iter", C.c_uint32), ("tier", C.c_uint32), ("seed", C.c_uint64), ("cx", C.c_double),
                ("cy", C.c_double), ("ps", C.c_double)]


_d4 = C.c_double * 4
_d2 = C.c_double * 2


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    def __init__(self, path=ORACLE_LIB):
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_compute_fractal_f.restype = C.c_float
        L.orc_compute_fractal_f.argtypes = [C.c_int, C.c_int, C.c_uint32, C.c_float, C.c_float, C.c_double,
                                            C.c_double]
        L.orc_compute_fractal_d.restype = C.c_float
        L.orc_compute_fractal_d.argtypes = [C.c_int, C.c_int, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                            C.c_double]
        L.orc_render_main.restype = None
        L.orc_render_main.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_uint32, C.c_uint32,
                                      _d4, C.c_uint32, C.c_float, C.c_uint32, C.c_void_p]
        L.orc_render_advanced.restype = None
        L.orc_render_advanced.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_uint32, C.c_uint32,
                                          _d4, C.c_uint32, C.c_float, C.c_uint32, _d4, C.c_void_p, C.c_long,
                                          C.c_uint32, C.c_uint32, C.c_void_p]
        L.orc_compose.restype = None
        L.orc_compose.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_long, C.c_uint32, C.c_uint32, C.c_void_p,
                                  C.c_uint32, C.c_float, C.c_int]
        L.orc_render_under_sampled.restype = None
        L.orc_render_under_sampled.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_uint32, C.c_uint32, _d4,
                                               C.c_uint32, C.c_uint32, C.c_void_p]
        L.orc_escape_grid.restype = C.c_uint64
        L.orc_escape_grid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_uint32, C.c_void_p, C.c_void_p]

        L.orc_frame.restype = C.c_uint64
        L.orc_frame.argtypes = [C.POINTER(FrameDesc), C.c_long, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]
        L.orc_frame_points_d.restype = None
        L.orc_frame_points_d.argtypes = [C.POINTER(FrameDesc), C.c_long, C.c_long, C.c_void_p, C.c_void_p]
        L.orc_mandelbrot_points_d.restype = C.c_uint64
        L.orc_mandelbrot_points_d.argtypes = [C.c_long, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]
        L.orc_max_threads.restype = C.c_int
        L.orc_hp_escape.restype = C.c_uint32
        L.orc_hp_escape.argtypes = [C.c_char_p, C.c_char_p, C.c_double, C.c_double, C.c_uint32, C.c_uint32,
                                    C.POINTER(C.c_double)]
        L.orc_hp_escape_batch.restype = None
        L.orc_hp_escape_batch.argtypes = [C.c_char_p, C.c_char_p, C.c_long, C.c_void_p, C.c_void_p, C.c_uint32,
                                          C.c_uint32, C.c_void_p, C.c_void_p]
        L.orc_set_newton.restype = None
        L.orc_set_newton.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.orc_compose_mode.restype = None
        L.orc_compose_mode.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_long, C.c_uint32, C.c_uint32,
                                       C.c_void_p, C.c_uint32, C.c_int, C.c_int]
        L.orc_batch_viewport.restype = C.c_uint64
        L.orc_batch_viewport.argtypes = [C.POINTER(Viewport), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_uint32, C.c_uint32]
        L.orc_frame_offsets.restype = None
        L.orc_frame_offsets.argtypes = [C.POINTER(FrameDesc), C.c_long, C.c_long, C.c_void_p, C.c_void_p]
        L.orc_sample_hash.restype = C.c_uint64
        L.orc_sample_hash.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]

    # -- computeFractal -------------------------------------------------------
    def compute_fractal(self, fractal, dbl, arith, max_iter, x, y, julia_c=(0.0, 0.0)):
        f = self.lib.orc_compute_fractal_d if dbl else self.lib.orc_compute_fractal_f
        return f(fractal, arith, max_iter, x, y, julia_c[0], julia_c[1])

    # -- kernels ----------------------------------------------------------------
    @staticmethod
    def _julia(julia_c):
        return _d2(*julia_c) if julia_c is not None else None

    def render_main(self, fractal, dbl, arith, w, h, rect, max_iter, max_ss, flags, julia_c=None):
        out = np.zeros((h, w), dtype=PIXEL_DTYPE)
        self.lib.orc_render_main(fractal, int(dbl), arith, _ptr(out), w * 16, w, h, _d4(*rect), max_iter, max_ss,
                                 flags, C.cast(self._julia(julia_c), C.c_void_p) if julia_c else None)
        return out

    def render_advanced(self, fractal, dbl, arith, w, h, rect, max_iter, max_ss, flags, rect_reused, inp, focus,
                        julia_c=None):
        inp = np.ascontiguousarray(inp)
        out = np.zeros((h, w), dtype=PIXEL_DTYPE)
        self.lib.orc_render_advanced(fractal, int(dbl), arith, _ptr(out), w * 16, w, h, _d4(*rect), max_iter,
                                     max_ss, flags, _d4(*rect_reused), _ptr(inp), inp.strides[0], focus[0], focus[1],
                                     C.cast(self._julia(julia_c), C.c_void_p) if julia_c else None)
        return out

    def compose(self, pix, palette, max_ss, visualize=False):
        pix = np.ascontiguousarray(pix)
        h, w = pix.shape
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        out = np.zeros((h, w), dtype=np.uint32)
        self.lib.orc_compose(_ptr(pix), pix.strides[0], _ptr(out), out.strides[0], w, h, _ptr(pal), len(pal),
                             max_ss, int(visualize))
        return out

    def render_under_sampled(self, fractal, arith, w, h, rect, max_iter, level, julia_c=None):
        out = np.zeros((h, w), dtype=PIXEL_DTYPE)
        self.lib.orc_render_under_sampled(fractal, arith, _ptr(out), w * 16, w, h, _d4(*rect), max_iter, level,
                                          C.cast(self._julia(julia_c), C.c_void_p) if julia_c else None)
        return out

    def escape_grid(self, fractal, dbl, arith, w, h, x0, y0, dx, dy, max_iter, julia_c=None, counts=True):
        out = np.zeros((h, w), dtype=np.uint32) if counts else None
        total = self.lib.orc_escape_grid(fractal, int(dbl), arith, w, h, x0, y0, dx, dy, max_iter,
                                         C.cast(self._julia(julia_c), C.c_void_p) if julia_c else None, _ptr(out))
        return total, out


    def frame(self, w, h, max_iter, spp, mode, dbl, arith, fractal, seed, center, pixel_size, julia_c=(0.0, 0.0),
              pix_start=0, pix_count=None, palette=None, interior_rgba=0xFF000000, smooth=True, pixels=True):
        """The library's frame path restated (orc_frame): returns dict with total,
        counts[n, spp], smooth[n, spp], pixels[n], rgba[n] for pixels
        [pix_start, pix_start + pix_count)."""
        n = w * h - pix_start if pix_count is None else pix_count
        d = FrameDesc(w, h, max_iter, spp, mode, int(dbl), arith, fractal, seed, center[0], center[1], pixel_size,
                      julia_c[0], julia_c[1])
        counts = np.zeros((n, spp), dtype=np.uint32)
        sm = np.zeros((n, spp), dtype=np.float32) if smooth else None
        px = np.zeros(n, dtype=PIXEL_DTYPE) if pixels else None
        pal = np.ascontiguousarray(palette, dtype=np.uint32) if palette is not None else None
        rgba = np.zeros(n, dtype=np.uint32) if pal is not None else None
        total = self.lib.orc_frame(C.byref(d), pix_start, n, _ptr(counts), _ptr(sm), _ptr(px), _ptr(rgba), _ptr(pal),
                                   len(pal) if pal is not None else 0, interior_rgba)
        return {"total": int(total), "counts": counts, "smooth": sm, "pixels": px, "rgba": rgba}

    def frame_points(self, w, h, spp, mode, seed, center, pixel_size, pix_start, pix_count):
        """binary64 sample points (xs, ys) of pixels [pix_start, pix_start + pix_count)."""
        d = FrameDesc(w, h, 0, spp, mode, 1, 0, 0, seed, center[0], center[1], pixel_size, 0.0, 0.0)
        xs = np.zeros(pix_count * spp, dtype=np.float64)
        ys = np.zeros(pix_count * spp, dtype=np.float64)
        self.lib.orc_frame_points_d(C.byref(d), pix_start, pix_count, _ptr(xs), _ptr(ys))
        return xs, ys

    def mandelbrot_points_d(self, xs, ys, max_iter, arith=ARITH_PARITY):
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        ys = np.ascontiguousarray(ys, dtype=np.float64)
        out = np.zeros(len(xs), dtype=np.uint32)
        total = self.lib.orc_mandelbrot_points_d(len(xs), _ptr(xs), _ptr(ys), max_iter, arith, _ptr(out))
        return int(total), out

    def hp_escape(self, cx_hex, cy_hex, dcx, dcy, bits, max_iter):
        r2 = C.c_double()
        i = self.lib.orc_hp_escape(cx_hex.encode(), cy_hex.encode(), dcx, dcy, bits, max_iter, C.byref(r2))
        return i, r2.value

    def hp_escape_batch(self, cx_hex, cy_hex, dcx, dcy, bits, max_iter):
        dcx = np.ascontiguousarray(dcx, dtype=np.float64)
        dcy = np.ascontiguousarray(dcy, dtype=np.float64)
        counts = np.zeros(len(dcx), dtype=np.uint32)
        r2 = np.zeros(len(dcx), dtype=np.float64)
        self.lib.orc_hp_escape_batch(cx_hex.encode(), cy_hex.encode(), len(dcx), _ptr(dcx), _ptr(dcy), bits,
                                     max_iter, _ptr(counts), _ptr(r2))
        return counts, r2

    def frame_offsets(self, w, h, spp, mode, seed, pixel_size, pix_start, pix_count):
        """Plane offsets (dcx, dcy) from the centre of frame samples of pixels [pix_start, +pix_count)."""
        d = FrameDesc(w, h, 0, spp, mode, 1, 0, 0, seed, 0.0, 0.0, pixel_size, 0.0, 0.0)
        xs = np.zeros(pix_count * spp, dtype=np.float64)
        ys = np.zeros(pix_count * spp, dtype=np.float64)
        self.lib.orc_frame_offsets(C.byref(d), pix_start, pix_count, _ptr(xs), _ptr(ys))
        return xs, ys

    def batch_viewport(self, w, h, spp, mode, max_iter, tier, seed, center, ps, palette=None,
                       interior_rgba=0xFF000000):
        v = Viewport(w, h, spp, mode, max_iter, tier, seed, center[0], center[1], ps)
        counts = np.zeros(w * h * spp, dtype=np.uint32)
        sm = np.zeros(w * h * spp, dtype=np.float32)
        pal = np.ascontiguousarray(palette, dtype=np.uint32) if palette is not None else None
        rgba = np.zeros(w * h, dtype=np.uint32) if pal is not None else None
        total = self.lib.orc_batch_viewport(C.byref(v), _ptr(counts), _ptr(sm), _ptr(rgba), _ptr(pal),
                                            len(pal) if pal is not None else 0, interior_rgba)
        return {"total": int(total), "counts": counts, "smooth": sm, "rgba": rgba}

    def set_newton(self, roots=(1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378), coefficients=(-1, 0, 0, 1),
                   magnifier=11):
        """The Newton modules' constants: roots (re, im) x3, coefficients c0..c3, colorMagnifier."""
        r = np.ascontiguousarray(roots, dtype=np.float64)
        c = np.ascontiguousarray(coefficients, dtype=np.float64)
        self.lib.orc_set_newton(_ptr(r), _ptr(c), magnifier)

    def compose_mode(self, pix, palette, mode, magnifier=1):
        pix = np.ascontiguousarray(pix)
        h, w = pix.shape
        pal = np.ascontiguousarray(palette if palette is not None else [0], dtype=np.uint32)
        out = np.zeros((h, w), dtype=np.uint32)
        self.lib.orc_compose_mode(_ptr(pix), pix.strides[0], _ptr(out), out.strides[0], w, h, _ptr(pal), len(pal),
                                  mode, magnifier)
        return out

    def max_threads(self):
        return self.lib.orc_max_threads()

    def sample_hash(self, seed, pixel, sample, axis):
        return self.lib.orc_sample_hash(seed, pixel, sample, axis)


class Reference:
    """The reference's own computeFractal (host build of src/main/cuda/fractals/*.cu)."""

    def __init__(self, path=REF_LIB):
        self.lib = C.CDLL(path)
        L = self.lib
        for n in ("ref_mandelbrot_f", "ref_julia_f"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [C.c_uint, C.c_float, C.c_float]
        for n in ("ref_mandelbrot_d", "ref_julia_d"):
            getattr(L, n).restype = C.c_float
            getattr(L, n).argtypes = [C.c_uint, C.c_double, C.c_double]
        L.ref_julia_set_c.restype = None
        L.ref_julia_set_c.argtypes = [C.c_double, C.c_double]
        L.ref_mandelbrot_colorize.restype = C.c_uint
        L.ref_mandelbrot_colorize.argtypes = [C.c_void_p, C.c_uint, C.c_float]
        L.ref_mandelbrot_grid.restype = C.c_ulonglong
        L.ref_mandelbrot_grid.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_uint, C.c_int, C.c_void_p]
        L.ref_mandelbrot_points_d.restype = C.c_ulonglong
        L.ref_mandelbrot_points_d.argtypes = [C.c_size_t, C.c_void_p, C.c_void_p, C.c_uint, C.c_int, C.c_void_p]
        L.ref_max_threads.restype = C.c_int
        L.ref_newton_set.restype = None
        L.ref_newton_set.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.ref_newton_f.restype = C.c_float
        L.ref_newton_f.argtypes = [C.c_int, C.c_uint, C.c_float, C.c_float]
        L.ref_newton_d.restype = C.c_float
        L.ref_newton_d.argtypes = [C.c_int, C.c_uint, C.c_double, C.c_double]
        L.ref_newton_colorize.restype = C.c_uint
        L.ref_newton_colorize.argtypes = [C.c_int, C.c_void_p, C.c_uint, C.c_float]

    def mandelbrot(self, dbl, max_iter, x, y):
        return (self.lib.ref_mandelbrot_d if dbl else self.lib.ref_mandelbrot_f)(max_iter, x, y)

    def julia(self, dbl, max_iter, x, y, c):
        self.lib.ref_julia_set_c(c[0], c[1])
        return (self.lib.ref_julia_d if dbl else self.lib.ref_julia_f)(max_iter, x, y)

    def colorize(self, palette, value):
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        return self.lib.ref_mandelbrot_colorize(_ptr(pal), len(pal), value)

    def grid(self, dbl, w, h, x0, y0, dx, dy, max_iter, threads=0, counts=True):
        out = np.zeros((h, w), dtype=np.uint32) if counts else None
        total = self.lib.ref_mandelbrot_grid(int(dbl), w, h, x0, y0, dx, dy, max_iter, threads, _ptr(out))
        return total, out

    def points_d(self, xs, ys, max_iter, threads=0):
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        ys = np.ascontiguousarray(ys, dtype=np.float64)
        out = np.zeros(len(xs), dtype=np.uint32)
        total = self.lib.ref_mandelbrot_points_d(len(xs), _ptr(xs), _ptr(ys), max_iter, threads, _ptr(out))
        return total, out

    def hp_escape(self, cx_hex, cy_hex, dcx, dcy, bits, max_iter):
        r2 = C.c_double()
        i = self.lib.orc_hp_escape(cx_hex.encode(), cy_hex.encode(), dcx, dcy, bits, max_iter, C.byref(r2))
        return i, r2.value

    def hp_escape_batch(self, cx_hex, cy_hex, dcx, dcy, bits, max_iter):
        dcx = np.ascontiguousarray(dcx, dtype=np.float64)
        dcy = np.ascontiguousarray(dcy, dtype=np.float64)
        counts = np.zeros(len(dcx), dtype=np.uint32)
        r2 = np.zeros(len(dcx), dtype=np.float64)
        self.lib.orc_hp_escape_batch(cx_hex.encode(), cy_hex.encode(), len(dcx), _ptr(dcx), _ptr(dcy), bits,
                                     max_iter, _ptr(counts), _ptr(r2))
        return counts, r2

    def frame_offsets(self, w, h, spp, mode, seed, pixel_size, pix_start, pix_count):
        """Plane offsets (dcx, dcy) from the centre of frame samples of pixels [pix_start, +pix_count)."""
        d = FrameDesc(w, h, 0, spp, mode, 1, 0, 0, seed, 0.0, 0.0, pixel_size, 0.0, 0.0)
        xs = np.zeros(pix_count * spp, dtype=np.float64)
        ys = np.zeros(pix_count * spp, dtype=np.float64)
        self.lib.orc_frame_offsets(C.byref(d), pix_start, pix_count, _ptr(xs), _ptr(ys))
        return xs, ys

    def batch_viewport(self, w, h, spp, mode, max_iter, tier, seed, center, ps, palette=None,
                       interior_rgba=0xFF000000):
        v = Viewport(w, h, spp, mode, max_iter, tier, seed, center[0], center[1], ps)
        counts = np.zeros(w * h * spp, dtype=np.uint32)
        sm = np.zeros(w * h * spp, dtype=np.float32)
        pal = np.ascontiguousarray(palette, dtype=np.uint32) if palette is not None else None
        rgba = np.zeros(w * h, dtype=np.uint32) if pal is not None else None
        total = self.lib.orc_batch_viewport(C.byref(v), _ptr(counts), _ptr(sm), _ptr(rgba), _ptr(pal),
                                            len(pal) if pal is not None else 0, interior_rgba)
        return {"total": int(total), "counts": counts, "smooth": sm, "rgba": rgba}

    def max_threads(self):
        return self.lib.ref_max_threads()

    def newton_set(self, roots, coefficients, magnifier):
        r = np.ascontiguousarray(roots, dtype=np.float64)
        c = np.ascontiguousarray(coefficients, dtype=np.float64)
        self.lib.ref_newton_set(_ptr(r), _ptr(c), magnifier)

    def newton(self, kind, dbl, max_iter, x, y):
        return (self.lib.ref_newton_d if dbl else self.lib.ref_newton_f)(kind, max_iter, x, y)

    def newton_colorize(self, kind, palette, value):
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        return self.lib.ref_newton_colorize(kind, _ptr(pal), len(pal), value)


def c1_grid():
    """The plain binary32 workload (C1) as a point grid: 1024x1024 pixel centres
    of the plane [-2, 1] x [-1.5, 1.5], maxIter 1000 -> (w, h, x0, y0, dx, dy,
    max_iter)."""
    w = h = 1024
    dx = 3.0 / 1024
    return w, h, -2.0 + dx / 2, 1.5 - dx / 2, dx, dx, 1000
