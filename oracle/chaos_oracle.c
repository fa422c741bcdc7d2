/*
 * chaos_oracle.c -- CPU restatement of the reference's fractal-kernel path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py call it to produce the
 * expected answer.  Nothing in the product (the CUDA library, the drop-in
 * module, the Python host layer) links, loads or calls it.
 *
 * Every function names the reference source it restates (paths relative to
 * the chaos-ultra project root; gen.cu = src/main/cuda/fractalRendererGeneric.cu).
 * The reference is CUDA; its warp-synchronous parts (the 8x4 warp tile of
 * getImageIndexes and the __all_sync votes of sampleTheFractal) are restated
 * here as explicit lock-step loops over the lanes of one tile.
 *
 * Build with -ffp-contract=off: the restatement rounds every product and sum
 * separately, as the reference kernel does when nvcc is told --fmad=false.
 * The "fma" arithmetic variant restates, with explicit fma() calls, the
 * operation sequence the CUDA fast path uses, so it is bit-exact as well.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    float value;
    float weight;
    uint8_t is_reused;
    uint8_t pad[3];
    float weight_of_new_samples;
} orc_pixel_info; /* pixel_info_t, src/main/cuda/helpers.cuh:106-130 (16 bytes) */

enum { ORC_MANDELBROT = 0, ORC_JULIA = 1 }; /* 2..4: the Newton modules (newton_oracle.cpp) */

/* Newton modules' constants (roots, coefficients c0..c3, colorMagnifier). */
static double g_newton_roots[6] = {1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378};
static double g_newton_coeffs[4] = {-1, 0, 0, 1};
static int g_newton_magnifier = 11;

void orc_set_newton(const double roots[6], const double coeffs[4], int magnifier)
{
    memcpy(g_newton_roots, roots, sizeof g_newton_roots);
    memcpy(g_newton_coeffs, coeffs, sizeof g_newton_coeffs);
    g_newton_magnifier = magnifier;
}

float orc_newton_compute_f(int fractal, uint32_t max_iter, float x, float y, const double *roots, const double *coeffs);
float orc_newton_compute_d(int fractal, uint32_t max_iter, double x, double y, const double *roots,
                           const double *coeffs);
enum { ORC_ARITH_FMA = 0, ORC_ARITH_PARITY = 1, ORC_ARITH_CONTRACTED = 2 }; /* same numbering as CHAOS_ARITH_* */
/* Served float-float frames (binary64 kernels only): the escape loop of the
 * library's ff_step from the binary64 sample point (chaos_device.cuh
 * compute_fractal with ARITH_FLOATFLOAT). */
enum { ORC_ARITH_FLOATFLOAT = 3 };
static float orc_compute_fractal_ff(int fractal, uint32_t max_iter, double px, double py, double jcx, double jcy);

/* kernel flag bits, gen.cu:157-161 */
#define ORC_FLAG_ADAPTIVE_SS (1u << 0)
#define ORC_FLAG_FOVEATION (1u << 2)
#define ORC_FLAG_SAMPLE_REUSE (1u << 3)
#define ORC_FLAG_IS_ZOOMING (1u << 4)
#define ORC_FLAG_ZOOMING_IN (1u << 5)

#define ORC_MAX_SUPER_SAMPLING 64u /* gen.cu:12 */
#define ORC_ADAPTIVE_THRESHOLD 10u /* gen.cu:93 */

/* ------------------------------------------------------------------------ */
/* Escape loops                                                              */
/* ------------------------------------------------------------------------ */

/* Reference loop: src/main/cuda/fractals/mandelbrot.cu:16-21 and
 * src/main/cuda/fractals/julia.cu:10-15.  Products and sums are rounded one by
 * one (the file is compiled with -ffp-contract=off). */
static uint32_t esc_parity_f(uint32_t max_iter, float x, float y, float cx, float cy, float *r2_exit)
{
    uint32_t i = 0;
    while (i < max_iter && x * x + y * y < 4) {
        float xn = x * x - y * y + cx;
        y = 2 * x * y + cy;
        x = xn;
        ++i;
    }
    *r2_exit = x * x + y * y;
    return i;
}

static uint32_t esc_parity_d(uint32_t max_iter, double x, double y, double cx, double cy, double *r2_exit)
{
    uint32_t i = 0;
    while (i < max_iter && x * x + y * y < 4) {
        double xn = x * x - y * y + cx;
        y = 2 * x * y + cy;
        x = xn;
        ++i;
    }
    *r2_exit = x * x + y * y;
    return i;
}

/* The fused-multiply-add step of the CUDA fast path:
 *   r2 = fma(x, x, y*y)            escape test, continue while r2 < 4
 *   x' = fma(x, x, fma(-y, y, cx))
 *   y' = fma(x + x, y, cy)
 * The iteration is the same map z <- z^2 + c; only the rounding differs. */
static uint32_t esc_fma_f(uint32_t max_iter, float x, float y, float cx, float cy, float *r2_exit)
{
    uint32_t i = 0;
    float r2;
    for (;;) {
        r2 = fmaf(x, x, y * y);
        if (!(i < max_iter && r2 < 4.0f)) break;
        float t = fmaf(-y, y, cx);
        float xn = fmaf(x, x, t);
        float yn = fmaf(x + x, y, cy);
        x = xn;
        y = yn;
        ++i;
    }
    *r2_exit = r2;
    return i;
}

static uint32_t esc_fma_d(uint32_t max_iter, double x, double y, double cx, double cy, double *r2_exit)
{
    uint32_t i = 0;
    double r2;
    for (;;) {
        r2 = fma(x, x, y * y);
        if (!(i < max_iter && r2 < 4.0)) break;
        double t = fma(-y, y, cx);
        double xn = fma(x, x, t);
        double yn = fma(x + x, y, cy);
        x = xn;
        y = yn;
        ++i;
    }
    *r2_exit = r2;
    return i;
}

/* The reference loop as nvcc compiles it with contraction on (its default):
 * the squares feed both the test and x', so they stay rounded products, and
 * only y' = 2*x*y + cy becomes one fused multiply-add.  Established by
 * comparing the reference's default sm_103a build with candidate roundings on
 * the same points. */
static uint32_t esc_contracted_f(uint32_t max_iter, float x, float y, float cx, float cy, float *r2_exit)
{
    uint32_t i = 0;
    float r2;
    for (;;) {
        float xx = x * x, yy = y * y;
        r2 = xx + yy;
        if (!(i < max_iter && r2 < 4.0f)) break;
        float xn = (xx - yy) + cx;
        float yn = fmaf(x + x, y, cy);
        x = xn;
        y = yn;
        ++i;
    }
    *r2_exit = r2;
    return i;
}

static uint32_t esc_contracted_d(uint32_t max_iter, double x, double y, double cx, double cy, double *r2_exit)
{
    uint32_t i = 0;
    double r2;
    for (;;) {
        double xx = x * x, yy = y * y;
        r2 = xx + yy;
        if (!(i < max_iter && r2 < 4.0)) break;
        double xn = (xx - yy) + cx;
        double yn = fma(x + x, y, cy);
        x = xn;
        y = yn;
        ++i;
    }
    *r2_exit = r2;
    return i;
}

static uint32_t esc_any_f(int arith, uint32_t max_iter, float x, float y, float cx, float cy, float *r2)
{
    return arith == ORC_ARITH_FMA          ? esc_fma_f(max_iter, x, y, cx, cy, r2)
           : arith == ORC_ARITH_CONTRACTED ? esc_contracted_f(max_iter, x, y, cx, cy, r2)
                                           : esc_parity_f(max_iter, x, y, cx, cy, r2);
}

static uint32_t esc_any_d(int arith, uint32_t max_iter, double x, double y, double cx, double cy, double *r2)
{
    return arith == ORC_ARITH_FMA          ? esc_fma_d(max_iter, x, y, cx, cy, r2)
           : arith == ORC_ARITH_CONTRACTED ? esc_contracted_d(max_iter, x, y, cx, cy, r2)
                                           : esc_parity_d(max_iter, x, y, cx, cy, r2);
}

/* computeFractal<float>: Mandelbrot starts at z=0 with c=point and maps an
 * interior point (i == maxIterations) to 0 (mandelbrot.cu:11-25); Julia starts
 * at z=point with c=(Real)julia_c and returns i unchanged (julia.cu:5-17). */
float orc_compute_fractal_f(int fractal, int arith, uint32_t max_iter, float px, float py, double jcx, double jcy)
{
    float r2;
    uint32_t i;
    if (fractal >= 2) return orc_newton_compute_f(fractal, max_iter, px, py, g_newton_roots, g_newton_coeffs);
    if (fractal == ORC_MANDELBROT) {
        i = esc_any_f(arith, max_iter, 0.f, 0.f, px, py, &r2);
        if (i == max_iter) return 0;
        return (float)i;
    }
    float cx = (float)jcx, cy = (float)jcy;
    i = esc_any_f(arith, max_iter, px, py, cx, cy, &r2);
    return (float)i;
}

float orc_compute_fractal_d(int fractal, int arith, uint32_t max_iter, double px, double py, double jcx, double jcy)
{
    double r2;
    uint32_t i;
    if (fractal >= 2) return orc_newton_compute_d(fractal, max_iter, px, py, g_newton_roots, g_newton_coeffs);
    if (arith == ORC_ARITH_FLOATFLOAT) return orc_compute_fractal_ff(fractal, max_iter, px, py, jcx, jcy);
    if (fractal == ORC_MANDELBROT) {
        i = esc_any_d(arith, max_iter, 0.0, 0.0, px, py, &r2);
        if (i == max_iter) return 0;
        return (float)i;
    }
    i = esc_any_d(arith, max_iter, px, py, jcx, jcy, &r2);
    return (float)i;
}

/* ------------------------------------------------------------------------ */
/* Reference-mode sampling (fractalRenderMain / fractalRenderAdvanced)       */
/* ------------------------------------------------------------------------ */

typedef struct {
    int fractal;
    int dbl;   /* 0: Rectangle<float> kernel, 1: Rectangle<double> kernel */
    int arith; /* ORC_ARITH_* */
    uint32_t w, h;
    float rf[4];  /* lb.x, lb.y, rt.x, rt.y as the float kernel receives them */
    double rd[4]; /* same, double kernel */
    uint32_t max_iter;
    double jcx, jcy;
} orc_view;

/* One sample of sampleTheFractal: sample offset (gen.cu:104-117), plane point
 * (gen.cu:97, 119-124) and the truncation of computeFractal's float result to
 * uint (gen.cu:126). */
static uint32_t sample_escape(const orc_view *v, uint32_t px, uint32_t py, uint32_t i, float sample_count_f)
{
    const uint32_t skip_first = 2;
    if (v->dbl) {
        double dx, dy;
        if (i <= skip_first) {
            dx = dy = (double)i / (double)(skip_first + 1);
        } else {
            float spr_f = sqrtf(sample_count_f - (float)skip_first);
            uint32_t spr = (uint32_t)roundf(spr_f);
            float fx = (float)((i - skip_first) % spr) / spr_f;
            float fy = (float)((i - skip_first) / spr) / spr_f;
            dx = fx;
            dy = fy;
        }
        double psx = (v->rd[2] - v->rd[0]) / (double)v->w;
        double psy = (v->rd[3] - v->rd[1]) / (double)v->h;
        /* the contracted build fuses the x coordinate's product into its add */
        double cx = v->arith == ORC_ARITH_CONTRACTED ? fma((double)px + dx, psx, v->rd[0])
                                                     : v->rd[0] + ((double)px + dx) * psx;
        double cy = v->rd[3] + (-((double)py + dy)) * psy;
        return (uint32_t)orc_compute_fractal_d(v->fractal, v->arith, v->max_iter, cx, cy, v->jcx, v->jcy);
    } else {
        float dx, dy;
        if (i <= skip_first) {
            dx = dy = (float)i / (float)(skip_first + 1);
        } else {
            float spr_f = sqrtf(sample_count_f - (float)skip_first);
            uint32_t spr = (uint32_t)roundf(spr_f);
            dx = (float)((i - skip_first) % spr) / spr_f;
            dy = (float)((i - skip_first) / spr) / spr_f;
        }
        float psx = (v->rf[2] - v->rf[0]) / (float)v->w;
        float psy = (v->rf[3] - v->rf[1]) / (float)v->h;
        float cx = v->arith == ORC_ARITH_CONTRACTED ? fmaf((float)px + dx, psx, v->rf[0])
                                                    : v->rf[0] + ((float)px + dx) * psx;
        float cy = v->rf[3] + (-((float)py + dy)) * psy;
        return (uint32_t)orc_compute_fractal_f(v->fractal, v->arith, v->max_iter, cx, cy, v->jcx, v->jcy);
    }
}

/* computeDispersion, gen.cu:24-34: variance-to-mean ratio over the first
 * data_length stored samples, divided by (n-1) in unsigned arithmetic.  The
 * reference passes data_length = i and stores only 10 samples; for i > 10 it
 * reads past its local array.  Here such reads are skipped (the sum covers the
 * 10 stored samples, the divisor stays i-1). */
static float dispersion(const float *data, uint32_t data_length, float mean)
{
    uint32_t n = data_length;
    float variance = 0;
    uint32_t m = data_length < ORC_ADAPTIVE_THRESHOLD ? data_length : ORC_ADAPTIVE_THRESHOLD;
    for (uint32_t k = 0; k < m; k++) {
        float d = data[k] - mean;
        float sq = d * d;
        variance = variance + sq;
    }
    variance /= (float)(uint32_t)(n - 1);
    return variance / mean;
}

/* sampleTheFractal, gen.cu:85-155, for the lanes of one warp that reach the
 * same call site together.  Every lane carries its own sampleCountF (the
 * reference's in/out argument); the votes (__all_sync over the active lanes)
 * are evaluated across exactly the lanes passed in. */
static void sample_lockstep(const orc_view *v, int n, const uint32_t *px, const uint32_t *py,
                            float *sample_count_f, int adaptive, uint32_t *result)
{
    uint32_t sample_count[32], sum[32];
    float samples[32][ORC_ADAPTIVE_THRESHOLD];
    int live[32];
    int any = 0;
    for (int l = 0; l < n; l++) {
        live[l] = !(sample_count_f[l] < 1);
        if (!live[l]) { /* gen.cu:87-90 */
            sample_count_f[l] = 0;
            result[l] = 0;
            continue;
        }
        uint32_t sc = (uint32_t)roundf(sample_count_f[l]);
        sample_count[l] = sc < ORC_MAX_SUPER_SAMPLING ? sc : ORC_MAX_SUPER_SAMPLING;
        sum[l] = 0;
        any = 1;
    }
    if (!any) return;
    /* The loop bound is uniform across the live lanes: sampleCountF is uniform
     * at every reference call site and the votes keep it so. */
    for (uint32_t i = 0;; i++) {
        int running = 0;
        for (int l = 0; l < n; l++)
            if (live[l] && i < sample_count[l]) running = 1;
        if (!running) break;
        float disp[32];
        int want_vote = 0;
        for (int l = 0; l < n; l++) {
            if (!live[l] || !(i < sample_count[l])) continue;
            uint32_t e = sample_escape(v, px[l], py[l], i, sample_count_f[l]);
            sum[l] += e;
            if (i < ORC_ADAPTIVE_THRESHOLD) samples[l][i] = (float)e;
            if ((adaptive && (i > 0 && i < ORC_ADAPTIVE_THRESHOLD)) || (i == sample_count[l] / 2)) {
                float mean = (float)(sum[l] / (i + 1));
                disp[l] = dispersion(samples[l], i, mean);
                want_vote = 1;
            }
        }
        if (!want_vote) continue;
        /* gen.cu:140-149; all lanes take the branch together */
        int all_eq = 1, all_lo = 1, all_le1 = 1;
        for (int l = 0; l < n; l++) {
            if (!live[l] || !(i < sample_count[l])) continue;
            if (i == 1 && !(fabsf(samples[l][0] - samples[l][1]) < FLT_EPSILON)) all_eq = 0;
            if (!(disp[l] < 0.01f)) all_lo = 0;
            if (!(disp[l] <= 1)) all_le1 = 0;
        }
        for (int l = 0; l < n; l++) {
            if (!live[l] || !(i < sample_count[l])) continue;
            if (i == 1 && all_eq)
                sample_count[l] = i + 1;
            else if (all_lo)
                sample_count[l] = i + 1;
            else if (all_le1 && i >= sample_count[l] / 2)
                sample_count[l] = i + 1;
        }
    }
    for (int l = 0; l < n; l++) {
        if (!live[l]) continue;
        result[l] = sum[l] / sample_count[l];
        sample_count_f[l] = (float)sample_count[l];
    }
}

/* Lane order of one warp (getImageIndexes, gen.cu:43-53, blockDim.x == 32):
 * lane l covers pixel (x0 + 4*(l/16) + l%4, y0 + (l/4)%4). */
static void tile_lanes(uint32_t x0, uint32_t y0, uint32_t *lx, uint32_t *ly)
{
    for (uint32_t l = 0; l < 32; l++) {
        lx[l] = x0 + 4 * (l / 16) + l % 4;
        ly[l] = y0 + (l / 4) % 4;
    }
}

static orc_pixel_info *pixel_at(void *base, long pitch, uint32_t x, uint32_t y)
{
    return (orc_pixel_info *)((char *)base + (size_t)y * (size_t)pitch) + x;
}

static void make_view(orc_view *v, int fractal, int dbl, int arith, uint32_t w, uint32_t h, const double rect[4],
                      uint32_t max_iter, const double julia_c[2])
{
    v->fractal = fractal;
    v->dbl = dbl;
    v->arith = arith;
    v->w = w;
    v->h = h;
    for (int k = 0; k < 4; k++) {
        v->rf[k] = (float)rect[k];
        v->rd[k] = rect[k];
    }
    v->max_iter = max_iter;
    v->jcx = julia_c ? julia_c[0] : 0.0;
    v->jcy = julia_c ? julia_c[1] : 0.0;
}

/* fractalRenderMain, gen.cu:168-181: one 8x4 warp tile at a time.  The output
 * record is pixel_info_t(result, sampleCount): value, weight, isReused=false,
 * weightOfNewSamples=0. */
void orc_render_main(int fractal, int dbl, int arith, void *out, long pitch, uint32_t w, uint32_t h,
                     const double rect[4], uint32_t max_iter, float max_ss, uint32_t flags, const double julia_c[2])
{
    orc_view v;
    make_view(&v, fractal, dbl, arith, w, h, rect, max_iter, julia_c);
    uint32_t tiles_x = (w + 7) / 8, tiles_y = (h + 3) / 4;
#pragma omp parallel for schedule(dynamic)
    for (long t = 0; t < (long)tiles_x * tiles_y; t++) {
        uint32_t x0 = 8 * (uint32_t)(t % tiles_x), y0 = 4 * (uint32_t)(t / tiles_x);
        uint32_t lx[32], ly[32], px[32], py[32], res[32];
        float scf[32];
        tile_lanes(x0, y0, lx, ly);
        int n = 0;
        for (int l = 0; l < 32; l++) {
            if (lx[l] >= w || ly[l] >= h) continue;
            px[n] = lx[l];
            py[n] = ly[l];
            scf[n] = max_ss;
            n++;
        }
        if (!n) continue;
        sample_lockstep(&v, n, px, py, scf, (flags & ORC_FLAG_ADAPTIVE_SS) != 0, res);
        for (int l = 0; l < n; l++) {
            orc_pixel_info *o = pixel_at(out, pitch, px[l], py[l]);
            memset(o, 0, sizeof *o);
            o->value = (float)res[l];
            o->weight = scf[l];
        }
    }
}

/* getWarpingOriginOfSampleReuse, gen.cu:194-203 */
static void warping_origin(const orc_view *v, const double old_rect[4], uint32_t px, uint32_t py, float *ox, float *oy)
{
    uint32_t qy = v->h - py;
    float rx, ry;
    if (v->dbl) {
        double sx = v->rd[2] - v->rd[0], sy = v->rd[3] - v->rd[1];
        /* contracted: the position in the plane is one fused multiply-add */
        int fz = v->arith == ORC_ARITH_CONTRACTED;
        double ppx = fz ? fma((double)px / (double)v->w, sx, v->rd[0]) : (double)px / (double)v->w * sx + v->rd[0];
        double ppy = fz ? fma((double)qy / (double)v->h, sy, v->rd[1]) : (double)qy / (double)v->h * sy + v->rd[1];
        double osx = old_rect[2] - old_rect[0], osy = old_rect[3] - old_rect[1];
        rx = (float)((ppx - old_rect[0]) / osx);
        ry = (float)((ppy - old_rect[1]) / osy);
    } else {
        float o0 = (float)old_rect[0], o1 = (float)old_rect[1], o2 = (float)old_rect[2], o3 = (float)old_rect[3];
        float sx = v->rf[2] - v->rf[0], sy = v->rf[3] - v->rf[1];
        int fz = v->arith == ORC_ARITH_CONTRACTED;
        float ppx = fz ? fmaf((float)px / (float)v->w, sx, v->rf[0]) : (float)px / (float)v->w * sx + v->rf[0];
        float ppy = fz ? fmaf((float)qy / (float)v->h, sy, v->rf[1]) : (float)qy / (float)v->h * sy + v->rf[1];
        rx = (ppx - o0) / (o2 - o0);
        ry = (ppy - o1) / (o3 - o1);
    }
    *ox = rx * (float)v->w;
    float oyv = ry * (float)v->h;
    *oy = v->arith == ORC_ARITH_CONTRACTED ? fmaf(-ry, (float)v->h, (float)v->h) : (float)v->h - oyv;
}

/* readFromArrayUsingFiltering<float>, gen.cu:259-302.  Contracted: every
 * term after the first is fused onto the sum so far, the first pair as
 * fma(w00, T00, w10 * T10). */
static void read_filtered(int arith, const void *in, long pitch, float x, float y, float *value, float *weight)
{
    uint32_t i = (uint32_t)floorf(x), j = (uint32_t)floorf(y);
    float alpha = x - (float)i, beta = y - (float)j;
    const orc_pixel_info *a = pixel_at((void *)in, pitch, i, j);
    const orc_pixel_info *b = pixel_at((void *)in, pitch, i + 1, j);
    const orc_pixel_info *c = pixel_at((void *)in, pitch, i, j + 1);
    const orc_pixel_info *d = pixel_at((void *)in, pitch, i + 1, j + 1);
    float w00 = (1 - alpha) * (1 - beta), w10 = alpha * (1 - beta), w01 = (1 - alpha) * beta, w11 = alpha * beta;
    float r, ww;
    if (arith == ORC_ARITH_CONTRACTED) {
        r = fmaf(w00, a->value, w10 * b->value);
        r = fmaf(w01, c->value, r);
        r = fmaf(w11, d->value, r);
        ww = fmaf(w00, a->weight, w10 * b->weight);
        ww = fmaf(w01, c->weight, ww);
        ww = fmaf(w11, d->weight, ww);
    } else {
        r = w00 * a->value + w10 * b->value;
        r = r + w01 * c->value;
        r = r + w11 * d->value;
        ww = w00 * a->weight + w10 * b->weight;
        ww = ww + w01 * c->weight;
        ww = ww + w11 * d->weight;
    }
    *value = r;
    *weight = ww;
}

/* getFoveationAdvisedSampleCount + linearMapping, gen.cu:209-257.
 * atanf here is the C library's; CUDA's atanf may differ in the last place,
 * which can move a pixel across a foveation threshold. */
static void foveation(int arith, uint32_t px, uint32_t py, uint32_t fx, uint32_t fy, float max_ss, float *advised,
                      int *inside)
{
    const float pi_f = 3.14159265358979f;
    const float screen_distance = 60.0f, pixel_cm = 0.02652f;
    uint32_t nx = px - px % 8, ny = py - py % 4;
    float foveal = max_ss >= 1 ? 5.5f : (float)(5.5 * (double)max_ss);
    float peripheral = 60;
    float ddx = (float)fx - (float)nx, ddy = (float)fy - (float)ny;
    /* contracted: the sum of squares and k*x + q are fused */
    float sq = arith == ORC_ARITH_CONTRACTED ? fmaf(ddx, ddx, ddy * ddy) : ddx * ddx + ddy * ddy;
    float dist = sqrtf(sq) * pixel_cm;
    float angle = atanf(dist / screen_distance) * 180 / pi_f;
    /* linearMapping<float>(angle, foveal, peripheral, 1, 0) */
    float k = (0.0f - 1.0f) / (peripheral - foveal);
    float q = (peripheral * 1.0f - 0.0f * foveal) / (peripheral - foveal);
    float lin = arith == ORC_ARITH_CONTRACTED ? fmaf(k, angle, q) : k * angle + q;
    float rel = (float)fmin(1.0, (double)lin);
    float adv = max_ss * rel;
    int in = 0;
    if (angle <= foveal) {
        adv = (float)fmax(1.0, (double)adv);
        in = 1;
    }
    *advised = adv;
    *inside = in;
}

/* fractalRenderAdvanced, gen.cu:307-368.  Lanes of one warp that take the
 * same sampleTheFractal call site vote together. */
void orc_render_advanced(int fractal, int dbl, int arith, void *out, long pitch, uint32_t w, uint32_t h,
                         const double rect[4], uint32_t max_iter, float max_ss, uint32_t flags,
                         const double rect_reused[4], const void *in, long in_pitch, uint32_t focus_x,
                         uint32_t focus_y, const double julia_c[2])
{
    orc_view v;
    make_view(&v, fractal, dbl, arith, w, h, rect, max_iter, julia_c);
    uint32_t tiles_x = (w + 7) / 8, tiles_y = (h + 3) / 4;
    int adaptive = (flags & ORC_FLAG_ADAPTIVE_SS) != 0;
#pragma omp parallel for schedule(dynamic)
    for (long t = 0; t < (long)tiles_x * tiles_y; t++) {
        uint32_t x0 = 8 * (uint32_t)(t % tiles_x), y0 = 4 * (uint32_t)(t / tiles_x);
        uint32_t lx[32], ly[32];
        tile_lanes(x0, y0, lx, ly);
        orc_pixel_info res[32];
        float adv[32], reused_v[32], reused_w[32];
        int inside[32], reusing[32], valid[32];
        for (int l = 0; l < 32; l++) {
            valid[l] = lx[l] < w && ly[l] < h;
            if (!valid[l]) continue;
            adv[l] = max_ss;
            inside[l] = 0;
            if ((flags & ORC_FLAG_FOVEATION) && (flags & ORC_FLAG_IS_ZOOMING) && (flags & ORC_FLAG_ZOOMING_IN))
                foveation(arith, lx[l], ly[l], focus_x, focus_y, max_ss, &adv[l], &inside[l]);
            reusing[l] = 0;
            if (flags & ORC_FLAG_SAMPLE_REUSE) {
                float ox, oy;
                warping_origin(&v, rect_reused, lx[l], ly[l], &ox, &oy);
                int oix = (int)roundf(ox), oiy = (int)roundf(oy);
                /* frames narrower than 5 pixels reuse nothing: there the unsigned
                   w - 2 of the reference's test can admit a corner outside the frame */
                if (w < 5 || h < 5 || oix < 2 || (uint32_t)oix >= w - 2 || oiy < 2 || (uint32_t)oiy >= h - 2) {
                    reusing[l] = 0;
                } else {
                    read_filtered(arith, in, in_pitch, ox, oy, &reused_v[l], &reused_w[l]);
                    reusing[l] = !(reused_w[l] < 0.1);
                }
            }
        }
        /* group A: reusing lanes inside the focus area while zooming in */
        uint32_t pa[32], qa[32], ra[32], ia[32];
        float sa[32];
        int na = 0;
        /* group B: lanes that do not reuse */
        uint32_t pb[32], qb[32], rb[32], ib[32];
        float sb[32];
        int nb = 0;
        for (int l = 0; l < 32; l++) {
            if (!valid[l]) continue;
            memset(&res[l], 0, sizeof res[l]);
            if (reusing[l]) {
                res[l].value = reused_v[l];
                res[l].weight = reused_w[l];
                res[l].is_reused = 1;
                res[l].weight_of_new_samples = 0;
                if ((flags & ORC_FLAG_ZOOMING_IN) && inside[l]) {
                    pa[na] = lx[l];
                    qa[na] = ly[l];
                    sa[na] = adv[l];
                    ia[na] = (uint32_t)l;
                    na++;
                }
            } else {
                float sc = adv[l];
                if (sc < 1) sc = 1;
                pb[nb] = lx[l];
                qb[nb] = ly[l];
                sb[nb] = sc;
                ib[nb] = (uint32_t)l;
                nb++;
            }
        }
        if (na) {
            sample_lockstep(&v, na, pa, qa, sa, adaptive, ra);
            for (int k = 0; k < na; k++) {
                int l = (int)ia[k];
                float samples = (float)ra[k];
                float sc = sa[k];
                float rw = reused_w[l] * 0.75f;
                res[l].weight_of_new_samples = sc;
                res[l].weight = rw + sc;
                float add = samples * sc;
                float num = arith == ORC_ARITH_CONTRACTED ? fmaf(reused_v[l], rw, add) : reused_v[l] * rw + add;
                res[l].value = num / res[l].weight;
            }
        }
        if (nb) {
            sample_lockstep(&v, nb, pb, qb, sb, adaptive, rb);
            for (int k = 0; k < nb; k++) {
                int l = (int)ib[k];
                res[l].value = (float)rb[k];
                res[l].weight = sb[k];
            }
        }
        for (int l = 0; l < 32; l++)
            if (valid[l]) *pixel_at(out, pitch, lx[l], ly[l]) = res[l];
    }
}

/* colorizeSampleCount, gen.cu:67-77.  The channels are `char`; the reference
 * toolchain (x86-64, signed char) converts 255*rel with a saturating
 * float-to-s8 conversion, so a channel tops out at 0x7f. */
static uint32_t colorize_sample_count(uint32_t sample_count, uint32_t full)
{
    if (sample_count > full) sample_count = full;
    float rel = (float)sample_count / (float)full;
    float f = 255 * rel;
    int c = (int)f;
    if (c > 127) c = 127;
    if (c < -128) c = -128;
    uint32_t b = (uint32_t)(uint8_t)(int8_t)c;
    return b | (b << 8) | (b << 16) | 0xff000000u;
}

/* compose, gen.cu:455-475 with colorize of mandelbrot.cu:27-35 / julia.cu:19-27:
 * palette index len - (round(value) % len) - 1; the RGBA word (R in the low
 * byte) goes to out[y*out_pitch/4 + x]. */
void orc_compose(const void *in, long pitch, uint32_t *out, long out_pitch, uint32_t w, uint32_t h,
                 const uint32_t *palette, uint32_t palette_len, float max_ss, int visualize_sample_count)
{
#pragma omp parallel for schedule(static)
    for (long y = 0; y < (long)h; y++) {
        for (uint32_t x = 0; x < w; x++) {
            const orc_pixel_info *p = pixel_at((void *)in, pitch, x, (uint32_t)y);
            uint32_t color;
            if (visualize_sample_count) {
                double m = fmax(1.0, (double)max_ss);
                uint32_t full = (uint32_t)m;
                color = colorize_sample_count((uint32_t)p->weight, full);
                if (p->is_reused) color = colorize_sample_count((uint32_t)p->weight_of_new_samples, full);
            } else {
                uint32_t vi = (uint32_t)roundf(p->value);
                uint32_t idx = palette_len - (vi % palette_len) - 1;
                color = palette[idx];
            }
            *(uint32_t *)((char *)out + (size_t)y * (size_t)out_pitch + 4 * (size_t)x) = color;
        }
    }
}

/* fractalRenderUnderSampled, gen.cu:478-503 (float plane, every level-th
 * pixel, weight 1/level). */
void orc_render_under_sampled(int fractal, int arith, void *out, long pitch, uint32_t w, uint32_t h,
                              const double rect[4], uint32_t max_iter, uint32_t level, const double julia_c[2])
{
    float lbx = (float)rect[0], lby = (float)rect[1], rtx = (float)rect[2], rty = (float)rect[3];
    float pw = (rtx - lbx) / (float)w;
    float ph = (rty - lby) / (float)h;
    double jx = julia_c ? julia_c[0] : 0, jy = julia_c ? julia_c[1] : 0;
    for (uint32_t y = 0; y < h; y += level) {
        if (y >= h - level) break;
        for (uint32_t x = 0; x < w; x += level) {
            if (x >= w - level) break;
            float cx = lbx + (float)x * pw;
            float cy = rty - (float)y * ph;
            uint32_t e = (uint32_t)orc_compute_fractal_f(fractal, arith, max_iter, cx, cy, jx, jy);
            orc_pixel_info *o = pixel_at(out, pitch, x, y);
            memset(o, 0, sizeof *o);
            o->value = (float)e;
            o->weight = 1 / (float)level;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Escape-count grids (plain per-sample escape counts, CPU baseline)         */
/* ------------------------------------------------------------------------ */

/* Escape count per pixel for the point c = (x0 + px*dx, y0 - py*dy), one
 * sample per pixel: counts[py*w+px] = iterations taken (max_iter for interior),
 * as the pixel-iteration metric counts them.  Returns the sum of counts. */
uint64_t orc_escape_grid(int fractal, int dbl, int arith, uint32_t w, uint32_t h, double x0, double y0, double dx,
                         double dy, uint32_t max_iter, const double julia_c[2], uint32_t *counts)
{
    uint64_t total = 0;
    double jx = julia_c ? julia_c[0] : 0, jy = julia_c ? julia_c[1] : 0;
#pragma omp parallel for schedule(dynamic) reduction(+ : total)
    for (long y = 0; y < (long)h; y++) {
        for (uint32_t x = 0; x < w; x++) {
            uint32_t i;
            if (dbl) {
                double cx = x0 + (double)x * dx, cy = y0 - (double)y * dy, r2;
                double zx = fractal == ORC_MANDELBROT ? 0.0 : cx, zy = fractal == ORC_MANDELBROT ? 0.0 : cy;
                double ccx = fractal == ORC_MANDELBROT ? cx : jx, ccy = fractal == ORC_MANDELBROT ? cy : jy;
                i = arith == ORC_ARITH_FMA ? esc_fma_d(max_iter, zx, zy, ccx, ccy, &r2)
                                           : esc_parity_d(max_iter, zx, zy, ccx, ccy, &r2);
            } else {
                float cx = (float)x0 + (float)x * (float)dx, cy = (float)y0 - (float)y * (float)dy, r2;
                float zx = fractal == ORC_MANDELBROT ? 0.f : cx, zy = fractal == ORC_MANDELBROT ? 0.f : cy;
                float ccx = fractal == ORC_MANDELBROT ? cx : (float)jx, ccy = fractal == ORC_MANDELBROT ? cy : (float)jy;
                i = arith == ORC_ARITH_FMA ? esc_fma_f(max_iter, zx, zy, ccx, ccy, &r2)
                                           : esc_parity_f(max_iter, zx, zy, ccx, ccy, &r2);
            }
            if (counts) counts[(size_t)y * w + x] = i;
            total += i;
        }
    }
    return total;
}

/* ------------------------------------------------------------------------ */
/* Frames of independent samples (the library's k_frame / chaos_render_frame) */
/* ------------------------------------------------------------------------ */
/* Not a reference kernel: this restates the frame path the GB300 library adds
 * (pixel-centre and jittered sampling, smooth iteration count, palette with
 * linear interpolation), so its escape counts can be checked bit for bit and
 * its smooth values / colours within a stated tolerance. */

typedef struct {
    uint32_t w, h, max_iter, spp, mode, dbl, arith, fractal;
    uint64_t seed;
    double center_x, center_y, pixel_size, jcx, jcy;
} orc_frame_desc;

/* SplitMix64 output function (Steele, Lea, Flood, OOPSLA 2014). */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t orc_sample_hash(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t axis)
{
    return mix64(seed ^ mix64(((uint64_t)pixel << 7) | ((uint64_t)sample << 1) | axis));
}

static float smooth_value(uint32_t i, float r2, uint32_t max_iter)
{
    if (i >= max_iter) return (float)max_iter;
    if (!(r2 < 3.0e38f)) return (float)i;
    float l = 0.5f * log2f(r2);
    return (float)(i + 1u) - log2f(l);
}

static void palette_lerp(const uint32_t *pal, uint32_t len, float nu, float ch[4])
{
    float fl = (float)len;
    float t = fmodf(nu, fl);
    if (t < 0.f) t = t + fl;
    uint32_t i0 = (uint32_t)t;
    if (i0 >= len) i0 = len - 1u;
    float f = t - (float)i0;
    uint32_t i1 = i0 + 1u == len ? 0u : i0 + 1u;
    uint32_t c0 = pal[i0], c1 = pal[i1];
    for (int k = 0; k < 4; k++) {
        float a0 = (float)((c0 >> (8 * k)) & 255u), a1 = (float)((c1 >> (8 * k)) & 255u);
        ch[k] = fmaf(a1 - a0, f, a0);
    }
}

static uint32_t pack_mean_rgba(const float acc[4], uint32_t spp)
{
    uint32_t out = 0;
    float n = (float)spp;
    for (int k = 0; k < 4; k++) {
        float v = acc[k] / n + 0.5f;
        v = v < 255.f ? v : 255.f;
        out |= ((uint32_t)v & 255u) << (8 * k);
    }
    return out;
}

/* Pixels [pix_start, pix_start + pix_count) of the frame.  Outputs are indexed
 * relative to pix_start: counts/smooth[(p - pix_start)*spp + s],
 * pixels/rgba[p - pix_start].  Returns the pixel-iterations of those pixels. */
uint64_t orc_frame(const orc_frame_desc *d, long pix_start, long pix_count, uint32_t *counts, float *smooth,
                   orc_pixel_info *pixels, uint32_t *rgba, const uint32_t *palette, uint32_t palette_len,
                   uint32_t interior_rgba)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (long q = 0; q < pix_count; q++) {
        uint32_t pix = (uint32_t)(pix_start + q);
        uint32_t px = pix % d->w, py = pix / d->w;
        float acc_v = 0.f, acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (uint32_t s = 0; s < d->spp; s++) {
            uint32_t i;
            float r2f;
            if (d->dbl) {
                double ox = 0.5, oy = 0.5, r2;
                if (d->mode == 1) {
                    ox = (double)(orc_sample_hash(d->seed, pix, s, 0) >> 11) * 0x1p-53;
                    oy = (double)(orc_sample_hash(d->seed, pix, s, 1) >> 11) * 0x1p-53;
                }
                double dxp = ((double)px + ox) - 0.5 * d->w, dyp = ((double)py + oy) - 0.5 * d->h;
                double cx = fma(dxp, d->pixel_size, d->center_x), cy = fma(-dyp, d->pixel_size, d->center_y);
                double zx = 0, zy = 0, kx = cx, ky = cy;
                if (d->fractal == ORC_JULIA) {
                    zx = cx;
                    zy = cy;
                    kx = d->jcx;
                    ky = d->jcy;
                }
                i = d->arith == ORC_ARITH_FMA ? esc_fma_d(d->max_iter, zx, zy, kx, ky, &r2)
                                              : esc_parity_d(d->max_iter, zx, zy, kx, ky, &r2);
                r2f = (float)r2;
            } else {
                float ox = 0.5f, oy = 0.5f, r2;
                if (d->mode == 1) {
                    ox = (float)(uint32_t)(orc_sample_hash(d->seed, pix, s, 0) >> 40) * 0x1p-24f;
                    oy = (float)(uint32_t)(orc_sample_hash(d->seed, pix, s, 1) >> 40) * 0x1p-24f;
                }
                float ps = (float)d->pixel_size, ctx = (float)d->center_x, cty = (float)d->center_y;
                float dxp = ((float)px + ox) - (float)(0.5 * d->w), dyp = ((float)py + oy) - (float)(0.5 * d->h);
                float cx = fmaf(dxp, ps, ctx), cy = fmaf(-dyp, ps, cty);
                float zx = 0, zy = 0, kx = cx, ky = cy;
                if (d->fractal == ORC_JULIA) {
                    zx = cx;
                    zy = cy;
                    kx = (float)d->jcx;
                    ky = (float)d->jcy;
                }
                i = d->arith == ORC_ARITH_FMA ? esc_fma_f(d->max_iter, zx, zy, kx, ky, &r2)
                                              : esc_parity_f(d->max_iter, zx, zy, kx, ky, &r2);
                r2f = r2;
            }
            int escaped = i < d->max_iter;
            float nu = smooth_value(i, r2f, d->max_iter);
            size_t sidx = (size_t)q * d->spp + s;
            if (counts) counts[sidx] = i;
            if (smooth) smooth[sidx] = nu;
            total += i;
            float v = escaped ? nu : (d->fractal == ORC_MANDELBROT ? 0.f : (float)d->max_iter);
            acc_v = acc_v + v;
            if (rgba) {
                float ch[4];
                if (escaped) {
                    palette_lerp(palette, palette_len, nu, ch);
                } else {
                    for (int k = 0; k < 4; k++) ch[k] = (float)((interior_rgba >> (8 * k)) & 255u);
                }
                for (int k = 0; k < 4; k++) acc[k] = acc[k] + ch[k];
            }
        }
        if (pixels) {
            memset(&pixels[q], 0, sizeof pixels[q]);
            pixels[q].value = acc_v / (float)d->spp;
            pixels[q].weight = (float)d->spp;
        }
        if (rgba) rgba[q] = pack_mean_rgba(acc, d->spp);
    }
    return total;
}

/* Plane points of the frame samples (binary64 frames), in the order of
 * orc_frame's outputs: xs/ys[(p - pix_start)*spp + s]. */
void orc_frame_points_d(const orc_frame_desc *d, long pix_start, long pix_count, double *xs, double *ys)
{
    for (long q = 0; q < pix_count; q++) {
        uint32_t pix = (uint32_t)(pix_start + q);
        uint32_t px = pix % d->w, py = pix / d->w;
        for (uint32_t s = 0; s < d->spp; s++) {
            double ox = 0.5, oy = 0.5;
            if (d->mode == 1) {
                ox = (double)(orc_sample_hash(d->seed, pix, s, 0) >> 11) * 0x1p-53;
                oy = (double)(orc_sample_hash(d->seed, pix, s, 1) >> 11) * 0x1p-53;
            }
            double dxp = ((double)px + ox) - 0.5 * d->w, dyp = ((double)py + oy) - 0.5 * d->h;
            xs[(size_t)q * d->spp + s] = fma(dxp, d->pixel_size, d->center_x);
            ys[(size_t)q * d->spp + s] = fma(-dyp, d->pixel_size, d->center_y);
        }
    }
}

/* Escape counts of a list of binary64 points, Mandelbrot, the reference loop
 * (rounded arithmetic) or the fma variant; interior points count max_iter.
 * OpenMP over points.  Returns the pixel-iteration total. */
uint64_t orc_mandelbrot_points_d(long n, const double *xs, const double *ys, uint32_t max_iter, int arith,
                                 uint32_t *counts)
{
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : total)
    for (long k = 0; k < n; k++) {
        double r2;
        uint32_t i = arith == ORC_ARITH_FMA ? esc_fma_d(max_iter, 0.0, 0.0, xs[k], ys[k], &r2)
                                            : esc_parity_d(max_iter, 0.0, 0.0, xs[k], ys[k], &r2);
        if (counts) counts[k] = i;
        total += i;
    }
    return total;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* High-precision direct iteration (the deep-zoom oracle)                     */
/* ------------------------------------------------------------------------ */
/* Signed fixed point with 32-bit limbs: value = sign * sum_{k=0..L} w[k] *
 * 2^(32(k-L)), w[L] the integer part.  Independent of the library's own
 * multi-word code (64-bit limbs); pinned against mpmath by the tests. */
#define HP_MAX 64 /* up to 2048 fraction bits */
typedef struct {
    int L;
    int neg;
    uint32_t w[HP_MAX + 1];
} hpnum;

static int hp_iszero(const hpnum *a)
{
    for (int k = 0; k <= a->L; k++)
        if (a->w[k]) return 0;
    return 1;
}

static int hp_cmpmag(const hpnum *a, const hpnum *b)
{
    for (int k = a->L; k >= 0; k--)
        if (a->w[k] != b->w[k]) return a->w[k] < b->w[k] ? -1 : 1;
    return 0;
}

static void hp_addsub(const hpnum *a, const hpnum *b, int negate_b, hpnum *r)
{
    int bneg = b->neg ^ negate_b;
    r->L = a->L;
    if (a->neg == bneg) {
        uint64_t c = 0;
        for (int k = 0; k <= a->L; k++) {
            c += (uint64_t)a->w[k] + b->w[k];
            r->w[k] = (uint32_t)c;
            c >>= 32;
        }
        r->neg = a->neg;
    } else {
        const hpnum *x = a, *y = b;
        int sign = a->neg;
        if (hp_cmpmag(a, b) < 0) {
            x = b;
            y = a;
            sign = bneg;
        }
        int64_t br = 0;
        for (int k = 0; k <= a->L; k++) {
            int64_t d = (int64_t)x->w[k] - y->w[k] - br;
            br = d < 0;
            r->w[k] = (uint32_t)(d + (br ? ((int64_t)1 << 32) : 0));
        }
        r->neg = sign;
    }
    if (hp_iszero(r)) r->neg = 0;
}

static void hp_mul(const hpnum *a, const hpnum *b, hpnum *r)
{
    int L = a->L;
    uint64_t col[2 * HP_MAX + 4];
    memset(col, 0, sizeof(uint64_t) * (size_t)(2 * L + 4));
    uint32_t p[2 * HP_MAX + 4];
    /* column sums of 32x32 products, carried as we go */
    for (int i = 0; i <= L; i++) {
        uint64_t carry = 0;
        for (int j = 0; j <= L; j++) {
            uint64_t t = (uint64_t)a->w[i] * b->w[j] + col[i + j] + carry;
            col[i + j] = t & 0xffffffffu;
            carry = t >> 32;
        }
        int k = i + L + 1;
        while (carry) {
            uint64_t t = col[k] + carry;
            col[k] = t & 0xffffffffu;
            carry = t >> 32;
            k++;
        }
    }
    for (int k = 0; k < 2 * L + 4; k++) p[k] = (uint32_t)col[k];
    r->L = L;
    for (int k = 0; k <= L; k++) r->w[k] = p[k + L];
    r->neg = (a->neg != b->neg) && !hp_iszero(r);
}

static void hp_from_double(double d, int L, hpnum *r)
{
    memset(r, 0, sizeof *r);
    r->L = L;
    if (d == 0.0) return;
    r->neg = d < 0;
    d = fabs(d);
    int e;
    double m = frexp(d, &e);
    uint64_t mant = (uint64_t)ldexp(m, 53);
    int shift = e - 53 + 32 * L; /* bit position of the mantissa's lsb */
    for (int b = 0; b < 53; b++) {
        if (!((mant >> b) & 1)) continue;
        int pos = shift + b;
        if (pos < 0 || pos >= 32 * (L + 1)) continue;
        r->w[pos / 32] |= 1u << (pos % 32);
    }
    if (hp_iszero(r)) r->neg = 0;
}

static double hp_to_double(const hpnum *a)
{
    double v = 0;
    for (int k = a->L; k >= 0 && k >= a->L - 3; k--) v += ldexp((double)a->w[k], 32 * (k - a->L));
    return a->neg ? -v : v;
}

static int hp_parse_hex(const char *s, int L, hpnum *r)
{
    memset(r, 0, sizeof *r);
    r->L = L;
    int neg = 0;
    if (*s == '-') {
        neg = 1;
        s++;
    }
    uint32_t ip = 0;
    while (*s >= '0' && *s <= '9') ip = ip * 10 + (uint32_t)(*s++ - '0');
    r->w[L] = ip;
    if (*s == '.') {
        s++;
        int bit = 32 * L;
        while (*s) {
            int v;
            char c = *s++;
            if (c >= '0' && c <= '9')
                v = c - '0';
            else if (c >= 'a' && c <= 'f')
                v = c - 'a' + 10;
            else if (c >= 'A' && c <= 'F')
                v = c - 'A' + 10;
            else
                return 0;
            bit -= 4;
            if (bit >= 0) r->w[bit / 32] |= (uint32_t)v << (bit % 32);
        }
    }
    r->neg = neg && !hp_iszero(r);
    return 1;
}

/* Mandelbrot at c = C + (dcx, dcy) in `bits` of fixed-point fraction:
 * continue while |z|^2 < 4 and i < max_iter (the reference loop's test).
 * Returns i; *r2 = |z_i|^2 as a double. */
uint32_t orc_hp_escape(const char *cx_hex, const char *cy_hex, double dcx, double dcy, uint32_t bits,
                       uint32_t max_iter, double *r2)
{
    int L = (int)((bits + 31) / 32);
    if (L > HP_MAX) L = HP_MAX;
    hpnum cx, cy, dx, dy, zx, zy, xx, yy, xy, t;
    hp_parse_hex(cx_hex, L, &cx);
    hp_parse_hex(cy_hex, L, &cy);
    hp_from_double(dcx, L, &dx);
    hp_from_double(dcy, L, &dy);
    hp_addsub(&cx, &dx, 0, &t);
    cx = t;
    hp_addsub(&cy, &dy, 0, &t);
    cy = t;
    memset(&zx, 0, sizeof zx);
    memset(&zy, 0, sizeof zy);
    zx.L = zy.L = L;
    uint32_t i = 0;
    double rr = 0;
    for (;;) {
        hp_mul(&zx, &zx, &xx);
        hp_mul(&zy, &zy, &yy);
        double x2 = hp_to_double(&xx), y2 = hp_to_double(&yy);
        rr = x2 + y2;
        if (!(i < max_iter && rr < 4.0)) break;
        hp_mul(&zx, &zy, &xy);
        hp_addsub(&xx, &yy, 1, &t);
        hp_addsub(&t, &cx, 0, &zx);
        hp_addsub(&xy, &xy, 0, &t);
        hp_addsub(&t, &cy, 0, &zy);
        ++i;
    }
    if (r2) *r2 = rr;
    return i;
}

void orc_hp_escape_batch(const char *cx_hex, const char *cy_hex, long n, const double *dcx, const double *dcy,
                         uint32_t bits, uint32_t max_iter, uint32_t *counts, double *r2)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (long k = 0; k < n; k++) {
        double rr;
        counts[k] = orc_hp_escape(cx_hex, cy_hex, dcx[k], dcy[k], bits, max_iter, &rr);
        if (r2) r2[k] = rr;
    }
}

/* The plane offsets dc of frame samples relative to the centre, in the order
 * of orc_frame's outputs (perturbation frames): dc = ((p + o) - n/2) * ps. */
void orc_frame_offsets(const orc_frame_desc *d, long pix_start, long pix_count, double *dcx, double *dcy)
{
    for (long q = 0; q < pix_count; q++) {
        uint32_t pix = (uint32_t)(pix_start + q);
        uint32_t px = pix % d->w, py = pix / d->w;
        for (uint32_t s = 0; s < d->spp; s++) {
            double ox = 0.5, oy = 0.5;
            if (d->mode == 1) {
                ox = (double)(orc_sample_hash(d->seed, pix, s, 0) >> 11) * 0x1p-53;
                oy = (double)(orc_sample_hash(d->seed, pix, s, 1) >> 11) * 0x1p-53;
            }
            dcx[(size_t)q * d->spp + s] = (((double)px + ox) - 0.5 * d->w) * d->pixel_size;
            dcy[(size_t)q * d->spp + s] = -(((double)py + oy) - 0.5 * d->h) * d->pixel_size;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Batched viewports (the library's k_batch) and float-float arithmetic      */
/* ------------------------------------------------------------------------ */

typedef struct {
    float hi, lo;
} ff_t;

static ff_t ff_fast_two_sum(float a, float b)
{
    float s = a + b;
    ff_t r = {s, b - (s - a)};
    return r;
}
static ff_t ff_from_double(double d)
{
    float hi = (float)d;
    ff_t r = {hi, (float)(d - (double)hi)};
    return r;
}

/* Knuth's two-sum. */
static float ff_two_sum(float a, float b, float *err)
{
    float s = a + b;
    float bb = s - a;
    *err = (a - (s - bb)) + (b - bb);
    return s;
}

/* The library's float-float step (chaos_frame.cuh ff_step): unnormalised
 * products, two-sums of the leading terms, error terms summed in a fixed
 * order, one normalisation per coordinate. */
static void ff_step(ff_t *x, ff_t *y, ff_t cx, ff_t cy)
{
    float px = x->hi * x->hi;
    float ex = fmaf(x->hi, x->hi, -px);
    ex = fmaf(x->hi + x->hi, x->lo, ex);
    float py = y->hi * y->hi;
    float ey = fmaf(y->hi, y->hi, -py);
    ey = fmaf(y->hi + y->hi, y->lo, ey);
    float pxy = x->hi * y->hi;
    float exy = fmaf(x->hi, y->hi, -pxy);
    exy = fmaf(x->hi, y->lo, exy);
    exy = fmaf(x->lo, y->hi, exy);
    float e1, e2, e3;
    float s = ff_two_sum(px, -py, &e1);
    float t = ff_two_sum(s, cx.hi, &e2);
    float e = ex - ey;
    e = e + e1;
    e = e + e2;
    e = e + cx.lo;
    ff_t xn = ff_fast_two_sum(t, e);
    float u = ff_two_sum(pxy + pxy, cy.hi, &e3);
    float f = fmaf(2.f, exy, e3) + cy.lo;
    *y = ff_fast_two_sum(u, f);
    *x = xn;
}

static uint32_t esc_ff_from(uint32_t max_iter, ff_t x, ff_t y, ff_t cx, ff_t cy, float *r2_exit)
{
    uint32_t i = 0;
    float r2;
    for (;;) {
        r2 = fmaf(x.hi, x.hi, y.hi * y.hi);
        if (!(i < max_iter && r2 < 4.0f)) break;
        ff_step(&x, &y, cx, cy);
        ++i;
    }
    *r2_exit = r2;
    return i;
}

/* computeFractal's escape value with the float-float loop: Mandelbrot from
 * z = 0 (interior -> 0), Julia from z = point with c = julia_c. */
static float orc_compute_fractal_ff(int fractal, uint32_t max_iter, double px, double py, double jcx, double jcy)
{
    float r2;
    ff_t zero = {0.f, 0.f};
    if (fractal == ORC_MANDELBROT) {
        uint32_t i = esc_ff_from(max_iter, zero, zero, ff_from_double(px), ff_from_double(py), &r2);
        return i == max_iter ? 0.f : (float)i;
    }
    return (float)esc_ff_from(max_iter, ff_from_double(px), ff_from_double(py), ff_from_double(jcx),
                              ff_from_double(jcy), &r2);
}

static uint32_t esc_ff(uint32_t max_iter, ff_t cx, ff_t cy, float *r2_exit)
{
    ff_t x = {0.f, 0.f}, y = {0.f, 0.f};
    uint32_t i = 0;
    float r2;
    for (;;) {
        r2 = fmaf(x.hi, x.hi, y.hi * y.hi);
        if (!(i < max_iter && r2 < 4.0f)) break;
        ff_step(&x, &y, cx, cy);
        ++i;
    }
    *r2_exit = r2;
    return i;
}

typedef struct {
    uint32_t w, h, spp, mode, max_iter, tier; /* tier: 0 binary32, 1 binary64, 2 float-float, 5 binary64 rounded */
    uint64_t seed;
    double cx, cy, ps;
} orc_viewport;

/* One viewport of a batch: sample point in binary64 (fma), rounded to the
 * tier, Mandelbrot with fused multiply-adds (binary32/64), float-float, or
 * the reference's rounded binary64 loop (mandelbrot.cu:16-21); outputs as
 * orc_frame.  Returns the pixel-iterations. */
uint64_t orc_batch_viewport(const orc_viewport *v, uint32_t *counts, float *smooth, uint32_t *rgba,
                            const uint32_t *palette, uint32_t palette_len, uint32_t interior_rgba)
{
    uint64_t total = 0;
    long n = (long)v->w * v->h;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (long q = 0; q < n; q++) {
        uint32_t pix = (uint32_t)q, px = pix % v->w, py = pix / v->w;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (uint32_t s = 0; s < v->spp; s++) {
            double ox = 0.5, oy = 0.5;
            if (v->mode == 1) {
                ox = (double)(orc_sample_hash(v->seed, pix, s, 0) >> 11) * 0x1p-53;
                oy = (double)(orc_sample_hash(v->seed, pix, s, 1) >> 11) * 0x1p-53;
            }
            double dxp = ((double)px + ox) - 0.5 * v->w, dyp = ((double)py + oy) - 0.5 * v->h;
            double cxd = fma(dxp, v->ps, v->cx), cyd = fma(-dyp, v->ps, v->cy);
            uint32_t i;
            float r2f;
            if (v->tier == 0) {
                i = esc_fma_f(v->max_iter, 0.f, 0.f, (float)cxd, (float)cyd, &r2f);
            } else if (v->tier == 1) {
                double r2;
                i = esc_fma_d(v->max_iter, 0.0, 0.0, cxd, cyd, &r2);
                r2f = (float)r2;
            } else if (v->tier == 5) { /* binary64 rounded as computeFractal<double> */
                double r2;
                i = esc_parity_d(v->max_iter, 0.0, 0.0, cxd, cyd, &r2);
                r2f = (float)r2;
            } else {
                i = esc_ff(v->max_iter, ff_from_double(cxd), ff_from_double(cyd), &r2f);
            }
            int escaped = i < v->max_iter;
            float nu = smooth_value(i, r2f, v->max_iter);
            size_t sidx = (size_t)q * v->spp + s;
            if (counts) counts[sidx] = i;
            if (smooth) smooth[sidx] = nu;
            total += i;
            if (rgba) {
                float ch[4];
                if (escaped) {
                    palette_lerp(palette, palette_len, nu, ch);
                } else {
                    for (int k = 0; k < 4; k++) ch[k] = (float)((interior_rgba >> (8 * k)) & 255u);
                }
                for (int k = 0; k < 4; k++) acc[k] = acc[k] + ch[k];
            }
        }
        if (rgba) rgba[q] = pack_mean_rgba(acc, v->spp);
    }
    return total;
}

/* compose with a module's colouring: mode 0 palette (mandelbrot/julia), 1 one
 * colour per root (newton_wired.cu:67-80, newton_generic.cu:75-88), 2 palette
 * with stride colorMagnifier (newton_iterations.cu:70-78). */
void orc_compose_mode(const void *in, long pitch, uint32_t *out, long out_pitch, uint32_t w, uint32_t h,
                      const uint32_t *palette, uint32_t palette_len, int mode, int magnifier)
{
    for (uint32_t y = 0; y < h; y++) {
        for (uint32_t x = 0; x < w; x++) {
            const orc_pixel_info *p = pixel_at((void *)in, pitch, x, y);
            uint32_t vi = (uint32_t)roundf(p->value), color;
            if (mode == 1)
                color = vi == 1 ? 0xff0000ffu : vi == 2 ? 0xff00ff00u : vi == 3 ? 0xffff0000u : 0xff000000u;
            else if (mode == 2)
                color = palette[palette_len - (vi * (uint32_t)magnifier % palette_len) - 1];
            else
                color = palette[palette_len - (vi % palette_len) - 1];
            *(uint32_t *)((char *)out + (size_t)y * (size_t)out_pitch + 4 * (size_t)x) = color;
        }
    }
}
