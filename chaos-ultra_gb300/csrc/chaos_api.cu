// chaos_api.cu -- the C ABI of libchaos_gb300.so (declared in include/chaos_gb300.h).
//
// Host-side mirror of the reference's JCuda layer:
//   chaos_module    FractalRenderingModule + its kernels and constants
//                   (J/cudarenderer/FractalRenderingModule.java, Module*.java)
//   chaos_renderer  CudaFractalRenderer: renderQuality / renderFast, the pitched
//                   sample-reuse double buffer, precision selection
//                   (J/cudarenderer/CudaFractalRenderer.java,
//                   DeviceMemoryDoubleBuffer2D.java, RenderingKernel.java)
// Every entry returns a status code; the message of the last failure is kept
// per thread (chaos_last_error).  Nothing here traps or aborts.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "chaos_kernels.cuh"
#include "chaos_trace.h"

using namespace chaos;

static_assert(sizeof(chaos_pixel_info) == sizeof(PixelInfo), "pixel record size");

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(CHAOS_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define CHAOS_CUDA(call, what)                       \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

// Per-device state: SM count and a ring of work counters.  Each persistent
// launch takes the next slot and zeroes it on its own stream first, so
// launches in flight on different streams use different counters (up to
// kCounterSlots of them at once).
constexpr int kMaxDevices = 64;
constexpr uint32_t kCounterSlots = 4096;

struct DeviceState {
    std::once_flag once;
    cudaError_t init_error = cudaSuccess;
    int sms = 0;
    uint32_t *counters = nullptr;
    std::atomic<uint32_t> next{0};
};
DeviceState g_devices[kMaxDevices];

int device_state(DeviceState **out)
{
    int dev = 0;
    CHAOS_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(CHAOS_ERR_UNSUPPORTED, "device %d out of range", dev);
    DeviceState &d = g_devices[dev];
    std::call_once(d.once, [&]() {
        cudaError_t e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaMalloc(&d.counters, 2 * kCounterSlots * sizeof(uint32_t));
        d.init_error = e;
    });
    if (d.init_error != cudaSuccess) return cuda_fail(d.init_error, "device set-up");
    *out = &d;
    return CHAOS_OK;
}

int take_counter(DeviceState *d, cudaStream_t s, uint32_t **counter)
{
    uint32_t slot = d->next.fetch_add(1, std::memory_order_relaxed) % kCounterSlots;
    *counter = d->counters + slot;
    CHAOS_CUDA(cudaMemsetAsync(*counter, 0, sizeof(uint32_t), s), "cudaMemsetAsync(work counter)");
    return CHAOS_OK;
}

// The status word that goes with a counter slot (a launch with a time limit
// and no status word of the caller's), zeroed on the stream.
int take_status(const DeviceState *d, const uint32_t *counter, cudaStream_t s, uint32_t **status)
{
    *status = d->counters + kCounterSlots + (counter - d->counters);
    CHAOS_CUDA(cudaMemsetAsync(*status, 0, sizeof(uint32_t), s), "cudaMemsetAsync(status word)");
    return CHAOS_OK;
}

// A launch's time limit in ns (0: none); false when the limit is negative or not finite.
bool budget_of(double seconds, unsigned long long *ns)
{
    if (!(seconds >= 0.0) || !std::isfinite(seconds)) return false;
    const double t = seconds * 1e9;
    *ns = seconds == 0.0 ? 0ull : t < 1.0 ? 1ull : t > 1.8e19 ? 18000000000000000000ull : (unsigned long long)t;
    return true;
}

// After a synchronous launch with a time limit: CHAOS_ERR_TIMEOUT when its
// status word says that the limit ran out.
int read_status(const uint32_t *status, cudaStream_t s, double seconds)
{
    uint32_t bits = 0;
    CHAOS_CUDA(cudaMemcpyAsync(&bits, status, sizeof bits, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(status)");
    CHAOS_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (bits & RUN_STATUS_TIMEOUT)
        return fail(CHAOS_ERR_TIMEOUT, "the launch ran past its time limit of %g s: outputs incomplete", seconds);
    return CHAOS_OK;
}

int finish(cudaError_t launch, cudaStream_t s, bool sync)
{
    if (launch != cudaSuccess) return cuda_fail(launch, "kernel launch");
    if (sync) CHAOS_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return CHAOS_OK;
}

template <class R> bool finite4(const R r[4])
{
    for (int k = 0; k < 4; k++)
        if (!std::isfinite((double)r[k])) return false;
    return true;
}

// Image sizes the reference host accepts: grid dims of ceil(n/32) < 65536
// (CudaFractalRenderer.java:247-253); the pixel count also has to fit an
// unsigned work index.
int check_size(uint32_t w, uint32_t h)
{
    if (w == 0 || h == 0) return fail(CHAOS_ERR_INVALID_ARGUMENT, "width and height must be positive (%u x %u)", w, h);
    if ((w + 31u) / 32u > 65535u || (h + 31u) / 32u > 65535u)
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "width/height must be smaller than %u", 65535u * 32u);
    if ((uint64_t)w * (uint64_t)h > (1ull << 31)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "image too large");
    return CHAOS_OK;
}

int check_pitched(const void *p, long pitch, uint32_t w, const char *what)
{
    if (!p) return fail(CHAOS_ERR_INVALID_ARGUMENT, "%s is NULL", what);
    if (pitch < (long)(16u * w)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "%s pitch %ld < 16*width", what, pitch);
    if (((uintptr_t)p & 3u) || (pitch & 3)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "%s must be 4-byte aligned", what);
    return CHAOS_OK;
}

struct FractalInfo {
    const char *name;
    int kind;
};
// Registered modules: the module file name and the name the Java GUI shows
// (CudaFractalRendererProvider.java:19-31, modules/Module*.java constructors).
const FractalInfo kFractals[] = {
    {"mandelbrot", FRACTAL_MANDELBROT},          {"julia", FRACTAL_JULIA},
    {"newton_wired", FRACTAL_NEWTON_WIRED},      {"newton wired", FRACTAL_NEWTON_WIRED},
    {"newton_generic", FRACTAL_NEWTON_GENERIC},  {"newton generic", FRACTAL_NEWTON_GENERIC},
    {"newton_iterations", FRACTAL_NEWTON_ITERATIONS}, {"newton colored by iterations", FRACTAL_NEWTON_ITERATIONS}};
const char *kDisplayNames[] = {"mandelbrot", "julia", "newton wired", "newton generic",
                               "newton colored by iterations"};

// ---- the JSON subset of the Newton modules' custom parameters -------------
// {"coefficients": [a3, a2, a1, a0], "roots": [[re, im], x3], "colorMagnifier": n}
// (ModuleNewtonGeneric.parseJsonToParams, ModuleNewtonIterations.java:15-24)
struct JsonValue {
    enum Kind { NUMBER, ARRAY, OBJECT, OTHER } kind = OTHER;
    double number = 0;
    std::vector<JsonValue> items;
    std::vector<std::pair<std::string, JsonValue>> members;
};

void json_ws(const char *&p)
{
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++;
}

bool json_parse(const char *&p, JsonValue &v, int depth = 0)
{
    if (depth > 16) return false;
    json_ws(p);
    if (*p == '[') {
        p++;
        v.kind = JsonValue::ARRAY;
        json_ws(p);
        if (*p == ']') {
            p++;
            return true;
        }
        for (;;) {
            JsonValue item;
            if (!json_parse(p, item, depth + 1)) return false;
            v.items.push_back(item);
            json_ws(p);
            if (*p == ',') {
                p++;
                continue;
            }
            if (*p == ']') {
                p++;
                return true;
            }
            return false;
        }
    }
    if (*p == '{') {
        p++;
        v.kind = JsonValue::OBJECT;
        json_ws(p);
        if (*p == '}') {
            p++;
            return true;
        }
        for (;;) {
            json_ws(p);
            if (*p != '"') return false;
            const char *q = ++p;
            while (*p && *p != '"') p++;
            if (*p != '"') return false;
            std::string key(q, p - q);
            p++;
            json_ws(p);
            if (*p != ':') return false;
            p++;
            JsonValue item;
            if (!json_parse(p, item, depth + 1)) return false;
            v.members.emplace_back(key, item);
            json_ws(p);
            if (*p == ',') {
                p++;
                continue;
            }
            if (*p == '}') {
                p++;
                return true;
            }
            return false;
        }
    }
    char *end = nullptr;
    double d = std::strtod(p, &end);
    if (end == p) return false;
    v.kind = JsonValue::NUMBER;
    v.number = d;
    p = end;
    return true;
}

const JsonValue *json_member(const JsonValue &o, const char *key)
{
    for (const auto &m : o.members)
        if (m.first == key) return &m.second;
    return nullptr;
}

int arith_of(int arith)
{
    return arith == CHAOS_ARITH_PARITY ? ARITH_PARITY : arith == CHAOS_ARITH_CONTRACTED ? ARITH_CONTRACTED : ARITH_FMA;
}

double float_ulp(float f)  // java.lang.Math.ulp(float)
{
    f = std::fabs(f);
    if (!std::isfinite(f)) return INFINITY;
    if (f < 0x1p-126f) return 0x1p-149;
    int e;
    std::frexp(f, &e);
    return std::ldexp(1.0, e - 24);
}

double double_ulp(double d)  // java.lang.Math.ulp(double)
{
    d = std::fabs(d);
    if (!std::isfinite(d)) return INFINITY;
    if (d < 0x1p-1022) return 0x1p-1074;
    int e;
    std::frexp(d, &e);
    return std::ldexp(1.0, e - 53);
}

}  // namespace

namespace chaos {
// shared with the other translation units of the library (chaos_perturb.cu)
int api_fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int api_device_counter(cudaStream_t s, uint32_t **counter, int *sms)
{
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    *sms = d->sms;
    return take_counter(d, s, counter);
}

int api_device_status(const uint32_t *counter, cudaStream_t s, uint32_t **status)
{
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    return take_status(d, counter, s, status);
}

bool api_budget(double seconds, unsigned long long *ns) { return budget_of(seconds, ns); }

int api_read_status(const uint32_t *status, cudaStream_t s, double seconds) { return read_status(status, s, seconds); }
}  // namespace chaos

struct chaos_module {
    int fractal = FRACTAL_MANDELBROT;
    std::string name;
    bool visualize = false;
    double julia_c[2] = {0.0, 0.0};
    NewtonParams newton{};
};


const char *chaos_last_error(void) { return g_last_error.c_str(); }

const char *chaos_version(void) { return "chaos_gb300 0.1 (sm_103a)"; }

const char *chaos_available_fractals(void)
{
    return "mandelbrot,julia,newton wired,newton generic,newton colored by iterations";
}

int chaos_module_open(const char *fractal_name, chaos_module **out)
{
    if (!fractal_name || !out) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    for (const FractalInfo &f : kFractals) {
        if (std::strcmp(f.name, fractal_name) == 0) {
            chaos_module *m = new (std::nothrow) chaos_module();
            if (!m) return fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
            m->fractal = f.kind;
            m->name = kDisplayNames[f.kind];
            // The Newton modules start from their supplyDefaultValues parameters
            // (ModuleNewtonGeneric.java:67-74, ModuleNewtonIterations.java:26-33).
            const double roots[6] = {1, 0, -0.5, 0.86602540378, -0.5, -0.86602540378};
            const double coefficients[4] = {-1, 0, 0, 1};  // z^3 - 1, stored c0..c3
            std::memcpy(m->newton.roots, roots, sizeof roots);
            std::memcpy(m->newton.coefficients, coefficients, sizeof coefficients);
            m->newton.color_magnifier = 11;
            *out = m;
            return CHAOS_OK;
        }
    }
    return fail(CHAOS_ERR_UNKNOWN_FRACTAL, "Unknown fractal: %s", fractal_name);
}

int chaos_module_close(chaos_module *m)
{
    delete m;
    return CHAOS_OK;
}

const char *chaos_module_fractal_name(const chaos_module *m) { return m ? m->name.c_str() : ""; }

int chaos_module_write_constant(chaos_module *m, const char *name, const void *src, size_t size)
{
    if (!m || !name || !src) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (std::strcmp(name, "VISUALIZE_SAMPLE_COUNT") == 0) {
        if (size != 1) return fail(CHAOS_ERR_INVALID_ARGUMENT, "VISUALIZE_SAMPLE_COUNT is 1 byte, got %zu", size);
        m->visualize = *static_cast<const uint8_t *>(src) != 0;
        return CHAOS_OK;
    }
    if (m->fractal == FRACTAL_JULIA && std::strcmp(name, "julia_c") == 0) {
        if (size != sizeof m->julia_c) return fail(CHAOS_ERR_INVALID_ARGUMENT, "julia_c is 16 bytes, got %zu", size);
        std::memcpy(m->julia_c, src, sizeof m->julia_c);
        return CHAOS_OK;
    }
    const bool generic = m->fractal == FRACTAL_NEWTON_GENERIC || m->fractal == FRACTAL_NEWTON_ITERATIONS;
    if (generic && std::strcmp(name, "roots") == 0) {
        if (size != sizeof m->newton.roots) return fail(CHAOS_ERR_INVALID_ARGUMENT, "roots is 48 bytes, got %zu", size);
        std::memcpy(m->newton.roots, src, sizeof m->newton.roots);
        return CHAOS_OK;
    }
    if (generic && std::strcmp(name, "coefficients") == 0) {
        if (size != sizeof m->newton.coefficients)
            return fail(CHAOS_ERR_INVALID_ARGUMENT, "coefficients is 32 bytes, got %zu", size);
        std::memcpy(m->newton.coefficients, src, sizeof m->newton.coefficients);
        return CHAOS_OK;
    }
    if (m->fractal == FRACTAL_NEWTON_ITERATIONS && std::strcmp(name, "colorMagnifier") == 0) {
        if (size != sizeof(int)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "colorMagnifier is 4 bytes, got %zu", size);
        std::memcpy(&m->newton.color_magnifier, src, sizeof(int));
        return CHAOS_OK;
    }
    return fail(CHAOS_ERR_NOT_FOUND, "no constant named %s in module %s", name, m->name.c_str());
}

int chaos_module_set_custom_params(chaos_module *m, const char *text)
{
    if (!m || !text) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->fractal == FRACTAL_NEWTON_GENERIC || m->fractal == FRACTAL_NEWTON_ITERATIONS) {
        const char *p = text;
        JsonValue v;
        if (!json_parse(p, v) || v.kind != JsonValue::OBJECT)
            return fail(CHAOS_ERR_INVALID_ARGUMENT, "custom parameters must be a JSON object");
        const JsonValue *c = json_member(v, "coefficients"), *r = json_member(v, "roots");
        if (!c || !r || c->kind != JsonValue::ARRAY || r->kind != JsonValue::ARRAY)
            return fail(CHAOS_ERR_INVALID_ARGUMENT, "\"coefficients\" and \"roots\" arrays are required");
        if (c->items.size() != 4) return fail(CHAOS_ERR_INVALID_ARGUMENT, "expecting 4 coefficients");
        if (r->items.size() != 3) return fail(CHAOS_ERR_INVALID_ARGUMENT, "expecting 3 roots");
        NewtonParams np = m->newton;
        for (int k = 0; k < 4; k++) {
            if (c->items[k].kind != JsonValue::NUMBER) return fail(CHAOS_ERR_INVALID_ARGUMENT, "bad coefficient");
            np.coefficients[3 - k] = c->items[k].number;  // the user writes the highest power first
        }
        for (int k = 0; k < 3; k++) {
            const JsonValue &root = r->items[k];
            if (root.kind != JsonValue::ARRAY || root.items.size() != 2 || root.items[0].kind != JsonValue::NUMBER ||
                root.items[1].kind != JsonValue::NUMBER)
                return fail(CHAOS_ERR_INVALID_ARGUMENT, "Found a root that is not represented as [real, imag].");
            np.roots[2 * k] = root.items[0].number;
            np.roots[2 * k + 1] = root.items[1].number;
        }
        if (m->fractal == FRACTAL_NEWTON_ITERATIONS) {
            const JsonValue *mag = json_member(v, "colorMagnifier");
            if (mag) {
                if (mag->kind != JsonValue::NUMBER) return fail(CHAOS_ERR_INVALID_ARGUMENT, "bad colorMagnifier");
                np.color_magnifier = (int)mag->number;
            }
        }
        m->newton = np;
        return CHAOS_OK;
    }
    if (m->fractal != FRACTAL_JULIA) return CHAOS_OK;  // ModuleMandelbrot / ModuleNewtonWired ignore theirs
    // ModuleJulia: numbers separated by ',' or ';' (parseParamsAsDoubles,
    // FractalRenderingModule.java:233-241); the first two are julia_c.
    std::vector<double> vals;
    std::string s(text);
    size_t start = 0;
    while (start <= s.size()) {
        size_t end = s.find_first_of(",;", start);
        if (end == std::string::npos) end = s.size();
        std::string tok = s.substr(start, end - start);
        size_t a = tok.find_first_not_of(" \t\r\n"), b = tok.find_last_not_of(" \t\r\n");
        if (a == std::string::npos) return fail(CHAOS_ERR_INVALID_ARGUMENT, "empty number in \"%s\"", text);
        tok = tok.substr(a, b - a + 1);
        char *endp = nullptr;
        errno = 0;
        double v = std::strtod(tok.c_str(), &endp);
        if (!endp || *endp != '\0' || errno == ERANGE)
            return fail(CHAOS_ERR_INVALID_ARGUMENT, "not a number: \"%s\"", tok.c_str());
        vals.push_back(v);
        start = end + 1;
        if (end == s.size()) break;
    }
    if (vals.size() < 2) return fail(CHAOS_ERR_INVALID_ARGUMENT, "julia needs two numbers, got \"%s\"", text);
    m->julia_c[0] = vals[0];
    m->julia_c[1] = vals[1];
    return CHAOS_OK;
}

int chaos_module_default_view(const chaos_module *m, double *cx, double *cy, double *zoom, uint32_t *max_iter,
                              float *max_ss)
{
    if (!m || !cx || !cy || !zoom || !max_iter || !max_ss) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m->fractal == FRACTAL_MANDELBROT) {  // ModuleMandelbrot.java:20-25
        *cx = -0.5;
        *cy = 0.0;
        *zoom = 2.0;
        *max_iter = 1600;
        *max_ss = 5.f;
    } else {  // Model.resetRenderingValuesToDefault (Model.java:284-294) + the module's supplyDefaultValues
        *cx = 0.0;
        *cy = 0.0;
        *zoom = 4.0;
        *max_iter = m->fractal == FRACTAL_JULIA ? 900 : 200;  // ModuleJulia.java:40-49, ModuleNewton*.java
        *max_ss = 2.f;
    }
    return CHAOS_OK;
}

// ---- reference-mode kernels ----------------------------------------------

template <class R>
static int render_main(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t w, uint32_t h, const R rect[4],
                       uint32_t max_iter, float max_ss, uint32_t flags, int arith, cudaStream_t s, bool sync)
{
    TraceRange trace_("fractalRenderMain");
    if (!m || !rect) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = check_size(w, h);
    if (rc) return rc;
    if ((rc = check_pitched(out, pitch, w, "output"))) return rc;
    if (!finite4(rect)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "plane segment must be finite");
    if (max_iter < 1) return fail(CHAOS_ERR_INVALID_ARGUMENT, "maxIterations must be a positive number");
    if (!(max_ss >= 1.f) || !std::isfinite(max_ss))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "maxSuperSampling must be >= 1 (got %g)", (double)max_ss);
    DeviceState *d;
    if ((rc = device_state(&d))) return rc;
    MainArgs<R> a{};
    a.out = out;
    a.pitch = pitch;
    a.size = UInt2{w, h};
    a.image = Rect<R>{rect[0], rect[1], rect[2], rect[3]};
    a.max_iter = max_iter;
    a.max_ss = max_ss;
    a.flags = flags;
    a.jcx = m->julia_c[0];
    a.jcy = m->julia_c[1];
    a.newton = m->newton;
    a.tiles_x = (w + 7u) / 8u;
    a.n_tiles = a.tiles_x * ((h + 3u) / 4u);
    if ((rc = take_counter(d, s, &a.counter))) return rc;
    return finish(launch_main<R>(a, arith_of(arith), m->fractal, d->sms, s), s, sync);
}

template <class R>
static int render_advanced(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t w, uint32_t h,
                           const R rect[4], uint32_t max_iter, float max_ss, uint32_t flags, const R rect_reused[4],
                           const chaos_pixel_info *in, long in_pitch, uint32_t fx, uint32_t fy, int arith,
                           cudaStream_t s, bool sync)
{
    TraceRange trace_("fractalRenderAdvanced");
    if (!m || !rect || !rect_reused) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = check_size(w, h);
    if (rc) return rc;
    if ((rc = check_pitched(out, pitch, w, "output"))) return rc;
    if ((rc = check_pitched(in, in_pitch, w, "input"))) return rc;
    if (!finite4(rect) || !finite4(rect_reused)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "plane segments must be finite");
    if (max_iter < 1) return fail(CHAOS_ERR_INVALID_ARGUMENT, "maxIterations must be a positive number");
    if (!(max_ss > 0.f) || !std::isfinite(max_ss))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "maxSuperSampling must be > 0 (got %g)", (double)max_ss);
    const char *ib = reinterpret_cast<const char *>(in), *ob = reinterpret_cast<const char *>(out);
    if (ib < ob + (size_t)pitch * h && ob < ib + (size_t)in_pitch * h)
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "input and output buffers overlap");
    DeviceState *d;
    if ((rc = device_state(&d))) return rc;
    AdvancedArgs<R> a{};
    a.m.out = out;
    a.m.pitch = pitch;
    a.m.size = UInt2{w, h};
    a.m.image = Rect<R>{rect[0], rect[1], rect[2], rect[3]};
    a.m.max_iter = max_iter;
    a.m.max_ss = max_ss;
    a.m.flags = flags;
    a.m.jcx = m->julia_c[0];
    a.m.jcy = m->julia_c[1];
    a.m.newton = m->newton;
    a.m.tiles_x = (w + 7u) / 8u;
    a.m.n_tiles = a.m.tiles_x * ((h + 3u) / 4u);
    a.image_reused = Rect<R>{rect_reused[0], rect_reused[1], rect_reused[2], rect_reused[3]};
    a.in = in;
    a.in_pitch = in_pitch;
    a.focus = UInt2{fx, fy};
    if ((rc = take_counter(d, s, &a.m.counter))) return rc;
    return finish(launch_advanced<R>(a, arith_of(arith), m->fractal, d->sms, s), s, sync);
}

int chaos_render_main_f32(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                          const float rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                          int arith, void *stream)
{
    return render_main<float>(m, out, pitch, width, height, rect, max_iterations, max_super_sampling, flags, arith,
                              (cudaStream_t)stream, true);
}

int chaos_render_main_f64(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                          const double rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                          int arith, void *stream)
{
    return render_main<double>(m, out, pitch, width, height, rect, max_iterations, max_super_sampling, flags, arith,
                               (cudaStream_t)stream, true);
}

int chaos_render_advanced_f32(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                              const float rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                              const float rect_reused[4], const chaos_pixel_info *in, long in_pitch, uint32_t focus_x,
                              uint32_t focus_y, int arith, void *stream)
{
    return render_advanced<float>(m, out, pitch, width, height, rect, max_iterations, max_super_sampling, flags,
                                  rect_reused, in, in_pitch, focus_x, focus_y, arith, (cudaStream_t)stream, true);
}

int chaos_render_advanced_f64(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                              const double rect[4], uint32_t max_iterations, float max_super_sampling, uint32_t flags,
                              const double rect_reused[4], const chaos_pixel_info *in, long in_pitch,
                              uint32_t focus_x, uint32_t focus_y, int arith, void *stream)
{
    return render_advanced<double>(m, out, pitch, width, height, rect, max_iterations, max_super_sampling, flags,
                                   rect_reused, in, in_pitch, focus_x, focus_y, arith, (cudaStream_t)stream, true);
}

static int compose_impl(chaos_module *m, const chaos_pixel_info *in, long pitch, uint32_t *out, long out_pitch,
                        uint32_t w, uint32_t h, const uint32_t *palette, uint32_t palette_len, float max_ss,
                        cudaStream_t s, bool sync)
{
    TraceRange trace_("compose");
    if (!m) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL module");
    int rc = check_size(w, h);
    if (rc) return rc;
    if ((rc = check_pitched(in, pitch, w, "input"))) return rc;
    if (!out || out_pitch < (long)(4u * w) || ((uintptr_t)out & 3u) || (out_pitch & 3))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "bad output buffer");
    const bool roots_only = m->fractal == FRACTAL_NEWTON_WIRED || m->fractal == FRACTAL_NEWTON_GENERIC;
    if (!m->visualize && !roots_only && (!palette || palette_len == 0))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "palette required (length > 0)");
    ComposeArgs a{};
    a.in = in;
    a.pitch = pitch;
    a.out = out;
    a.out_pitch = out_pitch;
    a.w = w;
    a.h = h;
    a.palette = palette;
    a.palette_len = palette_len;
    a.max_ss = max_ss;
    a.visualize = m->visualize;
    a.color_mode = m->fractal == FRACTAL_NEWTON_WIRED || m->fractal == FRACTAL_NEWTON_GENERIC ? COLOR_ROOTS
                   : m->fractal == FRACTAL_NEWTON_ITERATIONS                                 ? COLOR_MAGNIFIED
                                                                                              : COLOR_PALETTE;
    a.magnifier = m->newton.color_magnifier;
    return finish(launch_compose(a, s), s, sync);
}

int chaos_compose(chaos_module *m, const chaos_pixel_info *in, long pitch, uint32_t *out_rgba, long out_pitch,
                  uint32_t width, uint32_t height, const uint32_t *palette, uint32_t palette_len,
                  float max_super_sampling, void *stream)
{
    return compose_impl(m, in, pitch, out_rgba, out_pitch, width, height, palette, palette_len, max_super_sampling,
                        (cudaStream_t)stream, true);
}

int chaos_render_under_sampled(chaos_module *m, chaos_pixel_info *out, long pitch, uint32_t width, uint32_t height,
                               const float rect[4], uint32_t max_iterations, uint32_t level, void *stream)
{
    if (!m || !rect) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = check_size(width, height);
    if (rc) return rc;
    if ((rc = check_pitched(out, pitch, width, "output"))) return rc;
    if (level < 1) return fail(CHAOS_ERR_INVALID_ARGUMENT, "underSamplingLevel must be at least 1, current value: %u", level);
    if (!finite4(rect)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "plane segment must be finite");
    cudaStream_t s = (cudaStream_t)stream;
    const Rect<float> r{rect[0], rect[1], rect[2], rect[3]};
    if (m->fractal >= FRACTAL_NEWTON_WIRED)
        return finish(
            launch_under_sampled_newton(out, pitch, width, height, r, max_iterations, level, m->fractal, m->newton, s),
            s, true);
    return finish(launch_under_sampled(out, pitch, width, height, r, max_iterations, level, m->fractal,
                                       m->julia_c[0], m->julia_c[1], s),
                  s, true);
}

int chaos_debug(chaos_module *m)
{
    if (!m) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL module");
    return finish(launch_debug(m->fractal, 0), 0, true);
}

int chaos_select_precision(const double rect[4], uint32_t width, uint32_t height)
{
    if (!rect || width == 0 || height == 0) return CHAOS_PRECISION_DOUBLE;
    double pw = std::fabs(rect[2] - rect[0]) / (double)width;
    double ph = std::fabs(rect[3] - rect[1]) / (double)height;
    int p = CHAOS_PRECISION_SINGLE;
    if (pw < float_ulp((float)rect[0]) || ph < float_ulp((float)rect[1])) p = CHAOS_PRECISION_DOUBLE;
    if (pw < double_ulp(rect[0]) || ph < double_ulp(rect[1])) p = CHAOS_PRECISION_TOO_BIG;
    return p;
}

// ---- frames ---------------------------------------------------------------

// `status_used` (may be NULL): where an unsynchronised call with a time
// limit and no out->status reports the status word it gave the kernel.
template <class R>
static int frame_impl(const chaos_frame_desc *dsc, const chaos_frame_out *o, cudaStream_t s, bool sync,
                      uint32_t **status_used)
{
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    FrameArgs<R> a{};
    a.w = dsc->width;
    a.h = dsc->height;
    a.spp = dsc->samples_per_pixel;
    a.mode = dsc->sample_mode;
    a.max_iter = dsc->max_iterations;
    a.n_pix = dsc->width * dsc->height;
    a.seed = dsc->seed;
    a.center_x = (R)dsc->center_x;
    a.center_y = (R)dsc->center_y;
    a.ps = (R)dsc->pixel_size;
    a.half_w = (R)(0.5 * dsc->width);
    a.half_h = (R)(0.5 * dsc->height);
    a.jcx = (R)dsc->julia_cx;
    a.jcy = (R)dsc->julia_cy;
    a.counts = o->counts;
    a.smooth = o->smooth;
    a.pixels = reinterpret_cast<PixelInfo *>(o->pixels);
    a.pixels_pitch = o->pixels_pitch;
    a.rgba = o->rgba;
    a.palette = o->palette;
    a.palette_len = o->palette_len;
    a.interior_rgba = o->interior_rgba;
    a.total = o->total_iterations;
    a.skipped = o->cycle_skipped;
    budget_of(dsc->time_limit_s, &a.budget_ns);
    if ((rc = take_counter(d, s, &a.counter))) return rc;
    a.status = o->status;
    if (a.budget_ns && !a.status) {
        if (!sync && !status_used)
            return fail(CHAOS_ERR_INVALID_ARGUMENT, "a time limit on an unsynchronised frame needs out->status");
        if ((rc = take_status(d, a.counter, s, &a.status))) return rc;
    }
    if (status_used) *status_used = a.budget_ns ? a.status : nullptr;
    if ((rc = finish(launch_frame<R>(a, arith_of(dsc->arith), (int)dsc->fractal, d->sms, s), s, sync))) return rc;
    return sync && a.budget_ns ? read_status(a.status, s, dsc->time_limit_s) : CHAOS_OK;
}

static int frame_entry(const chaos_frame_desc *dsc, const chaos_frame_out *o, cudaStream_t s, bool sync,
                       uint32_t **status_used = nullptr)
{
    if (!dsc || !o) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    int rc = check_size(dsc->width, dsc->height);
    if (rc) return rc;
    if (dsc->samples_per_pixel < 1 || dsc->samples_per_pixel > 64)
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "samples_per_pixel must be 1..64");
    if (dsc->sample_mode == CHAOS_SAMPLES_CENTER && dsc->samples_per_pixel != 1)
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "pixel-centre sampling takes one sample per pixel");
    if (dsc->sample_mode > CHAOS_SAMPLES_JITTER) return fail(CHAOS_ERR_INVALID_ARGUMENT, "unknown sample mode");
    if (dsc->fractal > 1) return fail(CHAOS_ERR_UNKNOWN_FRACTAL, "unknown fractal id %u", dsc->fractal);
    if (!std::isfinite(dsc->center_x) || !std::isfinite(dsc->center_y) || !(dsc->pixel_size > 0) ||
        !std::isfinite(dsc->pixel_size))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "centre and pixel size must be finite, pixel size > 0");
    if ((uint64_t)dsc->width * dsc->height * dsc->samples_per_pixel > (1ull << 32))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "too many samples");
    if (o->pixels && (rc = check_pitched(o->pixels, o->pixels_pitch, dsc->width, "pixels"))) return rc;
    if (o->rgba && (!o->palette || o->palette_len == 0))
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "rgba output needs a palette");
    if (dsc->arith != CHAOS_ARITH_FMA && dsc->arith != CHAOS_ARITH_PARITY)
        return fail(CHAOS_ERR_UNSUPPORTED, "frames take CHAOS_ARITH_FMA or CHAOS_ARITH_PARITY");
    unsigned long long ns = 0;
    if (!budget_of(dsc->time_limit_s, &ns)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "time_limit_s must be >= 0");
    if (dsc->tier == CHAOS_TIER_F32) return frame_impl<float>(dsc, o, s, sync, status_used);
    if (dsc->tier == CHAOS_TIER_F64) return frame_impl<double>(dsc, o, s, sync, status_used);
    return fail(CHAOS_ERR_UNSUPPORTED, "unknown tier %u", dsc->tier);
}

int chaos_render_frame_async(const chaos_frame_desc *desc, const chaos_frame_out *out, void *stream)
{
    TraceRange trace_("chaos_render_frame");
    return frame_entry(desc, out, (cudaStream_t)stream, false);
}

int chaos_render_frame(const chaos_frame_desc *desc, const chaos_frame_out *out, void *stream)
{
    TraceRange trace_("chaos_render_frame");
    return frame_entry(desc, out, (cudaStream_t)stream, true);
}

namespace {
// Per-thread device buffers of chaos_render_frame_host.
struct HostFrameWorkspace {
    int device = -1;
    uint32_t *rgba = nullptr;
    size_t rgba_words = 0;
    uint32_t *palette = nullptr;
    size_t palette_words = 0;
    unsigned long long *total = nullptr;
    ~HostFrameWorkspace()
    {
        // the CUDA context may already be gone at thread exit; errors are ignored
        if (rgba) cudaFree(rgba);
        if (palette) cudaFree(palette);
        if (total) cudaFree(total);
    }
};
thread_local HostFrameWorkspace g_host_ws;

int grow(uint32_t **p, size_t *have, size_t need)
{
    if (*have >= need) return CHAOS_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, need * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(frame workspace)");
    *have = need;
    return CHAOS_OK;
}
}  // namespace

int chaos_render_frame_host(const chaos_frame_desc *desc, const uint32_t *palette, uint32_t palette_len,
                            uint32_t interior_rgba, uint32_t *rgba_host, unsigned long long *total_host, void *stream)
{
    TraceRange trace_("chaos_render_frame_host");
    if (!desc || !palette || palette_len == 0 || !rgba_host)
        return fail(CHAOS_ERR_INVALID_ARGUMENT, "desc, palette and rgba_host are required");
    int rc = check_size(desc->width, desc->height);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    HostFrameWorkspace &ws = g_host_ws;
    int dev = 0;
    CHAOS_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (ws.device != dev) {  // buffers belong to one device; start over on another
        if (ws.rgba) cudaFree(ws.rgba);
        if (ws.palette) cudaFree(ws.palette);
        if (ws.total) cudaFree(ws.total);
        ws.rgba = ws.palette = nullptr;
        ws.total = nullptr;
        ws.rgba_words = ws.palette_words = 0;
        ws.device = dev;
    }
    size_t n = (size_t)desc->width * desc->height;
    if ((rc = grow(&ws.rgba, &ws.rgba_words, n))) return rc;
    if ((rc = grow(&ws.palette, &ws.palette_words, palette_len))) return rc;
    if (!ws.total) CHAOS_CUDA(cudaMalloc(&ws.total, sizeof(unsigned long long)), "cudaMalloc(total)");
    CHAOS_CUDA(cudaMemcpyAsync(ws.palette, palette, palette_len * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
               "cudaMemcpyAsync(palette)");
    CHAOS_CUDA(cudaMemsetAsync(ws.total, 0, sizeof(unsigned long long), s), "cudaMemsetAsync(total)");
    chaos_frame_out o{};
    o.rgba = ws.rgba;
    o.palette = ws.palette;
    o.palette_len = palette_len;
    o.interior_rgba = interior_rgba;
    o.total_iterations = ws.total;
    uint32_t *status = nullptr;
    if ((rc = frame_entry(desc, &o, s, false, &status))) return rc;
    CHAOS_CUDA(cudaMemcpyAsync(rgba_host, ws.rgba, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
               "cudaMemcpyAsync(rgba)");
    unsigned long long total = 0;
    CHAOS_CUDA(cudaMemcpyAsync(&total, ws.total, sizeof total, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(total)");
    CHAOS_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (total_host) *total_host = total;
    return status ? read_status(status, s, desc->time_limit_s) : CHAOS_OK;
}

int chaos_measure_fma_peak(uint32_t tier, double *flops_per_second)
{
    if (!flops_per_second || tier > CHAOS_TIER_F64) return fail(CHAOS_ERR_INVALID_ARGUMENT, "bad argument");
    DeviceState *d;
    int rc = device_state(&d);
    if (rc) return rc;
    const bool dbl = tier == CHAOS_TIER_F64;
    const int blocks = d->sms * 8;  // 2048 threads per SM
    double *sink = nullptr;
    CHAOS_CUDA(cudaMalloc(&sink, sizeof(double)), "cudaMalloc(sink)");
    cudaEvent_t a = nullptr, b = nullptr;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    uint32_t iters = dbl ? (1u << 12) : (1u << 16);
    float ms = 0.f;
    cudaError_t e = cudaSuccess;
    for (int round = 0; round < 8 && e == cudaSuccess; round++) {  // grow until a launch takes >= 50 ms
        e = launch_fma_peak(dbl, blocks, iters, sink, 0);
        if (e == cudaSuccess) e = cudaEventRecord(a, 0);
        if (e == cudaSuccess) e = launch_fma_peak(dbl, blocks, iters, sink, 0);
        if (e == cudaSuccess) e = cudaEventRecord(b, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (ms >= 50.f) break;
        iters *= 4;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(e, "fma peak probe");
    double flops = (double)blocks * 256.0 * (double)iters * 8.0 * 2.0;
    *flops_per_second = flops / (ms * 1e-3);
    return CHAOS_OK;
}


// ---- renderer -------------------------------------------------------------

struct chaos_renderer {
    chaos_module *m = nullptr;
    bool initialized = false;
    uint32_t w = 0, h = 0;
    PixelInfo *buf[2] = {nullptr, nullptr};
    size_t pitch[2] = {0, 0};
    bool switched = false;
    bool primary_dirty = true;
    uint32_t *rgba = nullptr;
    size_t rgba_pitch = 0;
    uint32_t *palette = nullptr;
    uint32_t palette_len = 0;
    bool has_last = false;
    chaos_rendering_model last{};
};

namespace {

void free_renderer_memory(chaos_renderer *r)
{
    for (int k = 0; k < 2; k++) {
        if (r->buf[k]) cudaFree(r->buf[k]);
        r->buf[k] = nullptr;
    }
    if (r->rgba) cudaFree(r->rgba);
    if (r->palette) cudaFree(r->palette);
    r->rgba = nullptr;
    r->palette = nullptr;
}

// DeviceMemoryDoubleBuffer2D.switch2DBuffers / resetBufferOrder (:78-95)
void switch_buffers(chaos_renderer *r)
{
    std::swap(r->buf[0], r->buf[1]);
    std::swap(r->pitch[0], r->pitch[1]);
    r->switched = !r->switched;
}

uint32_t main_flags(const chaos_rendering_model *m)  // KernelMain.setParamsFromModel
{
    uint32_t f = 0;
    if (m->use_adaptive_super_sampling) f |= CHAOS_FLAG_ADAPTIVE_SS;
    if (m->visualise_sample_count) f |= CHAOS_FLAG_VISUALIZE_SAMPLE_COUNT;
    return f;
}

uint32_t advanced_flags(const chaos_rendering_model *m)  // KernelAdvanced.setParamsFromModel
{
    uint32_t f = main_flags(m);
    if (m->use_foveated_rendering) f |= CHAOS_FLAG_FOVEATION;
    if (m->use_sample_reuse) f |= CHAOS_FLAG_SAMPLE_REUSE;
    if (m->zooming) f |= CHAOS_FLAG_IS_ZOOMING;
    if (m->zooming_in) f |= CHAOS_FLAG_ZOOMING_IN;
    return f;
}

int check_model(const chaos_rendering_model *m)
{
    double rect[4] = {m->left_bottom_x, m->left_bottom_y, m->right_top_x, m->right_top_y};
    if (!finite4(rect)) return fail(CHAOS_ERR_INVALID_ARGUMENT, "Argument segment must be a finite float");
    if (m->max_iterations < 1) return fail(CHAOS_ERR_INVALID_ARGUMENT, "maxIterations must be a positive number");
    return CHAOS_OK;
}

int compose_output(chaos_renderer *r, const chaos_rendering_model *model)
{
    return compose_impl(r->m, reinterpret_cast<const chaos_pixel_info *>(r->buf[0]), (long)r->pitch[0], r->rgba,
                        (long)r->rgba_pitch, r->w, r->h, r->palette, r->palette_len, model->max_super_sampling, 0,
                        true);
}

}  // namespace


int chaos_renderer_create(chaos_module *m, chaos_renderer **out)
{
    if (!m || !out) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    chaos_renderer *r = new (std::nothrow) chaos_renderer();
    if (!r) return fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
    r->m = m;
    *out = r;
    return CHAOS_OK;
}

int chaos_renderer_initialize(chaos_renderer *r, uint32_t width, uint32_t height, const uint32_t *palette,
                              uint32_t palette_len)
{
    if (!r) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL renderer");
    if (r->initialized) return fail(CHAOS_ERR_STATE, "Already initialized.");
    int rc = check_size(width, height);
    if (rc) return rc;
    if (!palette || palette_len == 0) return fail(CHAOS_ERR_INVALID_ARGUMENT, "palette required");
    r->w = width;
    r->h = height;
    for (int k = 0; k < 2; k++) {
        cudaError_t e = cudaMallocPitch(&r->buf[k], &r->pitch[k], 16u * (size_t)width, height);
        if (e != cudaSuccess) {
            free_renderer_memory(r);
            return cuda_fail(e, "cudaMallocPitch(sample-reuse buffer)");
        }
    }
    cudaError_t e = cudaMallocPitch(&r->rgba, &r->rgba_pitch, 4u * (size_t)width, height);
    if (e == cudaSuccess) e = cudaMalloc(&r->palette, 4u * (size_t)palette_len);
    if (e == cudaSuccess) e = cudaMemcpy(r->palette, palette, 4u * (size_t)palette_len, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_renderer_memory(r);
        return cuda_fail(e, "renderer allocation");
    }
    r->palette_len = palette_len;
    r->switched = false;
    r->primary_dirty = true;
    r->has_last = false;
    r->initialized = true;
    return CHAOS_OK;
}

int chaos_renderer_free_resources(chaos_renderer *r)
{
    if (!r) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL renderer");
    if (!r->initialized) return fail(CHAOS_ERR_STATE, "Already free.");
    free_renderer_memory(r);
    r->initialized = false;
    return CHAOS_OK;
}

int chaos_renderer_render_quality(chaos_renderer *r, chaos_rendering_model *model)
{
    TraceRange trace_("renderQuality");
    if (!r || !model) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!r->initialized) return fail(CHAOS_ERR_STATE, "Renderer has to be initialized first");
    int rc = check_model(model);
    if (rc) return rc;
    r->m->visualize = model->visualise_sample_count != 0;  // setModuleConstants
    double rect[4] = {model->left_bottom_x, model->left_bottom_y, model->right_top_x, model->right_top_y};
    int prec = chaos_select_precision(rect, r->w, r->h);
    model->floating_point_precision = prec;
    if (r->switched) switch_buffers(r);  // memory.resetBufferOrder()
    uint32_t flags = main_flags(model);
    if (prec == CHAOS_PRECISION_SINGLE) {
        float rf[4] = {(float)rect[0], (float)rect[1], (float)rect[2], (float)rect[3]};
        rc = render_main<float>(r->m, reinterpret_cast<chaos_pixel_info *>(r->buf[0]), (long)r->pitch[0], r->w, r->h,
                                rf, model->max_iterations, model->max_super_sampling, flags, model->arith, 0, true);
    } else {
        rc = render_main<double>(r->m, reinterpret_cast<chaos_pixel_info *>(r->buf[0]), (long)r->pitch[0], r->w,
                                 r->h, rect, model->max_iterations, model->max_super_sampling, flags, model->arith, 0,
                                 true);
    }
    if (rc) return rc;
    if ((rc = compose_output(r, model))) return rc;
    r->last = *model;
    r->has_last = true;
    r->primary_dirty = false;
    model->sample_reuse_cache_dirty = 0;
    return CHAOS_OK;
}

int chaos_renderer_render_fast(chaos_renderer *r, chaos_rendering_model *model)
{
    TraceRange trace_("renderFast");
    if (!r || !model) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!r->initialized) return fail(CHAOS_ERR_STATE, "Renderer has to be initialized first");
    int rc = check_model(model);
    if (rc) return rc;
    r->m->visualize = model->visualise_sample_count != 0;
    if (model->sample_reuse_cache_dirty || r->primary_dirty || !r->has_last)
        return chaos_renderer_render_quality(r, model);
    double rect[4] = {model->left_bottom_x, model->left_bottom_y, model->right_top_x, model->right_top_y};
    double old[4] = {r->last.left_bottom_x, r->last.left_bottom_y, r->last.right_top_x, r->last.right_top_y};
    int prec = chaos_select_precision(rect, r->w, r->h);
    model->floating_point_precision = prec;
    uint32_t flags = advanced_flags(model);
    uint32_t fx = (uint32_t)model->mouse_focus_x, fy = (uint32_t)model->mouse_focus_y;
    chaos_pixel_info *out = reinterpret_cast<chaos_pixel_info *>(r->buf[1]);
    const chaos_pixel_info *in = reinterpret_cast<const chaos_pixel_info *>(r->buf[0]);
    if (prec == CHAOS_PRECISION_SINGLE) {
        float rf[4] = {(float)rect[0], (float)rect[1], (float)rect[2], (float)rect[3]};
        float of[4] = {(float)old[0], (float)old[1], (float)old[2], (float)old[3]};
        rc = render_advanced<float>(r->m, out, (long)r->pitch[1], r->w, r->h, rf, model->max_iterations,
                                    model->max_super_sampling, flags, of, in, (long)r->pitch[0], fx, fy, model->arith,
                                    0, true);
    } else {
        rc = render_advanced<double>(r->m, out, (long)r->pitch[1], r->w, r->h, rect, model->max_iterations,
                                     model->max_super_sampling, flags, old, in, (long)r->pitch[0], fx, fy,
                                     model->arith, 0, true);
    }
    if (rc) return rc;
    switch_buffers(r);
    if ((rc = compose_output(r, model))) return rc;
    r->last = *model;
    return CHAOS_OK;
}

int chaos_renderer_output(const chaos_renderer *r, const uint32_t **rgba, long *rgba_pitch,
                          const chaos_pixel_info **primary, long *primary_pitch)
{
    if (!r) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL renderer");
    if (!r->initialized) return fail(CHAOS_ERR_STATE, "Renderer has to be initialized first");
    if (rgba) *rgba = r->rgba;
    if (rgba_pitch) *rgba_pitch = (long)r->rgba_pitch;
    if (primary) *primary = reinterpret_cast<const chaos_pixel_info *>(r->buf[0]);
    if (primary_pitch) *primary_pitch = (long)r->pitch[0];
    return CHAOS_OK;
}

int chaos_renderer_read_output(const chaos_renderer *r, uint32_t *host_rgba)
{
    if (!r || !host_rgba) return fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!r->initialized) return fail(CHAOS_ERR_STATE, "Renderer has to be initialized first");
    CHAOS_CUDA(cudaMemcpy2D(host_rgba, 4u * (size_t)r->w, r->rgba, r->rgba_pitch, 4u * (size_t)r->w, r->h,
                            cudaMemcpyDeviceToHost),
               "cudaMemcpy2D(output)");
    return CHAOS_OK;
}

int chaos_renderer_destroy(chaos_renderer *r)
{
    if (!r) return CHAOS_OK;
    if (r->initialized) free_renderer_memory(r);
    delete r;
    return CHAOS_OK;
}

