// chaos_serve.cu -- serving concurrent zoom sessions.
//
// A server holds sessions.  Each session is one viewer zooming toward a
// target: its reuse buffers (two pitched pixel_info_t arrays), its RGBA8
// output, its work counter and its pixel-iteration counter stay on the device
// for the session's lifetime, and the session owns one CUDA stream.  Opening
// a session is admitted against the server's HBM budget (the bytes it will
// hold); a session that does not fit is refused with CHAOS_ERR_OUT_OF_MEMORY
// and allocates nothing.
//
// A frame request enqueues, on the session's stream, the reference renderer's
// frame: renderQuality for the first frame (fractalRenderMain + compose),
// renderFast afterwards (fractalRenderAdvanced reusing the previous frame,
// buffer swap, compose) -- the call sequence of
// J/cudarenderer/CudaFractalRenderer.java:159-206 -- and a host callback that
// stamps the completion time.  Requests return at once, so frames of different
// sessions that arrive while others run are on the GPU together (continuous
// batching: their persistent kernels share the SMs as blocks retire), while a
// session's own frames stay in order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "chaos_kernels.cuh"

namespace chaos {
int api_fail(int code, const char *fmt, ...);  // chaos_api.cu
int api_orbit_create_d(double center_x, double center_y, uint32_t bits, uint32_t max_iterations,
                       chaos_orbit **out);  // chaos_perturb.cu
int api_perturb_enqueue(const chaos_frame_desc *desc, const chaos_orbit *orbit, const chaos_frame_out *out,
                        cudaStream_t stream, uint32_t *counter);  // chaos_perturb.cu
}
using namespace chaos;

namespace {

using Clock = std::chrono::steady_clock;

struct FrameRecord {
    uint32_t session = 0, frame = 0;
    double arrival = 0, start = 0;
    std::atomic<double> done{-1.0};
    int32_t precision = 0;
    struct chaos_server *server = nullptr;
};

struct Session {
    chaos_session_desc d{};
    bool open = false;
    cudaStream_t stream = nullptr;
    PixelInfo *buf[2] = {nullptr, nullptr};
    size_t pitch[2] = {0, 0};
    uint32_t *rgba = nullptr;
    size_t rgba_pitch = 0;
    uint32_t *counter = nullptr;
    unsigned long long *iters = nullptr;
    size_t bytes = 0;
    bool has_prev = false;
    double prev_rect[4] = {0, 0, 0, 0};
    double cx = 0, cy = 0, span = 0;
    double off_x = 0, off_y = 0;  // frame centre - target, zoomed alongside (deep frames)
    chaos_orbit *orbit = nullptr;  // reference orbit of the target, once frames go past binary64
    uint32_t orbit_bits = 0;
    uint32_t frames = 0;
};

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

size_t session_bytes(const chaos_session_desc &d)
{
    return 2 * round_up(16 * (size_t)d.width, 512) * d.height + round_up(4 * (size_t)d.width, 512) * d.height + 4096;
}

void rect_of(const Session &s, double r[4])
{
    double hw = 0.5 * s.span, hh = 0.5 * s.span * (double)s.d.height / (double)s.d.width;
    r[0] = s.cx - hw;
    r[1] = s.cy - hh;
    r[2] = s.cx + hw;
    r[3] = s.cy + hh;
}

void free_session(Session &s)
{
    if (s.stream) cudaStreamSynchronize(s.stream);
    for (int k = 0; k < 2; k++)
        if (s.buf[k]) cudaFree(s.buf[k]);
    if (s.rgba) cudaFree(s.rgba);
    if (s.counter) cudaFree(s.counter);
    if (s.iters) cudaFree(s.iters);
    if (s.orbit) chaos_orbit_destroy(s.orbit);
    if (s.stream) cudaStreamDestroy(s.stream);
    s = Session();
}

}  // namespace

struct chaos_server {
    int device = -1;
    int sms = 0;
    size_t budget = 0, used = 0;
    uint32_t *palette = nullptr;
    uint32_t palette_len = 0;
    std::vector<Session> sessions;
    std::deque<FrameRecord> records;
    std::mutex mu;
    Clock::time_point t0 = Clock::now();
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

static void CUDART_CB frame_done(void *p)
{
    FrameRecord *r = static_cast<FrameRecord *>(p);
    r->done.store(r->server->now());
}

double chaos_server_clock(const chaos_server *s) { return s ? s->now() : 0.0; }

int chaos_server_create(size_t hbm_budget_bytes, const uint32_t *palette, uint32_t palette_len, chaos_server **out)
{
    if (!out || !palette || palette_len == 0 || palette_len > 4096)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "a host palette of 1..4096 entries is required");
    chaos_server *s = new (std::nothrow) chaos_server();
    if (!s) return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    s->budget = hbm_budget_bytes;
    cudaError_t e = cudaMalloc(&s->palette, palette_len * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(s->palette, palette, palette_len * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (s->palette) cudaFree(s->palette);
        delete s;
        return api_fail(CHAOS_ERR_CUDA, "server palette: %s", cudaGetErrorString(e));
    }
    s->palette_len = palette_len;
    *out = s;
    return CHAOS_OK;
}

int chaos_server_session_bytes(const chaos_session_desc *d, size_t *bytes)
{
    if (!d || !bytes) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    *bytes = session_bytes(*d);
    return CHAOS_OK;
}

int chaos_server_open(chaos_server *s, const chaos_session_desc *d, uint32_t *session)
{
    if (!s || !d || !session) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (d->width == 0 || d->height == 0 || (uint64_t)d->width * d->height > (1ull << 31))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "bad session size");
    if (d->max_iterations < 1 || !(d->max_super_sampling >= 1.f))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "maxIterations >= 1 and maxSuperSampling >= 1 required");
    if (!(d->span > 0) || !std::isfinite(d->span) || !std::isfinite(d->center_x) || !std::isfinite(d->center_y) ||
        !std::isfinite(d->target_x) || !std::isfinite(d->target_y) || !(d->zoom_per_frame >= 1.0))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "bad plane / zoom");
    if (d->fractal > 1) return api_fail(CHAOS_ERR_UNKNOWN_FRACTAL, "unknown fractal id %u", d->fractal);
    size_t bytes = session_bytes(*d);
    std::lock_guard<std::mutex> g(s->mu);
    if (s->used + bytes > s->budget)
        return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "session needs %zu bytes, %zu of %zu budget left", bytes,
                        s->budget - s->used, s->budget);
    Session ss;
    ss.d = *d;
    cudaError_t e = cudaStreamCreateWithFlags(&ss.stream, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; k++)
        e = cudaMallocPitch(&ss.buf[k], &ss.pitch[k], 16u * (size_t)d->width, d->height);
    if (e == cudaSuccess) e = cudaMallocPitch(&ss.rgba, &ss.rgba_pitch, 4u * (size_t)d->width, d->height);
    if (e == cudaSuccess) e = cudaMalloc(&ss.counter, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&ss.iters, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(ss.iters, 0, sizeof(unsigned long long), ss.stream);
    if (e != cudaSuccess) {
        free_session(ss);
        return api_fail(CHAOS_ERR_CUDA, "session allocation: %s", cudaGetErrorString(e));
    }
    ss.bytes = bytes;
    ss.open = true;
    ss.cx = d->center_x;
    ss.cy = d->center_y;
    ss.span = d->span;
    ss.off_x = d->center_x - d->target_x;
    ss.off_y = d->center_y - d->target_y;
    s->used += bytes;
    uint32_t id = 0;
    while (id < s->sessions.size() && s->sessions[id].open) id++;
    if (id == s->sessions.size()) s->sessions.push_back(Session());
    s->sessions[id] = ss;
    *session = id;
    return CHAOS_OK;
}

int chaos_server_close(chaos_server *s, uint32_t session)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    if (session >= s->sessions.size() || !s->sessions[session].open)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
    s->used -= s->sessions[session].bytes;
    free_session(s->sessions[session]);
    return CHAOS_OK;
}

template <class R>
static cudaError_t enqueue_frame(chaos_server *srv, Session &s, const double rect[4], bool fast, int prec)
{
    const chaos_session_desc &d = s.d;
    cudaError_t e = cudaMemsetAsync(s.counter, 0, sizeof(uint32_t), s.stream);
    if (e != cudaSuccess) return e;
    MainArgs<R> m{};
    m.size = UInt2{d.width, d.height};
    m.image = Rect<R>{(R)rect[0], (R)rect[1], (R)rect[2], (R)rect[3]};
    m.max_iter = d.max_iterations;
    m.max_ss = d.max_super_sampling;
    m.jcx = d.julia_cx;
    m.jcy = d.julia_cy;
    m.tiles_x = (d.width + 7u) / 8u;
    m.n_tiles = m.tiles_x * ((d.height + 3u) / 4u);
    m.counter = s.counter;
    m.total = s.iters;
    int arith = d.arith == CHAOS_ARITH_PARITY ? ARITH_PARITY : ARITH_FMA;
    (void)prec;
    if (!fast) {
        m.out = s.buf[0];
        m.pitch = (long)s.pitch[0];
        m.flags = d.flags & CHAOS_FLAG_ADAPTIVE_SS;  // KernelMain carries only the adaptive / visualise bits
        e = launch_main<R>(m, arith, (int)d.fractal, srv->sms, s.stream);
    } else {
        AdvancedArgs<R> a{};
        a.m = m;
        a.m.out = s.buf[1];
        a.m.pitch = (long)s.pitch[1];
        a.m.flags = d.flags | CHAOS_FLAG_IS_ZOOMING | CHAOS_FLAG_ZOOMING_IN;
        a.image_reused = Rect<R>{(R)s.prev_rect[0], (R)s.prev_rect[1], (R)s.prev_rect[2], (R)s.prev_rect[3]};
        a.in = s.buf[0];
        a.in_pitch = (long)s.pitch[0];
        // the zoom target's pixel is the viewer's focus (foveation centre)
        double fx = (d.target_x - rect[0]) / (rect[2] - rect[0]) * d.width;
        double fy = (rect[3] - d.target_y) / (rect[3] - rect[1]) * d.height;
        fx = std::min(std::max(fx, 0.0), (double)(d.width - 1));
        fy = std::min(std::max(fy, 0.0), (double)(d.height - 1));
        a.focus = UInt2{(uint32_t)fx, (uint32_t)fy};
        e = launch_advanced<R>(a, arith, (int)d.fractal, srv->sms, s.stream);
    }
    return e;
}

// A frame past binary64 (the reference stops there): perturbation around the
// session's target with binary64 differences, one sample per pixel centre, into
// the session's pixel buffer, then compose.  The target's reference orbit is
// computed once (again only when the zoom needs more bits) and stays resident
// with the session.  The frame centre sits at off from the target, which keeps
// its place on screen as the zoom goes on.
static int submit_deep_locked(chaos_server *srv, Session &s, uint32_t session, double arrival)
{
    const chaos_session_desc &d = s.d;
    const double ps = s.span / d.width;
    const uint32_t need = (uint32_t)std::min(1536.0, std::max(128.0, std::ceil((-std::log2(ps) + 96.0) / 64.0) * 64.0));
    if (!s.orbit || s.orbit_bits < need) {
        if (s.orbit) {
            cudaStreamSynchronize(s.stream);  // frames in flight still read it
            chaos_orbit_destroy(s.orbit);
            s.orbit = nullptr;
        }
        int rc = api_orbit_create_d(d.target_x, d.target_y, need, d.max_iterations, &s.orbit);
        if (rc != CHAOS_OK) return rc;
        s.orbit_bits = need;
    }
    srv->records.emplace_back();
    FrameRecord &r = srv->records.back();
    r.session = session;
    r.frame = s.frames;
    r.arrival = arrival;
    r.start = srv->now();
    r.precision = CHAOS_PRECISION_TOO_BIG;
    r.server = srv;
    chaos_frame_desc fd{};
    fd.width = d.width;
    fd.height = d.height;
    fd.max_iterations = d.max_iterations;
    fd.samples_per_pixel = 1;
    fd.sample_mode = CHAOS_SAMPLES_CENTER;
    fd.tier = CHAOS_TIER_PERTURB_F64;
    fd.center_x = s.off_x;
    fd.center_y = s.off_y;
    fd.pixel_size = ps;
    chaos_frame_out fo{};
    fo.pixels = reinterpret_cast<chaos_pixel_info *>(s.buf[0]);
    fo.pixels_pitch = (long)s.pitch[0];
    fo.total_iterations = s.iters;
    int rc = api_perturb_enqueue(&fd, s.orbit, &fo, s.stream, nullptr);
    if (rc != CHAOS_OK) {
        r.done.store(-2.0);
        return rc;
    }
    ComposeArgs c{};
    c.in = s.buf[0];
    c.pitch = (long)s.pitch[0];
    c.out = s.rgba;
    c.out_pitch = (long)s.rgba_pitch;
    c.w = d.width;
    c.h = d.height;
    c.palette = srv->palette;
    c.palette_len = srv->palette_len;
    c.max_ss = 1.f;
    c.visualize = false;
    cudaError_t e = launch_compose(c, s.stream);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(s.stream, frame_done, &r);
    if (e != cudaSuccess) {
        r.done.store(-2.0);
        return api_fail(CHAOS_ERR_CUDA, "frame enqueue: %s", cudaGetErrorString(e));
    }
    rect_of(s, s.prev_rect);
    s.has_prev = true;
    s.frames++;
    return CHAOS_OK;
}

static int submit_locked(chaos_server *srv, uint32_t session, double arrival)
{
    if (session >= srv->sessions.size() || !srv->sessions[session].open)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
    Session &s = srv->sessions[session];
    const chaos_session_desc &d = s.d;
    bool fast = s.has_prev;
    if (fast) {  // RenderingController.zoomAt: the target keeps its place on screen
        double z = d.zoom_per_frame;
        s.cx = d.target_x + (s.cx - d.target_x) / z;
        s.cy = d.target_y + (s.cy - d.target_y) / z;
        s.off_x /= z;
        s.off_y /= z;
        s.span /= z;
    }
    double rect[4];
    rect_of(s, rect);
    int prec = chaos_select_precision(rect, d.width, d.height);
    if (prec == CHAOS_PRECISION_TOO_BIG && d.fractal == 0 && s.span / d.width >= 1e-290)
        return submit_deep_locked(srv, s, session, arrival);
    srv->records.emplace_back();
    FrameRecord &r = srv->records.back();
    r.session = session;
    r.frame = s.frames;
    r.arrival = arrival;
    r.start = srv->now();
    r.precision = prec;
    r.server = srv;
    cudaError_t e = prec == CHAOS_PRECISION_SINGLE ? enqueue_frame<float>(srv, s, rect, fast, prec)
                                                   : enqueue_frame<double>(srv, s, rect, fast, prec);
    if (e == cudaSuccess && fast) {
        std::swap(s.buf[0], s.buf[1]);
        std::swap(s.pitch[0], s.pitch[1]);
    }
    if (e == cudaSuccess) {
        ComposeArgs c{};
        c.in = s.buf[0];
        c.pitch = (long)s.pitch[0];
        c.out = s.rgba;
        c.out_pitch = (long)s.rgba_pitch;
        c.w = d.width;
        c.h = d.height;
        c.palette = srv->palette;
        c.palette_len = srv->palette_len;
        c.max_ss = d.max_super_sampling;
        c.visualize = false;
        e = launch_compose(c, s.stream);
    }
    if (e == cudaSuccess) e = cudaLaunchHostFunc(s.stream, frame_done, &r);
    if (e != cudaSuccess) {
        r.done.store(-2.0);
        return api_fail(CHAOS_ERR_CUDA, "frame enqueue: %s", cudaGetErrorString(e));
    }
    std::copy(rect, rect + 4, s.prev_rect);
    s.has_prev = true;
    s.frames++;
    return CHAOS_OK;
}

int chaos_server_submit(chaos_server *s, uint32_t session, double arrival_s)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    return submit_locked(s, session, arrival_s);
}

int chaos_server_drain(chaos_server *s)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    for (Session &ss : s->sessions) {
        if (!ss.open) continue;
        cudaError_t e = cudaStreamSynchronize(ss.stream);
        if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "drain: %s", cudaGetErrorString(e));
    }
    return CHAOS_OK;
}

int chaos_server_run_trace(chaos_server *s, const uint32_t *sessions, const double *arrival_s, uint32_t n)
{
    if (!s || (n && (!sessions || !arrival_s))) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    const double base = s->now();
    for (uint32_t k = 0; k < n; k++) {
        const double due = base + arrival_s[k];
        for (;;) {  // sleep, then spin for the last 100 us
            double left = due - s->now();
            if (left <= 0) break;
            if (left > 2e-4)
                std::this_thread::sleep_for(std::chrono::duration<double>(left - 1e-4));
            else
                std::this_thread::yield();
        }
        int rc = chaos_server_submit(s, sessions[k], due);
        if (rc) return rc;
    }
    return chaos_server_drain(s);
}

int chaos_server_records(chaos_server *s, chaos_frame_record *out, uint32_t max, uint32_t *n)
{
    if (!s || !n) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> g(s->mu);
    uint32_t k = 0;
    for (const FrameRecord &r : s->records) {
        if (k >= max || !out) {
            k++;
            continue;
        }
        out[k].session = r.session;
        out[k].frame = r.frame;
        out[k].arrival_s = r.arrival;
        out[k].start_s = r.start;
        out[k].done_s = r.done.load();
        out[k].precision = r.precision;
        k++;
    }
    *n = k;
    return CHAOS_OK;
}

int chaos_server_read(chaos_server *s, uint32_t session, uint32_t *host_rgba, unsigned long long *pixel_iterations)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    if (session >= s->sessions.size() || !s->sessions[session].open)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
    Session &ss = s->sessions[session];
    cudaError_t e = cudaStreamSynchronize(ss.stream);
    if (e == cudaSuccess && host_rgba)
        e = cudaMemcpy2D(host_rgba, 4u * (size_t)ss.d.width, ss.rgba, ss.rgba_pitch, 4u * (size_t)ss.d.width,
                         ss.d.height, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && pixel_iterations)
        e = cudaMemcpy(pixel_iterations, ss.iters, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "read: %s", cudaGetErrorString(e));
    return CHAOS_OK;
}

int chaos_server_usage(const chaos_server *s, size_t *used, size_t *budget)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    if (used) *used = s->used;
    if (budget) *budget = s->budget;
    return CHAOS_OK;
}

int chaos_server_destroy(chaos_server *s)
{
    if (!s) return CHAOS_OK;
    for (Session &ss : s->sessions)
        if (ss.open) free_session(ss);
    if (s->palette) cudaFree(s->palette);
    delete s;
    return CHAOS_OK;
}
