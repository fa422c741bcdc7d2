// chaos_serve.cu -- serving concurrent zoom sessions with continuous batching.
//
// A server holds sessions.  Each session is one viewer zooming toward a
// target; its two pitched pixel_info_t reuse buffers, its RGBA8 image and its
// pixel-iteration counter are allocated when its first frame is admitted
// (against the server's HBM budget) and stay on the device until it closes,
// together with the target's reference orbit once the zoom passes binary64.
//
// Requests (chaos_server_submit) only enter a queue.  One scheduler thread
// per server owns all GPU work:
//   1. it reaps finished launches (their frames complete; slots free up; a
//      closing session whose last frame finished releases its buffers);
//   2. it admits queued requests in arrival order while frame slots are free
//      and memory fits, at most one frame per session per launch (a
//      session's frames stay in order), and expires requests that waited
//      past the wait limit;
//   3. it renders every admitted frame of all sessions in one launch: the
//      frame table goes to the device in one copy, one persistent kernel per
//      (precision, arithmetic, fractal, frame kind) present pulls strips of
//      8x4 tiles of all its frames from one work counter and composes each
//      pixel as it stores it (the kernels of one launch run side by side on
//      the launch slot's streams); perturbation frames and their compose
//      follow, and a host callback marks the launch's end.
// A frame completes as soon as the warp that finishes its last strip
// publishes it (a done word in host-mapped memory), not when its launch
// ends: the scheduler polls those words, so a small frame is not held back
// by a large one in the same launch.  A session's next frame is admitted
// once its previous frame has completed, into a new launch on another slot
// that runs beside the launches still on the GPU (continuous batching: new
// frames enter while others run, up to max_launches_in_flight launches).
//
// The frame sequence per session is the reference renderer's:
// renderQuality for the first frame (fractalRenderMain + compose), then
// renderFast (fractalRenderAdvanced reusing the previous frame, buffer swap,
// compose), J/cudarenderer/CudaFractalRenderer.java:159-206, with the zoom
// step of RenderingController.zoomAt (J/rendering/RenderingController.java:
// 130-150).
//
// Cancel and time limit: every kernel of a launch checks, per claimed strip
// of tiles, the frame's cancel word (host-mapped memory the host sets when a
// session closes; read one strip ahead so its latency hides behind the
// strip's work) and the launch's device-time budget (%globaltimer since the
// block started).  A stopped frame skips its remaining tiles and its status
// word records why; the host turns that into the frame record's status.
// Every host wait has a limit (call_timeout_s); no kernel waits on anything.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/chaos_gb300.h"
#include "chaos_refmode.cuh"
#include "chaos_trace.h"

namespace chaos {
int api_fail(int code, const char *fmt, ...);  // chaos_api.cu
int api_orbit_create_d(double center_x, double center_y, uint32_t bits, uint32_t max_iterations,
                       chaos_orbit **out);  // chaos_perturb.cu
int api_perturb_enqueue(const chaos_frame_desc *desc, const chaos_orbit *orbit, const chaos_frame_out *out,
                        cudaStream_t stream, uint32_t *counter);  // chaos_perturb.cu

// ---------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------

constexpr uint32_t SERVE_MAX_FRAMES = 256;  // frames per launch
constexpr uint32_t SERVE_GROUPS = 32;       // frame kind x precision x arithmetic x fractal

// Kernel group of a frame: ((renderFast * 2 + binary64) * 4 + arithmetic) * 2 + fractal.
__host__ __device__ constexpr uint32_t serve_group(bool adv, bool dbl, int arith, int fractal)
{
    return ((((adv ? 1u : 0u) * 2u + (dbl ? 1u : 0u)) * 4u + (uint32_t)arith) * 2u) + (uint32_t)fractal;
}
__host__ __device__ constexpr bool group_binary64(uint32_t g) { return (g / 8u) % 2u == 1u; }
constexpr uint32_t SERVE_STATUS_CANCELLED = 1u, SERVE_STATUS_TIMEOUT = 2u;

template <class R> struct ServeFrame {
    AdvancedArgs<R> a;               // frame parameters (a.in etc. for renderFast frames)
    uint32_t advanced;               // 1: fractalRenderAdvanced, 0: fractalRenderMain
    uint32_t slot;                   // the frame's index in the launch (status, done words)
    uint32_t chunk;                  // tiles per job
    uint32_t n_jobs;                 // jobs of this frame
    const volatile uint32_t *cancel; // host-mapped; nonzero stops the frame
    uint32_t *rgba;                  // the frame's image, composed tile by tile
    long rgba_pitch;
    float compose_max_ss;
    uint32_t pad_;
};

// Everything a launch sends to the device, copied in one piece.  Jobs of a
// kernel: job_begin[g][f] .. job_begin[g][f+1] are frame f of group g.
struct ServeTable {
    ServeFrame<float> f32[SERVE_MAX_FRAMES];   // binary32 frames, grouped
    ServeFrame<double> f64[SERVE_MAX_FRAMES];  // binary64 frames, grouped
    uint32_t job_begin[SERVE_GROUPS][SERVE_MAX_FRAMES + 1];
    ComposeArgs compose[SERVE_MAX_FRAMES];     // perturbation frames (composed after their kernel)
    uint32_t compose_begin[SERVE_MAX_FRAMES + 1];
    uint32_t counters[32];                     // one work counter per kernel (zero on arrival)
    uint32_t status[SERVE_MAX_FRAMES];         // SERVE_STATUS_* bits per frame (zero on arrival)
    uint32_t jobs_done[SERVE_MAX_FRAMES];      // finished jobs per frame (zero on arrival)
};

__device__ __forceinline__ uint32_t find_frame(const uint32_t *begin, uint32_t n, uint32_t job)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (begin[mid] <= job)
            lo = mid;
        else
            hi = mid - 1u;
    }
    return lo;
}

// Tiles of every frame of one group (ADV: renderFast frames, else
// renderQuality frames).  A job is a strip of `chunk` tiles of one frame
// (chunk > 1 for large frames, whose reuse tiles take few loads each); the
// next job is claimed while this one renders.  Each pixel is composed into
// the frame's RGBA8 image as soon as its record is stored (compose is
// per pixel, gen.cu:455-475), and the warp that finishes a frame's last job
// publishes the frame: a system-scope fence, then the frame's done word in
// host-mapped memory (1 | status << 8), so the host completes frames one by
// one while the launch goes on.
template <class R, int A, int F, bool ADV>
__global__ void __launch_bounds__(PERSIST_THREADS)
    k_serve(const ServeFrame<R> *__restrict__ frames, const uint32_t *__restrict__ job_begin, uint32_t n_frames,
            uint32_t *counter, uint32_t *status, uint32_t *jobs_done, volatile uint32_t *done_words,
            unsigned long long *const *totals, unsigned long long budget_ns, const uint32_t *palette,
            uint32_t palette_len)
{
    __shared__ uint32_t s_pal[4096];
    __shared__ uint32_t s_begin[SERVE_MAX_FRAMES + 1];
    for (uint32_t k = threadIdx.x; k <= n_frames; k += blockDim.x) s_begin[k] = job_begin[k];
    for (uint32_t k = threadIdx.x; k < palette_len; k += blockDim.x) s_pal[k] = palette[k];
    __syncthreads();
    const uint32_t n_jobs = s_begin[n_frames];
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long t0 = global_ns();
    uint32_t cur = 0xffffffffu;  // frame of the previous job
    uint32_t seen = 0;           // cancel word of frame `cur` read one job ago
    bool stopped = false;
    uint32_t claim = 0;
    if (lane == 0) claim = atomicAdd(counter, 1u);
    for (;;) {
        const uint32_t job = __shfl_sync(FULL, claim, 0);
        if (job >= n_jobs) break;
        const uint32_t f = find_frame(s_begin, n_frames, job);
        const ServeFrame<R> &fr = frames[f];
        if (f != cur) {
            cur = f;
            seen = 0;
            stopped = false;
        }
        uint32_t stop = 0;
        if (lane == 0) {
            if (seen)
                stop = SERVE_STATUS_CANCELLED;
            else if (budget_ns && global_ns() - t0 > budget_ns)
                stop = SERVE_STATUS_TIMEOUT;
            if (stop && !stopped) atomicOr(&status[fr.slot], stop);
            seen = fr.cancel ? *fr.cancel : 0u;  // used at the next job of this frame
            claim = atomicAdd(counter, 1u);
        }
        stop = __shfl_sync(FULL, stop, 0);
        unsigned long long iters = 0;
        if (stop) {
            stopped = true;
        } else {
            SampleGeometry<R> g = make_geometry(fr.a.m.image, fr.a.m.size, fr.a.m.max_iter, fr.a.m.jcx, fr.a.m.jcy);
            const uint32_t t_first = (job - s_begin[f]) * fr.chunk;
            const uint32_t t_end = min(t_first + fr.chunk, fr.a.m.n_tiles);
            TileCursor c(t_first, fr.a.m.tiles_x);
            for (uint32_t t = t_first; t < t_end; t++, c.next(fr.a.m.tiles_x)) {
                const uint32_t x0 = c.x0(), y0 = c.y0();
                PixelInfo rec;
                if constexpr (ADV)
                    rec = render_advanced_tile<R, A, F>(g, fr.a.m.image, fr.a.image_reused, fr.a.m.out, fr.a.m.pitch,
                                                        fr.a.m.size, fr.a.in, fr.a.in_pitch, fr.a.focus, x0, y0, lane,
                                                        fr.a.m.max_ss, fr.a.m.flags, iters);
                else
                    rec = render_main_tile<R, A, F>(g, fr.a.m.out, fr.a.m.pitch, fr.a.m.size, x0, y0, lane,
                                                    fr.a.m.max_ss, fr.a.m.flags, iters);
                const UInt2 p = tile_pixel(x0, y0, lane);
                if (p.x < fr.a.m.size.x && p.y < fr.a.m.size.y) {
                    uint32_t *row = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(fr.rgba) +
                                                                 (size_t)p.y * (size_t)fr.rgba_pitch);
                    row[p.x] = compose_pixel(rec, s_pal, palette_len, fr.compose_max_ss, false, COLOR_PALETTE, 1);
                }
            }
        }
        // the job is finished (rendered or skipped): its pixel-iterations go to
        // the session's counter, then the job is counted; the last one
        // publishes the frame (after which nothing here touches its buffers)
        add_total(totals[fr.slot], iters, lane);
        __threadfence();
        __syncwarp();
        if (lane == 0) {
            const uint32_t prev = atomicAdd(&jobs_done[fr.slot], 1u);
            if (prev + 1u == fr.n_jobs) {
                __threadfence_system();
                const uint32_t st = atomicOr(&status[fr.slot], 0u);
                done_words[fr.slot] = 1u | (st << 8);
            }
        }
    }
}

// compose (gen.cu:455-475) of every frame of a launch: a warp takes a run of
// 128 pixels of one row of one frame (as k_compose).
__global__ void __launch_bounds__(256)
    k_compose_frames(const ComposeArgs *__restrict__ frames, const uint32_t *__restrict__ begin, uint32_t n_frames,
                     const uint32_t *palette, uint32_t palette_len)
{
    __shared__ uint32_t s_pal[4096];
    __shared__ uint32_t s_begin[SERVE_MAX_FRAMES + 1];
    for (uint32_t k = threadIdx.x; k < palette_len; k += blockDim.x) s_pal[k] = palette[k];
    for (uint32_t k = threadIdx.x; k <= n_frames; k += blockDim.x) s_begin[k] = begin[k];
    __syncthreads();
    constexpr int RUN = 4;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n_jobs = s_begin[n_frames];
    const uint32_t warps = gridDim.x * (blockDim.x / 32u);
    for (uint32_t job = blockIdx.x * (blockDim.x / 32u) + (threadIdx.x >> 5); job < n_jobs; job += warps) {
        const uint32_t f = find_frame(s_begin, n_frames, job);
        const ComposeArgs &c = frames[f];
        const uint32_t runs = (c.w + 32u * RUN - 1u) / (32u * RUN);
        const uint32_t local = job - s_begin[f];
        const uint32_t y = local / runs, x0 = 32u * RUN * (local % runs);
        PixelInfo p[RUN];
#pragma unroll
        for (int k = 0; k < RUN; k++) {
            const uint32_t x = x0 + 32u * k + lane;
            if (x < c.w) p[k] = load_pixel(pixel_ptr(c.in, c.pitch, x, y));
        }
        uint32_t *row = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(c.out) + (size_t)y * (size_t)c.out_pitch);
#pragma unroll
        for (int k = 0; k < RUN; k++) {
            const uint32_t x = x0 + 32u * k + lane;
            if (x < c.w) row[x] = compose_pixel(p[k], s_pal, palette_len, c.max_ss, false, COLOR_PALETTE, 1);
        }
    }
}

template <class R, int A, int F, bool ADV> static int serve_occupancy()
{
    static const int occ = occupancy(k_serve<R, A, F, ADV>, PERSIST_THREADS);
    return occ;
}

// What every kernel of a launch shares.
struct ServeLaunchArgs {
    uint32_t *status, *jobs_done;
    volatile uint32_t *done_words;
    unsigned long long *const *totals;
    unsigned long long budget_ns;
    const uint32_t *palette;
    uint32_t palette_len;
    int sms;
};

template <class R, int A, int F, bool ADV>
static cudaError_t launch_serve_t(const ServeFrame<R> *frames, const uint32_t *begin, uint32_t n_frames,
                                  uint32_t n_jobs, uint32_t *counter, const ServeLaunchArgs &L, cudaStream_t s)
{
    const int occ = serve_occupancy<R, A, F, ADV>();
    k_serve<R, A, F, ADV><<<grid_for(n_jobs, occ, L.sms), PERSIST_THREADS, 0, s>>>(
        frames, begin, n_frames, counter, L.status, L.jobs_done, L.done_words, L.totals, L.budget_ns, L.palette,
        L.palette_len);
    return cudaGetLastError();
}

template <class R>
static cudaError_t launch_serve(uint32_t group, const ServeFrame<R> *frames, const uint32_t *begin,
                                uint32_t n_frames, uint32_t n_jobs, uint32_t *counter, const ServeLaunchArgs &L,
                                cudaStream_t s)
{
    const uint32_t a = (group / 2u) % 4u, f = group % 2u;
    const bool adv = group >= 16u;
#define CHAOS_SERVE_CASE(AA, FF)                                                                                    \
    if (a == AA && f == FF)                                                                                         \
        return adv ? launch_serve_t<R, AA, FF, true>(frames, begin, n_frames, n_jobs, counter, L, s)                \
                   : launch_serve_t<R, AA, FF, false>(frames, begin, n_frames, n_jobs, counter, L, s);
    CHAOS_SERVE_CASE(ARITH_PARITY, FRACTAL_MANDELBROT)
    CHAOS_SERVE_CASE(ARITH_PARITY, FRACTAL_JULIA)
    CHAOS_SERVE_CASE(ARITH_FMA, FRACTAL_MANDELBROT)
    CHAOS_SERVE_CASE(ARITH_FMA, FRACTAL_JULIA)
    CHAOS_SERVE_CASE(ARITH_CONTRACTED, FRACTAL_MANDELBROT)
    CHAOS_SERVE_CASE(ARITH_CONTRACTED, FRACTAL_JULIA)
    if constexpr (sizeof(R) == 8) {
        CHAOS_SERVE_CASE(ARITH_FLOATFLOAT, FRACTAL_MANDELBROT)
        CHAOS_SERVE_CASE(ARITH_FLOATFLOAT, FRACTAL_JULIA)
    }
#undef CHAOS_SERVE_CASE
    return cudaErrorInvalidValue;
}

}  // namespace chaos
using namespace chaos;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

namespace {

using Clock = std::chrono::steady_clock;
constexpr uint32_t kRecordRing = 1u << 16;
constexpr int kForkStreams = 3;     // per launch slot, beside its own stream
constexpr int kMaxLaunchSlots = 6;
constexpr uint32_t kMaxSessions = 4096;  // session slots (reused once released)
constexpr uint32_t kMaxDeepPerLaunch = 16;

enum RecordState : uint8_t { REC_FREE = 0, REC_WAITING, REC_ADMITTED, REC_DONE };

struct Record {
    chaos_frame_record r{};
    RecordState state = REC_FREE;
};

struct Session {
    chaos_session_desc d{};
    uint64_t generation = 0;                   // bumped when the slot takes a new session
    bool open = false, closing = false, resident = false;
    uint32_t reading = 0;                      // reads in progress (no admission meanwhile)
    PixelInfo *buf[2] = {nullptr, nullptr};    // buf[0]: latest frame, buf[1]: the one before
    size_t pitch = 0;
    uint32_t *rgba = nullptr;
    size_t rgba_pitch = 0;
    unsigned long long *iters = nullptr;
    size_t bytes = 0;
    bool has_prev = false;                     // a frame has been admitted (renderFast from now on)
    double prev_rect[4] = {0, 0, 0, 0};
    double cx = 0, cy = 0, span = 0;
    double off_x = 0, off_y = 0;               // frame centre - target, zoomed alongside (deep frames)
    chaos_orbit *orbit = nullptr;
    uint32_t orbit_bits = 0;
    uint32_t submitted = 0;                    // frames requested so far
    uint32_t waiting = 0, in_flight = 0;
    bool in_forming = false;                   // has a frame in the launch being built
    volatile uint32_t *cancel_host = nullptr;  // this slot's host-mapped cancel word
    const volatile uint32_t *cancel_dev = nullptr;
    chaos_served_frame last{};                 // the latest admitted frame
    bool last_valid = false;
    uint64_t last_record = 0;                  // record of the latest admitted frame
};

struct Launch {
    uint64_t seq = 0;
    int slot = 0;
    std::vector<uint64_t> records;  // frame k of the launch -> record id
    std::vector<uint32_t> sessions;
    std::vector<uint8_t> deep;      // perturbation frames complete with the launch
    std::vector<uint8_t> finished;  // frames completed so far
    std::atomic<double> done_at{-1.0};
    struct chaos_server *server = nullptr;
    bool failed = false;
};

// A launch slot: its tables, its streams (launches in different slots run
// side by side), and the host-mapped done words its kernels write.
struct LaunchSlot {
    ServeTable *host = nullptr;    // pinned
    ServeTable *dev = nullptr;
    uint32_t *status_host = nullptr;  // pinned copy of dev->status after the launch
    unsigned long long **totals_host = nullptr;  // pinned: per frame, its session's counter
    unsigned long long **totals_dev = nullptr;
    volatile uint32_t *done_host = nullptr;  // pinned, mapped: per frame 1 | status << 8 once finished
    uint32_t *done_dev = nullptr;
    cudaStream_t stream = nullptr, fork[kForkStreams] = {};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, table_ready = nullptr;
    cudaEvent_t fork_done[kForkStreams] = {};
    bool busy = false;
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

int internal_arith(int32_t a)
{
    return a == CHAOS_ARITH_PARITY ? ARITH_PARITY : a == CHAOS_ARITH_CONTRACTED ? ARITH_CONTRACTED : ARITH_FMA;
}

}  // namespace

struct chaos_server {
    int device = -1;
    int sms = 0;
    size_t budget = 0, used = 0;
    uint32_t *palette = nullptr;
    uint32_t palette_len = 0;
    chaos_server_config cfg{64, 4, 30.0, 0.0, 120.0};

    std::mutex mu;                    // all state below
    std::condition_variable changed;  // frames finished, sessions released (waiters: drain, read, close)
    std::vector<std::unique_ptr<Session>> sessions;
    std::deque<uint64_t> waiting;     // record ids in arrival order
    std::vector<Record> ring = std::vector<Record>(kRecordRing);
    uint64_t next_record = 0;
    uint32_t in_flight = 0;
    std::deque<std::unique_ptr<Launch>> launches;
    std::vector<std::unique_ptr<Launch>> failed_launches;
    uint64_t launch_seq = 0;
    LaunchSlot slots[kMaxLaunchSlots];
    cudaStream_t stream = nullptr;  // buffer frees
    std::vector<chaos_orbit *> retired_orbits;  // freed by the scheduler once their launches ended
    uint32_t *cancel_words = nullptr;           // pinned, mapped: one per session slot
    uint32_t *cancel_words_dev = nullptr;

    std::thread scheduler;
    bool stop = false;
    std::mutex wake_mu;  // wake-ups of the scheduler (host callbacks never take `mu`)
    std::condition_variable wake;
    std::atomic<uint64_t> epoch{0};

    Clock::time_point t0 = Clock::now();
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void poke()
    {
        {
            std::lock_guard<std::mutex> g(wake_mu);
            epoch.fetch_add(1);
        }
        wake.notify_all();
    }
    Record &rec(uint64_t id) { return ring[id % kRecordRing]; }
};

namespace {

void CUDART_CB launch_done(void *p)
{
    Launch *l = static_cast<Launch *>(p);
    chaos_server *srv = l->server;  // `l` may be reaped as soon as done_at is set
    l->done_at.store(srv->now());
    srv->poke();
}

void release_session_locked(chaos_server *srv, Session &s)
{
    for (int k = 0; k < 2; k++)
        if (s.buf[k]) cudaFreeAsync(s.buf[k], srv->stream);
    if (s.rgba) cudaFreeAsync(s.rgba, srv->stream);
    if (s.iters) cudaFreeAsync(s.iters, srv->stream);
    s.buf[0] = s.buf[1] = nullptr;
    s.rgba = nullptr;
    s.iters = nullptr;
    if (s.resident) srv->used -= s.bytes;
    s.resident = false;
    if (s.orbit) srv->retired_orbits.push_back(s.orbit);
    s.orbit = nullptr;
    s.open = false;
    s.closing = false;
    s.last_valid = false;
}

void finish_record_locked(chaos_server *srv, uint64_t id, int status, double done, double gpu_ms)
{
    Record &rc = srv->rec(id);
    rc.r.status = status;
    rc.r.done_s = done;
    rc.r.gpu_ms = gpu_ms;
    rc.state = REC_DONE;
}

void complete_frame_locked(chaos_server *srv, Launch &l, size_t k, int status, double done)
{
    l.finished[k] = 1;
    finish_record_locked(srv, l.records[k], status, done, -1.0);
    Session &s = *srv->sessions[l.sessions[k]];
    s.in_flight--;
    srv->in_flight--;
    if (s.closing && s.in_flight == 0 && s.waiting == 0) release_session_locked(srv, s);
}

int frame_status(uint32_t bits)
{
    return (bits & SERVE_STATUS_CANCELLED) ? CHAOS_ERR_STATE : (bits & SERVE_STATUS_TIMEOUT) ? CHAOS_ERR_TIMEOUT
                                                                                             : CHAOS_OK;
}

// Frames the kernels have published complete one by one; a launch whose last
// operation (and completion callback) has run completes the rest (its
// perturbation frames) and frees its slot.
void reap_locked(chaos_server *srv)
{
    bool any = false;
    const double now = srv->now();
    for (auto it = srv->launches.begin(); it != srv->launches.end();) {
        Launch &l = **it;
        LaunchSlot &sl = srv->slots[l.slot];
        if (!l.failed)
            for (size_t k = 0; k < l.records.size(); k++) {
                if (l.finished[k] || l.deep[k]) continue;
                const uint32_t w = sl.done_host[k];
                if (w & 1u) {
                    complete_frame_locked(srv, l, k, frame_status(w >> 8), now);
                    any = true;
                }
            }
        bool ended = l.failed;
        if (!ended && l.done_at.load() >= 0) ended = true;
        if (!ended && !l.failed) {
            cudaError_t q = cudaEventQuery(sl.ev1);
            if (q != cudaErrorNotReady && q != cudaSuccess) {
                l.failed = true;  // the stream failed: the callback never runs
                ended = true;
            }
        }
        if (!ended) {
            ++it;
            continue;
        }
        float gpu_ms = 0.f;
        if (!l.failed) cudaEventElapsedTime(&gpu_ms, sl.ev0, sl.ev1);
        const double done = l.done_at.load() >= 0 ? l.done_at.load() : now;
        for (size_t k = 0; k < l.records.size(); k++) {
            if (!l.finished[k]) {
                int st = l.failed ? CHAOS_ERR_CUDA : frame_status(sl.status_host[k]);
                complete_frame_locked(srv, l, k, st, done);
            }
            srv->rec(l.records[k]).r.gpu_ms = gpu_ms;
        }
        sl.busy = false;
        // a failed launch's callback may still run: keep it until the server goes
        if (l.failed) srv->failed_launches.push_back(std::move(*it));
        it = srv->launches.erase(it);
        any = true;
    }
    if (any && srv->launches.empty() && !srv->retired_orbits.empty()) {
        // nothing on the GPU reads them any more
        std::vector<chaos_orbit *> dead;
        dead.swap(srv->retired_orbits);
        for (chaos_orbit *o : dead) chaos_orbit_destroy(o);
    }
    if (any) srv->changed.notify_all();
}

void expire_locked(chaos_server *srv, double now)
{
    if (!(srv->cfg.max_wait_s > 0)) return;
    bool any = false;
    for (auto it = srv->waiting.begin(); it != srv->waiting.end();) {
        Record &rc = srv->rec(*it);
        if (now - rc.r.arrival_s > srv->cfg.max_wait_s) {
            Session &s = *srv->sessions[rc.r.session];
            finish_record_locked(srv, *it, CHAOS_ERR_TIMEOUT, now, 0.0);
            s.waiting--;
            it = srv->waiting.erase(it);
            any = true;
        } else {
            ++it;
        }
    }
    if (any) srv->changed.notify_all();
}

// The session's buffers, allocated on the stream of the launch that first
// uses them (stream-ordered, so nothing waits).
bool allocate_session_locked(chaos_server *srv, Session &s, cudaStream_t st)
{
    const chaos_session_desc &d = s.d;
    s.pitch = round_up(16 * (size_t)d.width, 512);
    s.rgba_pitch = round_up(4 * (size_t)d.width, 512);
    cudaError_t e = cudaMallocAsync((void **)&s.buf[0], s.pitch * d.height, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&s.buf[1], s.pitch * d.height, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&s.rgba, s.rgba_pitch * d.height, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&s.iters, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.iters, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) {
        api_fail(CHAOS_ERR_CUDA, "session buffers: %s", cudaGetErrorString(e));
        for (int k = 0; k < 2; k++)
            if (s.buf[k]) cudaFreeAsync(s.buf[k], st);
        if (s.rgba) cudaFreeAsync(s.rgba, st);
        if (s.iters) cudaFreeAsync(s.iters, st);
        s.buf[0] = s.buf[1] = nullptr;
        s.rgba = nullptr;
        s.iters = nullptr;
        return false;
    }
    s.resident = true;
    srv->used += s.bytes;
    return true;
}

// The deep frame's orbit precision for the session's current pixel size.
uint32_t orbit_bits_for(const Session &s)
{
    const double ps = s.span / s.d.width;
    return (uint32_t)std::min(1536.0, std::max(128.0, std::ceil((-std::log2(ps) + 96.0) / 64.0) * 64.0));
}

// Next frame's plane and precision (the zoom step of RenderingController.zoomAt).
void advance_zoom(Session &s, double rect[4], int &prec, bool &deep)
{
    const chaos_session_desc &d = s.d;
    if (s.has_prev) {  // the target keeps its place on screen
        double z = d.zoom_per_frame;
        s.cx = d.target_x + (s.cx - d.target_x) / z;
        s.cy = d.target_y + (s.cy - d.target_y) / z;
        s.off_x /= z;
        s.off_y /= z;
        s.span /= z;
    }
    rect_of(s, rect);
    prec = chaos_select_precision(rect, d.width, d.height);
    if (d.flags & CHAOS_SESSION_FLAG_BINARY64) {
        if (prec == CHAOS_PRECISION_SINGLE) prec = CHAOS_PRECISION_DOUBLE;
    } else if (prec == CHAOS_PRECISION_DOUBLE && d.arith == CHAOS_ARITH_FMA) {
        // float-float while the pixel is at least 2^-42 of the plane's magnitude
        const double m = std::max(std::max(std::fabs(s.cx), std::fabs(s.cy)), 1.0 / 256.0);
        if (s.span / d.width >= std::ldexp(m, -42)) prec = CHAOS_PRECISION_FLOATFLOAT;
    }
    deep = prec == CHAOS_PRECISION_TOO_BIG && d.fractal == 0 && s.span / d.width >= 1e-290;
}

template <class R>
void fill_frame(ServeFrame<R> &f, const Session &s, const double rect[4], bool fast, uint32_t slot,
                uint32_t flags)
{
    const chaos_session_desc &d = s.d;
    std::memset(&f, 0, sizeof f);
    MainArgs<R> &m = f.a.m;
    m.size = UInt2{d.width, d.height};
    m.image = Rect<R>{(R)rect[0], (R)rect[1], (R)rect[2], (R)rect[3]};
    m.max_iter = d.max_iterations;
    m.max_ss = d.max_super_sampling;
    m.flags = flags;
    m.jcx = d.julia_cx;
    m.jcy = d.julia_cy;
    m.tiles_x = (d.width + 7u) / 8u;
    m.n_tiles = m.tiles_x * ((d.height + 3u) / 4u);
    f.advanced = fast ? 1u : 0u;
    f.slot = slot;
    f.cancel = s.cancel_dev;
    f.rgba = s.rgba;
    f.rgba_pitch = (long)s.rgba_pitch;
    f.compose_max_ss = d.max_super_sampling;
    if (fast) {
        // this frame writes buf[1] (the older one) from buf[0]; the swap happens on admission
        m.out = s.buf[1];
        m.pitch = (long)s.pitch;
        f.a.image_reused = Rect<R>{(R)s.prev_rect[0], (R)s.prev_rect[1], (R)s.prev_rect[2], (R)s.prev_rect[3]};
        f.a.in = s.buf[0];
        f.a.in_pitch = (long)s.pitch;
        double fx = (d.target_x - rect[0]) / (rect[2] - rect[0]) * d.width;
        double fy = (rect[3] - d.target_y) / (rect[3] - rect[1]) * d.height;
        fx = std::min(std::max(fx, 0.0), (double)(d.width - 1));
        fy = std::min(std::max(fy, 0.0), (double)(d.height - 1));
        f.a.focus = UInt2{(uint32_t)fx, (uint32_t)fy};
    } else {
        m.out = s.buf[0];
        m.pitch = (long)s.pitch;
    }
}

struct Forming {
    struct Item {
        uint64_t record;
        uint32_t session;
        int prec;
        bool deep, fast;
        double rect[4];
        uint32_t group;  // kernel group (not deep)
    };
    std::vector<Item> items;
    int slot = -1;  // launch slot the frames go to
};

// Build and enqueue one launch of the admitted frames (under the lock: only
// asynchronous CUDA calls).
int enqueue_launch_locked(chaos_server *srv, Forming &fm)
{
    TraceRange trace_("chaos_server launch");
    const int slot_id = fm.slot;
    LaunchSlot &sl = srv->slots[slot_id];
    ServeTable &T = *sl.host;
    std::memset(T.counters, 0, sizeof T.counters);
    std::memset(T.status, 0, sizeof T.status);
    std::memset(T.jobs_done, 0, sizeof T.jobs_done);
    std::unique_ptr<Launch> L(new Launch());
    L->seq = ++srv->launch_seq;
    L->slot = slot_id;
    L->server = srv;
    const size_t n = fm.items.size();
    L->deep.assign(n, 0);
    L->finished.assign(n, 0);
    for (size_t k = 0; k < n; k++) sl.done_host[k] = 0u;

    // frames per group (binary32 frames in f32[], binary64 in f64[]); within a
    // group the smaller frames come first, so they finish first
    uint32_t n_group[SERVE_GROUPS] = {0};
    uint32_t first_of[SERVE_GROUPS] = {0};
    for (auto &it : fm.items)
        if (!it.deep) n_group[it.group]++;
    uint32_t n32 = 0, n64 = 0;
    for (uint32_t g = 0; g < SERVE_GROUPS; g++) {
        if (!group_binary64(g)) {
            first_of[g] = n32;
            n32 += n_group[g];
        } else {
            first_of[g] = n64;
            n64 += n_group[g];
        }
    }
    std::vector<uint32_t> order(n);
    for (uint32_t k = 0; k < n; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const chaos_session_desc &a = srv->sessions[fm.items[x].session]->d;
        const chaos_session_desc &b = srv->sessions[fm.items[y].session]->d;
        return (uint64_t)a.width * a.height < (uint64_t)b.width * b.height;
    });
    uint32_t fill[SERVE_GROUPS] = {0};
    uint64_t tiles_all = 0;
    uint32_t n_deep = 0;
    for (uint32_t k = 0; k < n; k++) {
        auto &it = fm.items[k];
        Session &s = *srv->sessions[it.session];
        L->records.push_back(it.record);
        L->sessions.push_back(it.session);
        sl.totals_host[k] = s.iters;
        L->deep[k] = it.deep ? 1 : 0;
        if (!it.deep) continue;
        // perturbation frames are composed after their own kernel
        ComposeArgs &c = T.compose[n_deep++];
        std::memset(&c, 0, sizeof c);
        c.in = s.buf[0];
        c.pitch = (long)s.pitch;
        c.out = s.rgba;
        c.out_pitch = (long)s.rgba_pitch;
        c.w = s.d.width;
        c.h = s.d.height;
        c.max_ss = 1.f;
        c.color_mode = COLOR_PALETTE;
        c.magnifier = 1;
    }
    for (uint32_t k : order) {
        auto &it = fm.items[k];
        if (it.deep) continue;
        Session &s = *srv->sessions[it.session];
        const chaos_session_desc &d = s.d;
        const uint32_t flags = it.fast ? (d.flags & 0xffffu) | CHAOS_FLAG_IS_ZOOMING | CHAOS_FLAG_ZOOMING_IN
                                       : (d.flags & CHAOS_FLAG_ADAPTIVE_SS);
        const uint32_t g = it.group;
        const uint32_t idx = first_of[g] + fill[g]++;
        if (!group_binary64(g))
            fill_frame<float>(T.f32[idx], s, it.rect, it.fast, k, flags);
        else
            fill_frame<double>(T.f64[idx], s, it.rect, it.fast, k, flags);
        tiles_all += (uint64_t)((d.width + 7u) / 8u) * ((d.height + 3u) / 4u);
    }
    // strips of tiles per job, as for single frames: up to 4 while every
    // resident warp still gets 8 jobs
    const int occ_hint = 5;
    const uint32_t chunk = tile_chunk_for((uint32_t)std::min<uint64_t>(tiles_all, 0xffffffffu), occ_hint, srv->sms, 4);
    for (uint32_t g = 0; g < SERVE_GROUPS; g++) {
        uint32_t acc = 0;
        for (uint32_t j = 0; j < n_group[g]; j++) {
            T.job_begin[g][j] = acc;
            uint32_t tiles;
            if (!group_binary64(g)) {
                ServeFrame<float> &f = T.f32[first_of[g] + j];
                f.chunk = chunk;
                f.n_jobs = (f.a.m.n_tiles + chunk - 1) / chunk;
                tiles = f.n_jobs;
            } else {
                ServeFrame<double> &f = T.f64[first_of[g] + j];
                f.chunk = chunk;
                f.n_jobs = (f.a.m.n_tiles + chunk - 1) / chunk;
                tiles = f.n_jobs;
            }
            acc += tiles;
        }
        T.job_begin[g][n_group[g]] = acc;
    }
    uint32_t cacc = 0;
    for (uint32_t k = 0; k < n_deep; k++) {
        T.compose_begin[k] = cacc;
        cacc += ((T.compose[k].w + 127u) / 128u) * T.compose[k].h;
    }
    T.compose_begin[n_deep] = cacc;

    // the table, then the kernels of each group side by side, then the
    // perturbation frames and their compose, status back, completion
    cudaStream_t s0 = sl.stream;
    cudaError_t e = cudaEventRecord(sl.ev0, s0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.dev, sl.host, sizeof(ServeTable), cudaMemcpyHostToDevice, s0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.totals_dev, sl.totals_host, SERVE_MAX_FRAMES * sizeof(unsigned long long *),
                            cudaMemcpyHostToDevice, s0);
    if (e == cudaSuccess) e = cudaEventRecord(sl.table_ready, s0);
    ServeLaunchArgs LA{};
    LA.status = sl.dev->status;
    LA.jobs_done = sl.dev->jobs_done;
    LA.done_words = sl.done_dev;
    LA.totals = sl.totals_dev;
    LA.budget_ns = srv->cfg.frame_time_limit_s > 0 ? (unsigned long long)(srv->cfg.frame_time_limit_s * 1e9) : 0ull;
    LA.palette = srv->palette;
    LA.palette_len = srv->palette_len;
    LA.sms = srv->sms;
    // the first group on the slot's own stream, the others on its fork streams
    int used = 0;
    for (uint32_t g = 0; g < SERVE_GROUPS && e == cudaSuccess; g++) {
        if (!n_group[g]) continue;
        const uint32_t n_jobs = T.job_begin[g][n_group[g]];
        cudaStream_t fs = used == 0 ? s0 : sl.fork[(used - 1) % kForkStreams];
        if (used >= 1 && used <= kForkStreams) e = cudaStreamWaitEvent(fs, sl.table_ready, 0);
        if (e != cudaSuccess) break;
        if (!group_binary64(g))
            e = launch_serve<float>(g, sl.dev->f32 + first_of[g], sl.dev->job_begin[g], n_group[g], n_jobs,
                                    &sl.dev->counters[g], LA, fs);
        else
            e = launch_serve<double>(g, sl.dev->f64 + first_of[g], sl.dev->job_begin[g], n_group[g], n_jobs,
                                     &sl.dev->counters[g], LA, fs);
        used++;
    }
    for (int k = 0; k < std::min(used - 1, kForkStreams) && e == cudaSuccess; k++) {
        e = cudaEventRecord(sl.fork_done[k], sl.fork[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, sl.fork_done[k], 0);
    }
    // perturbation frames (a session past binary64), one after another
    uint32_t deep_counter = SERVE_GROUPS;
    for (uint32_t k = 0; k < n && e == cudaSuccess; k++) {
        auto &it = fm.items[k];
        if (!it.deep) continue;
        Session &s = *srv->sessions[it.session];
        chaos_frame_desc fd{};
        fd.width = s.d.width;
        fd.height = s.d.height;
        fd.max_iterations = s.d.max_iterations;
        fd.samples_per_pixel = 1;
        fd.sample_mode = CHAOS_SAMPLES_CENTER;
        fd.tier = CHAOS_TIER_PERTURB_F64;
        fd.center_x = it.rect[0];  // offsets from the target, set on admission
        fd.center_y = it.rect[1];
        fd.pixel_size = it.rect[2];
        chaos_frame_out fo{};
        fo.pixels = reinterpret_cast<chaos_pixel_info *>(s.buf[0]);
        fo.pixels_pitch = (long)s.pitch;
        fo.total_iterations = s.iters;
        uint32_t *ctr = &sl.dev->counters[deep_counter < 32 ? deep_counter++ : 31];
        if (api_perturb_enqueue(&fd, s.orbit, &fo, s0, ctr) != CHAOS_OK) e = cudaErrorLaunchFailure;
    }
    if (e == cudaSuccess && cacc) {
        const unsigned warps_needed = (cacc + 7u) / 8u;
        const unsigned blocks = std::max(1u, std::min(warps_needed, (unsigned)srv->sms * 8u));
        k_compose_frames<<<blocks, 256, 0, s0>>>(sl.dev->compose, sl.dev->compose_begin, n_deep, srv->palette,
                                                 srv->palette_len);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.status_host, sl.dev->status, SERVE_MAX_FRAMES * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s0);
    if (e == cudaSuccess) e = cudaEventRecord(sl.ev1, s0);
    Launch *lp = L.get();
    if (e == cudaSuccess) e = cudaLaunchHostFunc(s0, launch_done, lp);
    if (e != cudaSuccess) {
        api_fail(CHAOS_ERR_CUDA, "serving launch: %s", cudaGetErrorString(e));
        L->failed = true;
    }
    sl.busy = true;
    srv->launches.push_back(std::move(L));
    return e == cudaSuccess ? CHAOS_OK : CHAOS_ERR_CUDA;
}

// Enqueue the launch (with the buffers as they were on admission), then the
// per-session bookkeeping: renderFast frames swap the two reuse buffers.
void commit_launch_locked(chaos_server *srv, Forming &fm)
{
    enqueue_launch_locked(srv, fm);
    for (auto &x : fm.items) {
        Session &s = *srv->sessions[x.session];
        s.in_forming = false;
        if (x.fast && !x.deep) std::swap(s.buf[0], s.buf[1]);
        if (!x.deep)
            std::copy(x.rect, x.rect + 4, s.prev_rect);
        else
            rect_of(s, s.prev_rect);
        s.has_prev = true;
    }
    srv->in_flight += (uint32_t)fm.items.size();
    fm.items.clear();
}

// Admission pass: returns true if it did something (a launch, or a reference
// orbit built), so that the scheduler loops again at once.  Building an orbit
// (a deep frame) happens without the lock.
bool admit_and_launch(chaos_server *srv, std::unique_lock<std::mutex> &lk)
{
    if (srv->waiting.empty()) return false;
    int slot = -1;
    uint32_t busy = 0;
    for (int k = 0; k < kMaxLaunchSlots; k++) {
        if (srv->slots[k].busy)
            busy++;
        else if (slot < 0)
            slot = k;
    }
    if (slot < 0 || busy >= srv->cfg.max_launches_in_flight) return false;
    Forming fm;
    fm.slot = slot;
    const cudaStream_t st = srv->slots[slot].stream;
    uint32_t n_deep = 0;
    bool memory_blocked = false;  // an earlier request waits for memory: no later one overtakes it for memory
    for (auto it = srv->waiting.begin(); it != srv->waiting.end();) {
        if (fm.items.size() >= SERVE_MAX_FRAMES) break;
        if (srv->in_flight + fm.items.size() >= srv->cfg.max_frames_in_flight) break;
        Record &rc = srv->rec(*it);
        Session &s = *srv->sessions[rc.r.session];
        // a session's next frame waits for its previous one (launches in
        // different slots run side by side)
        if (s.in_forming || s.in_flight || s.reading || s.closing) {
            ++it;
            continue;
        }
        if (!s.resident) {
            if (memory_blocked || srv->used + s.bytes > srv->budget) {
                memory_blocked = true;
                ++it;
                continue;
            }
            if (!allocate_session_locked(srv, s, st)) {
                finish_record_locked(srv, *it, CHAOS_ERR_CUDA, srv->now(), 0.0);
                s.waiting--;
                it = srv->waiting.erase(it);
                continue;
            }
        }
        // a deep frame needs the target's orbit at enough bits: build it
        // without the lock, then come back
        {
            Session probe = s;  // the zoom state this frame would have
            probe.orbit = nullptr;
            double r[4];
            int prec;
            bool deep;
            advance_zoom(probe, r, prec, deep);
            if (deep && (!s.orbit || s.orbit_bits < orbit_bits_for(probe))) {
                const uint32_t bits = orbit_bits_for(probe);
                const double tx = s.d.target_x, ty = s.d.target_y;
                const uint32_t mi = s.d.max_iterations;
                const uint32_t sid = rc.r.session;
                const uint64_t gen = s.generation;
                s.reading++;  // keeps the session out of admission meanwhile
                if (!fm.items.empty()) commit_launch_locked(srv, fm);
                lk.unlock();
                chaos_orbit *orbit = nullptr;
                int rc2 = api_orbit_create_d(tx, ty, bits, mi, &orbit);
                lk.lock();
                Session &s2 = *srv->sessions[sid];
                s2.reading--;
                if (rc2 == CHAOS_OK) {
                    if (s2.open && !s2.closing && s2.generation == gen) {
                        if (s2.orbit) srv->retired_orbits.push_back(s2.orbit);
                        s2.orbit = orbit;
                        s2.orbit_bits = bits;
                    } else {
                        srv->retired_orbits.push_back(orbit);
                    }
                } else {
                    // the frame cannot be rendered: it completes with the error
                    for (auto w = srv->waiting.begin(); w != srv->waiting.end(); ++w)
                        if (srv->rec(*w).r.session == sid && s2.generation == gen) {
                            finish_record_locked(srv, *w, rc2, srv->now(), 0.0);
                            s2.waiting--;
                            srv->waiting.erase(w);
                            srv->changed.notify_all();
                            break;
                        }
                }
                return true;
            }
        }
        Forming::Item item{};
        item.record = *it;
        item.session = rc.r.session;
        {
            Session probe = s;
            double r[4];
            int prec;
            bool deep;
            advance_zoom(probe, r, prec, deep);
            if (deep && n_deep >= kMaxDeepPerLaunch) {  // one work counter each; the rest go next launch
                ++it;
                continue;
            }
        }
        advance_zoom(s, item.rect, item.prec, item.deep);
        if (item.deep) n_deep++;
        item.fast = s.has_prev;
        if (item.deep) {
            // perturbation: offset of the frame centre from the target, pixel size
            item.rect[0] = s.off_x;
            item.rect[1] = s.off_y;
            item.rect[2] = s.span / s.d.width;
            item.rect[3] = 0;
            item.prec = CHAOS_PRECISION_TOO_BIG;
        } else {
            const int arith = item.prec == CHAOS_PRECISION_FLOATFLOAT ? ARITH_FLOATFLOAT : internal_arith(s.d.arith);
            item.group = serve_group(item.fast, item.prec != CHAOS_PRECISION_SINGLE, arith, s.d.fractal == 1 ? 1 : 0);
        }
        // bookkeeping of the admitted frame: the served-frame view, the swap
        double plane[4];
        rect_of(s, plane);
        chaos_served_frame &lf = s.last;
        lf.frame = rc.r.frame;
        lf.precision = item.prec;
        lf.advanced = (item.fast && !item.deep) ? 1u : 0u;
        lf.flags = item.fast ? (s.d.flags & 0xffffu) | CHAOS_FLAG_IS_ZOOMING | CHAOS_FLAG_ZOOMING_IN
                             : (s.d.flags & CHAOS_FLAG_ADAPTIVE_SS);
        lf.arith = s.d.arith;
        lf.max_iterations = s.d.max_iterations;
        lf.max_super_sampling = s.d.max_super_sampling;
        std::copy(plane, plane + 4, lf.rect);
        std::copy(s.prev_rect, s.prev_rect + 4, lf.rect_reused);
        if (item.fast && !item.deep) {
            double fx = (s.d.target_x - plane[0]) / (plane[2] - plane[0]) * s.d.width;
            double fy = (plane[3] - s.d.target_y) / (plane[3] - plane[1]) * s.d.height;
            lf.focus_x = (uint32_t)std::min(std::max(fx, 0.0), (double)(s.d.width - 1));
            lf.focus_y = (uint32_t)std::min(std::max(fy, 0.0), (double)(s.d.height - 1));
            // the frame writes buf[1] from buf[0]; afterwards buf[0] is the latest
            lf.pixels = reinterpret_cast<const chaos_pixel_info *>(s.buf[1]);
            lf.previous = reinterpret_cast<const chaos_pixel_info *>(s.buf[0]);
        } else {
            lf.focus_x = lf.focus_y = 0;
            lf.pixels = reinterpret_cast<const chaos_pixel_info *>(s.buf[0]);
            lf.previous = nullptr;
        }
        lf.pixels_pitch = (long)s.pitch;
        lf.previous_pitch = lf.previous ? (long)s.pitch : 0;
        s.last_valid = true;
        s.last_record = item.record;
        fm.items.push_back(item);
        s.in_forming = true;
        rc.state = REC_ADMITTED;
        rc.r.start_s = srv->now();
        rc.r.precision = item.prec;
        s.waiting--;
        s.in_flight++;
        it = srv->waiting.erase(it);
    }
    if (fm.items.empty()) return false;
    commit_launch_locked(srv, fm);
    return true;
}

void scheduler_main(chaos_server *srv)
{
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        const uint64_t seen = srv->epoch.load();
        reap_locked(srv);
        expire_locked(srv, srv->now());
        if (srv->stop && srv->launches.empty()) break;
        if (!srv->stop) {
            bool again = admit_and_launch(srv, lk);
            if (again) continue;
        }
        // wait for a callback, a request, or (with launches or waiting
        // requests) a short poll interval
        const bool busy = !srv->launches.empty() || !srv->waiting.empty();
        lk.unlock();
        {
            std::unique_lock<std::mutex> w(srv->wake_mu);
            srv->wake.wait_for(w, busy ? std::chrono::microseconds(200) : std::chrono::milliseconds(20),
                               [&] { return srv->epoch.load() != seen; });
        }
        lk.lock();
    }
}

// Wait (with the lock held) until pred() or the call limit.
template <class Pred> bool wait_locked(chaos_server *srv, std::unique_lock<std::mutex> &lk, Pred pred)
{
    const auto limit = std::chrono::duration<double>(srv->cfg.call_timeout_s > 0 ? srv->cfg.call_timeout_s : 120.0);
    return srv->changed.wait_for(lk, limit, pred);
}

Session *open_session(chaos_server *srv, uint32_t id)
{
    if (id >= srv->sessions.size() || !srv->sessions[id] || !srv->sessions[id]->open || srv->sessions[id]->closing)
        return nullptr;
    return srv->sessions[id].get();
}

}  // namespace

double chaos_server_clock(const chaos_server *s) { return s ? s->now() : 0.0; }

int chaos_server_create(size_t hbm_budget_bytes, const uint32_t *palette, uint32_t palette_len, chaos_server **out)
{
    if (!out || !palette || palette_len == 0 || palette_len > 4096)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "a host palette of 1..4096 entries is required");
    std::unique_ptr<chaos_server> s(new (std::nothrow) chaos_server());
    if (!s) return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    s->budget = hbm_budget_bytes;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->cancel_words, kMaxSessions * sizeof(uint32_t), cudaHostAllocMapped);
    if (e == cudaSuccess) {
        std::memset(s->cancel_words, 0, kMaxSessions * sizeof(uint32_t));
        e = cudaHostGetDevicePointer((void **)&s->cancel_words_dev, s->cancel_words, 0);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->palette, palette_len * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(s->palette, palette, palette_len * sizeof(uint32_t), cudaMemcpyHostToDevice);
    for (int k = 0; k < kMaxLaunchSlots && e == cudaSuccess; k++) {
        LaunchSlot &sl = s->slots[k];
        e = cudaMallocHost(&sl.host, sizeof(ServeTable));
        if (e == cudaSuccess) e = cudaMalloc(&sl.dev, sizeof(ServeTable));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.status_host, SERVE_MAX_FRAMES * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.totals_host, SERVE_MAX_FRAMES * sizeof(unsigned long long *));
        if (e == cudaSuccess) e = cudaMalloc(&sl.totals_dev, SERVE_MAX_FRAMES * sizeof(unsigned long long *));
        if (e == cudaSuccess) e = cudaHostAlloc((void **)&sl.done_host, SERVE_MAX_FRAMES * sizeof(uint32_t),
                                                cudaHostAllocMapped);
        if (e == cudaSuccess) {
            std::memset((void *)sl.done_host, 0, SERVE_MAX_FRAMES * sizeof(uint32_t));
            e = cudaHostGetDevicePointer((void **)&sl.done_dev, (void *)sl.done_host, 0);
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        for (int f = 0; f < kForkStreams && e == cudaSuccess; f++)
            e = cudaStreamCreateWithFlags(&sl.fork[f], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.table_ready, cudaEventDisableTiming);
        for (int f = 0; f < kForkStreams && e == cudaSuccess; f++)
            e = cudaEventCreateWithFlags(&sl.fork_done[f], cudaEventDisableTiming);
        if (e == cudaSuccess) std::memset(sl.host, 0, sizeof(ServeTable));
    }
    s->palette_len = palette_len;
    if (e != cudaSuccess) {
        int rc = api_fail(CHAOS_ERR_CUDA, "server set-up: %s", cudaGetErrorString(e));
        chaos_server_destroy(s.release());
        return rc;
    }
    chaos_server *srv = s.release();
    srv->scheduler = std::thread(scheduler_main, srv);
    *out = srv;
    return CHAOS_OK;
}

int chaos_server_configure(chaos_server *s, const chaos_server_config *c)
{
    if (!s || !c) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (c->max_frames_in_flight < 1 || c->max_frames_in_flight > 4096 || c->max_launches_in_flight < 1 ||
        c->max_launches_in_flight > (uint32_t)kMaxLaunchSlots || !(c->max_wait_s >= 0) ||
        !(c->frame_time_limit_s >= 0) || !(c->call_timeout_s >= 0))
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT,
                        "max_frames_in_flight 1..4096, max_launches_in_flight 1..%d, limits >= 0", kMaxLaunchSlots);
    std::lock_guard<std::mutex> g(s->mu);
    s->cfg = *c;
    s->poke();
    return CHAOS_OK;
}

int chaos_server_get_config(const chaos_server *s, chaos_server_config *c)
{
    if (!s || !c) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    *c = s->cfg;
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
    if (d->arith != CHAOS_ARITH_FMA && d->arith != CHAOS_ARITH_PARITY && d->arith != CHAOS_ARITH_CONTRACTED)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "unknown arithmetic %d", d->arith);
    const size_t bytes = session_bytes(*d);
    if (bytes > s->budget)
        return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "session needs %zu bytes, the whole budget is %zu", bytes, s->budget);
    std::unique_ptr<Session> ss(new (std::nothrow) Session());
    if (!ss) return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "out of host memory");
    ss->d = *d;
    ss->bytes = bytes;
    ss->open = true;
    ss->cx = d->center_x;
    ss->cy = d->center_y;
    ss->span = d->span;
    ss->off_x = d->center_x - d->target_x;
    ss->off_y = d->center_y - d->target_y;
    std::lock_guard<std::mutex> g(s->mu);
    // a slot whose session has been released is reused in place (waiters
    // hold pointers to slots; the generation tells sessions apart)
    uint32_t id = 0;
    while (id < s->sessions.size() &&
           (s->sessions[id]->open || s->sessions[id]->in_flight || s->sessions[id]->reading))
        id++;
    if (id >= kMaxSessions) return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "%u sessions are open", kMaxSessions);
    ss->cancel_host = s->cancel_words + id;
    ss->cancel_dev = s->cancel_words_dev + id;
    *ss->cancel_host = 0u;
    if (id == s->sessions.size()) {
        s->sessions.push_back(std::move(ss));
    } else {
        const uint64_t gen = s->sessions[id]->generation + 1;
        *s->sessions[id] = *ss;
        s->sessions[id]->generation = gen;
    }
    *session = id;
    return CHAOS_OK;
}

int chaos_server_close(chaos_server *s, uint32_t session)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    Session *ss = open_session(s, session);
    if (!ss) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
    // queued frames are dropped; frames on the GPU are cancelled
    const double t = s->now();
    for (auto it = s->waiting.begin(); it != s->waiting.end();) {
        if (s->rec(*it).r.session == session) {
            finish_record_locked(s, *it, CHAOS_ERR_STATE, t, 0.0);
            it = s->waiting.erase(it);
        } else {
            ++it;
        }
    }
    ss->waiting = 0;
    ss->closing = true;
    if (ss->in_flight) {
        *ss->cancel_host = 1u;
        s->poke();
        const uint64_t gen = ss->generation;
        if (!wait_locked(s, lk, [&] { return !ss->open || ss->generation != gen; }))
            return api_fail(CHAOS_ERR_TIMEOUT, "session %u: frames on the GPU did not finish in time", session);
    } else {
        release_session_locked(s, *ss);
    }
    s->changed.notify_all();
    s->poke();
    return CHAOS_OK;
}

int chaos_server_submit(chaos_server *s, uint32_t session, double arrival_s)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        Session *ss = open_session(s, session);
        if (!ss) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
        Record &rc = s->rec(s->next_record);
        if (rc.state == REC_WAITING || rc.state == REC_ADMITTED)
            return api_fail(CHAOS_ERR_OUT_OF_MEMORY, "%u frames are queued or in flight", kRecordRing);
        rc.r = chaos_frame_record{};
        rc.r.session = session;
        rc.r.frame = ss->submitted++;
        rc.r.arrival_s = arrival_s;
        rc.r.start_s = -1.0;
        rc.r.done_s = -1.0;
        rc.r.precision = -1;
        rc.state = REC_WAITING;
        s->waiting.push_back(s->next_record++);
        ss->waiting++;
    }
    s->poke();
    return CHAOS_OK;
}

int chaos_server_drain(chaos_server *s)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    if (!wait_locked(s, lk, [&] { return s->waiting.empty() && s->in_flight == 0; }))
        return api_fail(CHAOS_ERR_TIMEOUT, "drain: %zu frames waiting, %u on the GPU after %.0f s", s->waiting.size(),
                        s->in_flight, s->cfg.call_timeout_s);
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
    const uint64_t first = s->next_record > kRecordRing ? s->next_record - kRecordRing : 0;
    uint32_t k = 0;
    for (uint64_t id = first; id < s->next_record; id++, k++)
        if (out && k < max) out[k] = s->rec(id).r;
    *n = k;
    return CHAOS_OK;
}

int chaos_server_queue(chaos_server *s, uint32_t *waiting, uint32_t *in_flight)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    if (waiting) *waiting = (uint32_t)s->waiting.size();
    if (in_flight) *in_flight = s->in_flight;
    return CHAOS_OK;
}

// Wait until the session has nothing queued or on the GPU, and hold it out
// of admission; returns the session or null (error set).
static int quiesce(chaos_server *s, std::unique_lock<std::mutex> &lk, uint32_t session, Session **out)
{
    Session *ss = open_session(s, session);
    if (!ss) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "no open session %u", session);
    const uint64_t gen = ss->generation;
    auto quiet = [&] { return !ss->open || ss->generation != gen || (ss->waiting == 0 && ss->in_flight == 0); };
    if (!wait_locked(s, lk, quiet)) return api_fail(CHAOS_ERR_TIMEOUT, "session %u: frames did not finish in time", session);
    if (!ss->open || ss->closing || ss->generation != gen)
        return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "session %u was closed", session);
    *out = ss;
    return CHAOS_OK;
}

int chaos_server_read(chaos_server *s, uint32_t session, uint32_t *host_rgba, unsigned long long *pixel_iterations)
{
    if (!s) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    Session *ss = nullptr;
    int rc = quiesce(s, lk, session, &ss);
    if (rc) return rc;
    if (!ss->resident) {  // no frame yet
        if (pixel_iterations) *pixel_iterations = 0;
        if (host_rgba) std::memset(host_rgba, 0, 4u * (size_t)ss->d.width * ss->d.height);
        return CHAOS_OK;
    }
    ss->reading++;
    const uint32_t w = ss->d.width, h = ss->d.height;
    uint32_t *rgba = ss->rgba;
    const size_t rp = ss->rgba_pitch;
    unsigned long long *iters = ss->iters;
    lk.unlock();
    // the session's frames have finished (their launches ended), and none is
    // admitted while reading: plain copies
    cudaError_t e = cudaSuccess;
    if (host_rgba) e = cudaMemcpy2D(host_rgba, 4u * (size_t)w, rgba, rp, 4u * (size_t)w, h, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && pixel_iterations)
        e = cudaMemcpy(pixel_iterations, iters, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    lk.lock();
    ss->reading--;
    s->poke();
    if (e != cudaSuccess) return api_fail(CHAOS_ERR_CUDA, "read: %s", cudaGetErrorString(e));
    return CHAOS_OK;
}

int chaos_server_frame_state(chaos_server *s, uint32_t session, chaos_served_frame *out)
{
    if (!s || !out) return api_fail(CHAOS_ERR_INVALID_ARGUMENT, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    Session *ss = nullptr;
    int rc = quiesce(s, lk, session, &ss);
    if (rc) return rc;
    if (!ss->last_valid) return api_fail(CHAOS_ERR_STATE, "session %u has no finished frame", session);
    *out = ss->last;
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
    if (s->scheduler.joinable()) {
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->stop = true;
            // queued frames are dropped; frames on the GPU are cancelled
            for (uint64_t id : s->waiting) finish_record_locked(s, id, CHAOS_ERR_STATE, s->now(), 0.0);
            s->waiting.clear();
            for (auto &ss : s->sessions)
                if (ss && ss->open) {
                    ss->waiting = 0;
                    if (ss->cancel_host) *ss->cancel_host = 1u;
                }
        }
        s->poke();
        s->scheduler.join();  // ends once the launches on the GPU have ended
    }
    for (int k = 0; k < kMaxLaunchSlots; k++)
        if (s->slots[k].stream) cudaStreamSynchronize(s->slots[k].stream);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto &ss : s->sessions)
        if (ss && ss->open) release_session_locked(s, *ss);
    for (chaos_orbit *o : s->retired_orbits) chaos_orbit_destroy(o);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (int k = 0; k < kMaxLaunchSlots; k++) {
        LaunchSlot &sl = s->slots[k];
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.dev) cudaFree(sl.dev);
        if (sl.status_host) cudaFreeHost(sl.status_host);
        if (sl.totals_host) cudaFreeHost(sl.totals_host);
        if (sl.totals_dev) cudaFree(sl.totals_dev);
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        if (sl.table_ready) cudaEventDestroy(sl.table_ready);
        for (int f = 0; f < kForkStreams; f++) {
            if (sl.fork_done[f]) cudaEventDestroy(sl.fork_done[f]);
            if (sl.fork[f]) cudaStreamDestroy(sl.fork[f]);
        }
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done_host) cudaFreeHost((void *)sl.done_host);
    }
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->palette) cudaFree(s->palette);
    if (s->cancel_words) cudaFreeHost(s->cancel_words);
    delete s;
    return CHAOS_OK;
}
