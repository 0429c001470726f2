// capi.cu -- the extern "C" entry points declared in
// include/gstools_core_gb300.h: argument validation, per-device contexts,
// host staging for host-pointer calls, CUDA-event timing, error strings.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "internal.h"

namespace gsc {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string t_error;

int set_error(int code, const std::string &msg) {
    t_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? GSC_ERR_NOMEM
                     : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                         ? GSC_ERR_NO_DEVICE
                         : GSC_ERR_CUDA;
    cudaGetLastError();   // clear a non-sticky error so the next call is clean
    return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

const char *kernel_name(int32_t id) {
    static const char *names[K_COUNT] = {
        "mode_table", "plain_f64_scalar", "plain_f64_incompr", "plain_f64_libm",
        "split_reduce", "generic_f64", "sep_tables", "sep_tc_f16x3", "sep_tc_bf16x3",
        "grid_expand", "sep_tc_f16x5", "mixed_modes", "mixed_scalar", "mixed_incompr",
        "mixed_f64phase", "sep_f64_dmma", "fourier_scale", "batch_tables", "batch_plain",
        "batch_mixed", "sample_modes", "sep_split", "copy_h2d", "copy_d2h", "interleave",
        "mesh_check",
    };
    return (id >= 0 && id < K_COUNT) ? names[id] : "unknown";
}

// ---------------------------------------------------------------------------
// timing: CUDA events recorded on the launch stream around each kernel
// ---------------------------------------------------------------------------
struct TimingRec {
    int32_t id;
    cudaEvent_t a, b;
};
static thread_local bool t_timing = false;
static thread_local std::vector<TimingRec> t_recs;
static thread_local std::vector<cudaEvent_t> t_event_pool;

static cudaEvent_t pooled_event() {
    if (!t_event_pool.empty()) {
        cudaEvent_t e = t_event_pool.back();
        t_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void timing_reset(bool enabled) {
    for (auto &r : t_recs) {
        t_event_pool.push_back(r.a);
        t_event_pool.push_back(r.b);
    }
    t_recs.clear();
    t_timing = enabled;
}
bool timing_enabled() { return t_timing; }

TimedLaunch::TimedLaunch(cudaStream_t s) : st(s) {}

void TimedLaunch::begin(int32_t kid) {
    on = t_timing;
    id = kid;
    if (!on) return;
    TimingRec r{kid, pooled_event(), pooled_event()};
    if (!r.a || !r.b) {
        on = false;
        return;
    }
    cudaEventRecord(r.a, st);
    rec = t_recs.size();
    t_recs.push_back(r);
}

void TimedLaunch::end() {
    if (!on || rec >= t_recs.size()) return;
    cudaEventRecord(t_recs[rec].b, st);
}

// ---------------------------------------------------------------------------
// device contexts
// ---------------------------------------------------------------------------
static std::mutex g_ctx_mu;
static DeviceCtx *g_ctx[64] = {nullptr};


int get_ctx(int device, DeviceCtx **out) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return set_error(GSC_ERR_NO_DEVICE,
                         std::string("no usable CUDA device (") +
                             (e == cudaSuccess ? "count is 0" : cudaGetErrorString(e)) +
                             "); this library has no CPU path");
    }
    if (device < 0) GSC_CUDA(cudaGetDevice(&device));
    if (device >= count || device >= 64)
        return set_error(GSC_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if (!g_ctx[device]) {
        DeviceGuard g;
        GSC_TRY(g.set(device));
        auto *c = new DeviceCtx();
        c->device = device;
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->scratch_ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(c->scratch_ready, c->stream);
        if (e == cudaSuccess) e = cudaMalloc(&c->status, 256);
        if (e == cudaSuccess) e = cudaMemset(c->status, 0, 256);
        if (e != cudaSuccess) {
            // a context that failed half-way is released; the next call retries
            if (c->status) cudaFree(c->status);
            if (c->scratch_ready) cudaEventDestroy(c->scratch_ready);
            if (c->stream) cudaStreamDestroy(c->stream);
            delete c;
            return cuda_fail(e, "device context");
        }
        g_ctx[device] = c;
    }
    *out = g_ctx[device];
    return GSC_OK;
}

// ---------------------------------------------------------------------------
// per-device kernel set-up
// ---------------------------------------------------------------------------
struct OnceRegistry {
    std::mutex mu;
    std::vector<std::pair<const void *, int>> done;   // (key, device) pairs set up

    int run(const void *key, int device, const std::function<int()> &setup) {
        std::lock_guard<std::mutex> lk(mu);
        for (const auto &d : done)
            if (d.first == key && d.second == device) return GSC_OK;
        const int rc = setup();
        if (rc == GSC_OK) done.emplace_back(key, device);
        return rc;
    }
};
static OnceRegistry g_once;

int once_per_device(const void *key, int device, const std::function<int()> &setup) {
    return g_once.run(key, device, setup);
}

int smem_attr(const void *fn, size_t smem) {
    int device = 0;
    GSC_CUDA(cudaGetDevice(&device));
    return g_once.run(fn, device, [fn, smem]() -> int {
        GSC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
        return GSC_OK;
    });
}

// Allocation-failure injection (gsc_selftest_fail_alloc): -1 = off, k >= 0 =
// the k-th next allocation of a library buffer fails as out of memory.
static std::atomic<int> g_fail_alloc{-1};

static bool alloc_injected() {
    int v = g_fail_alloc.load();
    while (v >= 0) {
        if (g_fail_alloc.compare_exchange_weak(v, v - 1)) return v == 0;
    }
    return false;
}

int alloc_device(void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (alloc_injected())
        return set_error(GSC_ERR_NOMEM, std::string(what) + ": injected allocation failure");
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, what);
    }
    return GSC_OK;
}

int alloc_pinned(void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (alloc_injected())
        return set_error(GSC_ERR_NOMEM, std::string(what) + ": injected allocation failure");
    cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, what);
    }
    return GSC_OK;
}

static size_t grow_size(size_t bytes) {
    const size_t two_mb = size_t(2) << 20;
    size_t want = bytes + bytes / 4;
    return (want + two_mb - 1) / two_mb * two_mb;
}

int ensure_dev(DeviceCtx &ctx, DevBuf &buf, size_t bytes) {
    if (buf.bytes >= bytes && buf.ptr) return GSC_OK;
    if (buf.ptr) {
        // the old buffer may still be read by queued work on any stream
        GSC_CUDA(cudaEventSynchronize(ctx.scratch_ready));
        GSC_CUDA(cudaStreamSynchronize(ctx.stream));
        GSC_CUDA(cudaFree(buf.ptr));
        buf.ptr = nullptr;
        buf.bytes = 0;
    }
    const size_t n = grow_size(bytes);
    void *p = nullptr;
    GSC_TRY(alloc_device(&p, n, "cudaMalloc (scratch)"));
    buf.ptr = p;
    buf.bytes = n;
    return GSC_OK;
}

int ensure_pinned(DeviceCtx &ctx, size_t bytes) {
    if (ctx.pinned_bytes >= bytes && ctx.pinned) return GSC_OK;
    if (ctx.pinned) {
        GSC_CUDA(cudaStreamSynchronize(ctx.stream));
        GSC_CUDA(cudaFreeHost(ctx.pinned));
        ctx.pinned = nullptr;
        ctx.pinned_bytes = 0;
    }
    const size_t n = grow_size(bytes);
    void *p = nullptr;
    GSC_TRY(alloc_pinned(&p, n, "cudaHostAlloc (staging)"));
    ctx.pinned = p;
    ctx.pinned_bytes = n;
    return GSC_OK;
}

// ---------------------------------------------------------------------------
// options and validation
// ---------------------------------------------------------------------------

int resolve_opts(const gsc_opts *o, Resolved *r) {
    if (!o) return GSC_OK;
    if (o->struct_size < static_cast<int32_t>(sizeof(gsc_opts)))
        return set_error(GSC_ERR_INVALID, "gsc_opts.struct_size is smaller than sizeof(gsc_opts)");
    if (o->form < GSC_FORM_AUTO || o->form > GSC_FORM_SEP_F64)
        return set_error(GSC_ERR_INVALID, "unknown form");
    r->form = o->form;
    r->device = o->device;
    r->flags = o->flags;
    r->stream = static_cast<cudaStream_t>(o->stream);
    if (o->tolerance > 0) r->tolerance = o->tolerance;
    return GSC_OK;
}

static int check_sizes(int64_t dim, int64_t n_modes, int64_t n_points) {
    if (dim < 0 || n_modes < 0 || n_points < 0)
        return set_error(GSC_ERR_INVALID, "negative dimension, mode count or point count");
    if (dim > 65536) return set_error(GSC_ERR_INVALID, "dimension too large");
    return GSC_OK;
}

static int need_ptr(const void *p, bool needed, const char *name) {
    if (needed && !p) return set_error(GSC_ERR_INVALID, std::string(name) + " is NULL");
    return GSC_OK;
}

int check_device_ptr(const void *p, const char *name) {
    if (!p) return GSC_OK;
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GSC_ERR_INVALID, std::string(name) + " is not a CUDA pointer");
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged &&
        at.type != cudaMemoryTypeHost)
        return set_error(GSC_ERR_INVALID,
                         std::string(name) + " is not device-accessible memory");
    return GSC_OK;
}

static bool is_sep(int form) {
    return form == GSC_FORM_SEP_F16X3 || form == GSC_FORM_SEP_BF16X3 ||
           form == GSC_FORM_SEP_F16X5 || form == GSC_FORM_SEP_F64;
}

static int unstructured_form(const Resolved &r) {
    if (is_sep(r.form))
        return set_error(GSC_ERR_INVALID,
                         "separable (tensor-core) forms need a structured grid; use the "
                         "gsc_summate*_structured entry points");
    return GSC_OK;
}

// Largest max|err| / field RMS each form is validated to (tests and bench
// measure it); AUTO picks the fastest form whose bound fits the tolerance.
constexpr double kBoundSepF16x3 = 1e-5;
constexpr double kBoundSepF16x5 = 1e-6;
constexpr double kBoundMixed = 1e-6;

static bool is_mixed(int form) {
    return form == GSC_FORM_MIXED || form == GSC_FORM_MIXED_F64PHASE;
}

static int point_form(const Resolved &ro, const PlainArgs &a) {
    int f = ro.form;
    if (f == GSC_FORM_AUTO) f = ro.tolerance >= kBoundMixed ? GSC_FORM_MIXED : GSC_FORM_PLAIN_F64;
    const bool mixed_ok = a.dim >= 1 && a.dim <= 3 && !(a.incompr && a.dim == 1);
    return (is_mixed(f) && !mixed_ok) ? GSC_FORM_PLAIN_F64 : f;
}

// plain or mixed forms on explicit points (device pointers in `a`);
// range_flag: device word the mixed form sets when a wave number is past its
// integer phase range (see mixed_fx.cu)
static int run_points(DeviceCtx &ctx, const Resolved &ro, PlainArgs &a, cudaStream_t st,
                      int *range_flag) {
    const int f = point_form(ro, a);
    if (f == GSC_FORM_MIXED) return mixed_fx_run(ctx, a, range_flag, st);
    if (f == GSC_FORM_MIXED_F64PHASE) return mixed_run(ctx, a, true, st);
    a.variant = f == GSC_FORM_PLAIN_F64_LIBM ? 1 : 0;
    return plain_run(ctx, a, st);
}

static int structured_form(const Resolved &r, int64_t dim) {
    int f = r.form;
    if (f == GSC_FORM_AUTO)
        f = r.tolerance >= kBoundSepF16x3   ? GSC_FORM_SEP_F16X3
            : r.tolerance >= kBoundSepF16x5 ? GSC_FORM_SEP_F16X5
                                            : GSC_FORM_SEP_F64;
    if (is_sep(f) && dim < 2)   // 1-D: nothing to contract
        f = (r.form == GSC_FORM_AUTO && r.tolerance >= kBoundMixed) ? GSC_FORM_MIXED
                                                                  : GSC_FORM_PLAIN_F64;
    return f;
}

// Words of the per-device status buffer (256 bytes of device memory):
//   [0] sticky pipeline status: a bounded wait gave up (sm100.cuh codes)
//   [1] the last sep_f16x5 call's bound flag (written by every such call):
//       1 when its inputs break the exact leading sum's bound
//   [2] sticky: an explicit sep_f16x5 call on device pointers was flagged
//       and left its output invalid
//   [3] the last host-pointer mixed call's range flag (cleared by the call)
//       where the device does not map the pinned staging word that takes
//       it otherwise
//   [4] sticky: a mixed call on device pointers (or a batch) met a wave
//       number past the integer phase range (its output is invalid)
//   [5] the device half of a host call's flattened-mesh check: 1 when a
//       point differs from the candidate axes (cleared by the call)
//   [6] the range flag of the current device-pointer mixed call under AUTO
//       (cleared by the call; the plain FP64 launches behind it run on it)
//   [7] the range flag of the current host-array batch call (batch.cu;
//       cleared by the call)
constexpr int kStatusPipeline = 0, kStatusX5Flag = 1, kStatusX5Sticky = 2, kStatusFxFlag = 3,
              kStatusFxSticky = 4, kStatusMeshCheck = 5, kStatusFxDev = 6;

static const char *kFxRangeMsg =
    "mixed: a wave number times the largest coordinate exceeds 2^30 turns, past the range of "
    "its integer phase; the output is invalid.  Use form AUTO on host arrays (which recomputes "
    "such calls on the plain FP64 kernel) or plain";
static const char *kX5BoundMsg =
    "sep_f16x5: these inputs break the bound that keeps its leading sum exact (weights far "
    "from random, e.g. in phase at a grid point); the output is invalid.  Use form AUTO (which "
    "recomputes such calls on sep_f64) or sep_f64";

// Point kernels on device pointers.  A mixed call under AUTO writes its
// range flag to a word of its own, and the plain FP64 kernels are queued
// behind it, predicated on that word: a wave number past the integer
// phase's range is recomputed on the device, with no host synchronisation.
// An explicit mixed form leaves its output invalid and sets the sticky word.
static int run_points_dev(DeviceCtx &ctx, const Resolved &ro, PlainArgs &a, cudaStream_t st) {
    if (ro.form != GSC_FORM_AUTO || point_form(ro, a) != GSC_FORM_MIXED)
        return run_points(ctx, ro, a, st, ctx.status + kStatusFxSticky);
    int *flag = ctx.status + kStatusFxDev;
    GSC_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    GSC_TRY(run_points(ctx, ro, a, st, flag));
    PlainArgs b = a;
    b.variant = 0;
    b.run_if = flag;
    return plain_run(ctx, b, st);
}

// Reads and clears the sticky status words after the stream has finished.
static int check_status(DeviceCtx &ctx, cudaStream_t st) {
    int v[5] = {0, 0, 0, 0, 0};
    GSC_CUDA(cudaMemcpyAsync(v, ctx.status, sizeof(v), cudaMemcpyDeviceToHost, st));
    GSC_CUDA(cudaStreamSynchronize(st));
    if (v[kStatusPipeline] != 0 || v[kStatusX5Sticky] != 0 || v[kStatusFxSticky] != 0) {
        for (int w : {kStatusPipeline, kStatusX5Sticky, kStatusFxSticky})
            GSC_CUDA(cudaMemsetAsync(ctx.status + w, 0, sizeof(int), st));
        GSC_CUDA(cudaStreamSynchronize(st));
        if (v[kStatusPipeline] != 0)
            return set_error(GSC_ERR_KERNEL, "a tensor-core pipeline wait gave up (status " +
                                                 std::to_string(v[kStatusPipeline]) +
                                                 "); the output is invalid");
        if (v[kStatusX5Sticky] != 0) return set_error(GSC_ERR_KERNEL, kX5BoundMsg);
        return set_error(GSC_ERR_KERNEL, kFxRangeMsg);
    }
    return GSC_OK;
}

void parallel_copy(void *dst, const void *src, size_t n) {
    constexpr size_t kMinPart = size_t(4) << 20;
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::min<size_t>(std::min<size_t>(8, hw ? hw : 1), n / kMinPart);
    if (T <= 1) {
        memcpy(dst, src, n);
        return;
    }
    const size_t part = (n + T - 1) / T;
    std::vector<std::thread> th;
    th.reserve(T - 1);
    for (size_t t = 1; t < T; ++t) {
        const size_t o = t * part;
        if (o >= n) break;
        const size_t len = std::min(part, n - o);
        th.emplace_back([=] {
            memcpy(static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, len);
        });
    }
    memcpy(dst, src, std::min(part, n));
    for (auto &x : th) x.join();
}

int h2d_packed(cudaStream_t st, void *d, void *h, const std::vector<HostSrc> &segs) {
    constexpr size_t kChunk = size_t(64) << 20;
    if (segs.empty()) return GSC_OK;
    size_t total = 0, first = segs.front().off;
    for (const auto &sg : segs) {
        total = std::max(total, sg.off + sg.bytes);
        first = std::min(first, sg.off);
    }
    if (total <= first) return GSC_OK;
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::max<size_t>(1, std::min<size_t>(16, hw ? hw : 1));
    // bytes [a, b) of the packed image, from the segments they belong to
    // (segments in increasing offset order)
    auto copy_range = [&](size_t a, size_t b) {
        size_t k = static_cast<size_t>(
            std::upper_bound(segs.begin(), segs.end(), a,
                             [](size_t v, const HostSrc &x) { return v < x.off; }) - segs.begin());
        k = k > 0 ? k - 1 : 0;
        for (; k < segs.size() && segs[k].off < b; ++k) {
            const size_t lo = std::max(a, segs[k].off), hi = std::min(b, segs[k].off + segs[k].bytes);
            if (lo < hi && segs[k].src)
                memcpy(static_cast<char *>(h) + lo,
                       static_cast<const char *>(segs[k].src) + (lo - segs[k].off), hi - lo);
        }
    };
    for (size_t c0 = first; c0 < total; c0 += kChunk) {
        const size_t c1 = std::min(total, c0 + kChunk);
        const size_t n = c1 - c0;
        const size_t t_used = std::max<size_t>(1, std::min<size_t>(T, n / (size_t(1) << 20)));
        if (t_used == 1) {
            copy_range(c0, c1);
        } else {
            std::vector<std::thread> th;
            const size_t per = (n + t_used - 1) / t_used;
            for (size_t t = 1; t < t_used; ++t) {
                const size_t a = c0 + t * per, b = std::min(c1, a + per);
                if (a < b) th.emplace_back(copy_range, a, b);
            }
            copy_range(c0, std::min(c1, c0 + per));
            for (auto &x : th) x.join();
        }
        // this chunk's DMA runs while the host copies the next one
        GSC_CUDA(cudaMemcpyAsync(static_cast<char *>(d) + c0, static_cast<char *>(h) + c0, n,
                                 cudaMemcpyHostToDevice, st));
    }
    return GSC_OK;
}

int d2h_scatter(DeviceCtx &ctx, cudaStream_t st, const void *src, size_t n,
                const std::vector<HostSeg> &segs) {
    constexpr size_t kChunk = size_t(32) << 20;
    if (n == 0) return GSC_OK;
    // copies bytes [o, o + len) of the device range, staged at `stage`, to
    // the host segments they belong to
    size_t seg = 0, seg_start = 0;
    auto scatter = [&](const char *stage, size_t o, size_t len) {
        while (len > 0) {
            while (seg < segs.size() && o >= seg_start + segs[seg].bytes) {
                seg_start += segs[seg].bytes;
                ++seg;
            }
            if (seg >= segs.size()) return;
            const size_t in_seg = o - seg_start;
            const size_t take = std::min(len, segs[seg].bytes - in_seg);
            parallel_copy(static_cast<char *>(segs[seg].dst) + in_seg, stage, take);
            stage += take;
            o += take;
            len -= take;
        }
    };
    if (n <= kChunk) {
        GSC_TRY(ensure_pinned(ctx, n));
        GSC_CUDA(cudaMemcpyAsync(ctx.pinned, src, n, cudaMemcpyDeviceToHost, st));
        GSC_CUDA(cudaStreamSynchronize(st));
        scatter(static_cast<const char *>(ctx.pinned), 0, n);
        return GSC_OK;
    }
    GSC_TRY(ensure_pinned(ctx, 2 * kChunk));
    for (auto &e : ctx.stage_ev)
        if (!e) GSC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    char *pin[2] = {static_cast<char *>(ctx.pinned), static_cast<char *>(ctx.pinned) + kChunk};
    const size_t chunks = (n + kChunk - 1) / kChunk;
    for (size_t k = 0; k <= chunks; ++k) {
        if (k < chunks) {
            const size_t o = k * kChunk, len = std::min(kChunk, n - o);
            GSC_CUDA(cudaMemcpyAsync(pin[k & 1], static_cast<const char *>(src) + o, len,
                                     cudaMemcpyDeviceToHost, st));
            GSC_CUDA(cudaEventRecord(ctx.stage_ev[k & 1], st));
        }
        if (k > 0) {   // chunk k-1 is copied out while chunk k is in flight
            const size_t j = k - 1, o = j * kChunk, len = std::min(kChunk, n - o);
            GSC_CUDA(cudaEventSynchronize(ctx.stage_ev[j & 1]));
            scatter(pin[j & 1], o, len);
        }
    }
    return GSC_OK;
}

int d2h_staged(DeviceCtx &ctx, cudaStream_t st, void *dst, const void *src, size_t n) {
    return d2h_scatter(ctx, st, src, n, {HostSeg{dst, n}});
}

// Host memory the GPU reads or writes directly (pageable memory on a
// coherent host link moves at DMA speed once its pages exist): first-touch
// faults of fresh output arrays are the cost, so they are taken on host
// threads while the GPU computes.
void Prefault::start(void *p, size_t n) {
    if (p && n) start_many({HostSeg{p, n}});
}

void Prefault::start_many(const std::vector<HostSeg> &segs) {
    static const size_t kPage = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? static_cast<size_t>(v) : size_t(4096);
    }();
    const size_t page = kPage;
    // (segment, first page, end page) pieces, then an equal share per thread
    size_t total = 0;
    for (auto &sg : segs) total += sg.dst && sg.bytes ? (sg.bytes + page - 1) / page : 0;
    if (total == 0) return;
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::max<size_t>(1, std::min<size_t>(std::min<size_t>(8, hw ? hw : 1),
                                                          (total + 255) / 256));
    const size_t per = (total + T - 1) / T;
    auto touch_range = [segs, page](size_t a, size_t b) {   // global page indices [a, b)
        size_t first = 0;
        for (auto &sg : segs) {
            if (!sg.dst || !sg.bytes) continue;
            const size_t np = (sg.bytes + page - 1) / page;
            const size_t lo = std::max(a, first), hi = std::min(b, first + np);
            for (size_t i = lo; i < hi; ++i) {
                volatile char *c = static_cast<char *>(sg.dst) + std::min((i - first) * page, sg.bytes - 1);
                *c = 0;
            }
            first += np;
            if (first >= b) break;
        }
    };
    if (T == 1) {
        touch_range(0, total);
        return;
    }
    for (size_t t = 0; t < T; ++t) {
        const size_t a = t * per, b = std::min(total, a + per);
        if (a < b) th.emplace_back(touch_range, a, b);
    }
}

void Prefault::join() {
    for (auto &x : th) x.join();
    th.clear();
}

// Uploads a (rows, cols) host view to dense row-major device memory at
// d + off: large contiguous arrays go directly, others through the pinned
// buffer `h` at the same offset.
static int upload2(cudaStream_t st, double *d, double *h, size_t off, const double *src,
                   int64_t s0, int64_t s1, int64_t rows, int64_t cols);

// gathers a strided (rows, cols) host view into dense row-major dst
static void gather2(const double *src, int64_t s0, int64_t s1, int64_t rows, int64_t cols,
                    double *dst);

static int upload2(cudaStream_t st, double *d, double *h, size_t off, const double *src,
                   int64_t s0, int64_t s1, int64_t rows, int64_t cols) {
    const size_t n = static_cast<size_t>(rows * cols);
    if (n == 0) return GSC_OK;
    const bool contiguous = s1 == 1 && (rows == 1 || s0 == cols);
    if (contiguous && n * sizeof(double) >= (size_t(1) << 20)) {
        GSC_CUDA(cudaMemcpyAsync(d + off, src, n * sizeof(double), cudaMemcpyHostToDevice, st));
    } else {
        gather2(src, s0, s1, rows, cols, h + off);
        GSC_CUDA(cudaMemcpyAsync(d + off, h + off, n * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    return GSC_OK;
}

// Adds a (rows, cols) host view at element offset `off` of the packed input
// image: contiguous views as segments that h2d_packed copies, others gathered
// into h now.
static void stage2(std::vector<HostSrc> &segs, double *h, size_t off, const double *src,
                   int64_t s0, int64_t s1, int64_t rows, int64_t cols) {
    const size_t n = static_cast<size_t>(rows * cols);
    if (n == 0) return;
    const bool contiguous = s1 == 1 && (rows == 1 || s0 == cols);
    if (!contiguous) gather2(src, s0, s1, rows, cols, h + off);
    segs.push_back({contiguous ? static_cast<const void *>(src) : nullptr, off * sizeof(double),
                    n * sizeof(double)});
}

static void gather2(const double *src, int64_t s0, int64_t s1, int64_t rows, int64_t cols,
                    double *dst) {
    for (int64_t i = 0; i < rows; ++i) {
        const double *row = src + i * s0;
        double *o = dst + i * cols;
        if (s1 == 1) {
            parallel_copy(o, row, sizeof(double) * static_cast<size_t>(cols));
        } else {
            for (int64_t j = 0; j < cols; ++j) o[j] = row[j * s1];
        }
    }
}

// ---------------------------------------------------------------------------
// structured points passed as a list
// ---------------------------------------------------------------------------
constexpr int64_t kGridMinPoints = 4096;   // smaller grids are not worth routing

// Runs f(begin, end) over [0, n) on up to max_threads host threads (one for
// small n).
template <class F>
static void parallel_ranges(int64_t n, int64_t min_per_thread, F f, int64_t max_threads = 8) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t T = std::max<int64_t>(
        1, std::min<int64_t>(std::min<int64_t>(max_threads, hw ? hw : 1),
                             n / std::max<int64_t>(1, min_per_thread)));
    if (T <= 1) {
        f(int64_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    const int64_t per = (n + T - 1) / T;
    for (int64_t t = 1; t < T; ++t) {
        const int64_t a = t * per, b = std::min(n, a + per);
        if (a < b) th.emplace_back(f, a, b);
    }
    f(int64_t(0), std::min(n, per));
    for (auto &x : th) x.join();
}

// If pos (dim, P) may hold meshgrid(axes, indexing="ij") flattened in C
// order -- how GSTools lays out the points of a structured mesh before it
// calls summate -- returns true with the candidate axes, read from the run
// lengths of the first coordinates (a few reads per axis value).
static bool grid_candidate(const double *pos, int64_t sd, int64_t sp, int64_t dim, int64_t P,
                           std::vector<double> ax[3], int64_t n[3]) {
    if ((dim != 2 && dim != 3) || P < kGridMinPoints) return false;
    auto at = [=](int64_t d, int64_t i) { return pos[d * sd + i * sp]; };
    // axis 0 is constant over runs of L0 = n1 (* n2) points, axis 1 (3-D) over L1 = n2
    int64_t L0 = 1;
    while (L0 < P && at(0, L0) == at(0, 0)) ++L0;
    if (P % L0 != 0) return false;
    int64_t L1 = 1;
    if (dim == 3) {
        while (L1 < L0 && at(1, L1) == at(1, 0)) ++L1;
        if (L0 % L1 != 0) return false;
    }
    n[0] = P / L0;
    n[1] = dim == 3 ? L0 / L1 : L0;
    n[2] = dim == 3 ? L1 : 1;
    for (int d = 0; d < dim; ++d)
        if (n[d] < 2) return false;
    ax[0].resize(static_cast<size_t>(n[0]));
    ax[1].resize(static_cast<size_t>(n[1]));
    for (int64_t a = 0; a < n[0]; ++a) ax[0][a] = at(0, a * L0);
    for (int64_t b = 0; b < n[1]; ++b) ax[1][b] = at(1, b * L1);
    if (dim == 3) {
        ax[2].resize(static_cast<size_t>(n[2]));
        for (int64_t c = 0; c < n[2]; ++c) ax[2][c] = at(2, c);
    }
    return true;
}

// Every point of one x-slice of a C-order mesh against the candidate axes:
// the rows read once, with no early exit inside the slice, so that the
// compiler can vectorize the loads and compares (the check is bound by host
// memory bandwidth).  `good` stays an integer mask: a NaN coordinate
// compares unequal and fails the check.
__attribute__((optimize("O3"))) static bool grid_verify_rows(
    const double *__restrict__ p0, const double *__restrict__ p1, const double *__restrict__ p2,
    int64_t dim, const double *a0, const double *a1, const double *a2, int64_t a, int64_t n1,
    int64_t n2) {
    const int64_t L0 = n1 * n2;
    const double x0 = a0[a];
    uint64_t bad = 0;
    for (int64_t i = 0; i < L0; ++i) bad |= static_cast<uint64_t>(p0[i] != x0);
    if (dim == 3) {
        for (int64_t b = 0; b < n1; ++b) {
            const double x1 = a1[b];
            const double *r1 = p1 + b * n2, *r2 = p2 + b * n2;
            for (int64_t c = 0; c < n2; ++c)
                bad |= static_cast<uint64_t>(r1[c] != x1) | static_cast<uint64_t>(r2[c] != a2[c]);
        }
    } else {
        for (int64_t b = 0; b < n1; ++b) bad |= static_cast<uint64_t>(p1[b] != a1[b]);
    }
    return bad == 0;
}

// Every point of x-slices [a_begin, n0) of pos against the candidate axes,
// bit for bit, slice by slice on all host cores (the check reads those
// slices once; no divisions in the loops).
static bool grid_verify(const double *pos, int64_t sd, int64_t sp, int64_t dim,
                        const std::vector<double> ax[3], const int64_t n[3],
                        int64_t max_threads = 64, int64_t a_begin = 0) {
    auto at = [=](int64_t d, int64_t i) { return pos[d * sd + i * sp]; };
    std::atomic<bool> ok(true);
    const double *a0 = ax[0].data(), *a1 = ax[1].data(), *a2 = dim == 3 ? ax[2].data() : nullptr;
    const int64_t n1 = n[1], n2 = dim == 3 ? n[2] : 1, L0 = n1 * n2, L1 = n2;
    parallel_ranges(n[0] - a_begin, std::max<int64_t>(1, (int64_t(1) << 18) / L0), [&](int64_t s0, int64_t s1) {
        for (int64_t a = a_begin + s0; a < a_begin + s1 && ok.load(std::memory_order_relaxed); ++a) {
            const int64_t base = a * L0;
            bool good = true;
            if (sp == 1) {      // C-contiguous rows: the vectorizable form
                good = grid_verify_rows(pos + base, pos + sd + base,
                                        dim == 3 ? pos + 2 * sd + base : nullptr, dim, a0, a1, a2,
                                        a, n1, n2);
            } else {
                const double x0 = a0[a];
                for (int64_t i = 0; i < L0; ++i) good &= at(0, base + i) == x0;
                if (dim == 3) {
                    for (int64_t b = 0; b < n1; ++b) {
                        const double x1 = a1[b];
                        const int64_t off = base + b * L1;
                        for (int64_t c = 0; c < n2; ++c)
                            good &= (at(1, off + c) == x1) & (at(2, off + c) == a2[c]);
                    }
                } else {
                    for (int64_t b = 0; b < n1; ++b) good &= at(1, base + b) == a1[b];
                }
            }
            if (!good) ok.store(false, std::memory_order_relaxed);
        }
    }, max_threads);
    return ok.load();
}

static bool detect_grid(const double *pos, int64_t sd, int64_t sp, int64_t dim, int64_t P,
                        std::vector<double> ax[3], int64_t n[3]) {
    return grid_candidate(pos, sd, sp, dim, P, ax, n) && grid_verify(pos, sd, sp, dim, ax, n);
}

// [lo, hi) byte range spanned by a (rows, cols) view with element strides
static void view_span(const double *p, int64_t s0, int64_t s1, int64_t rows, int64_t cols,
                      uintptr_t &lo, uintptr_t &hi) {
    int64_t a = 0, b = 0;
    for (int64_t s : {s0 * (rows - 1), s1 * (cols - 1)}) (s < 0 ? a : b) += s;
    lo = reinterpret_cast<uintptr_t>(p + a);
    hi = reinterpret_cast<uintptr_t>(p + b + 1);
}

// The device's share of the check of a flattened mesh: x-slices [0, na) of
// C-ordered positions, and the candidate axes, read in place from host
// memory while the separable form computes.  bad is the result.
struct MeshCheck {
    const double *pos;       // host, rows of P contiguous coordinates
    int64_t sd;              // row stride (elements)
    int64_t na;              // x-slices checked on the device
    const double *ax[3];     // candidate axes, host
    int64_t n[3];
    int dim;
    int bad = 1;             // out: 0 only when every checked point matched
};

// Any point of slices [0, na) that differs from the candidate axes (or is
// NaN) sets *bad.  Warps take rows of contiguous points -- (x-slice, y) rows
// of n2 points in 3-D, x-slices of n1 points in 2-D -- so that the axis
// indices cost one division per row; lanes stride along the row with four
// iterations' host reads in flight.
__global__ void __launch_bounds__(1024) mesh_check_kernel(const double *__restrict__ pos,
                                                          int64_t sd, int64_t na, int64_t n1,
                                                          int64_t n2, int dim,
                                                          const double *__restrict__ a0,
                                                          const double *__restrict__ a1,
                                                          const double *__restrict__ a2, int *bad) {
    const int lane = static_cast<int>(threadIdx.x & 31);
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t L = dim == 3 ? n2 : n1;                 // points per row
    const int64_t rows = dim == 3 ? na * n1 : na;
    int miss = 0;
    for (int64_t row = warp; row < rows; row += n_warps) {
        const int64_t a = dim == 3 ? row / n1 : row;
        const double xa = a0[a];
        const double *px = pos + row * L, *py = px + sd;
        if (dim == 3) {
            const double yb = a1[row - a * n1];
            const double *pz = px + 2 * sd;
#pragma unroll 4
            for (int64_t c = lane; c < L; c += 32)
                miss |= (px[c] != xa) | (py[c] != yb) | (pz[c] != a2[c]);
        } else {
#pragma unroll 4
            for (int64_t c = lane; c < L; c += 32) miss |= (px[c] != xa) | (py[c] != a1[c]);
        }
    }
    if (__syncthreads_or(miss) && threadIdx.x == 0) atomicOr(bad, 1);
}

static int host_structured(const double *cov, int64_t cs_d, int64_t cs_n, const double *z1,
                           int64_t z1s, const double *z2, int64_t z2s, int64_t dim, int64_t N,
                           const double *const *ax, const int64_t *n, const int64_t *sx,
                           double *out, bool incompr, const gsc_opts *opts,
                           const double *sf, int64_t sfs, bool interleave = false,
                           MeshCheck *mc = nullptr);

static int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) {
        cudaGetLastError();
        d = 0;
    }
    return d;
}

// Whether kernels on `device` may read pageable host memory in place
// (coherent access through the host's page tables).
static bool pageable_access(int device) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return v != 0;
}

// ---------------------------------------------------------------------------
// host-pointer path shared by the scalar and incompressible summators
// ---------------------------------------------------------------------------
static int host_plain(const double *cov, int64_t cs_d, int64_t cs_n, const double *z1,
                      int64_t z1s, const double *z2, int64_t z2s, const double *pos,
                      int64_t ps_d, int64_t ps_p, int64_t dim, int64_t N, int64_t P,
                      double *out, int64_t os_d, int64_t os_p, bool incompr,
                      const gsc_opts *opts, const double *sf = nullptr, int64_t sfs = 0) {
    // sf != nullptr: Fourier method, spectrum factor sf[j * sfs] (scalar field)
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    GSC_TRY(check_sizes(dim, N, P));
    if (incompr && dim != 2 && dim != 3)
        return set_error(GSC_ERR_DIM, "Only two- and three-dimensional problems are supported.");
    GSC_TRY(need_ptr(cov, dim * N > 0, "cov_samples"));
    GSC_TRY(need_ptr(z1, N > 0, "z1"));
    GSC_TRY(need_ptr(z2, N > 0, "z2"));
    GSC_TRY(need_ptr(pos, dim * P > 0, "pos"));
    GSC_TRY(need_ptr(out, P > 0, "out"));
    GSC_TRY(unstructured_form(ro));
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    if (P == 0) return GSC_OK;
    const size_t n_sf = sf ? static_cast<size_t>(N) : 0;
    const int64_t nout = incompr ? dim : 1;

    // AUTO on a flattened structured mesh: the separable forms on its axes
    // (FP64 DMMA at the default tolerance, within the same 1e-12 bar)
    // The candidate axes come from the first coordinates' run lengths; the
    // check of every point (one read of the whole array on the host cores)
    // runs on a host thread while the GPU computes on the candidate axes.  A
    // check that fails discards that result: the point kernels recompute it.
    if (ro.form == GSC_FORM_AUTO) {
        std::vector<double> axv[3];
        int64_t n[3] = {1, 1, 1};
        if (grid_candidate(pos, ps_d, ps_p, dim, P, axv, n)) {
            const double *axp[3] = {axv[0].data(), axv[1].data(), dim == 3 ? axv[2].data() : nullptr};
            const int64_t sx[3] = {1, 1, 1};
            const bool c_out = os_p == 1 && (nout == 1 || os_d == P);
            const bool f_out = !c_out && os_d == 1 && os_p == nout;   // summate_incompr's layout
            std::unique_ptr<double[]> tmp;
            if (!c_out && !f_out) tmp.reset(new double[static_cast<size_t>(nout * P)]);
            double *dst = tmp ? tmp.get() : out;
            // the result may be written while the points are read only if
            // the two do not share memory
            uintptr_t plo, phi, olo, ohi;
            view_span(pos, ps_d, ps_p, dim, P, plo, phi);
            view_span(dst, tmp ? P : os_d, tmp ? 1 : os_p, nout, P, olo, ohi);
            const bool overlap_ok = ohi <= plo || phi <= olo;
            bool is_grid = false;
            int rc = GSC_OK;
            if (overlap_ok) {
                // one core stays free for this thread, which issues the GPU work
                const unsigned hw = std::thread::hardware_concurrency();
                const int64_t workers = std::max<int64_t>(1, static_cast<int64_t>(hw ? hw : 2) - 1);
                // Where the GPU reads pageable host memory in place, it checks
                // the first x-slices of C-ordered rows while the host cores
                // check the rest.  Its share f balances the host link, which
                // carries the device's reads and the result's copy (about 180
                // GB/s together on a GB300 node), against the host cores'
                // reads (about 82 GB/s while the copy writes into host
                // memory): f = 0.687 - 0.313 r, r = result bytes / mesh
                // bytes = components / dimensions (C2 0.58, C4 0.37)
                MeshCheck mc;
                const bool dev_check = ps_p == 1 && n[0] >= 4 &&
                                       static_cast<size_t>(dim * P) * sizeof(double) >= (size_t(32) << 20) &&
                                       pageable_access(ro.device >= 0 ? ro.device : current_device());
                if (dev_check) {
                    mc.pos = pos;
                    mc.sd = ps_d;
                    const int64_t f_milli = 687 - 313 * nout / dim;
                    mc.na = std::max<int64_t>(1, std::min<int64_t>(n[0] - 1, n[0] * f_milli / 1000));
                    for (int k = 0; k < 3; ++k) {
                        mc.ax[k] = k < dim ? axv[k].data() : nullptr;
                        mc.n[k] = n[k];
                    }
                    mc.dim = static_cast<int>(dim);
                }
                const int64_t a_host = dev_check ? mc.na : 0;
                bool host_ok = false;
                std::thread check([&] { host_ok = grid_verify(pos, ps_d, ps_p, dim, axv, n, workers, a_host); });
                rc = host_structured(cov, cs_d, cs_n, z1, z1s, z2, z2s, dim, N, axp, n, sx, dst,
                                     incompr, opts, sf, sfs, f_out, dev_check ? &mc : nullptr);
                check.join();
                is_grid = host_ok && (!dev_check || mc.bad == 0);
            } else if ((is_grid = grid_verify(pos, ps_d, ps_p, dim, axv, n))) {
                rc = host_structured(cov, cs_d, cs_n, z1, z1s, z2, z2s, dim, N, axp, n, sx, dst,
                                     incompr, opts, sf, sfs, f_out);
            }
            if (is_grid) {
                GSC_TRY(rc);
                if (tmp)
                    parallel_ranges(P, int64_t(1) << 18, [&](int64_t b, int64_t e) {
                        for (int64_t i = 0; i < nout; ++i)
                            for (int64_t p = b; p < e; ++p) out[i * os_d + p * os_p] = tmp[i * P + p];
                    });
                return GSC_OK;
            }
            timing_reset(ro.flags & GSC_FLAG_TIMING);   // not a grid: the point kernels below
        }
    }

    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    cudaStream_t st = ctx->stream;

    // C-ordered positions stay where they are when the GPU reads pageable
    // host memory coherently (GB300's host link with address translation,
    // cudaDevAttrPageableMemoryAccess): the kernels read them in place, once
    // per mode split, and no host core packs them into staging.  Dense modes of the scalar and incompressible methods are read
    // in place too, by the one kernel that turns them into per-mode records
    // (dimensions 1-3; the generic kernel of other dimensions reads every
    // mode per point, and Fourier weights are scaled into staging first): a
    // call then copies nothing to the GPU, which saves the copy's fixed cost
    // of about 20 us.
    const size_t n_cov = static_cast<size_t>(dim * N);
    const bool pageable = pageable_access(ctx->device);
    const bool pos_in_place = ps_p == 1 && (dim == 1 || ps_d == P) && pageable;
    const bool modes_in_place = !sf && N > 0 && dim >= 1 && dim <= 3 && cs_n == 1 &&
                                (dim == 1 || cs_d == N) && z1s == 1 && z2s == 1 && pageable;
    const size_t n_pos = pos_in_place ? 0 : static_cast<size_t>(dim * P);
    const size_t n_m = modes_in_place ? 0 : n_cov + 2 * static_cast<size_t>(N);
    const size_t n_in = n_m + n_sf + n_pos;
    const size_t n_out = static_cast<size_t>(nout * P);
    const size_t bytes = (n_in + n_out) * sizeof(double);
    GSC_TRY(ensure_pinned(*ctx, bytes + 64));           // + the range flag's slot
    GSC_TRY(ensure_dev(*ctx, ctx->io, bytes));

    double *h = static_cast<double *>(ctx->pinned);
    double *d = static_cast<double *>(ctx->io.ptr);
    volatile int *hflag = reinterpret_cast<volatile int *>(h + n_in + n_out);
    TimedLaunch tc(st);
    tc.begin(K_COPY_H2D);
    // the inputs as one packed image, moved through the pinned buffer in
    // chunks (a DMA straight from a large pageable array runs at a fraction
    // of the link)
    std::vector<HostSrc> segs;
    if (!modes_in_place) {
        stage2(segs, h, 0, cov, cs_d, cs_n, dim, N);
        stage2(segs, h, n_cov, z1, 0, z1s, 1, N);
        stage2(segs, h, n_cov + N, z2, 0, z2s, 1, N);
    }
    if (sf) stage2(segs, h, n_m, sf, 0, sfs, 1, N);
    if (!pos_in_place) stage2(segs, h, n_m + n_sf, pos, ps_d, ps_p, dim, P);
    GSC_TRY(h2d_packed(st, d, h, segs));
    tc.end();
    if (sf) GSC_TRY(fourier_scale(d + n_m, d + n_cov, d + n_cov + N, N, d + n_cov,
                                  d + n_cov + N, st));
    PlainArgs a;
    a.cov = modes_in_place ? cov : d;
    a.z1 = modes_in_place ? z1 : d + n_cov;
    a.z2 = modes_in_place ? z2 : d + n_cov + N;
    a.pos = pos_in_place ? pos : d + n_m + n_sf;
    a.dim = dim;
    a.n_modes = N;
    a.n_points = P;
    a.incompr = incompr;
    // a C-ordered or Fortran-ordered result leaves the device in its own
    // layout (the kernels write with the output's strides), so it moves in
    // one contiguous copy
    const bool c_order = os_p == 1 && (nout == 1 || os_d == P);
    const bool f_order = !c_order && os_d == 1 && os_p == nout;
    // A pinned C- or Fortran-ordered result (the Python layer's pool blocks)
    // is written by the kernels in place over the coherent host link: no
    // copy back and none of its fixed cost.  Not where the result's bytes
    // overlap an input that is read in place.
    bool direct_out = (c_order || f_order) && pageable && is_pinned_host(out);
    if (direct_out) {
        uintptr_t olo, ohi;
        view_span(out, os_d, os_p, nout, P, olo, ohi);
        auto apart = [&](const double *q, int64_t s0, int64_t s1, int64_t rows, int64_t cols) {
            uintptr_t lo, hi;
            view_span(q, s0, s1, rows, cols, lo, hi);
            return ohi <= lo || hi <= olo;
        };
        if (pos_in_place && !apart(pos, ps_d, ps_p, dim, P)) direct_out = false;
        if (modes_in_place && (!apart(cov, cs_d, cs_n, dim, N) || !apart(z1, 0, z1s, 1, N) ||
                               !apart(z2, 0, z2s, 1, N)))
            direct_out = false;
    }
    a.out = direct_out ? out : d + n_in;
    a.out_sd = f_order ? 1 : P;
    a.out_sp = f_order ? nout : 1;
    const bool fx = point_form(ro, a) == GSC_FORM_MIXED;
    // wave numbers past the mixed form's integer phase range: AUTO recomputes
    // on the plain FP64 kernel, an explicit mixed form reports it.  The
    // record kernel writes the range flag straight into its pinned host word
    // where the device maps that memory (no clearing launch, no read-back
    // copy), else into the device status word, which is copied back with the
    // result.  Either way one synchronisation; a flagged result is discarded.
    *hflag = 0;
    int *dflag = ctx->status + kStatusFxFlag;
    bool flag_mapped = false;
    if (fx) {
        void *dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, const_cast<int *>(hflag), 0) == cudaSuccess && dp) {
            dflag = static_cast<int *>(dp);
            flag_mapped = true;
        } else {
            cudaGetLastError();
            GSC_CUDA(cudaMemsetAsync(dflag, 0, sizeof(int), st));
        }
    }
    GSC_TRY(run_points(*ctx, ro, a, st, dflag));
    auto recompute = [&]() -> int {
        if (ro.form != GSC_FORM_AUTO) return set_error(GSC_ERR_KERNEL, kFxRangeMsg);
        Resolved rp = ro;
        rp.form = GSC_FORM_PLAIN_F64;
        return run_points(*ctx, rp, a, st, nullptr);
    };
    if (direct_out) {
        if (fx && !flag_mapped)
            GSC_CUDA(cudaMemcpyAsync(const_cast<int *>(hflag), dflag, sizeof(int),
                                     cudaMemcpyDeviceToHost, st));
        GSC_CUDA(cudaStreamSynchronize(st));
        if (*hflag) {
            *hflag = 0;
            GSC_TRY(recompute());
            GSC_CUDA(cudaStreamSynchronize(st));
        }
        return GSC_OK;
    }
    if (c_order || f_order) {
        Prefault pf;
        if (!is_pinned_host(out)) pf.start(out, n_out * sizeof(double));
        pf.join();
        for (int pass = 0; pass < 2; ++pass) {
            if (fx && pass == 0 && !flag_mapped)
                GSC_CUDA(cudaMemcpyAsync(const_cast<int *>(hflag), dflag, sizeof(int),
                                         cudaMemcpyDeviceToHost, st));
            tc.begin(K_COPY_D2H);
            GSC_CUDA(cudaMemcpyAsync(out, a.out, n_out * sizeof(double), cudaMemcpyDeviceToHost, st));
            tc.end();
            GSC_CUDA(cudaStreamSynchronize(st));
            if (!*hflag) return GSC_OK;
            *hflag = 0;
            GSC_TRY(recompute());
        }
        return GSC_OK;
    }
    if (fx) {
        if (!flag_mapped)
            GSC_CUDA(cudaMemcpyAsync(const_cast<int *>(hflag), dflag, sizeof(int),
                                     cudaMemcpyDeviceToHost, st));
        GSC_CUDA(cudaStreamSynchronize(st));
        if (*hflag) GSC_TRY(recompute());
    }
    double *ho = h + n_in;
    tc.begin(K_COPY_D2H);
    GSC_CUDA(cudaMemcpyAsync(ho, a.out, n_out * sizeof(double), cudaMemcpyDeviceToHost, st));
    tc.end();
    GSC_CUDA(cudaStreamSynchronize(st));
    parallel_ranges(P, int64_t(1) << 18, [&](int64_t b, int64_t e) {
        for (int64_t i = 0; i < nout; ++i)
            for (int64_t p = b; p < e; ++p) out[i * os_d + p * os_p] = ho[i * P + p];
    });
    return GSC_OK;
}

// Spectrum-scaled copies of z1, z2 for device-pointer Fourier calls, in the
// context's own buffer (the caller's arrays stay untouched).
static int scaled_modes(DeviceCtx &ctx, const double *sf, const double *&z1, const double *&z2,
                        int64_t N, cudaStream_t st) {
    if (N == 0) return GSC_OK;
    GSC_TRY(ensure_dev(ctx, ctx.zscaled, 2 * static_cast<size_t>(N) * sizeof(double)));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    double *zs = static_cast<double *>(ctx.zscaled.ptr);
    GSC_TRY(fourier_scale(sf, z1, z2, N, zs, zs + N, st));
    z1 = zs;
    z2 = zs + N;
    return GSC_OK;
}

static int dev_plain(const double *cov, const double *z1, const double *z2, const double *pos,
                     int64_t dim, int64_t N, int64_t P, double *out, bool incompr,
                     const gsc_opts *opts, bool fourier = false, const double *sf = nullptr) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    GSC_TRY(check_sizes(dim, N, P));
    if (incompr && dim != 2 && dim != 3)
        return set_error(GSC_ERR_DIM, "Only two- and three-dimensional problems are supported.");
    GSC_TRY(need_ptr(cov, dim * N > 0, "cov_samples"));
    GSC_TRY(need_ptr(z1, N > 0, "z1"));
    GSC_TRY(need_ptr(z2, N > 0, "z2"));
    GSC_TRY(need_ptr(pos, dim * P > 0, "pos"));
    GSC_TRY(need_ptr(out, P > 0, "out"));
    GSC_TRY(unstructured_form(ro));
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    if (P == 0) return GSC_OK;
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    GSC_TRY(check_device_ptr(cov, "cov_samples"));
    GSC_TRY(check_device_ptr(z1, "z1"));
    GSC_TRY(check_device_ptr(z2, "z2"));
    GSC_TRY(check_device_ptr(pos, "pos"));
    GSC_TRY(check_device_ptr(out, "out"));
    if (fourier) {
        GSC_TRY(need_ptr(sf, N > 0, "spectrum_factor"));
        if (N > 0) GSC_TRY(check_device_ptr(sf, "spectrum_factor"));
        GSC_TRY(scaled_modes(*ctx, sf, z1, z2, N, ro.stream));
    }
    PlainArgs a;
    a.cov = cov;
    a.z1 = z1;
    a.z2 = z2;
    a.pos = pos;
    a.dim = dim;
    a.n_modes = N;
    a.n_points = P;
    a.incompr = incompr;
    a.out = out;
    a.out_sd = P;
    a.out_sp = 1;
    return run_points_dev(*ctx, ro, a, ro.stream);
}

// ---------------------------------------------------------------------------
// structured grids
// ---------------------------------------------------------------------------
static int check_structured(int64_t dim, int64_t N, const int64_t *n, bool incompr) {
    GSC_TRY(check_sizes(dim, N, 0));
    if (dim < 1 || dim > 3)
        return set_error(incompr ? GSC_ERR_DIM : GSC_ERR_INVALID,
                         incompr ? "Only two- and three-dimensional problems are supported."
                                 : "structured grids need 1, 2 or 3 axes");
    if (incompr && dim == 1)
        return set_error(GSC_ERR_DIM, "Only two- and three-dimensional problems are supported.");
    for (int d = 0; d < dim; ++d)
        if (n[d] < 0) return set_error(GSC_ERR_INVALID, "negative axis length");
    int64_t P = 1;
    for (int d = 0; d < dim; ++d) {
        if (n[d] > 0 && P > (int64_t(1) << 40) / n[d])
            return set_error(GSC_ERR_INVALID, "grid too large");
        P *= n[d];
    }
    if (N > (int64_t(1) << 30)) return set_error(GSC_ERR_INVALID, "too many modes");
    return GSC_OK;
}

// All pointers are device pointers; out is (ncomp, P) row-major.
// host_call: the caller synchronises and reads the x5 bound flag itself
// (host-pointer entry points); else a device-pointer call, which queues the
// FP64 fallback behind an AUTO x5 launch.
static int run_structured(DeviceCtx &ctx, const Resolved &ro, const double *cov, const double *z1,
                          const double *z2, int64_t dim, int64_t N, const double *const *axis,
                          const int64_t *n, bool incompr, double *out, cudaStream_t st,
                          const std::function<int(int64_t, int64_t)> *on_rows = nullptr,
                          bool host_call = false) {
    int64_t P = 1;
    for (int d = 0; d < dim; ++d) P *= n[d];
    if (P == 0) return GSC_OK;
    const int form = structured_form(ro, dim);
    if (is_sep(form)) {
        SepArgs a;
        a.cov = cov;
        a.z1 = z1;
        a.z2 = z2;
        a.dim = dim;
        a.n_modes = N;
        for (int d = 0; d < 3; ++d) {
            a.axis[d] = d < dim ? axis[d] : nullptr;
            a.n[d] = d < dim ? n[d] : 1;
        }
        a.incompr = incompr;
        a.form = form;
        a.chunk_kblocks = 0;
        a.out = out;
        a.status = ctx.status;
        a.on_rows = on_rows;
        if (form == GSC_FORM_SEP_F16X5) {
            a.bound_flag = ctx.status + kStatusX5Flag;
            if (!host_call && ro.form != GSC_FORM_AUTO) a.bound_sticky = ctx.status + kStatusX5Sticky;
            GSC_TRY(sep_tc_run(ctx, a, st));
            if (!host_call && ro.form == GSC_FORM_AUTO) {
                // the FP64 form, queued behind: its launches do nothing unless
                // the x5 launch flagged these inputs
                SepArgs f = a;
                f.form = GSC_FORM_SEP_F64;
                f.on_rows = nullptr;
                f.bound_flag = f.bound_sticky = nullptr;
                f.run_if = ctx.status + kStatusX5Flag;
                GSC_TRY(sep_f64_run(ctx, f, st));
            }
            return GSC_OK;
        }
        return form == GSC_FORM_SEP_F64 ? sep_f64_run(ctx, a, st) : sep_tc_run(ctx, a, st);
    }
    // plain FP64 forms on the expanded grid
    const double *pos = axis[0];
    if (dim > 1) {
        GSC_TRY(ensure_dev(ctx, ctx.grid, static_cast<size_t>(dim * P) * sizeof(double)));
        GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
        TimedLaunch tl(st);
        tl.begin(K_GRID_EXPAND);
        GSC_TRY(grid_expand(axis, n, dim, static_cast<double *>(ctx.grid.ptr), st));
        tl.end();
        pos = static_cast<const double *>(ctx.grid.ptr);
    }
    PlainArgs a;
    a.cov = cov;
    a.z1 = z1;
    a.z2 = z2;
    a.pos = pos;
    a.dim = dim;
    a.n_modes = N;
    a.n_points = P;
    a.incompr = incompr;
    a.out = out;
    a.out_sd = P;
    a.out_sp = 1;
    Resolved rp = ro;
    // AUTO that chose the mixed form stays AUTO, which keeps its FP64 fallback
    rp.form = (ro.form == GSC_FORM_AUTO && form == GSC_FORM_MIXED) ? GSC_FORM_AUTO : form;
    return run_points_dev(ctx, rp, a, st);
}

static int host_structured(const double *cov, int64_t cs_d, int64_t cs_n, const double *z1,
                           int64_t z1s, const double *z2, int64_t z2s, int64_t dim, int64_t N,
                           const double *const *ax, const int64_t *n, const int64_t *sx,
                           double *out, bool incompr, const gsc_opts *opts,
                           const double *sf, int64_t sfs, bool interleave, MeshCheck *mc) {
    // interleave: out is a Fortran-ordered (nout, P) array, i.e. (P, nout)
    // row-major; the result is rearranged on the device before its copy
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    GSC_TRY(check_structured(dim, N, n, incompr));
    int64_t P = 1;
    for (int d = 0; d < dim; ++d) P *= n[d];
    GSC_TRY(need_ptr(cov, dim * N > 0, "cov_samples"));
    GSC_TRY(need_ptr(z1, N > 0, "z1"));
    GSC_TRY(need_ptr(z2, N > 0, "z2"));
    for (int d = 0; d < dim; ++d) GSC_TRY(need_ptr(ax[d], n[d] > 0, "axis"));
    GSC_TRY(need_ptr(out, P > 0, "out"));
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    if (P == 0) return GSC_OK;

    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    cudaStream_t st = ctx->stream;
    // The device's share of a flattened mesh's check runs on the second
    // stream, launched before the tables and the GEMM: its 16 blocks hold a
    // few SMs while they wait on host reads, and the GEMM takes the rest.
    // (Run after the GEMM instead, the call took 2.9 against 2.5 ms on the
    // 256^3 mesh.)  Its flag is read on every return path, with the context
    // still locked.
    struct CheckRead {
        MeshCheck *mc = nullptr;
        cudaStream_t s = nullptr;
        int *flag = nullptr;
        ~CheckRead() {
            if (!mc) return;
            int v = 1;
            if (cudaMemcpyAsync(&v, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                cudaGetLastError();
                v = 1;
            }
            mc->bad = v;
        }
    } check_read;
    auto launch_check = [&]() -> int {
        if (!mc) return GSC_OK;
        if (mc->na <= 0) {
            mc->bad = 0;
            return GSC_OK;
        }
        if (!ctx->stream2)
            GSC_CUDA(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
        // after the work queued before this call
        if (!ctx->chunk_ev)
            GSC_CUDA(cudaEventCreateWithFlags(&ctx->chunk_ev, cudaEventDisableTiming));
        GSC_CUDA(cudaEventRecord(ctx->chunk_ev, st));
        GSC_CUDA(cudaStreamWaitEvent(ctx->stream2, ctx->chunk_ev, 0));
        int *flag = ctx->status + kStatusMeshCheck;
        GSC_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream2));
        TimedLaunch tl(ctx->stream2);
        tl.begin(K_MESH_CHECK);
        mesh_check_kernel<<<16, 1024, 0, ctx->stream2>>>(
            mc->pos, mc->sd, mc->na, mc->n[1], mc->dim == 3 ? mc->n[2] : 1, mc->dim, mc->ax[0],
            mc->ax[1], mc->dim == 3 ? mc->ax[2] : nullptr, flag);
        tl.end();
        GSC_CUDA(cudaGetLastError());
        check_read.mc = mc;
        check_read.s = ctx->stream2;
        check_read.flag = flag;
        return GSC_OK;
    };

    const int64_t nout = incompr ? dim : 1;
    const size_t n_cov = static_cast<size_t>(dim * N);
    size_t n_ax = 0;
    for (int d = 0; d < dim; ++d) n_ax += static_cast<size_t>(n[d]);
    const size_t n_sf = sf ? static_cast<size_t>(N) : 0;
    const size_t n_in = n_cov + 2 * static_cast<size_t>(N) + n_sf + n_ax;
    const size_t n_out = static_cast<size_t>(nout * P);
    // inputs, and the two 32 MiB stages of the output copy
    GSC_TRY(ensure_pinned(*ctx, std::max(n_in * sizeof(double),
                                         std::min(n_out * sizeof(double), size_t(64) << 20))));
    if (nout == 1) interleave = false;
    GSC_TRY(ensure_dev(*ctx, ctx->io, (n_in + n_out * (interleave ? 2 : 1)) * sizeof(double) + 1024));
    double *h = static_cast<double *>(ctx->pinned);
    double *d = static_cast<double *>(ctx->io.ptr);
    TimedLaunch tc(st);
    tc.begin(K_COPY_H2D);
    GSC_TRY(upload2(st, d, h, 0, cov, cs_d, cs_n, dim, N));
    GSC_TRY(upload2(st, d, h, n_cov, z1, 0, z1s, 1, N));
    GSC_TRY(upload2(st, d, h, n_cov + N, z2, 0, z2s, 1, N));
    if (sf) GSC_TRY(upload2(st, d, h, n_cov + 2 * N, sf, 0, sfs, 1, N));
    size_t off = n_cov + 2 * N + n_sf;
    const double *dax[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < dim; ++k) {
        GSC_TRY(upload2(st, d, h, off, ax[k], 0, sx[k], 1, n[k]));
        dax[k] = d + off;
        off += static_cast<size_t>(n[k]);
    }
    tc.end();
    if (sf) GSC_TRY(fourier_scale(d + n_cov + 2 * N, d + n_cov, d + n_cov + N, N, d + n_cov,
                                  d + n_cov + N, st));
    // output buffer 128-byte aligned after the inputs
    double *dout = reinterpret_cast<double *>(
        (reinterpret_cast<uintptr_t>(d + n_in) + 127) & ~static_cast<uintptr_t>(127));
    double *dil = interleave ? dout + n_out : nullptr;       // (P, nout) layout
    // the rows [lo, hi) of the result, in the caller's layout, ready on st
    // for a copy: the device result itself or its interleaved rows
    auto result_rows = [&](int64_t lo, int64_t hi) -> int {
        if (interleave) GSC_TRY(interleave_rows(dout, nout, P, lo * n[dim - 1], hi * n[dim - 1], dil, st));
        return GSC_OK;
    };
    // A pinned result (resident pages) is copied in row ranges as the
    // launches that complete them are queued, on a second stream, so the
    // copy of one wave's rows overlaps the computing of the next.
    const bool pinned = is_pinned_host(out);
    const int64_t nn_last = n[dim - 1];                 // output elements per (slice, row)
    int64_t rows_copied = 0;
    bool copying = false;
    std::function<int(int64_t, int64_t)> on_rows = [&](int64_t lo, int64_t hi) -> int {
        if (!ctx->copy_stream)
            GSC_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        if (!ctx->chunk_ev)
            GSC_CUDA(cudaEventCreateWithFlags(&ctx->chunk_ev, cudaEventDisableTiming));
        GSC_TRY(result_rows(lo, hi));
        GSC_CUDA(cudaEventRecord(ctx->chunk_ev, st));
        GSC_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_ev, 0));
        copying = true;
        if (interleave) {
            const int64_t e0 = lo * nn_last * nout, ne = (hi - lo) * nn_last * nout;
            GSC_CUDA(cudaMemcpyAsync(out + e0, dil + e0, static_cast<size_t>(ne) * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx->copy_stream));
        } else {
            for (int64_t c = 0; c < nout; ++c)
                GSC_CUDA(cudaMemcpyAsync(out + c * P + lo * nn_last, dout + c * P + lo * nn_last,
                                         static_cast<size_t>((hi - lo) * nn_last) * sizeof(double),
                                         cudaMemcpyDeviceToHost, ctx->copy_stream));
        }
        rows_copied = hi;
        return GSC_OK;
    };
    GSC_TRY(launch_check());
    int rc = run_structured(*ctx, ro, d, d + n_cov, d + n_cov + N, dim, N, dax, n, incompr, dout,
                            st, pinned ? &on_rows : nullptr, true);
    if (copying) {
        // queued copies land in the caller's array: they finish before return
        const cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
        if (rc == GSC_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize (result copies)");
    }
    GSC_TRY(rc);
    if (!copying || rows_copied * nn_last != P) {
        // output pages are faulted in on host threads while the GPU computes;
        // the result then moves by DMA straight into the caller's array
        Prefault pf;
        if (!pinned) pf.start(out, n_out * sizeof(double));
        GSC_TRY(result_rows(0, P / nn_last));
        pf.join();
        tc.begin(K_COPY_D2H);
        GSC_CUDA(cudaMemcpyAsync(out, interleave ? dil : dout, n_out * sizeof(double),
                                 cudaMemcpyDeviceToHost, st));
        tc.end();
    }
    GSC_TRY(check_status(*ctx, st));
    if (structured_form(ro, dim) == GSC_FORM_SEP_F16X5) {
        // inputs past the exact leading sum's bound: AUTO recomputes on the
        // FP64 form, an explicit sep_f16x5 reports it
        int flag = 0;
        GSC_CUDA(cudaMemcpyAsync(&flag, ctx->status + kStatusX5Flag, sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
        GSC_CUDA(cudaStreamSynchronize(st));
        if (flag) {
            if (ro.form != GSC_FORM_AUTO) return set_error(GSC_ERR_KERNEL, kX5BoundMsg);
            Resolved rf = ro;
            rf.form = GSC_FORM_SEP_F64;
            GSC_TRY(run_structured(*ctx, rf, d, d + n_cov, d + n_cov + N, dim, N, dax, n, incompr,
                                   dout, st, nullptr, true));
            GSC_TRY(result_rows(0, P / nn_last));
            tc.begin(K_COPY_D2H);
            GSC_CUDA(cudaMemcpyAsync(out, interleave ? dil : dout, n_out * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
            tc.end();
            GSC_TRY(check_status(*ctx, st));
        }
    }
    return GSC_OK;
}

static int dev_structured(const double *cov, const double *z1, const double *z2, int64_t dim,
                          int64_t N, const double *const *ax, const int64_t *n, double *out,
                          bool incompr, const gsc_opts *opts, bool fourier = false,
                          const double *sf = nullptr) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    GSC_TRY(check_structured(dim, N, n, incompr));
    int64_t P = 1;
    for (int d = 0; d < dim; ++d) P *= n[d];
    GSC_TRY(need_ptr(cov, dim * N > 0, "cov_samples"));
    GSC_TRY(need_ptr(z1, N > 0, "z1"));
    GSC_TRY(need_ptr(z2, N > 0, "z2"));
    for (int d = 0; d < dim; ++d) GSC_TRY(need_ptr(ax[d], n[d] > 0, "axis"));
    GSC_TRY(need_ptr(out, P > 0, "out"));
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    if (P == 0) return GSC_OK;
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    GSC_TRY(check_device_ptr(cov, "cov_samples"));
    GSC_TRY(check_device_ptr(z1, "z1"));
    GSC_TRY(check_device_ptr(z2, "z2"));
    for (int d = 0; d < dim; ++d) GSC_TRY(check_device_ptr(ax[d], "axis"));
    GSC_TRY(check_device_ptr(out, "out"));
    if (fourier) {
        GSC_TRY(need_ptr(sf, N > 0, "spectrum_factor"));
        if (N > 0) GSC_TRY(check_device_ptr(sf, "spectrum_factor"));
        GSC_TRY(scaled_modes(*ctx, sf, z1, z2, N, ro.stream));
    }
    return run_structured(*ctx, ro, cov, z1, z2, dim, N, ax, n, incompr, out, ro.stream);
}

}  // namespace gsc

using namespace gsc;

extern "C" {

const char *gsc_version(void) { return "1.1.0+gb300"; }

const char *gsc_last_error(void) { return t_error.c_str(); }

int gsc_device_count(int32_t *count) {
    if (!count) return set_error(GSC_ERR_INVALID, "count is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return GSC_OK;
}

int gsc_last_timeline(int32_t *ids, double *start_ms, double *ms, int32_t cap) {
    int32_t n = 0;
    for (auto &r : t_recs) {
        if (n >= cap) break;
        float f = 0.f, s = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&f, r.a, r.b) != cudaSuccess ||
            cudaEventElapsedTime(&s, t_recs.front().a, r.a) != cudaSuccess) {
            cudaGetLastError();
            f = -1.f;
            s = -1.f;
        }
        if (ids) ids[n] = r.id;
        if (start_ms) start_ms[n] = s;
        if (ms) ms[n] = f;
        ++n;
    }
    return n;
}

int gsc_last_timings(int32_t *ids, double *ms, int32_t cap) {
    int32_t n = 0;
    for (auto &r : t_recs) {
        if (n >= cap) break;
        float f = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&f, r.a, r.b) != cudaSuccess) {
            cudaGetLastError();
            f = -1.f;
        }
        if (ids) ids[n] = r.id;
        if (ms) ms[n] = f;
        ++n;
    }
    return n;
}

const char *gsc_kernel_name(int32_t id) { return kernel_name(id); }

int gsc_summate_f64(const double *cov, int64_t cov_stride_d, int64_t cov_stride_n,
                    const double *z1, int64_t z1_stride, const double *z2, int64_t z2_stride,
                    const double *pos, int64_t pos_stride_d, int64_t pos_stride_p, int64_t dim,
                    int64_t n_modes, int64_t n_points, double *out, int64_t out_stride,
                    const gsc_opts *opts) {
    return host_plain(cov, cov_stride_d, cov_stride_n, z1, z1_stride, z2, z2_stride, pos,
                      pos_stride_d, pos_stride_p, dim, n_modes, n_points, out, 0, out_stride,
                      false, opts);
}

int gsc_summate_dev(const double *cov, const double *z1, const double *z2, const double *pos,
                    int64_t dim, int64_t n_modes, int64_t n_points, double *out,
                    const gsc_opts *opts) {
    return dev_plain(cov, z1, z2, pos, dim, n_modes, n_points, out, false, opts);
}

int gsc_summate_incompr_f64(const double *cov, int64_t cov_stride_d, int64_t cov_stride_n,
                            const double *z1, int64_t z1_stride, const double *z2,
                            int64_t z2_stride, const double *pos, int64_t pos_stride_d,
                            int64_t pos_stride_p, int64_t dim, int64_t n_modes,
                            int64_t n_points, double *out, int64_t out_stride_d,
                            int64_t out_stride_p, const gsc_opts *opts) {
    return host_plain(cov, cov_stride_d, cov_stride_n, z1, z1_stride, z2, z2_stride, pos,
                      pos_stride_d, pos_stride_p, dim, n_modes, n_points, out, out_stride_d,
                      out_stride_p, true, opts);
}

int gsc_summate_incompr_dev(const double *cov, const double *z1, const double *z2,
                            const double *pos, int64_t dim, int64_t n_modes, int64_t n_points,
                            double *out, const gsc_opts *opts) {
    return dev_plain(cov, z1, z2, pos, dim, n_modes, n_points, out, true, opts);
}

int gsc_summate_fourier_f64(const double *spectrum_factor, int64_t sf_stride, const double *modes,
                            int64_t modes_stride_d, int64_t modes_stride_n, const double *z1,
                            int64_t z1_stride, const double *z2, int64_t z2_stride,
                            const double *pos, int64_t pos_stride_d, int64_t pos_stride_p,
                            int64_t dim, int64_t n_modes, int64_t n_points, double *out,
                            int64_t out_stride, const gsc_opts *opts) {
    if (!spectrum_factor && n_modes > 0)
        return set_error(GSC_ERR_INVALID, "spectrum_factor is NULL");
    return host_plain(modes, modes_stride_d, modes_stride_n, z1, z1_stride, z2, z2_stride, pos,
                      pos_stride_d, pos_stride_p, dim, n_modes, n_points, out, 0, out_stride,
                      false, opts, n_modes > 0 ? spectrum_factor : nullptr, sf_stride);
}

int gsc_summate_fourier_dev(const double *spectrum_factor, const double *modes, const double *z1,
                            const double *z2, const double *pos, int64_t dim, int64_t n_modes,
                            int64_t n_points, double *out, const gsc_opts *opts) {
    return dev_plain(modes, z1, z2, pos, dim, n_modes, n_points, out, false, opts, true,
                     spectrum_factor);
}

int gsc_summate_dev_noalloc(const double *cov, const double *z1, const double *z2,
                            const double *pos, int64_t dim, int64_t n_modes, int64_t n_points,
                            double *out, const gsc_opts *opts) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    GSC_TRY(check_sizes(dim, n_modes, n_points));
    if (dim < 1 || dim > 3)
        return set_error(GSC_ERR_DIM, "gsc_summate_dev_noalloc supports dimensions 1, 2 and 3");
    if (ro.form != GSC_FORM_AUTO && ro.form != GSC_FORM_PLAIN_F64)
        return set_error(GSC_ERR_INVALID, "gsc_summate_dev_noalloc runs the plain FP64 form only");
    if (n_modes > kNoAllocModes)
        return set_error(GSC_ERR_INVALID, "gsc_summate_dev_noalloc takes at most " +
                                              std::to_string(kNoAllocModes) + " modes per call");
    GSC_TRY(need_ptr(cov, dim * n_modes > 0, "cov_samples"));
    GSC_TRY(need_ptr(z1, n_modes > 0, "z1"));
    GSC_TRY(need_ptr(z2, n_modes > 0, "z2"));
    GSC_TRY(need_ptr(pos, dim * n_points > 0, "pos"));
    GSC_TRY(need_ptr(out, n_points > 0, "out"));
    if (n_points == 0) return GSC_OK;
    // no library context here: its creation allocates (stream, status word)
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return set_error(GSC_ERR_NO_DEVICE, "no usable CUDA device; this library has no CPU path");
    }
    int device = ro.device;
    if (device < 0) GSC_CUDA(cudaGetDevice(&device));
    if (device >= count) return set_error(GSC_ERR_INVALID, "device ordinal out of range");
    DeviceGuard g;
    GSC_TRY(g.set(device));
    GSC_TRY(check_device_ptr(cov, "cov_samples"));
    GSC_TRY(check_device_ptr(z1, "z1"));
    GSC_TRY(check_device_ptr(z2, "z2"));
    GSC_TRY(check_device_ptr(pos, "pos"));
    GSC_TRY(check_device_ptr(out, "out"));
    PlainArgs a;
    a.cov = cov;
    a.z1 = z1;
    a.z2 = z2;
    a.pos = pos;
    a.dim = dim;
    a.n_modes = n_modes;
    a.n_points = n_points;
    a.incompr = false;
    a.out = out;
    a.out_sd = n_points;
    a.out_sp = 1;
    a.variant = 0;
    return plain_noalloc_run(device, a, ro.stream);
}

int gsc_device_status(int32_t device) {
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    GSC_CUDA(cudaEventSynchronize(ctx->scratch_ready));
    return check_status(*ctx, ctx->stream);
}

int gsc_release_buffers(int32_t device) {
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    // every user of the buffers records scratch_ready (device-pointer calls)
    // or runs on the context stream (host-pointer calls) before it returns
    GSC_CUDA(cudaEventSynchronize(ctx->scratch_ready));
    GSC_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->sampling_ev) GSC_CUDA(cudaEventSynchronize(ctx->sampling_ev));
    for (DevBuf *b : {&ctx->io, &ctx->scratch, &ctx->grid, &ctx->zscaled, &ctx->sampling}) {
        if (b->ptr) GSC_CUDA(cudaFree(b->ptr));
        b->ptr = nullptr;
        b->bytes = 0;
    }
    if (ctx->pinned) GSC_CUDA(cudaFreeHost(ctx->pinned));
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    if (ctx->sampling_pinned) GSC_CUDA(cudaFreeHost(ctx->sampling_pinned));
    ctx->sampling_pinned = nullptr;
    ctx->sampling_pinned_bytes = 0;
    for (gsc_batch *b : ctx->batch) gsc_batch_destroy(b);
    ctx->batch.clear();
    ctx->batch_sig.clear();
    return GSC_OK;
}

int gsc_selftest_fail_alloc(int32_t countdown) {
    if (countdown < -1) return set_error(GSC_ERR_INVALID, "countdown must be -1 or >= 0");
    g_fail_alloc.store(countdown);
    return GSC_OK;
}

int gsc_selftest_detect_grid(const double *pos, int64_t ps_d, int64_t ps_p, int64_t dim,
                             int64_t n_points, int64_t *n_axes) {
    if (!n_axes) return set_error(GSC_ERR_INVALID, "n_axes is NULL");
    n_axes[0] = n_axes[1] = n_axes[2] = 0;
    if (dim < 0 || n_points < 0) return set_error(GSC_ERR_INVALID, "negative dimension or count");
    if (n_points > 0 && !pos) return set_error(GSC_ERR_INVALID, "pos is NULL");
    std::vector<double> ax[3];
    int64_t n[3] = {0, 0, 0};
    if (n_points > 0 && detect_grid(pos, ps_d, ps_p, dim, n_points, ax, n)) {
        for (int d = 0; d < 3; ++d) n_axes[d] = d < dim ? n[d] : 0;
    }
    return GSC_OK;
}

int gsc_summate_structured_f64(const double *cov, int64_t cs_d, int64_t cs_n, const double *z1,
                               int64_t z1s, const double *z2, int64_t z2s, int64_t dim,
                               int64_t n_modes, const double *a0, int64_t n0, int64_t s0,
                               const double *a1, int64_t n1, int64_t s1, const double *a2,
                               int64_t n2, int64_t s2, double *out, const gsc_opts *opts) {
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2}, sx[3] = {s0, s1, s2};
    return host_structured(cov, cs_d, cs_n, z1, z1s, z2, z2s, dim, n_modes, ax, n, sx, out,
                           false, opts, nullptr, 0);
}

int gsc_summate_structured_dev(const double *cov, const double *z1, const double *z2,
                               int64_t dim, int64_t n_modes, const double *a0, int64_t n0,
                               const double *a1, int64_t n1, const double *a2, int64_t n2,
                               double *out, const gsc_opts *opts) {
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2};
    return dev_structured(cov, z1, z2, dim, n_modes, ax, n, out, false, opts);
}

int gsc_summate_incompr_structured_f64(const double *cov, int64_t cs_d, int64_t cs_n,
                                       const double *z1, int64_t z1s, const double *z2,
                                       int64_t z2s, int64_t dim, int64_t n_modes,
                                       const double *a0, int64_t n0, int64_t s0,
                                       const double *a1, int64_t n1, int64_t s1,
                                       const double *a2, int64_t n2, int64_t s2, double *out,
                                       const gsc_opts *opts) {
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2}, sx[3] = {s0, s1, s2};
    return host_structured(cov, cs_d, cs_n, z1, z1s, z2, z2s, dim, n_modes, ax, n, sx, out,
                           true, opts, nullptr, 0);
}

int gsc_summate_incompr_structured_dev(const double *cov, const double *z1, const double *z2,
                                       int64_t dim, int64_t n_modes, const double *a0,
                                       int64_t n0, const double *a1, int64_t n1,
                                       const double *a2, int64_t n2, double *out,
                                       const gsc_opts *opts) {
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2};
    return dev_structured(cov, z1, z2, dim, n_modes, ax, n, out, true, opts);
}

int gsc_summate_fourier_structured_f64(const double *spectrum_factor, int64_t sf_stride,
                                       const double *modes, int64_t ms_d, int64_t ms_n,
                                       const double *z1, int64_t z1s, const double *z2,
                                       int64_t z2s, int64_t dim, int64_t n_modes,
                                       const double *a0, int64_t n0, int64_t s0,
                                       const double *a1, int64_t n1, int64_t s1,
                                       const double *a2, int64_t n2, int64_t s2, double *out,
                                       const gsc_opts *opts) {
    if (!spectrum_factor && n_modes > 0)
        return set_error(GSC_ERR_INVALID, "spectrum_factor is NULL");
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2}, sx[3] = {s0, s1, s2};
    return host_structured(modes, ms_d, ms_n, z1, z1s, z2, z2s, dim, n_modes, ax, n, sx, out,
                           false, opts, n_modes > 0 ? spectrum_factor : nullptr, sf_stride);
}

int gsc_summate_fourier_structured_dev(const double *spectrum_factor, const double *modes,
                                       const double *z1, const double *z2, int64_t dim,
                                       int64_t n_modes, const double *a0, int64_t n0,
                                       const double *a1, int64_t n1, const double *a2,
                                       int64_t n2, double *out, const gsc_opts *opts) {
    const double *ax[3] = {a0, a1, a2};
    const int64_t n[3] = {n0, n1, n2};
    return dev_structured(modes, z1, z2, dim, n_modes, ax, n, out, false, opts, true,
                          spectrum_factor);
}

}  // extern "C"
