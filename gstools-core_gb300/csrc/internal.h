// internal.h -- declarations shared by the translation units of the GB300
// summator library.  Not installed; the public surface is
// include/gstools_core_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gstools_core_gb300.h"

namespace gsc {

// ---- status helpers -------------------------------------------------------
int set_error(int code, const std::string &msg);   // records msg, returns code
int cuda_fail(cudaError_t e, const char *what);     // GSC_ERR_CUDA / NOMEM

// GSC_OK, or the library's status for a failed CUDA call
inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? GSC_OK : cuda_fail(e, "CUDA call"); }

#define GSC_CUDA(call)                                         \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return ::gsc::cuda_fail(e_, #call); \
    } while (0)

#define GSC_TRY(expr)                  \
    do {                               \
        int rc_ = (expr);              \
        if (rc_ != GSC_OK) return rc_; \
    } while (0)

// ---- kernel ids (gsc_kernel_name / gsc_last_timings) ----------------------
enum KernelId : int32_t {
    K_MODE_TABLE = 0,      // per-mode angle tables and projector weights
    K_PLAIN_SCALAR = 1,    // FP64 scalar summator, table-driven sincos
    K_PLAIN_INCOMPR = 2,   // FP64 incompressible summator, table-driven sincos
    K_PLAIN_LIBM = 3,      // FP64 summators on CUDA's sincos()
    K_SPLIT_REDUCE = 4,    // ordered sum of mode-split partials
    K_GENERIC = 5,         // any dimension, one thread per point
    K_SEP_TABLES = 6,      // per-axis factor tables of the separable form
    K_SEP_TC_F16 = 7,      // tcgen05 separable contraction, f16 hi/lo split
    K_SEP_TC_BF16 = 8,     // tcgen05 separable contraction, bf16 hi/lo split
    K_GRID_EXPAND = 9,     // meshgrid of structured axes (plain form on grids)
    K_SEP_TC_F16X5 = 10,   // tcgen05 separable contraction, exact leading term
    K_MIXED_MODES = 11,    // per-mode records of the mixed form
    K_MIXED_SCALAR = 12,   // mixed form, integer phase, scalar field
    K_MIXED_INCOMPR = 13,  // mixed form, integer phase, vector field
    K_MIXED_F64PHASE = 14, // mixed form with the phase in FP64
    K_SEP_F64 = 15,        // separable contraction on the FP64 MMA
    K_FOURIER_SCALE = 16,  // spectrum factor folded into z1, z2 (Fourier method)
    K_BATCH_TABLES = 17,   // per-mode tables of every item of a batch
    K_BATCH_PLAIN = 18,    // persistent FP64 batch kernel (device work queue)
    K_BATCH_MIXED = 19,    // persistent mixed-precision batch kernel
    K_SAMPLE_MODES = 20,   // on-device spectral sampling (Philox4x32-10)
    K_SEP_SPLIT = 21,      // FP32 inputs of the x5 factor tables
    K_COPY_H2D = 22,       // host-to-device copies of a host-pointer call (not a kernel)
    K_COPY_D2H = 23,       // device-to-host copies of a host-pointer call (not a kernel)
    K_INTERLEAVE = 24,     // (nout, P) rows to the (P, nout) layout of a Fortran-ordered result
    K_MESH_CHECK = 25,     // the device's share of the check of a flattened mesh
    K_COUNT
};
const char *kernel_name(int32_t id);

// ---- per-device context ---------------------------------------------------
// A grow-only device buffer.  `ready` orders reuse across streams: every
// launch that touches the buffer waits on it first and records it after.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct DeviceCtx {
    int device = -1;
    cudaStream_t stream = nullptr;   // stream of host-pointer calls
    cudaEvent_t scratch_ready = nullptr;
    std::mutex mu;                   // serialises users of the buffers below
    DevBuf io;                       // inputs+outputs of host-pointer calls
    DevBuf scratch;                  // tables and partial sums
    void *pinned = nullptr;          // pinned host staging
    size_t pinned_bytes = 0;
    DevBuf grid;                     // expanded meshgrid for plain forms on grids
    DevBuf zscaled;                  // spectrum-scaled z1, z2 of device-pointer Fourier calls
    DevBuf sampling;                 // item table of on-device sampling calls
    void *sampling_pinned = nullptr; // its pinned staging, reused once its copy is done
    size_t sampling_pinned_bytes = 0;
    cudaEvent_t sampling_ev = nullptr;
    int *status = nullptr;           // sticky kernel status word (device)
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};   // pipelined device-to-host staging
    cudaStream_t copy_stream = nullptr;  // result copies overlapping later launches
    cudaStream_t stream2 = nullptr;      // second compute stream of grouped batch calls
    cudaEvent_t chunk_ev = nullptr;      // "rows so far are done" on the compute stream
    // plans of the last host-pointer batch call, one per group of items, and
    // their shape signatures (a plan is reused when its signature is equal)
    std::vector<gsc_batch *> batch;
    std::vector<std::vector<int64_t>> batch_sig;
};

// Makes `dev` current for the guard's lifetime.
struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    int set(int dev) {
        GSC_CUDA(cudaGetDevice(&prev));
        if (prev != dev) {
            GSC_CUDA(cudaSetDevice(dev));
            changed = true;
        }
        return GSC_OK;
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

// Options after defaults are applied (capi.cu).
struct Resolved {
    int form = GSC_FORM_AUTO;
    int device = -1;
    int flags = 0;
    cudaStream_t stream = nullptr;
    double tolerance = 1e-12;
};
int resolve_opts(const gsc_opts *o, Resolved *r);
// GSC_OK for NULL or device-accessible memory, else GSC_ERR_INVALID naming `name`.
int check_device_ptr(const void *p, const char *name);

// Returns the context of `device` (-1 = current), initialising it once.
int get_ctx(int device, DeviceCtx **out);

// One-time set-up of a kernel on one device.  Launch attributes such as
// cudaFuncAttributeMaxDynamicSharedMemorySize belong to the device that was
// current when they were set, so a process-wide "done" flag would leave every
// later device unconfigured.  `setup` runs with that device current, under a
// lock shared by all threads, until it succeeds once for the pair (key,
// device); later calls return GSC_OK without running it.
int once_per_device(const void *key, int device, const std::function<int()> &setup);
// cudaFuncSetAttribute(fn, MaxDynamicSharedMemorySize, smem) on the current
// device, once per (fn, device).
int smem_attr(const void *fn, size_t smem);
// Makes `buf` hold at least `bytes`; waits for in-flight users before growing.
// cudaMalloc / cudaHostAlloc with the allocation-failure injection of
// gsc_selftest_fail_alloc; GSC_ERR_NOMEM on failure, *p = nullptr.
int alloc_device(void **p, size_t bytes, const char *what);
int alloc_pinned(void **p, size_t bytes, const char *what);
int ensure_dev(DeviceCtx &ctx, DevBuf &buf, size_t bytes);
// true for page-locked host memory (host_pool.cu): its pages need no
// faulting in before a copy lands there
bool is_pinned_host(const void *p);
int ensure_pinned(DeviceCtx &ctx, size_t bytes);
// memcpy with up to 8 host threads for large blocks
void parallel_copy(void *dst, const void *src, size_t bytes);
// Host arrays packed back to back into pinned staging `h` and moved to the
// device range `d` (same byte offsets; segments in increasing offset order):
// chunks of 64 MiB are copied by all host cores, and each chunk's DMA runs
// while the next is copied.  One DMA per chunk instead of one pageable copy
// per array (each pageable copy pays a fixed cost in the driver, which
// dominates for many arrays of a few MB).
struct HostSrc {
    const void *src;  // null: the bytes are already at h + off (gathered there)
    size_t off;       // byte offset in h and d
    size_t bytes;
};
int h2d_packed(cudaStream_t st, void *d, void *h, const std::vector<HostSrc> &segs);
// Device -> pageable host through the pinned buffer in 32 MiB chunks, the DMA
// of one chunk overlapping the host copy of the previous one; returns after
// the data is in `dst` (synchronises `st`).
int d2h_staged(DeviceCtx &ctx, cudaStream_t st, void *dst, const void *src, size_t bytes);
// As d2h_staged for a device range whose consecutive pieces go to separate
// host arrays (segments in order, sizes summing to `bytes`).
struct HostSeg {
    void *dst;
    size_t bytes;
};
int d2h_scatter(DeviceCtx &ctx, cudaStream_t st, const void *src, size_t bytes,
                const std::vector<HostSeg> &segs);
// Faults in the pages of a host range on worker threads (start), so that a
// later device-to-host copy into it runs at DMA speed; join() waits.
struct Prefault {
    std::vector<std::thread> th;
    void start(void *p, size_t bytes);
    void start_many(const std::vector<HostSeg> &segs);
    void join();
    ~Prefault() { join(); }
};

// ---- autotuner cache (tuner.cu) ----------------------------------------------
// Tuned launch configurations keyed by text (device name, kernel family,
// shape buckets), in memory and, with a cache file, persisted.
bool tune_get(const std::string &key, int v[4]);
void tune_put(const std::string &key, const int v[4]);
int tune_mode();                  // 0 fixed defaults, 1 cached entries only, 2 tune on a miss
std::string device_name(int device);
int tune_bucket(double v);        // e with v in [2^(e-1), 2^e) (0 below 1)

// ---- timing ---------------------------------------------------------------
struct TimedLaunch {
    explicit TimedLaunch(cudaStream_t s);
    bool on = false;
    cudaStream_t st = nullptr;
    int32_t id = 0;
    size_t rec = 0;            // its record (timed launches may nest)
    void begin(int32_t kid);   // records a start event when timing is on
    void end();                // records the stop event
};
void timing_reset(bool enabled);
bool timing_enabled();

// ---- plain FP64 summators (plain.cu) --------------------------------------
struct PlainArgs {
    const double *cov;   // (dim, n_modes) row-major, device
    const double *z1;    // (n_modes), device
    const double *z2;
    const double *pos;   // (dim, n_points) row-major, device
    int64_t dim, n_modes, n_points;
    bool incompr;        // vector field (dim outputs) instead of scalar
    double *out;         // device
    int64_t out_sd, out_sp;  // element strides of out[i, p] (scalar: 0, 1)
    int variant;         // 0 table-driven sincos, 1 CUDA sincos()
    // plain_run only: null, or a device word; every launch does nothing
    // while the word is 0 (a fallback queued behind another form's launches)
    const int *run_if = nullptr;
};
int plain_run(DeviceCtx &ctx, const PlainArgs &a, cudaStream_t st);

// out[i*sd + p*sp] = sum over s of part[s][i][p], s ascending (plain.cu)
int split_reduce(const double *part, int64_t S, int64_t nout, int64_t P, double *out, int64_t sd,
                 int64_t sp, cudaStream_t st);

// ---- mixed-precision summators (mixed_fx.cu, mixed.cu) ------------------------
// GSC_FORM_MIXED: integer fixed-point phase, table and polynomial e^{i theta}
// (mixed_fx.cu).  range_flag (device word, may be null) is set to 1 when a
// wave number is too large for the integer phase at these positions (the
// output is then invalid).
int mixed_fx_run(DeviceCtx &ctx, const PlainArgs &a, int *range_flag, cudaStream_t st);
// GSC_FORM_MIXED_F64PHASE: FP64 phase, FP32 sincos polynomials (mixed.cu);
// f64phase = false forwards to mixed_fx_run.
int mixed_run(DeviceCtx &ctx, const PlainArgs &a, bool f64phase, cudaStream_t st);

// Allocation-free scalar summator (plain.cu): per-mode tables in a fixed
// device array of kNoAllocModes modes; `device` must be current.
constexpr int64_t kNoAllocModes = 1024;
int plain_noalloc_run(int device, const PlainArgs &a, cudaStream_t st);

// ---- separable tensor-core summators on structured grids (separable_tc.cu) --
struct SepArgs {
    const double *cov;        // (dim, n_modes) row-major, device
    const double *z1, *z2;    // (n_modes), device
    int64_t dim, n_modes;     // dim in {2, 3}
    const double *axis[3];    // device axes; axis[i] has n[i] points
    int64_t n[3];
    bool incompr;
    int form;                 // GSC_FORM_SEP_F16X3, _BF16X3 or _F16X5
    int chunk_kblocks;        // k-blocks per FP32 accumulation chunk, 0 = default
    double *out;              // (ncomp, prod n) row-major, device
    int *status;              // device status word (0 = ok)
    // sep_f16x5 only (device words, may be null): the call sets bound_flag
    // to 1 when the inputs break the exact main sum's bound (checked before
    // and while the GEMM runs; its output is then invalid), else 0, and sets
    // bound_sticky to 1 then
    int *bound_flag = nullptr;
    int *bound_sticky = nullptr;
    // sep_f64 only: null, or a device word; every launch of the call does
    // nothing while it is 0 (a fallback queued behind an x5 launch whose
    // bound_flag it is)
    const int *run_if = nullptr;
    // sep_f16x5 only: when set, the GEMM runs as one launch per wave of
    // whole row tiles and this is called after each launch is queued with
    // the (slice, row) range [lo, hi) whose output that launch completes,
    // so that the caller can queue its copy while the next launch computes
    const std::function<int(int64_t lo, int64_t hi)> *on_rows = nullptr;
};
int sep_tc_run(DeviceCtx &ctx, const SepArgs &a, cudaStream_t st);
int sep_f64_run(DeviceCtx &ctx, const SepArgs &a, cudaStream_t st);   // separable_f64.cu

// ---- batched ensembles (batch.cu, with kernels in plain.cu / mixed.cu) ------
// One realization of an ensemble as the device kernels see it.
struct BatchItem {
    const double *cov, *z1, *z2, *sf;   // sf: Fourier spectrum factor or nullptr
    const double *pos;                  // (dim, n_points) row-major
    double *out;                        // (nout, n_points) row-major
    double *part;                       // splits > 1: splits slots of nout * n_points
    int64_t n_modes, n_points, mode_off;   // mode_off: first row of the shared mode tables
    int32_t dim, incompr, splits, pad;
};
// One entry of the device work queue: a block of points of one item and one
// mode range (split) of it.
struct BatchUnit {
    int32_t item, split;
    int64_t p_first, jb, je;
};
constexpr int kBatchThreads = 128;   // threads per block of the batch kernels

// Per-mode tables of every item, one launch (plain.cu / mixed.cu).  mode_prefix
// has n_items + 1 entries (exclusive prefix sums of n_modes).
int batch_plain_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                       int64_t total_modes, void *wtab, double *rec, cudaStream_t st);
int batch_mixed_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                       int64_t total_modes, float *rec, double *rec64, cudaStream_t st);
// Persistent kernels fed from the work queue `units` through `counter`
// (zero before the launch).  Shared-memory bytes and occupancy per config:
size_t batch_plain_smem(int tile);
int batch_plain_occupancy(int R, int tile, int device);
int batch_mixed_occupancy(int R, bool f64phase, int device);
bool batch_plain_config_ok(int R, int tile);
bool batch_mixed_config_ok(int R);
int batch_plain_launch(int R, int tile, int blocks, const BatchItem *items,
                       const BatchUnit *units, int64_t n_units, int *counter, const void *wtab,
                       const double *rec, cudaStream_t st);
int batch_mixed_launch(int R, bool f64phase, int blocks, const BatchItem *items,
                       const BatchUnit *units, int64_t n_units, int *counter, const float *rec,
                       const double *rec64, cudaStream_t st);
constexpr int64_t kPlainTableBytesPerMode = 256 * 16;   // W_j[a], a < 256, double2
constexpr int64_t kPlainRecBytesPerMode = 12 * 8;
constexpr int64_t kMixedRecBytesPerMode = 20 * 4;
constexpr int64_t kMixedRec64BytesPerMode = 4 * 8;
constexpr int64_t kFxRecBytesPerMode = 64 * 4;      // mixed_fx.cu mode record
// Batched mixed form (mixed_fx.cu): records of every item's modes, the range
// words of every item's positions (4 x uint64 per item), the range flag.
int batch_fx_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                    int64_t total_modes, uint32_t *rec, unsigned long long *maxbits,
                    int *range_flag, cudaStream_t st);
bool batch_fx_config_ok(int R);
// scalar: the ensemble has no incompressible item (a kernel without those
// variants)
int batch_fx_occupancy(int R, bool scalar);
int batch_fx_launch(int R, bool scalar, int blocks, const BatchItem *items, const BatchUnit *units,
                    int64_t n_units, int *counter, const uint32_t *rec,
                    const unsigned long long *maxbits, cudaStream_t st);

// Fourier method (src/field.rs:219-249): z1s[j] = sf[j] * z1[j],
// z2s[j] = sf[j] * z2[j], device pointers; z1s may alias z1 (in place).
int fourier_scale(const double *sf, const double *z1, const double *z2, int64_t n, double *z1s,
                  double *z2s, cudaStream_t st);

// meshgrid(axis..., indexing="ij") flattened: pos[d * P + p], device
int grid_expand(const double *const *axis, const int64_t *n, int64_t dim, double *pos,
                cudaStream_t st);

// dst[p * nout + c] = src[c * P + p] for points p in [p0, p1): the rows of a
// (nout, P) result in the layout of a Fortran-ordered (nout, P) array
int interleave_rows(const double *src, int64_t nout, int64_t P, int64_t p0, int64_t p1,
                    double *dst, cudaStream_t st);

}  // namespace gsc
