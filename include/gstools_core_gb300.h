/*
 * gstools_core_gb300.h -- C ABI of the GB300 (sm_103a) spectral random-field
 * summators.  This is the seam a foreign caller links against: plain C
 * types, pointers and sizes; no CUDA, torch or C++ types in any signature.
 *
 * Reference interface being replaced (GeoStat-Framework/GSTools-Core 1.1.0):
 *   Rust   pub fn field::summator(cov_samples, z1, z2, pos, num_threads)
 *            src/field.rs:37-43            -> gsc_summate_f64
 *          pub fn field::summator_incompr(...)
 *            src/field.rs:97-103           -> gsc_summate_incompr_f64
 *          pub fn field::summator_fourier(...)
 *            src/field.rs:219-226          -> gsc_summate_fourier_f64
 *   Python gstools_core.summate / summate_incompr / summate_fourier (PyO3)
 *            src/lib.rs:33-48, 50-65, 67-84 -> same three entry points, bound
 *                                             by the package gstools_core
 *
 * Conventions
 *  - Arrays are float64.  Strides are in ELEMENTS (ndarray / numpy strides
 *    divided by 8), so any view the reference accepts can be passed as is:
 *    cov_samples[d, j] = cov[d * cov_stride_d + j * cov_stride_n], etc.
 *  - `*_f64` entry points take HOST pointers (what the Rust/PyO3 caller
 *    holds).  The call copies inputs to the GPU, runs, copies the result
 *    back into the caller-owned `out`, and returns when `out` is written.
 *  - `*_dev` entry points take DEVICE pointers to dense row-major arrays and
 *    enqueue on `opts->stream` without synchronising.
 *  - Every entry point returns GSC_OK (0) or a nonzero status; the message
 *    is available from gsc_last_error() on the calling thread.  Where the
 *    reference panics (shape asserts src/field.rs:44-46, 104-106; dimension
 *    src/field.rs:180) these return GSC_ERR_INVALID / GSC_ERR_DIM instead of
 *    aborting the process.
 *  - Calls are thread safe.  Host-pointer calls on one device are
 *    serialised; device-pointer calls order their use of the library's
 *    internal scratch buffers with CUDA events, so calls on different streams
 *    are correct but do not overlap.
 *  - There is no CPU fallback: without a usable CUDA device every compute
 *    entry point returns GSC_ERR_NO_DEVICE.
 */
#ifndef GSTOOLS_CORE_GB300_H
#define GSTOOLS_CORE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GSC_OK             0
#define GSC_ERR_INVALID    1  /* bad shape, stride, pointer or option       */
#define GSC_ERR_DIM        2  /* unsupported spatial dimension              */
#define GSC_ERR_CUDA       3  /* a CUDA runtime call failed                 */
#define GSC_ERR_NO_DEVICE  4  /* no usable CUDA device                      */
#define GSC_ERR_NOMEM      5  /* device or pinned host allocation failed    */
#define GSC_ERR_KERNEL     6  /* a kernel reported an error status          */

/* ---- computation forms ----------------------------------------------- */
#define GSC_FORM_AUTO       0  /* library choice for the requested tolerance */
#define GSC_FORM_PLAIN_F64  1  /* FP64 end to end, table-driven FP64 sincos   */
#define GSC_FORM_PLAIN_F64_LIBM 2  /* FP64 end to end on CUDA's sincos()    */
#define GSC_FORM_SEP_F16X3  3  /* structured grids: separable contraction on
                                  tcgen05 tensor cores, both operands split
                                  into f16 hi + lo, 3 products; max error
                                  about 5e-6 of the field RMS               */
#define GSC_FORM_SEP_BF16X3 4  /* as GSC_FORM_SEP_F16X3 with bf16 terms
                                  (about 5e-5)                                */
#define GSC_FORM_SEP_F16X5  5  /* structured grids, 5 products: the leading
                                  product on an integer grid that the FP32
                                  tensor-memory accumulator sums exactly
                                  (checked at every chunk boundary), the
                                  rest drained in chunks, FP64 output
                                  without FP32 rounding at the field's
                                  magnitude; max error below 1e-6 of the
                                  field RMS.  Inputs that break the bound
                                  (weights far from random) are flagged:
                                  see gsc_device_status                      */
#define GSC_FORM_MIXED      6  /* any points: phase k.x mod one turn in
                                  32-bit fixed point (two integer products
                                  and one exact FP32 product per dimension,
                                  within 2^-30 turns), FP32 table and
                                  polynomial sincos, FP32 sums per 64 modes
                                  with a compensated total; below 1e-6 of
                                  the field RMS.  |k| * max|x| beyond 2^30
                                  turns is flagged (see gsc_device_status)  */
#define GSC_FORM_MIXED_F64PHASE 7 /* as GSC_FORM_MIXED with the phase and its
                                  reduction in FP64                          */
#define GSC_FORM_SEP_F64    8  /* structured grids: separable contraction in
                                  FP64 on the double-precision MMA; FP64
                                  round-off (below 1e-12 of the field RMS)   */

/* ---- flags ----------------------------------------------------------- */
#define GSC_FLAG_TIMING     1  /* record per-kernel CUDA-event timings      */

/* AUTO on structured grids (2-D, 3-D) picks GSC_FORM_SEP_F16X3 for
 * tolerance >= 1e-5, GSC_FORM_SEP_F16X5 for tolerance >= 1e-6, else
 * GSC_FORM_SEP_F64; on
 * explicit points GSC_FORM_MIXED for tolerance >= 1e-6, else PLAIN_F64.
 *
 * Options.  Pass NULL for the defaults (form AUTO at tolerance 1e-12,
 * current device, library stream for host-pointer calls and the legacy
 * default stream for device-pointer calls). */
typedef struct gsc_opts {
    int32_t struct_size;  /* sizeof(gsc_opts); lets the struct grow       */
    int32_t form;         /* GSC_FORM_*                                   */
    int32_t device;       /* CUDA device ordinal, -1 = current device     */
    int32_t flags;        /* GSC_FLAG_*                                   */
    void   *stream;       /* cudaStream_t, NULL = see above               */
    double  tolerance;    /* max |err| / field RMS that AUTO may spend;
                             <= 0 means 1e-12 (the plain FP64 bar)        */
} gsc_opts;

/* ---- library information --------------------------------------------- */

/* Version string: the reference crate version this build mirrors plus the
 * GB300 build tag, e.g. "1.1.0+gb300". */
const char *gsc_version(void);

/* Message of the last failing call made on this thread ("" if none). */
const char *gsc_last_error(void);

/* Number of CUDA devices the library can use (0 when there are none). */
int gsc_device_count(int32_t *count);

/* Per-kernel timings of the last GSC_FLAG_TIMING call on this thread:
 * writes up to `cap` (name-index, milliseconds) pairs and returns how many
 * kernels were recorded.  Names come from gsc_kernel_name(). */
int gsc_last_timings(int32_t *kernel_ids, double *ms, int32_t cap);
/* The same records as a timeline: also each record's start in milliseconds
 * after the first record's start (the launches of all of the call's streams
 * on one clock).  Returns how many records were written. */
int gsc_last_timeline(int32_t *kernel_ids, double *start_ms, double *ms, int32_t cap);
const char *gsc_kernel_name(int32_t kernel_id);

/* Status of the kernels launched by device-pointer calls on `device`
 * (-1 = current): waits for them, returns GSC_OK or GSC_ERR_KERNEL (a
 * pipeline wait gave up; a GSC_FORM_MIXED call or batch met a wave number
 * whose phase exceeds its integer range; or an explicit GSC_FORM_SEP_F16X5
 * call met inputs past the bound that keeps its leading sum exact; the
 * output of that call is invalid), and clears the status.  Host-pointer
 * calls check it themselves.  With GSC_FORM_AUTO such calls are recomputed
 * on an FP64 form: host-pointer calls after the check; device-pointer calls
 * by an FP64 computation queued behind the mixed or x5 launches
 * (GSC_FORM_PLAIN_F64 or GSC_FORM_SEP_F64) that does nothing unless the
 * device flagged the inputs, and they leave no status. */
int gsc_device_status(int32_t device);

/* Frees the scratch memory the library keeps on `device` (-1 = current)
 * between calls: the input/output, table and staging buffers of host- and
 * device-pointer calls, their pinned host staging, and the cached plan of
 * gsc_summate_batch_f64.  Waits for the library's queued work first; the
 * next call allocates again.  Plans made with gsc_batch_create are the
 * caller's and stay.  No reference counterpart (the reference allocates per
 * call). */
int gsc_release_buffers(int32_t device);

/* Pinned host blocks for result arrays.  gsc_host_alloc returns a block of
 * page-locked host memory of at least `bytes` (rounded up to a multiple of
 * 64 KiB, or of 2 MiB above 2 MiB), taken
 * from the pool's free blocks of that rounded size when there is one;
 * gsc_host_free hands it back (the pool keeps up to GSC_HOST_POOL_MB MiB of
 * free blocks, default 2048, and releases the rest); gsc_host_pool_trim
 * releases every free block; gsc_host_pool_stats reports the bytes handed
 * out and the bytes cached.  Results written into such blocks by the
 * host-pointer entry points move by DMA with no page faults.  No reference
 * counterpart (the reference returns freshly allocated arrays,
 * src/lib.rs:47,64). */
int gsc_host_alloc(int64_t bytes, void **ptr);
int gsc_host_free(void *ptr);
int gsc_host_pool_trim(void);
int gsc_host_pool_stats(int64_t *live_bytes, int64_t *cached_bytes);

/* ---- scalar randomization method: src/field.rs:37-65 ------------------ */
/* u[p] = sum_j z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p)
 * cov (dim, n_modes), z1/z2 (n_modes), pos (dim, n_points), out (n_points).
 * Replaces field::summator (src/field.rs:37) / PyO3 summate (src/lib.rs:35). */
int gsc_summate_f64(const double *cov, int64_t cov_stride_d, int64_t cov_stride_n,
                    const double *z1, int64_t z1_stride,
                    const double *z2, int64_t z2_stride,
                    const double *pos, int64_t pos_stride_d, int64_t pos_stride_p,
                    int64_t dim, int64_t n_modes, int64_t n_points,
                    double *out, int64_t out_stride,
                    const gsc_opts *opts);

/* Device-pointer form: cov (dim, n_modes) row-major, pos (dim, n_points)
 * row-major, out (n_points).  Enqueued on opts->stream. */
int gsc_summate_dev(const double *cov, const double *z1, const double *z2,
                    const double *pos, int64_t dim, int64_t n_modes,
                    int64_t n_points, double *out, const gsc_opts *opts);

/* Allocation-free form of gsc_summate_dev.  It has no counterpart in the
 * reference.  It is for callers that may not have a library allocate device
 * memory -- a host whose own allocator owns the whole GPU, a real-time loop
 * that cannot block in the driver's allocator, a plug-in host that hands out
 * memory only from its arena.  The call allocates nothing: the plain FP64
 * kernel's per-mode tables live in a fixed array inside the library
 * (4 MiB + 96 KiB, held on every GPU that loads the library until exit), so
 * a call takes at most 1024 modes and returns GSC_ERR_INVALID beyond that.
 * Inputs and output are the caller's device arrays, as for gsc_summate_dev;
 * dim in {1, 2, 3}; forms AUTO or PLAIN_F64 only.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and
 * configures the kernel; make that first call before any stream capture.
 * All calls share the array, which keeps the last call's contents; kernels
 * of calls that overlap on the GPU race on it, so order such calls on one
 * stream or with events. */
int gsc_summate_dev_noalloc(const double *cov, const double *z1, const double *z2,
                            const double *pos, int64_t dim, int64_t n_modes,
                            int64_t n_points, double *out, const gsc_opts *opts);

/* ---- Fourier method: src/field.rs:219-249 ----------------------------- */
/* u[p] = sum_j sf[j] (z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p)) with k_j
 * the columns of `modes` (dim, n_modes) -- the equidistant Fourier grid --
 * and sf the spectrum factor sqrt(2 S(k_j dk)) (n_modes).  The factor is
 * folded into z1, z2 on the GPU (one rounding each), after which every form
 * of gsc_summate_f64 applies.  Replaces field::summator_fourier
 * (src/field.rs:219) / PyO3 summate_fourier (src/lib.rs:67-84). */
int gsc_summate_fourier_f64(const double *spectrum_factor, int64_t sf_stride,
                            const double *modes, int64_t modes_stride_d, int64_t modes_stride_n,
                            const double *z1, int64_t z1_stride,
                            const double *z2, int64_t z2_stride,
                            const double *pos, int64_t pos_stride_d, int64_t pos_stride_p,
                            int64_t dim, int64_t n_modes, int64_t n_points,
                            double *out, int64_t out_stride,
                            const gsc_opts *opts);

/* Device-pointer form: modes (dim, n_modes) and pos (dim, n_points)
 * row-major; spectrum_factor, z1, z2 (n_modes); out (n_points). */
int gsc_summate_fourier_dev(const double *spectrum_factor, const double *modes,
                            const double *z1, const double *z2, const double *pos,
                            int64_t dim, int64_t n_modes, int64_t n_points,
                            double *out, const gsc_opts *opts);

/* ---- incompressible vector field: src/field.rs:97-182 ----------------- */
/* u[i, p] = sum_j p_i(k_j) (z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p)),
 * p(k) = e_1 - k k_0 / |k|^2, dim in {2, 3}; out (dim, n_points) written
 * at out[i * out_stride_d + p * out_stride_p] (the reference returns the
 * Fortran-ordered array: out_stride_d = 1, out_stride_p = dim).
 * Replaces field::summator_incompr (src/field.rs:97) / PyO3 summate_incompr
 * (src/lib.rs:52). */
int gsc_summate_incompr_f64(const double *cov, int64_t cov_stride_d, int64_t cov_stride_n,
                            const double *z1, int64_t z1_stride,
                            const double *z2, int64_t z2_stride,
                            const double *pos, int64_t pos_stride_d, int64_t pos_stride_p,
                            int64_t dim, int64_t n_modes, int64_t n_points,
                            double *out, int64_t out_stride_d, int64_t out_stride_p,
                            const gsc_opts *opts);

/* Device-pointer form: out (dim, n_points) row-major. */
int gsc_summate_incompr_dev(const double *cov, const double *z1, const double *z2,
                            const double *pos, int64_t dim, int64_t n_modes,
                            int64_t n_points, double *out, const gsc_opts *opts);

/* ---- structured grids ------------------------------------------------ */
/* The scalar field of gsc_summate_f64 on the grid
 * meshgrid(axis0, axis1[, axis2], indexing="ij") flattened in C order, i.e.
 * the points GSTools passes to summate for a structured mesh:
 * p = (i0 * n1 + i1) * n2 + i2.  dim in {1, 2, 3}; axis d has n_d points
 * with element stride s_d (unused axes: NULL, 0, 0).  out[p], p < prod n_d,
 * contiguous.  Forms: GSC_FORM_SEP_* (tensor cores), GSC_FORM_PLAIN_* (the
 * plain kernel on the expanded grid) or AUTO.  New entry point: the
 * reference has no structured variant (its callers expand the grid). */
int gsc_summate_structured_f64(const double *cov, int64_t cov_stride_d, int64_t cov_stride_n,
                               const double *z1, int64_t z1_stride,
                               const double *z2, int64_t z2_stride,
                               int64_t dim, int64_t n_modes,
                               const double *axis0, int64_t n0, int64_t s0,
                               const double *axis1, int64_t n1, int64_t s1,
                               const double *axis2, int64_t n2, int64_t s2,
                               double *out, const gsc_opts *opts);

/* Device-pointer form: contiguous axes, out (prod n_d) contiguous. */
int gsc_summate_structured_dev(const double *cov, const double *z1, const double *z2,
                               int64_t dim, int64_t n_modes,
                               const double *axis0, int64_t n0,
                               const double *axis1, int64_t n1,
                               const double *axis2, int64_t n2,
                               double *out, const gsc_opts *opts);

/* Incompressible field on a structured grid (dim in {2, 3}): out is
 * (dim, prod n_d) row-major (component c at out + c * prod n_d). */
int gsc_summate_incompr_structured_f64(const double *cov, int64_t cov_stride_d,
                                       int64_t cov_stride_n,
                                       const double *z1, int64_t z1_stride,
                                       const double *z2, int64_t z2_stride,
                                       int64_t dim, int64_t n_modes,
                                       const double *axis0, int64_t n0, int64_t s0,
                                       const double *axis1, int64_t n1, int64_t s1,
                                       const double *axis2, int64_t n2, int64_t s2,
                                       double *out, const gsc_opts *opts);

int gsc_summate_incompr_structured_dev(const double *cov, const double *z1, const double *z2,
                                       int64_t dim, int64_t n_modes,
                                       const double *axis0, int64_t n0,
                                       const double *axis1, int64_t n1,
                                       const double *axis2, int64_t n2,
                                       double *out, const gsc_opts *opts);

/* Fourier-method field on a structured grid (the Fourier modes of a periodic
 * field lie on an equidistant grid, so the separable forms apply): as
 * gsc_summate_structured_f64 with the spectrum factor of
 * gsc_summate_fourier_f64.  No reference counterpart (callers of
 * summator_fourier expand the grid). */
int gsc_summate_fourier_structured_f64(const double *spectrum_factor, int64_t sf_stride,
                                       const double *modes, int64_t modes_stride_d,
                                       int64_t modes_stride_n,
                                       const double *z1, int64_t z1_stride,
                                       const double *z2, int64_t z2_stride,
                                       int64_t dim, int64_t n_modes,
                                       const double *axis0, int64_t n0, int64_t s0,
                                       const double *axis1, int64_t n1, int64_t s1,
                                       const double *axis2, int64_t n2, int64_t s2,
                                       double *out, const gsc_opts *opts);

int gsc_summate_fourier_structured_dev(const double *spectrum_factor, const double *modes,
                                       const double *z1, const double *z2,
                                       int64_t dim, int64_t n_modes,
                                       const double *axis0, int64_t n0,
                                       const double *axis1, int64_t n1,
                                       const double *axis2, int64_t n2,
                                       double *out, const gsc_opts *opts);

/* ---- batched ensembles ------------------------------------------------ */
/* Many realizations (items) with their own dimension, mode and point counts
 * summed by one persistent kernel fed from a device work queue, replayable
 * as a CUDA graph.  No reference counterpart: GSTools calls summate once per
 * realization; each item computes exactly what that call computes.  All
 * pointers are device pointers to dense row-major arrays: cov (dim, n_modes)
 * (Fourier: the mode grid), z1, z2, spectrum_factor (n_modes), pos
 * (dim, n_points), out (n_points), or (dim, n_points) for INCOMPR items. */
#define GSC_BATCH_SCALAR   0   /* field::summator           src/field.rs:37   */
#define GSC_BATCH_INCOMPR  1   /* field::summator_incompr   src/field.rs:97   */
#define GSC_BATCH_FOURIER  2   /* field::summator_fourier   src/field.rs:219  */

typedef struct gsc_batch_item {
    int32_t dim;                    /* 1, 2, 3 (INCOMPR: 2, 3)               */
    int32_t kind;                   /* GSC_BATCH_*                           */
    int64_t n_modes, n_points;
    const double *cov, *z1, *z2;
    const double *spectrum_factor;  /* FOURIER items only                    */
    const double *pos;
    double *out;
} gsc_batch_item;

/* Configuration of a plan.  Inputs (0 = let the autotuner choose):
 * points_per_thread (2, 4, 8), tile_modes (FP64 form: 8 or 16, with 2 or 4
 * points per thread), units_per_block (target work units per resident
 * block: how finely item modes are split).  gsc_batch_get_config fills all
 * fields with what the plan uses. */
typedef struct gsc_batch_config {
    int32_t struct_size;            /* sizeof(gsc_batch_config)              */
    int32_t points_per_thread;
    int32_t tile_modes;
    int32_t units_per_block;
    int32_t form;                   /* out: GSC_FORM_PLAIN_F64 / MIXED / ..   */
    int32_t blocks;                 /* out: persistent blocks launched       */
    int64_t units;                  /* out: work units in the queue          */
    int32_t max_splits;             /* out: largest mode split of an item    */
    int32_t tuned;                  /* out: 1 if this plan ran the autotuner */
    double  tune_ms;                /* out: GPU time spent tuning            */
    double  work;                   /* out: point*modes (x components)       */
} gsc_batch_config;

typedef struct gsc_batch gsc_batch;

/* Builds a plan on opts->device (forms AUTO, PLAIN_F64, MIXED,
 * MIXED_F64PHASE; AUTO is MIXED for tolerance >= 1e-6, else PLAIN_F64).  It
 * allocates the plan's device memory (tables, queue, split partials) and,
 * unless `config` fixes every choice or an ensemble of the same shape was
 * tuned before in this process, times the candidate configurations on this
 * ensemble's own data -- writing scratch values into the items' outputs --
 * and returns when done.  The item pointers are bound to the plan: change
 * the data in place between runs, not the pointers. */
int gsc_batch_create(const gsc_batch_item *items, int64_t count, const gsc_opts *opts,
                     const gsc_batch_config *config, gsc_batch **plan);

/* Enqueues one run of the whole ensemble on `stream` (cudaStream_t, NULL =
 * legacy default stream): tables, the persistent kernel, the split
 * reduction.  Allocates nothing and does not synchronise.  Runs of one plan
 * must not overlap each other on the GPU. */
int gsc_batch_run(gsc_batch *plan, void *stream);

/* As gsc_batch_run, through a CUDA graph of the run captured on the first
 * call (on a stream of the plan) and launched on `stream` afterwards. */
int gsc_batch_run_graph(gsc_batch *plan, void *stream);

int gsc_batch_get_config(const gsc_batch *plan, gsc_batch_config *config);

/* Frees the plan; its runs must have completed. */
int gsc_batch_destroy(gsc_batch *plan);

/* Host-pointer ensemble: items as for gsc_batch_create but with HOST
 * pointers to dense row-major arrays.  Packs the inputs into pinned staging
 * and copies them to the GPU, runs the ensemble (the plans of the previous
 * call on the device are reused when the shapes match), and copies every
 * output back before returning.  An ensemble of at least 4e9 point*modes and
 * 8 items runs as G = 4 groups of consecutive items (8 from 4e10 point*modes
 * and 16 items): the first and the last hold 1/(4G) of the work each, the
 * others share the rest equally; one plan each.  A group's inputs are copied while the
 * previous group computes, and its results while the next one computes.
 * Without a config (or with zero fields), the groups share one set of
 * launch choices, tuned on the group with the most work and cached under the
 * ensemble's shape.  A mixed-form item whose wave number times extent passes
 * 2^30 turns makes the call recompute the ensemble on GSC_FORM_PLAIN_F64
 * under GSC_FORM_AUTO and return GSC_ERR_KERNEL under an explicit
 * GSC_FORM_MIXED. */
int gsc_summate_batch_f64(const gsc_batch_item *items, int64_t count, const gsc_opts *opts,
                          const gsc_batch_config *config);

/* Configuration of the plan used by the last gsc_summate_batch_f64 call on
 * `device` (-1 = current); for a call run in groups, the first group's
 * launch choices with the units, work and tuning time of all groups. */
int gsc_last_batch_config(int32_t device, gsc_batch_config *config);

/* ---- autotuner cache ------------------------------------------------------ */
/* Launch choices that depend on a call's shape (points per thread and mode
 * splits of the mixed kernel, the batch planner's configuration) are timed on
 * the call's own data the first time a shape bucket is seen on a device and
 * kept, keyed by the device's name, the kernel family and the buckets.  With
 * a cache file the entries persist across processes: gsc_tune_cache_open
 * reads `path` if it exists and writes every new entry to it (NULL: memory
 * only); a file whose header, entries or checksum do not match is refused
 * (GSC_ERR_INVALID) and then neither read nor overwritten.  The environment
 * variable GSC_TUNE_CACHE names a file to open on first use.
 * gsc_tune_set_mode: 0 fixed default configurations, 1 cached entries only,
 * 2 (default, or GSC_TUNE) tune on a miss.  get/put/clear/size inspect the
 * cache (put writes an entry as the tuner does).  No reference counterpart:
 * the reference has no tunable launch parameters. */
int gsc_tune_cache_open(const char *path);
int gsc_tune_cache_size(int64_t *entries);
int gsc_tune_cache_get(const char *key, int32_t *values);
int gsc_tune_cache_put(const char *key, const int32_t *values);
int gsc_tune_cache_clear(void);
int gsc_tune_set_mode(int32_t mode);

/* ---- self-test of the failure path -------------------------------------- */
/* Runs one CTA that waits, with the bounded wait of the tensor-core
 * pipelines, on a barrier nothing completes; the wait gives up after
 * limit_us microseconds (1e3 .. 2e6), records its code in the device status
 * word and the kernel returns.  Returns what gsc_device_status returns:
 * GSC_ERR_KERNEL with the recorded code, after which the status is clear
 * and the device remains usable.  No reference counterpart. */
int gsc_selftest_wait_timeout(int32_t device, int64_t limit_us);

/* Issue rates of the instruction kinds the mixed form's inner loop is made
 * of, measured on `device` (-1 = current): rates[0] high 32-bit integer
 * multiply-adds (__umulhi), rates[1] low 32-bit integer multiply-adds,
 * rates[2] FP32 fused multiply-adds, each in thread operations per second
 * over the whole GPU (best of 3 launches of independent chains).  A
 * measurement for roofline accounting; no reference counterpart. */
int gsc_selftest_pipe_rates(int32_t device, double *rates);

/* Allocation-failure injection: the `countdown`-th next allocation of a
 * library buffer (0 = the next one; device scratch, pinned staging, batch
 * plan memory) fails as GSC_ERR_NOMEM with "injected allocation failure" in
 * the message, exactly as a real out-of-memory does, after which injection
 * is off again.  -1 switches it off.  Process-wide.  No reference
 * counterpart. */
int gsc_selftest_fail_alloc(int32_t countdown);

/* Structured-mesh recognition of the point entry points, on host arrays
 * alone (no device is touched): for pos (dim, n_points) with element
 * strides, sets n_axes[0..2] to the axis lengths when the points are
 * meshgrid(*axes, indexing="ij") flattened in C order, as GSTools passes a
 * structured mesh, every point compared with the rebuilt axes (n_axes[d] = 0
 * for d >= dim).  All three are 0 when the points are no such mesh or would
 * not be routed (dim not 2 or 3, fewer than 4096 points, an axis of one
 * point).  Returns GSC_OK, or GSC_ERR_INVALID for NULL pointers and negative
 * sizes.  No reference counterpart. */
int gsc_selftest_detect_grid(const double *pos, int64_t pos_stride_d, int64_t pos_stride_p,
                             int64_t dim, int64_t n_points, int64_t *n_axes);

/* Per-device kernel set-up, on the host only (no device is touched): the
 * registry that every launch path uses to set a kernel's launch attributes
 * once per (kernel, device) -- cudaFuncSetAttribute applies to the device
 * current at the time, so a process-wide flag would leave later devices
 * unconfigured -- is driven by `n_threads` threads (1 .. 64) at once over
 * `n_keys` stand-in kernels (1 .. 64) and `n_devices` stand-in device
 * ordinals (1 .. 64), each thread visiting every pair in its own order.
 * Every pair's set-up fails on its first attempt and succeeds on the second.
 * Sets *setups to the number of successful set-ups and returns GSC_OK when
 * each pair succeeded exactly once and was tried no more than twice, else
 * GSC_ERR_KERNEL.  No reference counterpart. */
int gsc_selftest_once_per_device(int32_t n_devices, int32_t n_keys, int32_t n_threads,
                                 int64_t *setups);

/* Work-queue check of the batch planner, on the host only (no device is
 * touched; the items' pointers are ignored): builds the cost-sorted work
 * queue that gsc_batch_create would build for `items` with configuration
 * `config` (points_per_thread, tile_modes, units_per_block) and `blocks`
 * resident blocks, applies `corruption` to it, and validates it the way
 * every plan's queue is validated before it is uploaded: each unit names an
 * item and split that exist, starts on a point-block boundary inside the
 * item and covers a mode range inside it, and every (point block, split) of
 * every item appears exactly once with the splits tiling [0, n_modes) in
 * order.  Returns GSC_OK for a valid queue, GSC_ERR_INVALID (with the
 * failing unit in the message) for a corrupt one.
 *   corruption 0 none, 1 drop a unit, 2 duplicate a unit, 3 item index out
 *   of range, 4 shift a unit's mode range, 5 misalign a unit's point block,
 *   6 split index out of range */
int gsc_selftest_batch_queue(const gsc_batch_item *items, int64_t count, int32_t form,
                             const gsc_batch_config *config, int32_t blocks,
                             int32_t corruption);

/* ---- on-device spectral sampling ---------------------------------------- */
/* The randomization method's inputs drawn on the GPU: wave vectors
 * cov (dim, n_modes) from a covariance model's spectral density and the
 * weights z1, z2 ~ N(0, 1).  No reference counterpart: GSTools draws them on
 * the host (RandMeth).  Every value is a function of (seed, realization,
 * mode) only (Philox4x32-10 counters), so realizations and modes can be
 * drawn in any order or subset with identical results.
 *   GAUSSIAN     k ~ N(0, 2 / len_scale^2) per component
 *   EXPONENTIAL  k = g / |n| / len_scale, g ~ N(0, I), n ~ N(0, 1)
 *                (multivariate Student-t, one degree of freedom) */
#define GSC_SPECTRUM_GAUSSIAN     0
#define GSC_SPECTRUM_EXPONENTIAL  1

typedef struct gsc_sample_item {
    int32_t spectrum;               /* GSC_SPECTRUM_*                        */
    int32_t dim;                    /* 1, 2, 3                               */
    int64_t n_modes;
    double  len_scale;              /* > 0                                   */
    int64_t realization;            /* counter word: one stream per value    */
    double *cov, *z1, *z2;          /* device outputs, (dim, n_modes), (n)   */
} gsc_sample_item;

/* All items in one launch on opts->stream (no synchronisation). */
int gsc_sample_modes_batch_dev(const gsc_sample_item *items, int64_t count, uint64_t seed,
                               const gsc_opts *opts);

/* One realization, device outputs. */
int gsc_sample_modes_dev(int32_t spectrum, int32_t dim, int64_t n_modes, double len_scale,
                         uint64_t seed, int64_t realization, double *cov, double *z1,
                         double *z2, const gsc_opts *opts);

/* One realization, host outputs (returns when they are written). */
int gsc_sample_modes_f64(int32_t spectrum, int32_t dim, int64_t n_modes, double len_scale,
                         uint64_t seed, int64_t realization, double *cov, double *z1,
                         double *z2, const gsc_opts *opts);

#ifdef __cplusplus
}
#endif

#endif /* GSTOOLS_CORE_GB300_H */
