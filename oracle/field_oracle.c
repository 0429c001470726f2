/*
 * field_oracle.c -- CPU restatement of GSTools-Core's randomization-method
 * summators (reference crate gstools-core 1.1.0, src/field.rs).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product path (gstools-core_gb300/) never links or calls it.
 *
 * Parity is pinned: the functions below reproduce the reference's own
 * known-answer tests (src/field.rs:359-381 summator, bit exact;
 * src/field.rs:384-430 summator_incompr, within the reference's own
 * assert_ulps_eq!(max_ulps = 6) rule; src/field.rs:334-356 summator_fourier,
 * bit exact).  See tests/test_oracle.py.
 *
 * Floating-point contract (what makes it bit exact against the Rust code):
 *   - compiled with -ffp-contract=off: Rust never contracts a*b+c into FMA;
 *   - phase = ((0 + k0*x0) + k1*x1) + k2*x2 ..., left to right, which is what
 *     ndarray 0.15's 1-D `dot` does for the strided columns of a C-order
 *     (d, N) array (src/field.rs:57), and what ShortVec::dot does
 *     (src/short_vec.rs:30-33);
 *   - glibc cos()/sin(): Rust's f64::cos/sin on linux-gnu call libm.
 *
 * All strides are in elements (not bytes), so any numpy view can be passed.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2
#define ORC_EDIM 3

/* --------------------------------------------------------------------- */
/* scalar summator: src/field.rs:37-65                                    */
/* --------------------------------------------------------------------- */

typedef struct {
    const double *cov; int64_t cs_d, cs_n;
    const double *z1; int64_t z1s;
    const double *z2; int64_t z2s;
    const double *pos; int64_t ps_d, ps_p;
    const double *sf; int64_t sfs;   /* spectrum factor (Fourier) or NULL */
    int64_t dim, n_modes, p_begin, p_end;
    double *out; int64_t os;
} scalar_job;

/* One point: the sequential fold over modes of src/field.rs:54-62
 * (summator) or src/field.rs:236-244 (summator_fourier). */
static double scalar_point(const scalar_job *jb, int64_t p)
{
    double sum = 0.0;
    for (int64_t j = 0; j < jb->n_modes; ++j) {
        double phase = 0.0;                      /* ndarray dot: 0 + sum_d */
        for (int64_t d = 0; d < jb->dim; ++d)
            phase = phase + jb->cov[d * jb->cs_d + j * jb->cs_n] *
                            jb->pos[d * jb->ps_d + p * jb->ps_p];
        double z1 = jb->z1[j * jb->z1s];
        double z2 = jb->z2[j * jb->z2s];
        double z12 = z1 * cos(phase) + z2 * sin(phase);   /* field.rs:58 */
        if (jb->sf)
            z12 = jb->sf[j * jb->sfs] * z12;              /* field.rs:243 */
        sum = sum + z12;                                  /* field.rs:60 */
    }
    return sum;
}

static void *scalar_worker(void *arg)
{
    scalar_job *jb = (scalar_job *)arg;
    for (int64_t p = jb->p_begin; p < jb->p_end; ++p)
        jb->out[p * jb->os] = scalar_point(jb, p);
    return NULL;
}

/* Parallel over points, like `Zip::from(pos.columns()).par_map_collect`
 * (src/field.rs:53).  Every point keeps the sequential mode order, so the
 * result does not depend on the thread count. */
static int run_scalar(scalar_job base, int64_t n_points, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (n_points < nthreads) nthreads = n_points > 0 ? (int)n_points : 1;
    if (nthreads == 1) {
        base.p_begin = 0; base.p_end = n_points;
        scalar_worker(&base);
        return ORC_OK;
    }
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
    scalar_job *jobs = malloc(sizeof(scalar_job) * (size_t)nthreads);
    if (!th || !jobs) { free(th); free(jobs); return ORC_ENOMEM; }
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = base;
        jobs[t].p_begin = n_points * t / nthreads;
        jobs[t].p_end = n_points * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, scalar_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return ORC_OK;
}

int orc_summator(const double *cov, int64_t cs_d, int64_t cs_n,
                 const double *z1, int64_t z1s,
                 const double *z2, int64_t z2s,
                 const double *pos, int64_t ps_d, int64_t ps_p,
                 int64_t dim, int64_t n_modes, int64_t n_points,
                 double *out, int64_t os, int nthreads)
{
    if (dim < 0 || n_modes < 0 || n_points < 0) return ORC_EINVAL;
    scalar_job jb = {cov, cs_d, cs_n, z1, z1s, z2, z2s, pos, ps_d, ps_p,
                     NULL, 0, dim, n_modes, 0, 0, out, os};
    return run_scalar(jb, n_points, nthreads);
}

/* summator_fourier: src/field.rs:219-249 (same fold, scaled per mode). */
int orc_summator_fourier(const double *sf, int64_t sfs,
                         const double *modes, int64_t ms_d, int64_t ms_n,
                         const double *z1, int64_t z1s,
                         const double *z2, int64_t z2s,
                         const double *pos, int64_t ps_d, int64_t ps_p,
                         int64_t dim, int64_t n_modes, int64_t n_points,
                         double *out, int64_t os, int nthreads)
{
    if (dim < 0 || n_modes < 0 || n_points < 0) return ORC_EINVAL;
    scalar_job jb = {modes, ms_d, ms_n, z1, z1s, z2, z2s, pos, ps_d, ps_p,
                     sf, sfs, dim, n_modes, 0, 0, out, os};
    return run_scalar(jb, n_points, nthreads);
}

/* --------------------------------------------------------------------- */
/* incompressible summator: src/field.rs:97-182                           */
/* --------------------------------------------------------------------- */

typedef struct {
    const double *cov; int64_t cs_d, cs_n;
    const double *z1; int64_t z1s;
    const double *z2; int64_t z2s;
    const double *pos; int64_t ps_d, ps_p;
    int64_t dim, n_points, j_begin, j_end;
    double *acc;            /* (n_points, dim) private accumulator */
} incompr_job;

/* The fold body of src/field.rs:135-156 for the mode range [j_begin, j_end),
 * accumulated into a zeroed (n_points, dim) array, as one rayon fold split
 * does with its `vec![ShortVec::zero(); pos.len()]` (src/field.rs:136). */
static void *incompr_worker(void *arg)
{
    incompr_job *jb = (incompr_job *)arg;
    const int64_t D = jb->dim;
    double k[3], x[3];
    for (int64_t j = jb->j_begin; j < jb->j_end; ++j) {
        for (int64_t d = 0; d < D; ++d) k[d] = jb->cov[d * jb->cs_d + j * jb->cs_n];
        double kk = 0.0;                               /* ShortVec::dot */
        for (int64_t d = 0; d < D; ++d) kk = kk + k[d] * k[d];
        double k_2 = k[0] / kk;                        /* field.rs:138 */
        double z1 = jb->z1[j * jb->z1s];
        double z2 = jb->z2[j * jb->z2s];
        for (int64_t p = 0; p < jb->n_points; ++p) {
            for (int64_t d = 0; d < D; ++d) x[d] = jb->pos[d * jb->ps_d + p * jb->ps_p];
            double phase = 0.0;                        /* field.rs:145 */
            for (int64_t d = 0; d < D; ++d) phase = phase + k[d] * x[d];
            double z12 = z1 * cos(phase) + z2 * sin(phase);   /* :146 */
            double *s = jb->acc + p * D;
            s[0] += (1.0 - k[0] * k_2) * z12;          /* field.rs:148 */
            for (int64_t d = 1; d < D; ++d)            /* field.rs:150-152 */
                s[d] -= k[d] * k_2 * z12;
        }
    }
    return NULL;
}

/* nthreads <= 1: one fold split over all modes, i.e. the single-threaded
 * reference.  nthreads > 1: contiguous mode chunks of at least 100 modes
 * (rayon `with_min_len(100)`, src/field.rs:134), each with its own
 * accumulator, then a left-to-right reduce (src/field.rs:158-163).  The
 * reference's own reduction tree depends on rayon's work splitting, so
 * results are compared by tolerance, exactly as the reference's test does. */
int orc_summator_incompr(const double *cov, int64_t cs_d, int64_t cs_n,
                         const double *z1, int64_t z1s,
                         const double *z2, int64_t z2s,
                         const double *pos, int64_t ps_d, int64_t ps_p,
                         int64_t dim, int64_t n_modes, int64_t n_points,
                         double *out, int64_t os_d, int64_t os_p, int nthreads)
{
    if (n_modes < 0 || n_points < 0) return ORC_EINVAL;
    if (dim != 2 && dim != 3) return ORC_EDIM;   /* field.rs:177-181 panics */
    int64_t chunks = nthreads < 1 ? 1 : nthreads;
    int64_t max_chunks = n_modes / 100;
    if (chunks > max_chunks) chunks = max_chunks;
    if (chunks < 1) chunks = 1;
    size_t acc_len = (size_t)n_points * (size_t)dim;
    double *acc = calloc(acc_len ? acc_len * (size_t)chunks : 1, sizeof(double));
    incompr_job *jobs = malloc(sizeof(incompr_job) * (size_t)chunks);
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)chunks);
    if (!acc || !jobs || !th) { free(acc); free(jobs); free(th); return ORC_ENOMEM; }
    for (int64_t c = 0; c < chunks; ++c) {
        incompr_job jb = {cov, cs_d, cs_n, z1, z1s, z2, z2s, pos, ps_d, ps_p,
                          dim, n_points, n_modes * c / chunks,
                          n_modes * (c + 1) / chunks, acc + acc_len * (size_t)c};
        jobs[c] = jb;
    }
    if (chunks == 1) {
        incompr_worker(&jobs[0]);
    } else {
        for (int64_t c = 0; c < chunks; ++c)
            pthread_create(&th[c], NULL, incompr_worker, &jobs[c]);
        for (int64_t c = 0; c < chunks; ++c) pthread_join(th[c], NULL);
        for (int64_t c = 1; c < chunks; ++c)           /* ShortVec::add */
            for (size_t i = 0; i < acc_len; ++i) acc[i] += acc[acc_len * (size_t)c + i];
    }
    /* (n_points, dim) -> out[d, p] (field.rs:166-174 returns the transpose) */
    for (int64_t p = 0; p < n_points; ++p)
        for (int64_t d = 0; d < dim; ++d)
            out[d * os_d + p * os_p] = acc[p * dim + d];
    free(acc); free(jobs); free(th);
    return ORC_OK;
}
