// plain.cu -- FP64 randomization-method summators for GB300 (sm_103a).
//
// Computes, in FP64 end to end,
//   scalar   u[p]    = sum_j z1_j cos(k_j.x_p) + z2_j sin(k_j.x_p)
//            (reference: src/field.rs:37-65)
//   incompr  u[i, p] = sum_j w_ij (z1_j cos(k_j.x_p) + z2_j sin(k_j.x_p)),
//            w_0j = 1 - k_0j k_0j/|k_j|^2, w_ij = -k_ij k_0j/|k_j|^2
//            (reference: src/field.rs:97-182)
//
// Design.  GB300's FP64 pipe is narrow, so the kernel is built to spend as
// few FP64 instructions per point*mode as possible while staying FP64
// accurate:
//  * phase k.x is formed exactly as the reference forms it:
//    ((k0*x0 + k1*x1) + k2*x2), no FMA, so every phase has the reference's
//    bits (src/field.rs:57, src/short_vec.rs:30-33);
//  * sincos is table driven (Tang-style): phase = n*(2pi/M) + r with a
//    two-constant Cody-Waite reduction (exact first step under FMA) and
//    |r| <= pi/M, M = 256; e^{ir} by short Taylor polynomials (truncation
//    below 5e-15), and the angle n*(2pi/M) folded into a per-mode table
//    W_j[a] = (z1_j - i z2_j) e^{i 2 pi a/M}, so
//    z1 cos(phase) + z2 sin(phase) = Re(W_j[n mod M] e^{ir})
//    = Re W cos r - Im W sin r: 18 FP64 operations per point*mode for d=3;
//  * per-mode tables live in global memory and are staged tile by tile into
//    shared memory with cp.async double buffering; each thread keeps R
//    points in registers, so one staged tile serves T*R points;
//  * phases beyond |k.x| ~ 1e13 (where the one-step reduction would lose
//    accuracy) take CUDA's sincos() for the whole tile (warp-uniform test);
//  * when there are too few points to fill 152 SMs, the modes are split
//    across blockIdx.y and the partial sums are added in split order by a
//    second kernel (deterministic; no atomics).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>

#include "internal.h"

namespace gsc {
namespace {

constexpr int kM = 256;                             // table angles per turn
constexpr double kInvStep = 40.74366543152521;      // M / (2 pi)
constexpr double kStepHi = 0.02454369260617026;     // fl(2 pi / M) = fl(pi)/128
constexpr double kStepLo = 9.567553118338697e-19;   // fl(2 pi / M - kStepHi)
constexpr double kRound = 6755399441055744.0;       // 1.5 * 2^52: x + kRound rounds x
constexpr double kSafePhase = 1.0e13;               // table path bound on |k.x|
constexpr int kRec = 12;                            // doubles per mode record
constexpr int kThreads = 128;                       // threads per block
constexpr int kTileModes = 8;                       // modes per staged tile
constexpr int64_t kChunkModes = 16384;              // modes per table build
static_assert(kThreads == kBatchThreads, "batch units assume the plain block size");

// Mode record layout (doubles): k0 k1 k2 | sum|k| | z1 z2 | w0 w1 w2 | pad
enum { R_K0 = 0, R_KABS = 3, R_Z1 = 4, R_Z2 = 5, R_W0 = 6 };

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---------------------------------------------------------------------------
// Per-mode tables: W_j[a] = (z1 - i z2) e^{i 2 pi a / M} and the mode record.
// grid (nc), block (kM)
// ---------------------------------------------------------------------------
// Table row a (thread) and, for a == 0, the record of mode j.
__device__ __forceinline__ void mode_entry(const double *__restrict__ cov, double z1j, double z2j,
                                           int64_t dim, int64_t n_modes, int64_t j, int incompr,
                                           int want_table, double2 *__restrict__ wrow,
                                           double *__restrict__ r) {
    const int a = threadIdx.x;
    if (want_table) {
        double s, c;
        sincospi(a * (1.0 / (kM / 2)), &s, &c);       // angle 2 pi a / M
        wrow[a] = make_double2(z1j * c + z2j * s, z1j * s - z2j * c);
    }
    if (a == 0) {
        double k[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < dim && d < 3; ++d) k[d] = cov[d * n_modes + j];
        r[R_K0 + 0] = k[0];
        r[R_K0 + 1] = k[1];
        r[R_K0 + 2] = k[2];
        r[R_KABS] = fabs(k[0]) + fabs(k[1]) + fabs(k[2]);
        r[R_Z1] = z1j;
        r[R_Z2] = z2j;
        double w0 = 0.0, w1 = 0.0, w2 = 0.0;
        if (incompr) {
            // src/field.rs:138: k_2 = k0 / k.k, ShortVec::dot order, no FMA
            double kk = 0.0;
            for (int d = 0; d < dim; ++d) kk = __dadd_rn(kk, __dmul_rn(k[d], k[d]));
            const double k_2 = __ddiv_rn(k[0], kk);
            w0 = __dadd_rn(1.0, -__dmul_rn(k[0], k_2));          // :148
            w1 = -__dmul_rn(k[1], k_2);                            // :150-152
            w2 = -__dmul_rn(k[2], k_2);
        }
        r[R_W0 + 0] = w0;
        r[R_W0 + 1] = w1;
        r[R_W0 + 2] = w2;
        r[9] = r[10] = r[11] = 0.0;
    }
}

__global__ void __launch_bounds__(kM)
mode_table_kernel(const double *__restrict__ cov, const double *__restrict__ z1,
                  const double *__restrict__ z2, int64_t dim, int64_t n_modes, int64_t j0,
                  int incompr, int want_table, double2 *__restrict__ wtab,
                  double *__restrict__ rec, const int *__restrict__ run_if) {
    if (run_if && *run_if == 0) return;      // a predicated launch that is not wanted
    const int64_t jl = blockIdx.x;
    const int64_t j = j0 + jl;
    mode_entry(cov, z1[j], z2[j], dim, n_modes, j, incompr, want_table, wtab + jl * kM,
               rec + jl * kRec);
}

// item owning global row g: the last i with prefix[i] <= g
__device__ __forceinline__ int64_t owner_of(const int64_t *__restrict__ prefix, int64_t n,
                                            int64_t g) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Tables of every item of a batch: grid (total modes), block (kM).  The
// Fourier factor, where present, multiplies z1 and z2 first.
__global__ void __launch_bounds__(kM)
batch_table_kernel(const BatchItem *__restrict__ items, const int64_t *__restrict__ prefix,
                   int64_t n_items, double2 *__restrict__ wtab, double *__restrict__ rec) {
    const int64_t g = blockIdx.x;
    const BatchItem &it = items[owner_of(prefix, n_items, g)];
    const int64_t j = g - it.mode_off;
    double z1j = it.z1[j], z2j = it.z2[j];
    if (it.sf) {
        const double f = it.sf[j];
        z1j = __dmul_rn(f, z1j);
        z2j = __dmul_rn(f, z2j);
    }
    mode_entry(it.cov, z1j, z2j, it.dim, it.n_modes, j, it.incompr, 1, wtab + g * kM,
               rec + g * kRec);
}

// phase = k.x in the reference's order (ndarray dot on strided columns)
template <int D>
__device__ __forceinline__ double phase_of(const double *k, const double *x) {
    double ph = __dmul_rn(k[0], x[0]);
    if (D > 1) ph = __dadd_rn(ph, __dmul_rn(k[1], x[1]));
    if (D > 2) ph = __dadd_rn(ph, __dmul_rn(k[2], x[2]));
    return ph;
}

// z1 cos(ph) + z2 sin(ph) through the mode's angle table (see file header).
__device__ __forceinline__ double table_term(double ph, const double2 *__restrict__ tab) {
    const double s = fma(ph, kInvStep, kRound);
    const double n = s - kRound;
    const int a = __double2loint(s) & (kM - 1);
    double r = fma(-n, kStepHi, ph);          // exact
    r = fma(-n, kStepLo, r);
    const double r2 = r * r;
    const double cr = fma(r2, fma(r2, 1.0 / 24.0, -0.5), 1.0);
    const double sr = fma(r * r2, fma(r2, 1.0 / 120.0, -1.0 / 6.0), r);
    const double2 w = tab[a];
    return fma(w.x, cr, -(w.y * sr));
}

// ---------------------------------------------------------------------------
// One block's work: the kThreads*R points starting at p_first (thread t owns
// p_first + t + r*kThreads), modes [jb, je) of the staged tables `wtab`,
// `rec` (indices relative to them), TILE modes per staged tile.  The sums are
// written (accumulate=0) or added (accumulate=1) at dst + i*sd + p*sp.
// Shared memory: 2 * TILE * (kM*16 [table] + kRec*8) bytes at `smem`.
// ---------------------------------------------------------------------------
template <int D, int R, bool INC, bool LIBM, int TILE>
__device__ __forceinline__ void plain_block(const double *__restrict__ pos, int64_t P,
                                            int64_t p_first, const double2 *__restrict__ wtab,
                                            const double *__restrict__ rec, int64_t jb,
                                            int64_t je, int accumulate, double *__restrict__ dst,
                                            int64_t sd, int64_t sp, unsigned char *smem) {
    constexpr int NOUT = INC ? D : 1;
    constexpr int TAB_BYTES = LIBM ? 0 : TILE * kM * 16;
    constexpr int REC_BYTES = TILE * kRec * 8;
    constexpr int STAGE = TAB_BYTES + REC_BYTES;

    const int tid = threadIdx.x;
    const int64_t p0 = p_first + tid;

    double x[R][D];
    double acc[R][NOUT];
    double xabs = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t p = p0 + r * kThreads;
        double s = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            x[r][d] = p < P ? pos[d * P + p] : 0.0;
            s += fabs(x[r][d]);
        }
        xabs = fmax(xabs, s);
#pragma unroll
        for (int i = 0; i < NOUT; ++i) acc[r][i] = 0.0;
    }
    // warp-uniform bound on |x| for the table-path range test
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) xabs = fmax(xabs, __shfl_xor_sync(0xffffffffu, xabs, o));

    auto stage_tile = [&](int buf, int64_t t0) {
        const int tm = static_cast<int>(min(static_cast<int64_t>(TILE), je - t0));
        unsigned char *base = smem + buf * STAGE;
        if (!LIBM) {
            const int chunks = tm * kM;                      // 16-byte chunks
            const double2 *src = wtab + (t0)*kM;
            for (int c = tid; c < chunks; c += kThreads) cp_async16(base + c * 16, src + c);
        }
        const int rchunks = tm * kRec / 2;
        const double *rsrc = rec + t0 * kRec;
        for (int c = tid; c < rchunks; c += kThreads)
            cp_async16(base + TAB_BYTES + c * 16, rsrc + 2 * c);
        cp_async_commit();
    };

    if (jb < je) stage_tile(0, jb);
    int buf = 0;
    for (int64_t t0 = jb; t0 < je; t0 += TILE, buf ^= 1) {
        const int tm = static_cast<int>(min(static_cast<int64_t>(TILE), je - t0));
        if (t0 + TILE < je) {
            stage_tile(buf ^ 1, t0 + TILE);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const unsigned char *base = smem + buf * STAGE;
        const double2 *tab = reinterpret_cast<const double2 *>(base);
        const double *rc = reinterpret_cast<const double *>(base + TAB_BYTES);
        for (int m = 0; m < tm; ++m) {
            const double *mr = rc + m * kRec;
            double k[3] = {mr[R_K0], mr[R_K0 + 1], mr[R_K0 + 2]};
            double w[3] = {mr[R_W0], mr[R_W0 + 1], mr[R_W0 + 2]};
            const bool table_ok = !LIBM && (mr[R_KABS] * xabs < kSafePhase);
            if (table_ok) {
                const double2 *mt = tab + m * kM;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const double z12 = table_term(phase_of<D>(k, x[r]), mt);
                    if (INC) {
#pragma unroll
                        for (int i = 0; i < NOUT; ++i) acc[r][i] = fma(w[i], z12, acc[r][i]);
                    } else {
                        acc[r][0] = __dadd_rn(acc[r][0], z12);
                    }
                }
            } else {
                const double z1 = mr[R_Z1], z2 = mr[R_Z2];
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    double sn, cs;
                    sincos(phase_of<D>(k, x[r]), &sn, &cs);
                    const double z12 = __dadd_rn(__dmul_rn(z1, cs), __dmul_rn(z2, sn));
                    if (INC) {
#pragma unroll
                        for (int i = 0; i < NOUT; ++i) acc[r][i] = fma(w[i], z12, acc[r][i]);
                    } else {
                        acc[r][0] = __dadd_rn(acc[r][0], z12);
                    }
                }
            }
        }
        __syncthreads();   // buffer `buf` is refilled two tiles later
    }

#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t p = p0 + r * kThreads;
        if (p >= P) continue;
#pragma unroll
        for (int i = 0; i < NOUT; ++i) {
            double *o = dst + i * sd + p * sp;
            *o = accumulate ? *o + acc[r][i] : acc[r][i];
        }
    }
}

// ---------------------------------------------------------------------------
// Main kernel.  grid (ceil(P / (T*R)), splits), block T.
// Split s handles modes [s*mps, min(nc, (s+1)*mps)) of the current chunk and
// writes (accumulate=0) or adds (accumulate=1) its sums at
// dst + s*split_stride + i*sd + p*sp.
// ---------------------------------------------------------------------------
template <int D, int R, bool INC, bool LIBM>
__global__ void __launch_bounds__(kThreads)
plain_kernel(const double *__restrict__ pos, int64_t P, const double2 *__restrict__ wtab,
             const double *__restrict__ rec, int64_t nc, int64_t mps, int accumulate,
             double *__restrict__ dst, int64_t sd, int64_t sp, int64_t split_stride,
             const int *__restrict__ run_if) {
    if (run_if && *run_if == 0) return;      // a predicated launch that is not wanted
    extern __shared__ __align__(16) unsigned char smem[];
    const int64_t jb = static_cast<int64_t>(blockIdx.y) * mps;
    const int64_t je = min(nc, jb + mps);
    plain_block<D, R, INC, LIBM, kTileModes>(
        pos, P, static_cast<int64_t>(blockIdx.x) * (kThreads * R), wtab, rec, jb, je, accumulate,
        dst + static_cast<int64_t>(blockIdx.y) * split_stride, sd, sp, smem);
}

// ---------------------------------------------------------------------------
// Persistent batch kernel: each block takes the next unit of the device work
// queue (atomic counter) until the queue is empty.  A unit is one point block
// of one item and one of its mode ranges; its sums go to the item's output,
// or to its split slot when the item's modes are split.
// ---------------------------------------------------------------------------
template <int R, int TILE>
__global__ void __launch_bounds__(kThreads)
batch_plain_kernel(const BatchItem *__restrict__ items, const BatchUnit *__restrict__ units,
                   int64_t n_units, int *__restrict__ counter, const double2 *__restrict__ wtab,
                   const double *__restrict__ rec) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_unit;
    for (;;) {
        __syncthreads();                     // s_unit of the previous unit is consumed
        if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1);
        __syncthreads();
        const int64_t u = s_unit;
        if (u >= n_units) break;
        const BatchUnit w = units[u];
        const BatchItem &it = items[w.item];
        const int64_t P = it.n_points;
        const int64_t nout = it.incompr ? it.dim : 1;
        double *dst = it.splits > 1 ? it.part + static_cast<int64_t>(w.split) * nout * P : it.out;
        const double2 *wt = wtab + it.mode_off * kM;
        const double *rc = rec + it.mode_off * kRec;
        switch (it.dim * 2 + it.incompr) {
            case 2:
                plain_block<1, R, false, false, TILE>(it.pos, P, w.p_first, wt, rc, w.jb, w.je, 0,
                                                      dst, P, 1, smem);
                break;
            case 4:
                plain_block<2, R, false, false, TILE>(it.pos, P, w.p_first, wt, rc, w.jb, w.je, 0,
                                                      dst, P, 1, smem);
                break;
            case 5:
                plain_block<2, R, true, false, TILE>(it.pos, P, w.p_first, wt, rc, w.jb, w.je, 0,
                                                     dst, P, 1, smem);
                break;
            case 6:
                plain_block<3, R, false, false, TILE>(it.pos, P, w.p_first, wt, rc, w.jb, w.je, 0,
                                                      dst, P, 1, smem);
                break;
            case 7:
                plain_block<3, R, true, false, TILE>(it.pos, P, w.p_first, wt, rc, w.jb, w.je, 0,
                                                     dst, P, 1, smem);
                break;
            default:
                break;                       // rejected on the host
        }
    }
}

// out[i*sd + p*sp] = sum_s part[s][i][p], s ascending
__global__ void split_reduce_kernel(const double *__restrict__ part, int64_t S, int64_t nout,
                                    int64_t P, double *__restrict__ out, int64_t sd, int64_t sp,
                                    const int *__restrict__ run_if) {
    if (run_if && *run_if == 0) return;      // a predicated launch that is not wanted
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nout * P) return;
    const int64_t i = t / P, p = t - i * P;
    double s = 0.0;
    for (int64_t k = 0; k < S; ++k) s += part[k * nout * P + t];
    out[i * sd + p * sp] = s;
}

// Any dimension (0 or > 3), scalar field: one thread per point, CUDA sincos.
__global__ void generic_kernel(const double *__restrict__ cov, const double *__restrict__ z1,
                               const double *__restrict__ z2, const double *__restrict__ pos,
                               int64_t dim, int64_t N, int64_t P, double *__restrict__ out,
                               int64_t sp, const int *__restrict__ run_if) {
    if (run_if && *run_if == 0) return;      // a predicated launch that is not wanted
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double sum = 0.0;
    for (int64_t j = 0; j < N; ++j) {
        double ph = 0.0;
        for (int64_t d = 0; d < dim; ++d) ph = __dadd_rn(ph, __dmul_rn(cov[d * N + j], pos[d * P + p]));
        double sn, cs;
        sincos(ph, &sn, &cs);
        sum = __dadd_rn(sum, __dadd_rn(__dmul_rn(z1[j], cs), __dmul_rn(z2[j], sn)));
    }
    out[p * sp] = sum;
}

template <int D, int R, bool INC, bool LIBM>
int launch_main(dim3 grid, size_t smem, cudaStream_t st, const double *pos, int64_t P,
                const double2 *wtab, const double *rec, int64_t nc, int64_t mps, int accumulate,
                double *dst, int64_t sd, int64_t sp, int64_t split_stride, const int *run_if) {
    auto fn = plain_kernel<D, R, INC, LIBM>;
    GSC_TRY(smem_attr(reinterpret_cast<const void *>(fn), smem));   // once per device
    fn<<<grid, kThreads, smem, st>>>(pos, P, wtab, rec, nc, mps, accumulate, dst, sd, sp,
                                     split_stride, run_if);
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

template <int R, bool INC, bool LIBM>
int dispatch_dim(int64_t dim, dim3 grid, size_t smem, cudaStream_t st, const double *pos,
                 int64_t P, const double2 *wtab, const double *rec, int64_t nc, int64_t mps,
                 int accumulate, double *dst, int64_t sd, int64_t sp, int64_t split_stride,
                 const int *run_if = nullptr) {
    switch (dim) {
        case 1:
            if (!INC)
                return launch_main<1, R, INC, LIBM>(grid, smem, st, pos, P, wtab, rec, nc, mps,
                                                    accumulate, dst, sd, sp, split_stride, run_if);
            break;
        case 2:
            return launch_main<2, R, INC, LIBM>(grid, smem, st, pos, P, wtab, rec, nc, mps,
                                                accumulate, dst, sd, sp, split_stride, run_if);
        case 3:
            return launch_main<3, R, INC, LIBM>(grid, smem, st, pos, P, wtab, rec, nc, mps,
                                                accumulate, dst, sd, sp, split_stride, run_if);
    }
    return set_error(GSC_ERR_DIM, "unsupported dimension for the plain kernel");
}

int sm_count(int device) {
    static std::atomic<int> cached[64];   // zero-initialised (static storage)
    if (device >= 0 && device < 64) {
        const int c = cached[device].load(std::memory_order_relaxed);
        if (c) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0)
        n = 152;
    if (device >= 0 && device < 64) cached[device].store(n, std::memory_order_relaxed);
    return n;
}

__global__ void grid_expand_kernel(const double *__restrict__ a0, const double *__restrict__ a1,
                                   const double *__restrict__ a2, int64_t n0, int64_t n1,
                                   int64_t n2, int dim, double *__restrict__ pos) {
    const int64_t P = n0 * n1 * n2;
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int64_t i2 = p % n2, i01 = p / n2, i1 = i01 % n1, i0 = i01 / n1;
    if (dim == 2) {
        // (n0, n1) grid: p = i0 * n1 + i1 with n2 == 1
        pos[p] = a0[i0];
        pos[P + p] = a1[i1];
    } else {
        pos[p] = a0[i0];
        pos[P + p] = a1[i1];
        pos[2 * P + p] = a2[i2];
    }
}

// (nout, P) rows -> (P, nout) for the points [p0, p0 + n): each thread moves
// one point's nout values (coalesced reads per component; a warp's nout
// stores cover one contiguous run of 32 * nout values).
__global__ void interleave_kernel(const double *__restrict__ src, int nout, int64_t P, int64_t p0,
                                  int64_t n, double *__restrict__ dst) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p = p0 + i;
    for (int c = 0; c < nout; ++c) dst[p * nout + c] = src[c * P + p];
}

// Fourier method: the spectrum factor multiplies z1 cos + z2 sin of its mode
// (src/field.rs:241-242), so folding it into z1, z2 once per call lets every
// summator form compute the Fourier field unchanged.
__global__ void fourier_scale_kernel(const double *__restrict__ sf, const double *z1,
                                     const double *z2, int64_t n, double *z1s, double *z2s) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double f = sf[j], a = z1[j], b = z2[j];
    z1s[j] = __dmul_rn(f, a);
    z2s[j] = __dmul_rn(f, b);
}

}  // namespace

int fourier_scale(const double *sf, const double *z1, const double *z2, int64_t n, double *z1s,
                  double *z2s, cudaStream_t st) {
    if (n == 0) return GSC_OK;
    TimedLaunch tl(st);
    tl.begin(K_FOURIER_SCALE);
    fourier_scale_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(sf, z1, z2, n, z1s,
                                                                                z2s);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

int split_reduce(const double *part, int64_t S, int64_t nout, int64_t P, double *out, int64_t sd,
                 int64_t sp, cudaStream_t st) {
    TimedLaunch tl(st);
    tl.begin(K_SPLIT_REDUCE);
    const int64_t tot = nout * P;
    split_reduce_kernel<<<static_cast<unsigned>((tot + 255) / 256), 256, 0, st>>>(part, S, nout, P,
                                                                                 out, sd, sp, nullptr);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

int grid_expand(const double *const *axis, const int64_t *n, int64_t dim, double *pos,
                cudaStream_t st) {
    const int64_t n2 = dim == 3 ? n[2] : 1;
    const int64_t P = n[0] * n[1] * n2;
    if (P == 0) return GSC_OK;
    grid_expand_kernel<<<static_cast<unsigned>((P + 255) / 256), 256, 0, st>>>(
        axis[0], axis[1], dim == 3 ? axis[2] : nullptr, n[0], n[1], n2, static_cast<int>(dim), pos);
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

int interleave_rows(const double *src, int64_t nout, int64_t P, int64_t p0, int64_t p1,
                    double *dst, cudaStream_t st) {
    const int64_t n = p1 - p0;
    if (n <= 0) return GSC_OK;
    TimedLaunch tl(st);
    tl.begin(K_INTERLEAVE);
    interleave_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(
        src, static_cast<int>(nout), P, p0, n, dst);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

int plain_run(DeviceCtx &ctx, const PlainArgs &a, cudaStream_t st) {
    constexpr int R = 4;
    const int64_t P = a.n_points, N = a.n_modes, dim = a.dim;
    if (P == 0) return GSC_OK;
    const int64_t nout = a.incompr ? dim : 1;
    const bool libm = a.variant == 1;

    if (!a.incompr && (dim == 0 || dim > 3)) {
        TimedLaunch tl(st);
        tl.begin(K_GENERIC);
        const int tpb = 128;
        generic_kernel<<<static_cast<unsigned>((P + tpb - 1) / tpb), tpb, 0, st>>>(
            a.cov, a.z1, a.z2, a.pos, dim, N, P, a.out, a.out_sp, a.run_if);
        tl.end();
        GSC_CUDA(cudaGetLastError());
        return GSC_OK;
    }
    if (a.incompr && dim != 2 && dim != 3)
        return set_error(GSC_ERR_DIM, "Only two- and three-dimensional problems are supported.");

    // ---- launch geometry ---------------------------------------------------
    const int64_t pts_per_block = static_cast<int64_t>(kThreads) * R;
    const int64_t bx = (P + pts_per_block - 1) / pts_per_block;
    if (bx > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many points for one launch");
    const int64_t chunk = std::min<int64_t>(N, kChunkModes);
    const int64_t want_blocks = static_cast<int64_t>(sm_count(ctx.device)) * 6;
    int64_t S = std::max<int64_t>(1, (want_blocks + bx - 1) / bx);
    S = std::min<int64_t>(S, std::max<int64_t>(1, chunk / (2 * kTileModes)));
    S = std::min<int64_t>(S, 64);
    int64_t mps = chunk > 0 ? (chunk + S - 1) / S : 0;
    mps = (mps + kTileModes - 1) / kTileModes * kTileModes;
    if (mps > 0) S = std::max<int64_t>(1, (chunk + mps - 1) / mps);
    if (N == 0) S = 1;

    // ---- scratch: tables of one chunk, mode records, split partials --------
    const size_t tab_bytes = libm ? 0 : static_cast<size_t>(chunk) * kM * sizeof(double2);
    const size_t rec_bytes = static_cast<size_t>(chunk) * kRec * sizeof(double);
    const size_t part_bytes = S > 1 ? static_cast<size_t>(S) * nout * P * sizeof(double) : 0;
    const size_t off_rec = (tab_bytes + 255) / 256 * 256;
    const size_t off_part = off_rec + (rec_bytes + 255) / 256 * 256;
    GSC_TRY(ensure_dev(ctx, ctx.scratch, off_part + part_bytes + 256));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    unsigned char *sbase = static_cast<unsigned char *>(ctx.scratch.ptr);
    double2 *wtab = reinterpret_cast<double2 *>(sbase);
    double *rec = reinterpret_cast<double *>(sbase + off_rec);
    double *part = reinterpret_cast<double *>(sbase + off_part);

    double *dst = S > 1 ? part : a.out;
    const int64_t sd = S > 1 ? P : a.out_sd;
    const int64_t sp = S > 1 ? 1 : a.out_sp;
    const int64_t split_stride = S > 1 ? nout * P : 0;
    const size_t smem = 2 * ((libm ? 0 : kTileModes * kM * 16) + kTileModes * kRec * 8);
    const dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(S));

    int64_t j0 = 0;
    int first = 1;
    do {
        const int64_t nc = std::min<int64_t>(N - j0, kChunkModes);
        if (nc > 0) {
            TimedLaunch tl(st);
            tl.begin(K_MODE_TABLE);
            mode_table_kernel<<<static_cast<unsigned>(nc), kM, 0, st>>>(
                a.cov, a.z1, a.z2, dim, N, j0, a.incompr ? 1 : 0, libm ? 0 : 1, wtab, rec, a.run_if);
            tl.end();
            GSC_CUDA(cudaGetLastError());
        }
        const int64_t mps_c = nc > 0 ? std::min<int64_t>(mps, nc) : 0;
        const dim3 g(grid.x, static_cast<unsigned>(
                                 nc > 0 ? std::min<int64_t>(S, (nc + mps_c - 1) / mps_c) : 1));
        // on later chunks, splits past the end of a short chunk are not
        // launched and keep their sums
        const dim3 gl = first ? grid : g;
        TimedLaunch tl(st);
        tl.begin(a.incompr ? K_PLAIN_INCOMPR : (libm ? K_PLAIN_LIBM : K_PLAIN_SCALAR));
        int rc;
        if (a.incompr) {
            rc = libm ? dispatch_dim<R, true, true>(dim, gl, smem, st, a.pos, P, wtab, rec, nc,
                                                    mps_c, !first, dst, sd, sp, split_stride, a.run_if)
                      : dispatch_dim<R, true, false>(dim, gl, smem, st, a.pos, P, wtab, rec, nc,
                                                     mps_c, !first, dst, sd, sp, split_stride, a.run_if);
        } else {
            rc = libm ? dispatch_dim<R, false, true>(dim, gl, smem, st, a.pos, P, wtab, rec, nc,
                                                     mps_c, !first, dst, sd, sp, split_stride, a.run_if)
                      : dispatch_dim<R, false, false>(dim, gl, smem, st, a.pos, P, wtab, rec, nc,
                                                      mps_c, !first, dst, sd, sp, split_stride, a.run_if);
        }
        tl.end();
        if (rc != GSC_OK) return rc;
        first = 0;
        j0 += nc;
    } while (j0 < N);

    if (S > 1) {
        TimedLaunch tl(st);
        tl.begin(K_SPLIT_REDUCE);
        const int64_t tot = nout * P;
        split_reduce_kernel<<<static_cast<unsigned>((tot + 255) / 256), 256, 0, st>>>(
            part, S, nout, P, a.out, a.out_sd, a.out_sp, a.run_if);
        tl.end();
        GSC_CUDA(cudaGetLastError());
    }
    GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
    return GSC_OK;
}

// ---- batched ensembles: tables and the persistent kernel ---------------------
int batch_plain_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                       int64_t total_modes, void *wtab, double *rec, cudaStream_t st) {
    if (total_modes == 0) return GSC_OK;
    if (total_modes > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many modes in the batch");
    TimedLaunch tl(st);
    tl.begin(K_BATCH_TABLES);
    batch_table_kernel<<<static_cast<unsigned>(total_modes), kM, 0, st>>>(
        items, mode_prefix, n_items, static_cast<double2 *>(wtab), rec);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

size_t batch_plain_smem(int tile) { return 2 * static_cast<size_t>(tile) * (kM * 16 + kRec * 8); }

namespace {
using BatchPlainFn = void (*)(const BatchItem *, const BatchUnit *, int64_t, int *,
                              const double2 *, const double *);
BatchPlainFn batch_plain_fn(int R, int tile) {
    if (tile == 8) {
        if (R == 2) return batch_plain_kernel<2, 8>;
        if (R == 4) return batch_plain_kernel<4, 8>;
        if (R == 8) return batch_plain_kernel<8, 8>;
    } else if (tile == 16) {
        if (R == 2) return batch_plain_kernel<2, 16>;
        if (R == 4) return batch_plain_kernel<4, 16>;
    }
    return nullptr;
}
int configure_batch_plain(BatchPlainFn fn, int tile) {
    return smem_attr(reinterpret_cast<const void *>(fn), batch_plain_smem(tile));   // per device
}
}  // namespace

bool batch_plain_config_ok(int R, int tile) { return batch_plain_fn(R, tile) != nullptr; }

int batch_plain_occupancy(int R, int tile, int device) {
    BatchPlainFn fn = batch_plain_fn(R, tile);
    if (!fn) return 0;
    if (configure_batch_plain(fn, tile) != GSC_OK) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kThreads, batch_plain_smem(tile)) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    (void)device;
    return n;
}

int batch_plain_launch(int R, int tile, int blocks, const BatchItem *items,
                       const BatchUnit *units, int64_t n_units, int *counter, const void *wtab,
                       const double *rec, cudaStream_t st) {
    BatchPlainFn fn = batch_plain_fn(R, tile);
    if (!fn) return set_error(GSC_ERR_INVALID, "unsupported batch configuration");
    GSC_TRY(configure_batch_plain(fn, tile));
    TimedLaunch tl(st);
    tl.begin(K_BATCH_PLAIN);
    fn<<<blocks, kThreads, batch_plain_smem(tile), st>>>(items, units, n_units, counter,
                                                         static_cast<const double2 *>(wtab), rec);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

}  // namespace gsc

// ---------------------------------------------------------------------------
// Allocation-free variant of the scalar FP64 summator.
//
// Some callers must not let a library allocate device memory: a host whose
// framework allocator already owns the whole device (a cudaMalloc from the
// library would fail or fragment that pool), a real-time loop that cannot
// afford to block in the driver's allocator, or a plug-in host that only
// permits memory from its own arena.  For them the per-mode tables of the
// plain kernel live in one fixed array compiled into the library, so a call
// allocates nothing; the caller passes the inputs and the output as usual.
//
// The array (4 MiB of tables + 96 KiB of mode records, enough for 1024
// modes) is held on every GPU that loads the library until the process
// exits.  All calls share it and it keeps the last call's contents; every
// call rewrites the part it reads, so nothing has to start at zero.  Calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) race on the array.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char
    gsc_noalloc_scratch[gsc::kNoAllocModes *
                        (gsc::kPlainTableBytesPerMode + gsc::kPlainRecBytesPerMode)];

namespace gsc {

// the array is sliced below as kNoAllocModes tables of kM double2 followed by
// kNoAllocModes records of kRec doubles: its size must follow those constants
static_assert(kPlainTableBytesPerMode == kM * sizeof(double2) &&
                  kPlainRecBytesPerMode == kRec * sizeof(double),
              "the fixed table array is sized from the plain kernel's per-mode layout");
static_assert(sizeof(gsc_noalloc_scratch) ==
                  kNoAllocModes * (kM * sizeof(double2) + kRec * sizeof(double)),
              "fixed table array size");

static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[64] = {nullptr};

// The device address of the fixed array on the current device, looked up
// once per device.  Host code cannot use the array's name as a device
// address: outside device code it names a host-side stand-in.
static int noalloc_address(int device, void **addr) {
    if (device < 0 || device >= 64) return set_error(GSC_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, gsc_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(fixed table array)");
        g_noalloc_addr[device] = p;
    }
    *addr = g_noalloc_addr[device];
    return GSC_OK;
}

int plain_noalloc_run(int device, const PlainArgs &a, cudaStream_t st) {
    constexpr int R = 4;
    const int64_t P = a.n_points, N = a.n_modes;
    if (N > kNoAllocModes)
        return set_error(GSC_ERR_INVALID, "gsc_summate_dev_noalloc takes at most " +
                                              std::to_string(kNoAllocModes) +
                                              " modes per call (its fixed table array holds "
                                              "that many); split the modes over several calls "
                                              "or use gsc_summate_dev");
    if (P == 0) return GSC_OK;
    void *scratch = nullptr;
    GSC_TRY(noalloc_address(device, &scratch));
    double2 *wtab = static_cast<double2 *>(scratch);
    double *rec = reinterpret_cast<double *>(static_cast<unsigned char *>(scratch) +
                                             kNoAllocModes * kM * sizeof(double2));
    const int64_t bx = (P + kThreads * R - 1) / (kThreads * R);
    if (bx > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many points for one launch");
    if (N > 0) {
        mode_table_kernel<<<static_cast<unsigned>(N), kM, 0, st>>>(a.cov, a.z1, a.z2, a.dim, N, 0,
                                                                      0, 1, wtab, rec, nullptr);
        GSC_CUDA(cudaGetLastError());
    }
    const size_t smem = 2 * (kTileModes * kM * 16 + kTileModes * kRec * 8);
    // one mode split: every point's modes are summed by one thread, in order
    return dispatch_dim<R, false, false>(a.dim, dim3(static_cast<unsigned>(bx), 1), smem, st,
                                         a.pos, P, wtab, rec, N, N, 0, a.out, P, a.out_sp, 0);
}

}  // namespace gsc
