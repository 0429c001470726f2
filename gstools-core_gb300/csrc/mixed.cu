// mixed.cu -- mixed-precision summators for unstructured points (sm_103a).
//
// Same sums as plain.cu (reference src/field.rs:37-65 and :97-182) for points
// without grid structure, where no tensor-core factorisation exists and every
// point*mode needs its own phase and sincos.  GB300 executes FP64 at 1/64 of
// the FP32 rate (1.89 vs 119 FMA per clock per SM), so this form keeps FP64
// accuracy only where it is needed and spends FP32 instructions:
//
//  * phase in turns, theta = kappa.x with kappa = k / 2pi, in double-float
//    (FP32 pairs): kappa = kh + kl per mode, x = xh + xl per point (48
//    significant bits each); per dimension p = kh*xh is split exactly into
//    p (rounded) and fma(kh, xh, -p), the integer turns rint(p) are dropped
//    exactly, and the small terms kh*xl + kl*xh are added in FP32.  The
//    reduced phase is accurate to |theta| * 2^-46 turns (2^-29 turns at
//    |k.x| = 1e6, where a plain FP32 product keeps no fraction at all) while
//    every dimension's product is at least one turn; where one is smaller,
//    the FP32 sum of the dimensions' fractions rounds at the total's ulp,
//    up to 2^-24 turns (3.7e-7 rad).  FP64 would spend 9 FP64 instructions
//    per point*mode here;
//  * sincos(2 pi theta): quadrant by rounding 4 theta, then sin/cos of
//    2 pi f, |f| <= 1/8, by polynomials fitted for this kernel (FP32
//    coefficients, max error 8.6e-8 / 5.8e-8 over the interval), corrected
//    to first order for the low part of the phase;
//  * z1 cos + z2 sin accumulated in FP32 over tiles of 32 modes with Kahan
//    compensation (plain FP32 sums alone reached 1.0e-6 of the field RMS on a
//    300-mode 1-D case), each tile folded into a double-float (TwoSum)
//    running total, converted to FP64 at the end: the compensated sum across
//    tiles is as accurate as FP64.
//
// The "mixed_f64phase" variant forms the phase and its reduction in FP64
// (the literal recipe: 5 FP64 instructions per point*mode) and shares the
// rest; it exists to measure what the double-float phase buys.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "dfturns.cuh"
#include "internal.h"

namespace gsc {
namespace {

constexpr int kMxThreads = 128;
static_assert(kMxThreads == kBatchThreads, "batch units assume the mixed block size");
constexpr int kMxR = 4;              // points per thread
constexpr int kMxTile = 32;          // modes per FP32 accumulation tile
// floats per mode: kh0 kh1 kh2 kl0 kl1 kl2 z1 z2 w0 w1 w2 - | (a_q, b_q), q = 0..3:
// the weights rotated by q quarter turns, z1 cos(t + q pi/2) + z2 sin(t + q pi/2)
// = a_q cos t + b_q sin t: (z1, z2), (z2, -z1), (-z1, -z2), (-z2, z1)
constexpr int kMxRec = 20;
constexpr int kMxRot = 12;           // offset of the rotated pairs
constexpr int kMxRec64 = 4;          // doubles per mode (FP64-phase variant): kappa0..2, -

__device__ __forceinline__ void mixed_mode_entry(const double *__restrict__ cov, double z1j,
                                                 double z2j, int64_t dim, int64_t n_modes,
                                                 int64_t j, int incompr, float *__restrict__ r,
                                                 double *__restrict__ r64) {
    double k[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < dim && d < 3; ++d) k[d] = cov[d * n_modes + j];
    for (int d = 0; d < 3; ++d) {
        const double kap = k[d] * kInv2Pi;
        const float hi = __double2float_rn(kap);
        r[d] = hi;
        r[3 + d] = __double2float_rn(kap - static_cast<double>(hi));
        r64[d] = kap;
    }
    r64[3] = 0.0;
    const float z1f = __double2float_rn(z1j), z2f = __double2float_rn(z2j);
    r[6] = z1f;
    r[7] = z2f;
    r[kMxRot + 0] = z1f;
    r[kMxRot + 1] = z2f;
    r[kMxRot + 2] = z2f;
    r[kMxRot + 3] = -z1f;
    r[kMxRot + 4] = -z1f;
    r[kMxRot + 5] = -z2f;
    r[kMxRot + 6] = -z2f;
    r[kMxRot + 7] = z1f;
    double w0 = 0.0, w1 = 0.0, w2 = 0.0;
    if (incompr) {   // projector as the reference forms it (src/field.rs:138-152)
        double kk = 0.0;
        for (int d = 0; d < dim; ++d) kk = __dadd_rn(kk, __dmul_rn(k[d], k[d]));
        const double k_2 = __ddiv_rn(k[0], kk);
        w0 = __dadd_rn(1.0, -__dmul_rn(k[0], k_2));
        w1 = -__dmul_rn(k[1], k_2);
        w2 = -__dmul_rn(k[2], k_2);
    }
    r[8] = __double2float_rn(w0);
    r[9] = __double2float_rn(w1);
    r[10] = __double2float_rn(w2);
    r[11] = 0.f;
}

__global__ void mixed_mode_kernel(const double *__restrict__ cov, const double *__restrict__ z1,
                                  const double *__restrict__ z2, int64_t dim, int64_t n_modes,
                                  int64_t j0, int64_t nc, int incompr, float *__restrict__ rec,
                                  double *__restrict__ rec64) {
    const int64_t jl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (jl >= nc) return;
    const int64_t j = j0 + jl;
    mixed_mode_entry(cov, z1[j], z2[j], dim, n_modes, j, incompr, rec + jl * kMxRec,
                     rec64 + jl * kMxRec64);
}

// Records of every item of a batch, one thread per mode (Fourier factor
// folded into z1, z2 first).
__global__ void batch_mixed_table_kernel(const BatchItem *__restrict__ items,
                                         const int64_t *__restrict__ prefix, int64_t n_items,
                                         int64_t total, float *__restrict__ rec,
                                         double *__restrict__ rec64) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int64_t lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const BatchItem &it = items[lo];
    const int64_t j = g - it.mode_off;
    double z1j = it.z1[j], z2j = it.z2[j];
    if (it.sf) {
        const double f = it.sf[j];
        z1j = __dmul_rn(f, z1j);
        z2j = __dmul_rn(f, z2j);
    }
    mixed_mode_entry(it.cov, z1j, z2j, it.dim, it.n_modes, j, it.incompr, rec + g * kMxRec,
                     rec64 + g * kMxRec64);
}

// (z1 cos + z2 sin)(2 pi (th + tl)), th in [-1/2, 1/2] turns, tl tiny:
// quadrant q by rounding 4 th, f = th - q/4 (exact, |f| <= 1/8), sin(2 pi f)
// = f S(f^2), cos(2 pi f) = C(f^2), first-order correction for tl; the
// rotation by q quarter turns is taken from the mode's rotated weight pairs
// `ab` (indexed by q mod 4) instead of permuting and negating sin and cos.
__device__ __forceinline__ float mixed_term(float th, float tl, const float2 *ab) {
    float s1, c1;
    const int qi = sincos_turns_reduced(th, tl, s1, c1);    // low bits: q mod 4
    const float2 w = ab[qi & 3];
    return fmaf(w.x, c1, w.y * s1);
}

// Kahan step: (sum, cmp) += a, cmp holding minus the lost low-order part
__device__ __forceinline__ void kahan_add(float &sum, float &cmp, float a) {
    const float y = a - cmp;
    const float t = sum + y;
    cmp = (t - sum) - y;
    sum = t;
}

// Knuth's TwoSum: (hi, lo) += a
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float a) {
    const float s = hi + a;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (a - bb);
    hi = s;
    lo += e;
}

// One block's work: the kMxThreads*R points from p_first (thread t owns
// p_first + t + r*kMxThreads), modes [jb, je) of the records `rec`, `rec64`;
// sums written (accumulate=0) or added at dst + i*sd + p*sp.  srec / srec64
// are shared-memory staging areas of kMxTile records.
template <int D, int R, bool INC, bool F64P>
__device__ __forceinline__ void mixed_block(const double *__restrict__ pos, int64_t P,
                                            int64_t p_first, const float *__restrict__ rec,
                                            const double *__restrict__ rec64, int64_t jb,
                                            int64_t je, int accumulate, double *__restrict__ dst,
                                            int64_t sd, int64_t sp, float *srec, double *srec64) {
    constexpr int NOUT = INC ? D : 1;
    constexpr int kMxR = R;
    const int tid = threadIdx.x;
    const int64_t p0 = p_first + tid;

    float xh[kMxR][D], xl[kMxR][D];
    double xd[kMxR][D];
    float hi[kMxR][NOUT], lo[kMxR][NOUT];
#pragma unroll
    for (int r = 0; r < kMxR; ++r) {
        const int64_t p = p0 + r * kMxThreads;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double x = p < P ? pos[d * P + p] : 0.0;
            xd[r][d] = x;
            xh[r][d] = __double2float_rn(x);
            xl[r][d] = __double2float_rn(x - static_cast<double>(xh[r][d]));
        }
#pragma unroll
        for (int i = 0; i < NOUT; ++i) hi[r][i] = lo[r][i] = 0.f;
    }

    for (int64_t t0 = jb; t0 < je; t0 += kMxTile) {
        const int tm = static_cast<int>(min(static_cast<int64_t>(kMxTile), je - t0));
        __syncthreads();
        for (int i = tid; i < tm * kMxRec; i += kMxThreads) srec[i] = rec[t0 * kMxRec + i];
        if (F64P)
            for (int i = tid; i < tm * kMxRec64; i += kMxThreads) srec64[i] = rec64[t0 * kMxRec64 + i];
        __syncthreads();
        float acc[kMxR][NOUT], cmp[kMxR][NOUT];
#pragma unroll
        for (int r = 0; r < kMxR; ++r)
#pragma unroll
            for (int i = 0; i < NOUT; ++i) acc[r][i] = cmp[r][i] = 0.f;
        for (int m = 0; m < tm; ++m) {
            const float *mr = srec + m * kMxRec;
            const float2 *ab = reinterpret_cast<const float2 *>(mr + kMxRot);
            float w[3] = {mr[8], mr[9], mr[10]};
#pragma unroll
            for (int r = 0; r < kMxR; ++r) {
                float th, tl;
                if (F64P) {
                    const double *kr = srec64 + m * kMxRec64;
                    double t = kr[0] * xd[r][0];
                    if (D > 1) t = fma(kr[1], xd[r][1], t);
                    if (D > 2) t = fma(kr[2], xd[r][2], t);
                    t -= rint(t);
                    th = __double2float_rn(t);
                    tl = 0.f;
                } else {
                    float a = 0.f, b = 0.f;
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const float kh = mr[d], kl = mr[3 + d];
                        const float pr = kh * xh[r][d];
                        const float e = fmaf(kh, xh[r][d], -pr);      // exact
                        a += pr - rintf(pr);   // fraction exact; the sum rounds below 1 turn
                        b = fmaf(kh, xl[r][d], fmaf(kl, xh[r][d], e + b));
                    }
                    const float a2 = a - rintf(a);
                    th = a2 + b;
                    tl = b - (th - a2);
                }
                const float z12 = mixed_term(th, tl, ab);
                if (INC) {
#pragma unroll
                    for (int i = 0; i < NOUT; ++i) kahan_add(acc[r][i], cmp[r][i], w[i] * z12);
                } else {
                    kahan_add(acc[r][0], cmp[r][0], z12);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kMxR; ++r)
#pragma unroll
            for (int i = 0; i < NOUT; ++i) {
                two_sum_add(hi[r][i], lo[r][i], acc[r][i]);
                lo[r][i] -= cmp[r][i];
            }
    }

    double *d0 = dst;
#pragma unroll
    for (int r = 0; r < kMxR; ++r) {
        const int64_t p = p0 + r * kMxThreads;
        if (p >= P) continue;
#pragma unroll
        for (int i = 0; i < NOUT; ++i) {
            const double v = static_cast<double>(hi[r][i]) + static_cast<double>(lo[r][i]);
            double *o = d0 + i * sd + p * sp;
            *o = accumulate ? *o + v : v;
        }
    }
}

// Four resident blocks per SM: the register budget this leaves (up to 128)
// lets the compiler interleave the R points' FP32 chains; the default budget
// (72 registers, 7 blocks) ran 30% slower on 16.7M points x 4096 modes.
template <int D, bool INC, bool F64P>
__global__ void __launch_bounds__(kMxThreads, 4)
mixed_kernel(const double *__restrict__ pos, int64_t P, const float *__restrict__ rec,
             const double *__restrict__ rec64, int64_t nc, int64_t mps, int accumulate,
             double *__restrict__ dst, int64_t sd, int64_t sp, int64_t split_stride) {
    __shared__ __align__(16) float srec[kMxTile * kMxRec];
    __shared__ __align__(16) double srec64[F64P ? kMxTile * kMxRec64 : 1];
    const int64_t jb = static_cast<int64_t>(blockIdx.y) * mps;
    const int64_t je = min(nc, jb + mps);
    mixed_block<D, kMxR, INC, F64P>(pos, P, static_cast<int64_t>(blockIdx.x) * (kMxThreads * kMxR),
                                    rec, rec64, jb, je, accumulate,
                                    dst + static_cast<int64_t>(blockIdx.y) * split_stride, sd, sp,
                                    srec, srec64);
}

// Persistent batch kernel (see batch_plain_kernel in plain.cu).
template <int R, bool F64P>
__global__ void __launch_bounds__(kMxThreads)
batch_mixed_kernel(const BatchItem *__restrict__ items, const BatchUnit *__restrict__ units,
                   int64_t n_units, int *__restrict__ counter, const float *__restrict__ rec,
                   const double *__restrict__ rec64) {
    __shared__ __align__(16) float srec[kMxTile * kMxRec];
    __shared__ __align__(16) double srec64[F64P ? kMxTile * kMxRec64 : 1];
    __shared__ int s_unit;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1);
        __syncthreads();
        const int64_t u = s_unit;
        if (u >= n_units) break;
        const BatchUnit w = units[u];
        const BatchItem &it = items[w.item];
        const int64_t P = it.n_points;
        const int64_t nout = it.incompr ? it.dim : 1;
        double *dst = it.splits > 1 ? it.part + static_cast<int64_t>(w.split) * nout * P : it.out;
        const float *rc = rec + it.mode_off * kMxRec;
        const double *rc64 = rec64 + it.mode_off * kMxRec64;
        switch (it.dim * 2 + it.incompr) {
            case 2:
                mixed_block<1, R, false, F64P>(it.pos, P, w.p_first, rc, rc64, w.jb, w.je, 0, dst,
                                               P, 1, srec, srec64);
                break;
            case 4:
                mixed_block<2, R, false, F64P>(it.pos, P, w.p_first, rc, rc64, w.jb, w.je, 0, dst,
                                               P, 1, srec, srec64);
                break;
            case 5:
                mixed_block<2, R, true, F64P>(it.pos, P, w.p_first, rc, rc64, w.jb, w.je, 0, dst,
                                              P, 1, srec, srec64);
                break;
            case 6:
                mixed_block<3, R, false, F64P>(it.pos, P, w.p_first, rc, rc64, w.jb, w.je, 0, dst,
                                               P, 1, srec, srec64);
                break;
            case 7:
                mixed_block<3, R, true, F64P>(it.pos, P, w.p_first, rc, rc64, w.jb, w.je, 0, dst,
                                              P, 1, srec, srec64);
                break;
            default:
                break;
        }
    }
}

template <int D, bool INC, bool F64P>
int launch_mixed(dim3 grid, cudaStream_t st, const double *pos, int64_t P, const float *rec,
                 const double *rec64, int64_t nc, int64_t mps, int accumulate, double *dst,
                 int64_t sd, int64_t sp, int64_t split_stride) {
    mixed_kernel<D, INC, F64P><<<grid, kMxThreads, 0, st>>>(pos, P, rec, rec64, nc, mps, accumulate,
                                                             dst, sd, sp, split_stride);
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

template <bool INC, bool F64P>
int dispatch_mixed(int64_t dim, dim3 grid, cudaStream_t st, const double *pos, int64_t P,
                   const float *rec, const double *rec64, int64_t nc, int64_t mps, int accumulate,
                   double *dst, int64_t sd, int64_t sp, int64_t split_stride) {
    switch (dim) {
        case 1:
            if (!INC)
                return launch_mixed<1, INC, F64P>(grid, st, pos, P, rec, rec64, nc, mps, accumulate,
                                                  dst, sd, sp, split_stride);
            break;
        case 2:
            return launch_mixed<2, INC, F64P>(grid, st, pos, P, rec, rec64, nc, mps, accumulate,
                                              dst, sd, sp, split_stride);
        case 3:
            return launch_mixed<3, INC, F64P>(grid, st, pos, P, rec, rec64, nc, mps, accumulate,
                                              dst, sd, sp, split_stride);
    }
    return set_error(GSC_ERR_DIM, "the mixed form supports dimensions 1, 2, 3 (incompressible: 2, 3)");
}

int mx_sm_count(int device) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0)
        n = 152;
    return n;
}

}  // namespace

int mixed_run(DeviceCtx &ctx, const PlainArgs &a, bool f64phase, cudaStream_t st) {
    // the double-float phase of GSC_FORM_MIXED became mixed_fx.cu's integer phase
    if (!f64phase) return mixed_fx_run(ctx, a, nullptr, st);
    const int64_t P = a.n_points, N = a.n_modes, dim = a.dim;
    if (P == 0) return GSC_OK;
    const int64_t nout = a.incompr ? dim : 1;
    if (dim < 1 || dim > 3 || (a.incompr && dim == 1))
        return set_error(GSC_ERR_DIM, "the mixed form supports dimensions 1, 2, 3 (incompressible: 2, 3)");
    constexpr int64_t kChunk = 1 << 20;   // modes per record build
    const int64_t pts_per_block = static_cast<int64_t>(kMxThreads) * kMxR;
    const int64_t bx = (P + pts_per_block - 1) / pts_per_block;
    if (bx > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many points for one launch");
    const int64_t chunk = std::min<int64_t>(N, kChunk);
    const int64_t want_blocks = static_cast<int64_t>(mx_sm_count(ctx.device)) * 8;
    int64_t S = std::max<int64_t>(1, (want_blocks + bx - 1) / bx);
    S = std::min<int64_t>(S, std::max<int64_t>(1, chunk / (2 * kMxTile)));
    S = std::min<int64_t>(S, 64);
    int64_t mps = chunk > 0 ? (chunk + S - 1) / S : 0;
    mps = (mps + kMxTile - 1) / kMxTile * kMxTile;
    if (mps > 0) S = std::max<int64_t>(1, (chunk + mps - 1) / mps);
    if (N == 0) S = 1;

    const size_t rec_bytes = static_cast<size_t>(chunk) * kMxRec * sizeof(float);
    const size_t rec64_bytes = static_cast<size_t>(chunk) * kMxRec64 * sizeof(double);
    const size_t part_bytes = S > 1 ? static_cast<size_t>(S) * nout * P * sizeof(double) : 0;
    const size_t off_rec64 = (rec_bytes + 255) / 256 * 256;
    const size_t off_part = off_rec64 + (rec64_bytes + 255) / 256 * 256;
    GSC_TRY(ensure_dev(ctx, ctx.scratch, off_part + part_bytes + 256));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    unsigned char *sbase = static_cast<unsigned char *>(ctx.scratch.ptr);
    float *rec = reinterpret_cast<float *>(sbase);
    double *rec64 = reinterpret_cast<double *>(sbase + off_rec64);
    double *part = reinterpret_cast<double *>(sbase + off_part);

    double *dst = S > 1 ? part : a.out;
    const int64_t sd = S > 1 ? P : a.out_sd;
    const int64_t sp = S > 1 ? 1 : a.out_sp;
    const int64_t split_stride = S > 1 ? nout * P : 0;
    const dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(S));

    int64_t j0 = 0;
    int first = 1;
    do {
        const int64_t nc = std::min<int64_t>(N - j0, kChunk);
        if (nc > 0) {
            TimedLaunch tl(st);
            tl.begin(K_MIXED_MODES);
            mixed_mode_kernel<<<static_cast<unsigned>((nc + 127) / 128), 128, 0, st>>>(
                a.cov, a.z1, a.z2, dim, N, j0, nc, a.incompr ? 1 : 0, rec, rec64);
            tl.end();
            GSC_CUDA(cudaGetLastError());
        }
        const int64_t mps_c = nc > 0 ? std::min<int64_t>(mps, nc) : 0;
        const dim3 g(grid.x, static_cast<unsigned>(
                                 nc > 0 ? std::min<int64_t>(S, (nc + mps_c - 1) / mps_c) : 1));
        const dim3 gl = first ? grid : g;
        TimedLaunch tl(st);
        tl.begin(K_MIXED_F64PHASE);
        int rc;
        if (a.incompr)
            rc = dispatch_mixed<true, true>(dim, gl, st, a.pos, P, rec, rec64, nc, mps_c, !first,
                                            dst, sd, sp, split_stride);
        else
            rc = dispatch_mixed<false, true>(dim, gl, st, a.pos, P, rec, rec64, nc, mps_c, !first,
                                             dst, sd, sp, split_stride);
        tl.end();
        if (rc != GSC_OK) return rc;
        first = 0;
        j0 += nc;
    } while (j0 < N);

    if (S > 1) GSC_TRY(split_reduce(part, S, nout, P, a.out, a.out_sd, a.out_sp, st));
    GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
    return GSC_OK;
}

// ---- batched ensembles ----------------------------------------------------------
int batch_mixed_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                       int64_t total_modes, float *rec, double *rec64, cudaStream_t st) {
    if (total_modes == 0) return GSC_OK;
    TimedLaunch tl(st);
    tl.begin(K_BATCH_TABLES);
    batch_mixed_table_kernel<<<static_cast<unsigned>((total_modes + 127) / 128), 128, 0, st>>>(
        items, mode_prefix, n_items, total_modes, rec, rec64);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

namespace {
using BatchMixedFn = void (*)(const BatchItem *, const BatchUnit *, int64_t, int *, const float *,
                              const double *);
// the FP64-phase variant only: GSC_FORM_MIXED batches run mixed_fx.cu's kernel
BatchMixedFn batch_mixed_fn(int R, bool f64p) {
    if (!f64p) return nullptr;
    if (R == 2) return batch_mixed_kernel<2, true>;
    if (R == 4) return batch_mixed_kernel<4, true>;
    if (R == 8) return batch_mixed_kernel<8, true>;
    return nullptr;
}
}  // namespace

bool batch_mixed_config_ok(int R) { return batch_mixed_fn(R, true) != nullptr; }

int batch_mixed_occupancy(int R, bool f64phase, int device) {
    BatchMixedFn fn = batch_mixed_fn(R, f64phase);
    if (!fn) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kMxThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    (void)device;
    return n;
}

int batch_mixed_launch(int R, bool f64phase, int blocks, const BatchItem *items,
                       const BatchUnit *units, int64_t n_units, int *counter, const float *rec,
                       const double *rec64, cudaStream_t st) {
    BatchMixedFn fn = batch_mixed_fn(R, f64phase);
    if (!fn) return set_error(GSC_ERR_INVALID, "unsupported batch configuration");
    TimedLaunch tl(st);
    tl.begin(K_BATCH_MIXED);
    fn<<<blocks, kMxThreads, 0, st>>>(items, units, n_units, counter, rec, rec64);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

}  // namespace gsc
