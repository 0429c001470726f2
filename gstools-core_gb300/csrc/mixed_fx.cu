// mixed_fx.cu -- the mixed-precision summators for unstructured points
// (form GSC_FORM_MIXED), sm_103a.
//
// Same sums as plain.cu (reference src/field.rs:37-65 and :97-182) for points
// without grid structure, where no tensor-core factorisation exists and every
// point*mode needs its own phase.  GB300 runs FP64 at 1/64 of the FP32
// rate, so the phase is formed in 32-bit integer arithmetic, where a product
// modulo 2^32 drops whole turns for free:
//
//  * phase in units of 2^-32 turn.  Per call and dimension d, positions are
//    taken as 61-bit fixed-point integers X = rint(x * 2^s_d) + 2^60 (s_d
//    from the largest |x_d|: exact for every FP64 coordinate below 2^53
//    units), split X = Xh 2^29 + Xl.  Per mode, B = kappa_d 2^(61 - s_d)
//    (kappa = k / 2 pi turns per unit) is held as BI + BF 2^-32.  Then
//      theta = sum_d  BI Xh + hi32(BF Xh) + hi32(BI * 8 Xl)   (mod 2^32)
//    is kappa.x (plus a per-mode constant folded into the table below) to
//    within 3 units per dimension (1.3e-8 rad for three dimensions, at any
//    |k.x| below 2^30 turns): three 32-bit integer multiply-adds per
//    dimension, where a double-float product takes eight FP32 instructions
//    and an FP64 one 1/64 of the pipe.  BI is stored biased by 2^31, so
//    both high products are unsigned; the bias's effect is a per-point
//    constant taken out once per point.  When every mode of a call (or batch
//    item) has |BI| < 2^20, sum_d BI Xl 2^-29 is one chain of FP32 fused
//    multiply-adds instead (the high products issue at a quarter of the
//    FP32 rate);
//  * e^{i theta}: theta + 2^27 + 16 selects by its top 4 bits one of 16
//    entries of the mode's table T[m] = (z1 - i z2) e^{2 pi i (m/16 - phi)}
//    (phi the per-mode constant; built in FP64 per mode, stored as FP32).
//    Bits 5..27 of the same word, placed under the exponent of 1.0f, give
//    1 + u 2^-23 exactly; minus 1.5 that is the remainder r in sixteenths
//    of a turn (|r| <= 1/2, rounded to 2^-27 turn by the + 16) with no
//    integer-to-float conversion.  sin and cos of r pi/8 are minimax
//    polynomials of degree 5 and 4 in r (within 6e-9), and the term is
//    Re(T e^{i r pi/8});
//  * the terms of eight modes are added (four pair sums), and the group sums
//    are summed in FP32 over tiles of 128 modes with Kahan compensation; each
//    tile is folded into a double-float (TwoSum) running total, converted to
//    FP64 at the end.
// Phases beyond 2^30 turns (|k| * max|x| > 6.7e9) do not fit the integer
// range; such calls are flagged in the range word (the caller recomputes them
// on the FP64 kernel or reports it).  Non-finite coordinates give NaN, as the
// reference does.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "dfturns.cuh"
#include "internal.h"

namespace gsc {
namespace {

constexpr int kFxThreads = 128;
static_assert(kFxThreads == kBatchThreads, "batch units assume the block size");
constexpr int kFxR = 4;                 // points per thread when untuned
constexpr int kFxW = 8;                 // target blocks per SM when untuned
constexpr int kFxTile = 128;            // modes per staged tile = accumulation tile (largest)
constexpr int kFxSplitModes = 64;       // mode splits are multiples of this
// 32-bit words per mode: [0..2] BI' (BI + 2^31), [3] w0, [4..6] BF, [7] w1,
// [8] w2 (projector weights of the incompressible field, FP32), [9..11] BI
// as FP32, [32..63] the table T[m] as (re, im) FP32 pairs; words 12..31 are
// unused.  A record is
// 256 bytes and the tile of records in shared memory 256-byte aligned, so
// a table starts on a 128-byte boundary (its entry's address is one OR) and
// its 16 entries fill the 32 shared-memory banks once: a warp's gather from
// them is free of bank conflicts.
constexpr int kFxTab = 32;
constexpr int kFxRecWords = 64;
static_assert(kFxRecWords * 4 == kFxRecBytesPerMode, "record layout");
// sin(r pi/8) = r (S1 + r^2 (S3 + r^2 S5)), cos(r pi/8) = C0 + r^2 (C2 + r^2
// C4) for r in sixteenths of a turn, |r| <= 1/2: minimax (Remez exchange on
// r^2 in [0, 1/4], absolute error) fits, rounded to FP32; with the rounded
// coefficients both stay within 6e-9 of sin and cos
constexpr float kFxS1 = 0.39269909262657166f, kFxS3 = -0.01009317860007286f,
                kFxS5 = 7.771774107823148e-05f;
constexpr float kFxC0 = 1.0f, kFxC2 = -0.07710610330104828f, kFxC4 = 0.000988987972959876f;
// 1.5 2^23: an FP32 sum that stays within 2^22 of it has ulp 1, and the
// integer it rounds to is its bit pattern minus 0x4B400000
constexpr float kFxMagic = 12582912.0f;
constexpr uint32_t kFxMagicBits = 0x4B400000u;
// the FP32 product form needs |BI| < 2^20 in every dimension (the sum of
// three products stays within 2^22 of the magic constant)
constexpr int32_t kFxSmallBI = 1 << 20;

// cos(2 pi m / 16), m = 0..15, to FP64 rounding (from cos(pi/8) =
// sqrt(2 + sqrt 2) / 2 and cos(pi/4) = sqrt(2) / 2)
__constant__ double kSixteenthCos[16] = {
    1.0, 0.9238795325112867, 0.7071067811865476, 0.38268343236508984,
    0.0, -0.38268343236508984, -0.7071067811865476, -0.9238795325112867,
    -1.0, -0.9238795325112867, -0.7071067811865476, -0.38268343236508984,
    0.0, 0.38268343236508984, 0.7071067811865476, 0.9238795325112867};

// Fixed-point scale s_d of dimension d from the largest finite |x_d|
// (bits of that non-negative double, 0 when none): |x| * 2^s < 2^60.
__device__ __forceinline__ int fx_scale(unsigned long long maxbits) {
    // e with m in [2^(e-1), 2^e): from the exponent field when m is normal
    // (what frexp returns), frexp itself for a subnormal m
    const int biased = static_cast<int>(maxbits >> 52);
    int e = 0;
    if (biased != 0) e = biased - 1022;
    else if (maxbits != 0ull) frexp(__longlong_as_double(static_cast<long long>(maxbits)), &e);
    return 60 - e;
}

// x 2^q, as ldexp(x, q) returns it (both round once, to nearest): a product
// with the power of two where that is a normal double
__device__ __forceinline__ double fx_ldexp(double x, int q) {
    if (q >= -1022 && q <= 1023)
        return x * __longlong_as_double(static_cast<long long>(q + 1023) << 52);
    return ldexp(x, q);
}

// Largest finite |x_d| of pos (dim, P) into maxbits[d] (as the bit pattern
// of a non-negative double, which orders like the value); maxbits zeroed
// before.  One warp-level reduction, then one atomic per warp and dimension.
__device__ __forceinline__ void fx_range_part(const double *__restrict__ pos, int64_t P, int dim,
                                              int64_t i0, int64_t stride,
                                              unsigned long long *maxbits) {
    unsigned long long m[3] = {0ull, 0ull, 0ull};
    for (int64_t i = i0; i < P; i += stride)
        for (int d = 0; d < dim && d < 3; ++d) {
            // |x| as bits (sign cleared), kept when finite
            const unsigned long long v =
                static_cast<unsigned long long>(__double_as_longlong(pos[d * P + i])) &
                0x7fffffffffffffffull;
            if (v < 0x7ff0000000000000ull) m[d] = max(m[d], v);
        }
    for (int d = 0; d < dim && d < 3; ++d) {
        unsigned long long v = m[d];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31) == 0 && v) atomicMax(maxbits + d, v);
    }
}

// Single calls: block b writes the largest finite |x_d| of its share of the
// points to part[3 b + d] (no atomics, nothing to zero first), and block 0
// clears the product-form word maxbits[3] that the record kernel sets.
constexpr int kFxRangeThreads = 256;
__global__ void __launch_bounds__(kFxRangeThreads)
fx_range_kernel(const double *__restrict__ pos, int64_t P, int dim,
                unsigned long long *__restrict__ part, unsigned long long *maxbits) {
    __shared__ unsigned long long wm[kFxRangeThreads / 32][3];
    unsigned long long m[3] = {0ull, 0ull, 0ull};
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < P; i += stride)
        for (int d = 0; d < dim && d < 3; ++d) {
            const unsigned long long v =
                static_cast<unsigned long long>(__double_as_longlong(pos[d * P + i])) &
                0x7fffffffffffffffull;
            if (v < 0x7ff0000000000000ull) m[d] = max(m[d], v);
        }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        unsigned long long v = m[d];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) wm[warp][d] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long v = 0ull;
        for (int w = 0; w < kFxRangeThreads / 32; ++w) v = max(v, wm[w][threadIdx.x]);
        part[3 * static_cast<int64_t>(blockIdx.x) + threadIdx.x] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) maxbits[3] = 0ull;
}

// The record of mode j (see kFxRecWords).  mb[d]: the range words of the
// positions (largest |x_d| as bits); small_word: set when a wave number
// needs the general product form.  range_flag (may be null) is set to 1
// when a wave number is too large for the integer phase at these positions.
__device__ void fx_mode_entry(const double *k, double z1, double z2, int dim, int incompr,
                              const unsigned long long *mb, unsigned long long *small_word,
                              uint32_t *__restrict__ r, int *range_flag) {
    bool finite = isfinite(z1) && isfinite(z2);
    bool small = true;                              // every |BI| < 2^20
    double phi = 0.0;                               // units of 2^-32 turn
    for (int d = 0; d < 3; ++d) {
        int32_t bi = 0;
        uint32_t bf = 0;
        if (d < dim) {
            finite = finite && isfinite(k[d]);
            const double B = fx_ldexp(k[d] * kInv2Pi, 61 - fx_scale(mb[d]));
            if (fabs(B) < 2147483648.0) {
                const long long bq = __double2ll_rn(B * 4294967296.0);  // B to 2^-32 (exact scaling)
                bi = static_cast<int32_t>(bq >> 32);
                bf = static_cast<uint32_t>(bq);
                // B 2^31 mod 2^32: what the offset 2^60 of X adds to theta
                phi += static_cast<double>(static_cast<uint32_t>(bq >> 1)) + 0.5 * (bq & 1);
            } else if (isfinite(B) && range_flag) {
                *range_flag = 1;
            }
        }
        r[d] = static_cast<uint32_t>(bi) + 0x80000000u;
        r[4 + d] = bf;
        r[9 + d] = __float_as_uint(static_cast<float>(bi));
        small = small && bi < kFxSmallBI && bi > -kFxSmallBI;
    }
    double w[3] = {0.0, 0.0, 0.0};
    if (incompr) {   // projector as the reference forms it (src/field.rs:138-152)
        double kk = 0.0;
        for (int d = 0; d < dim; ++d) kk = __dadd_rn(kk, __dmul_rn(k[d], k[d]));
        const double k_2 = __ddiv_rn(k[0], kk);
        w[0] = __dadd_rn(1.0, -__dmul_rn(k[0], k_2));
        w[1] = -__dmul_rn(k[1], k_2);
        w[2] = -__dmul_rn(k[2], k_2);
    }
    r[3] = __float_as_uint(__double2float_rn(w[0]));
    r[7] = __float_as_uint(__double2float_rn(w[1]));
    r[8] = __float_as_uint(__double2float_rn(w[2]));
    if (!small) atomicOr(small_word, 1ull);
    for (int q = 12; q < kFxTab; ++q) r[q] = 0u;
    // phi mod 2^32, exactly (0 <= phi < 3 2^32, a multiple of 1/2)
    phi -= 4294967296.0 * floor(phi * 2.3283064365386963e-10);
    // T[m] = (z1 - i z2) e^{-2 pi i phi / 2^32} e^{2 pi i m / 16}: one FP64
    // sincos for the mode's rotation, the sixteenth turns from a table (FP64
    // products, a few FP64 ulps)
    double s0, c0;
    sincos(phi * -1.4629180792671596e-09, &s0, &c0);
    const double ar = z1 * c0 + z2 * s0, ai = z1 * s0 - z2 * c0;   // (z1 - i z2) e^{i a}
    const float nanf_ = __int_as_float(0x7fffffff);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        const double cm = kSixteenthCos[m], sm = kSixteenthCos[(m + 12) & 15];   // sin = cos(. - 1/4)
        const float tr = __double2float_rn(ar * cm - ai * sm);
        const float ti = __double2float_rn(ar * sm + ai * cm);
        r[kFxTab + 2 * m] = __float_as_uint(finite ? tr : nanf_);
        r[kFxTab + 2 * m + 1] = __float_as_uint(finite ? ti : nanf_);
    }
}

// One warp of modes per block.  A record is one thread's dependent chain of
// FP64 operations (about 13 us on GB300 for any number of modes per warp),
// so the kernel takes that latency once.  Each block first reduces the range
// kernel's per-block maxima; block 0 stores them as the range words of the
// sums.
constexpr int kFxModeThreads = 32;
__global__ void __launch_bounds__(kFxModeThreads)
fx_mode_kernel(const double *__restrict__ cov, const double *__restrict__ z1,
               const double *__restrict__ z2, int dim, int64_t n_modes, int64_t j0, int64_t nc,
               int incompr, const unsigned long long *__restrict__ range_part, int range_blocks,
               unsigned long long *maxbits, uint32_t *__restrict__ rec, int *range_flag) {
    // the mode's inputs first (they may come over the host link), so that
    // their latency overlaps the reduction of the range words
    const int64_t jl = static_cast<int64_t>(blockIdx.x) * kFxModeThreads + threadIdx.x;
    const int64_t j = j0 + jl;
    const bool mine = jl < nc;
    double k[3] = {0.0, 0.0, 0.0}, z1j = 0.0, z2j = 0.0;
    if (mine) {
        for (int d = 0; d < dim && d < 3; ++d) k[d] = cov[d * n_modes + j];
        z1j = z1[j];
        z2j = z2[j];
    }
    unsigned long long mb[3] = {0ull, 0ull, 0ull};
    for (int b = threadIdx.x; b < range_blocks; b += kFxModeThreads)
        for (int d = 0; d < dim && d < 3; ++d)
            mb[d] = max(mb[d], range_part[3 * static_cast<int64_t>(b) + d]);
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mb[d] = max(mb[d], __shfl_xor_sync(0xffffffffu, mb[d], o));
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        maxbits[0] = mb[0];
        maxbits[1] = mb[1];
        maxbits[2] = mb[2];
    }
    if (!mine) return;
    fx_mode_entry(k, z1j, z2j, dim, incompr, mb, maxbits + 3, rec + jl * kFxRecWords, range_flag);
}

// Kahan step: (sum, cmp) += a, cmp holding minus the lost low-order part
__device__ __forceinline__ void fx_kahan(float &sum, float &cmp, float a) {
    const float y = a - cmp;
    const float t = sum + y;
    cmp = (t - sum) - y;
    sum = t;
}

// Knuth's TwoSum: (hi, lo) += a
__device__ __forceinline__ void fx_two_sum(float &hi, float &lo, float a) {
    const float s = hi + a;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (a - bb);
    hi = s;
    lo += e;
}

// FP32 pair at a 32-bit shared-memory address
__device__ __forceinline__ float2 fx_lds2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

// The term Re(T e^{i theta}) of one point*mode: c the point's constant,
// (xh, x8l / xlf) its coordinate words, (bi, bf / bif) the mode's
// wave-number words, tab the shared-memory address of the mode's
// 128-byte-aligned table.
template <int D, bool SMALL>
__device__ __forceinline__ float fx_term(uint32_t c, const uint32_t *xh, const uint32_t *x8l,
                                         const float *xlf, const uint32_t *bi, const uint32_t *bf,
                                         const float *bif, uint32_t tab) {
    uint32_t t = c;
    if constexpr (SMALL) {
        // sum_d BI Xl 2^-29 (every |BI| < 2^20) rounded to an integer by a
        // chain of FP32 fused multiply-adds into the mantissa of 1.5 2^23
        float v = kFxMagic;
#pragma unroll
        for (int d = 0; d < D; ++d) v = fmaf(bif[d], xlf[d], v);
        t += __float_as_uint(v);
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if constexpr (!SMALL) t += __umulhi(bi[d], x8l[d]);
        t += __umulhi(bf[d], xh[d]);
        t += bi[d] * xh[d];
    }
    // t = theta + 2^27 + 16: entry m = t >> 28 (theta to the nearest 1/16
    // turn) at byte 8 m of the table; bits 5..27 are the remainder plus
    // 1/32 turn in units of 2^-27 turn, as the mantissa of a float in [1, 2)
    const float2 T = fx_lds2(tab | ((t >> 25) & 0x78u));
    const float r = __uint_as_float(0x3F800000u | ((t >> 5) & 0x007FFFFFu)) - 1.5f;
    const float r2 = r * r;
    const float sn = r * fmaf(r2, fmaf(r2, kFxS5, kFxS3), kFxS1);
    const float cs = fmaf(r2, fmaf(r2, kFxC4, kFxC2), kFxC0);
    return fmaf(T.x, cs, -T.y * sn);
}

// The words of mode m of the staged tile: BI' and BF, BI as FP32, the
// projector weights (times scale; incompressible field only) and the
// shared-memory address of the table.
struct FxModeWords {
    uint32_t bi[3], bf[3];
    float bif[3], w[3];
    uint32_t tab;
};

template <bool INC>
__device__ __forceinline__ FxModeWords fx_mode_words(const uint32_t *srec, uint32_t sbase, int m,
                                                     float scale) {
    const uint32_t *mr = srec + m * kFxRecWords;
    const uint4 h0 = *reinterpret_cast<const uint4 *>(mr);         // BI'0..2, w0
    const uint4 h1 = *reinterpret_cast<const uint4 *>(mr + 4);     // BF0..2, w1
    const uint4 h2 = *reinterpret_cast<const uint4 *>(mr + 8);     // w2, BI0..2 as FP32
    FxModeWords o;
    o.bi[0] = h0.x; o.bi[1] = h0.y; o.bi[2] = h0.z;
    o.bf[0] = h1.x; o.bf[1] = h1.y; o.bf[2] = h1.z;
    o.bif[0] = __uint_as_float(h2.y);
    o.bif[1] = __uint_as_float(h2.z);
    o.bif[2] = __uint_as_float(h2.w);
    o.w[0] = o.w[1] = o.w[2] = 0.f;
    if (INC) {
        o.w[0] = scale * __uint_as_float(h0.w);
        o.w[1] = scale * __uint_as_float(h1.w);
        o.w[2] = scale * __uint_as_float(h2.x);
    }
    o.tab = sbase + static_cast<uint32_t>(m * kFxRecWords + kFxTab) * 4u;
    return o;
}

// One block's work: the kFxThreads*R points from p_first (thread t owns
// p_first + t + r*kFxThreads), modes [jb, je) of the records `rec`; sums
// written (accumulate=0) or added at dst + i*sd + p*sp.  maxbits: the
// positions' range words (scales); srec: shared staging of TILE records.
template <int D, int R, bool INC, bool SMALL, int TILE>
__device__ __forceinline__ void fx_block_(const double *__restrict__ pos, int64_t P, int64_t p_first,
                                         const uint32_t *__restrict__ rec, int64_t jb, int64_t je,
                                         int accumulate, double *__restrict__ dst, int64_t sd,
                                         int64_t sp, const unsigned long long *maxbits,
                                         uint32_t *srec) {
    constexpr int NOUT = INC ? D : 1;
    const int tid = threadIdx.x;
    const int64_t p0 = p_first + tid;

    int sc[D];
#pragma unroll
    for (int d = 0; d < D; ++d) sc[d] = fx_scale(maxbits[d]);
    // SMALL: every mode's |BI| < 2^20, and BI Xl 2^-29 is an FP32 product
    // (xlf = Xl 2^-29); otherwise a high integer product (x8l = 8 Xl)
    uint32_t xh[R][D], x8l[R][SMALL ? 1 : D], cp[R];
    float xlf[R][SMALL ? D : 1];
    bool bad[R];
    float hi[R][NOUT], lo[R][NOUT];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t p = p0 + r * kFxThreads;
        // 2^27 centres the remainder on the table entry, + 16 rounds it to
        // the 2^-27 turn the float takes, + D offsets the mean truncation of
        // the two high products per dimension
        uint32_t c = 0x08000000u + 16u + D;
        bad[r] = false;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double x = p < P ? pos[d * P + p] : 0.0;
            bad[r] = bad[r] || !isfinite(x);
            const long long X = isfinite(x) ? __double2ll_rn(ldexp(x, sc[d])) : 0ll;
            const unsigned long long Xp = static_cast<unsigned long long>(X) + (1ull << 60);
            const uint32_t h = static_cast<uint32_t>(Xp >> 29);
            const uint32_t l = static_cast<uint32_t>(Xp) & 0x1FFFFFFFu;
            xh[r][d] = h;
            if constexpr (SMALL) {
                xlf[r][d] = static_cast<float>(l) * 1.862645149230957e-09f;     // Xl 2^-29
                // the bias 2^31 of BI' adds 2^31 Xh (mod 2^32)
                c -= (h & 1u) << 31;
            } else {
                x8l[r][d] = l << 3;
                // the bias 2^31 of BI' adds 2^31 Xh (mod 2^32) and 4 Xl
                c -= 4u * l + ((h & 1u) << 31);
            }
        }
        // the FP32 products of the signed BI leave the bits of 1.5 2^23 in theta
        if constexpr (SMALL) c -= kFxMagicBits;
        cp[r] = c;
#pragma unroll
        for (int i = 0; i < NOUT; ++i) hi[r][i] = lo[r][i] = 0.f;
    }

    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(srec));
    for (int64_t t0 = jb; t0 < je; t0 += TILE) {
        const int tm = static_cast<int>(min(static_cast<int64_t>(TILE), je - t0));
        __syncthreads();
        {
            // the header (words 0..11) and the table (words 32..63) of each record
            const uint4 *src = reinterpret_cast<const uint4 *>(rec + t0 * kFxRecWords);
            uint4 *dstv = reinterpret_cast<uint4 *>(srec);
            for (int i = tid; i < tm * (kFxRecWords / 4); i += kFxThreads) {
                const int q = i & (kFxRecWords / 4 - 1);
                if (q < 3 || q >= kFxTab / 4) dstv[i] = src[i];
            }
        }
        __syncthreads();
        float acc[R][NOUT], cmp[R][NOUT];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int i = 0; i < NOUT; ++i) acc[r][i] = cmp[r][i] = 0.f;
        // modes in groups of eight: four pair sums per point, added, then one
        // Kahan step; a tile shorter than TILE (the last) goes in pairs,
        // the second mode of an odd tile's last pair counting zero times
        constexpr int kGroupPairs = 4;
        const int tq = tm == TILE ? TILE : 0;
        for (int m = 0; m < tq; m += 2 * kGroupPairs) {
            float pend[R][NOUT];
#pragma unroll
            for (int h = 0; h < kGroupPairs; ++h) {
                const FxModeWords ma = fx_mode_words<INC>(srec, sbase, m + 2 * h, 1.0f);
                const FxModeWords mb = fx_mode_words<INC>(srec, sbase, m + 2 * h + 1, 1.0f);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float ta = fx_term<D, SMALL>(cp[r], xh[r], x8l[r], xlf[r], ma.bi,
                                                       ma.bf, ma.bif, ma.tab);
                    const float tb = fx_term<D, SMALL>(cp[r], xh[r], x8l[r], xlf[r], mb.bi,
                                                       mb.bf, mb.bif, mb.tab);
#pragma unroll
                    for (int i = 0; i < NOUT; ++i) {
                        const float ps = INC ? fmaf(ma.w[i], ta, mb.w[i] * tb) : ta + tb;
                        if (h == 0)
                            pend[r][i] = ps;
                        else if (h < kGroupPairs - 1)
                            pend[r][i] += ps;
                        else
                            fx_kahan(acc[r][i], cmp[r][i], pend[r][i] + ps);
                    }
                }
            }
        }
        for (int m = tq; m < tm; m += 2) {
            const bool two = m + 1 < tm;
            const float sb = two ? 1.0f : 0.0f;
            const FxModeWords ma = fx_mode_words<INC>(srec, sbase, m, 1.0f);
            const FxModeWords mb = fx_mode_words<INC>(srec, sbase, two ? m + 1 : m, sb);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float ta = fx_term<D, SMALL>(cp[r], xh[r], x8l[r], xlf[r], ma.bi, ma.bf,
                                                   ma.bif, ma.tab);
                const float tb = fx_term<D, SMALL>(cp[r], xh[r], x8l[r], xlf[r], mb.bi, mb.bf,
                                                   mb.bif, mb.tab);
#pragma unroll
                for (int i = 0; i < NOUT; ++i)
                    fx_kahan(acc[r][i], cmp[r][i],
                             INC ? fmaf(ma.w[i], ta, mb.w[i] * tb) : fmaf(sb, tb, ta));
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int i = 0; i < NOUT; ++i) {
                fx_two_sum(hi[r][i], lo[r][i], acc[r][i]);
                lo[r][i] -= cmp[r][i];
            }
    }

#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t p = p0 + r * kFxThreads;
        if (p >= P) continue;
#pragma unroll
        for (int i = 0; i < NOUT; ++i) {
            double v = static_cast<double>(hi[r][i]) + static_cast<double>(lo[r][i]);
            if (bad[r]) v = __longlong_as_double(0x7ff8000000000000ll);
            double *o = dst + i * sd + p * sp;
            *o = accumulate ? *o + v : v;
        }
    }
}

// The block's work with the product form its modes allow: maxbits[3] is
// set when some mode of the call (or batch item) has |BI| >= 2^20; the
// branch is the same for the whole block.
template <int D, int R, bool INC, int TILE>
__device__ __forceinline__ void fx_block(const double *__restrict__ pos, int64_t P, int64_t p_first,
                                         const uint32_t *__restrict__ rec, int64_t jb, int64_t je,
                                         int accumulate, double *__restrict__ dst, int64_t sd,
                                         int64_t sp, const unsigned long long *maxbits,
                                         uint32_t *srec) {
    if (maxbits[3] == 0ull)
        fx_block_<D, R, INC, true, TILE>(pos, P, p_first, rec, jb, je, accumulate, dst, sd, sp,
                                         maxbits, srec);
    else
        fx_block_<D, R, INC, false, TILE>(pos, P, p_first, rec, jb, je, accumulate, dst, sd, sp,
                                          maxbits, srec);
}

// R points per thread (2, 4 or 8; the autotuner picks).  The launch bound
// leaves room for several resident blocks, so that the R points' integer and
// FP32 chains interleave with other warps'.  Tiles of 128 modes for R = 8
// (three blocks per SM, limited by registers); 64 for R = 2, 4, whose
// launches keep more blocks per SM than 32 KB tiles of shared memory allow.
template <int D, bool INC, int R>
__global__ void __launch_bounds__(kFxThreads, R >= 8 ? 3 : 4)
mixed_fx_kernel(const double *__restrict__ pos, int64_t P, const uint32_t *__restrict__ rec,
                const unsigned long long *__restrict__ maxbits, int64_t nc, int64_t mps,
                int accumulate, double *__restrict__ dst, int64_t sd, int64_t sp,
                int64_t split_stride) {
    constexpr int TILE = R >= 8 ? kFxTile : kFxTile / 2;
    __shared__ __align__(256) uint32_t srec[TILE * kFxRecWords];
    const int64_t jb = static_cast<int64_t>(blockIdx.y) * mps;
    const int64_t je = min(nc, jb + mps);
    fx_block<D, R, INC, TILE>(pos, P, static_cast<int64_t>(blockIdx.x) * (kFxThreads * R), rec, jb,
                              je, accumulate,
                              dst + static_cast<int64_t>(blockIdx.y) * split_stride, sd, sp,
                              maxbits, srec);
}

template <int D, bool INC>
int launch_fx(int R, dim3 grid, cudaStream_t st, const double *pos, int64_t P, const uint32_t *rec,
              const unsigned long long *maxbits, int64_t nc, int64_t mps, int accumulate,
              double *dst, int64_t sd, int64_t sp, int64_t split_stride) {
    if (R == 2)
        mixed_fx_kernel<D, INC, 2><<<grid, kFxThreads, 0, st>>>(pos, P, rec, maxbits, nc, mps,
                                                                accumulate, dst, sd, sp, split_stride);
    else if (R == 8)
        mixed_fx_kernel<D, INC, 8><<<grid, kFxThreads, 0, st>>>(pos, P, rec, maxbits, nc, mps,
                                                                accumulate, dst, sd, sp, split_stride);
    else
        mixed_fx_kernel<D, INC, 4><<<grid, kFxThreads, 0, st>>>(pos, P, rec, maxbits, nc, mps,
                                                                accumulate, dst, sd, sp, split_stride);
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

int dispatch_fx(int R, int64_t dim, bool inc, dim3 grid, cudaStream_t st, const double *pos,
                int64_t P, const uint32_t *rec, const unsigned long long *maxbits, int64_t nc,
                int64_t mps, int accumulate, double *dst, int64_t sd, int64_t sp,
                int64_t split_stride) {
    if (dim == 1 && !inc)
        return launch_fx<1, false>(R, grid, st, pos, P, rec, maxbits, nc, mps, accumulate, dst, sd,
                                   sp, split_stride);
    if (dim == 2)
        return inc ? launch_fx<2, true>(R, grid, st, pos, P, rec, maxbits, nc, mps, accumulate, dst,
                                        sd, sp, split_stride)
                   : launch_fx<2, false>(R, grid, st, pos, P, rec, maxbits, nc, mps, accumulate, dst,
                                         sd, sp, split_stride);
    if (dim == 3)
        return inc ? launch_fx<3, true>(R, grid, st, pos, P, rec, maxbits, nc, mps, accumulate, dst,
                                        sd, sp, split_stride)
                   : launch_fx<3, false>(R, grid, st, pos, P, rec, maxbits, nc, mps, accumulate, dst,
                                         sd, sp, split_stride);
    return set_error(GSC_ERR_DIM, "the mixed form supports dimensions 1, 2, 3 (incompressible: 2, 3)");
}

// Launch shape of one configuration: R points per thread, mode splits so that
// about W blocks per SM exist when the points alone are few.  W < 0 asks for
// whole waves instead: at most -W times the blocks that fit on the GPU at
// once (occ per SM), so that no partial wave is left (a small call whose
// blocks fill 1.3 waves runs at the speed of two).
struct FxShape {
    int R, W;
    int64_t bx, S, mps;
};
FxShape fx_shape(int R, int W, int64_t P, int64_t chunk, int sms, int occ = 4) {
    FxShape f{R, W, 0, 1, 0};
    const int64_t pts_per_block = static_cast<int64_t>(kFxThreads) * R;
    f.bx = (P + pts_per_block - 1) / pts_per_block;
    int64_t S;
    if (W < 0) {
        const int64_t slots = static_cast<int64_t>(sms) * std::max(1, occ) * (-W);
        S = std::max<int64_t>(1, slots / f.bx);
    } else {
        const int64_t want_blocks = static_cast<int64_t>(sms) * W;
        S = std::max<int64_t>(1, (want_blocks + f.bx - 1) / f.bx);
    }
    S = std::min<int64_t>(S, std::max<int64_t>(1, chunk / (2 * kFxSplitModes)));
    S = std::min<int64_t>(S, 64);
    int64_t mps = chunk > 0 ? (chunk + S - 1) / S : 0;
    mps = (mps + kFxSplitModes - 1) / kFxSplitModes * kFxSplitModes;
    if (mps > 0) S = std::max<int64_t>(1, (chunk + mps - 1) / mps);
    if (chunk == 0) S = 1;
    f.S = S;
    f.mps = mps;
    return f;
}

// Resident blocks per SM of the sums kernel for (dim, kind, R).
template <int D, bool INC>
int fx_occ_t(int R) {
    int n = 0;
    cudaError_t e;
    if (R == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mixed_fx_kernel<D, INC, 2>, kFxThreads, 0);
    else if (R == 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mixed_fx_kernel<D, INC, 8>, kFxThreads, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mixed_fx_kernel<D, INC, 4>, kFxThreads, 0);
    if (e != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 4;
    }
    return n;
}
int fx_occupancy(int64_t dim, bool inc, int R) {
    if (dim == 1) return fx_occ_t<1, false>(R);
    if (dim == 2) return inc ? fx_occ_t<2, true>(R) : fx_occ_t<2, false>(R);
    return inc ? fx_occ_t<3, true>(R) : fx_occ_t<3, false>(R);
}

int fx_sm_count(int device) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 152;
    }
    return n;
}

// ---- batched ensembles ------------------------------------------------------------
// Range words of every item: the kBatchRangeBlocks blocks (blockIdx.y) of
// column blockIdx.x walk item blockIdx.x's positions.  Small blocks, so
// that the next ensemble's tables fit beside a persistent kernel's last
// blocks instead of waiting for whole SMs.
constexpr int kBatchRangeThreads = 128, kBatchRangeBlocks = 8;
__global__ void __launch_bounds__(kBatchRangeThreads)
batch_fx_range_kernel(const BatchItem *__restrict__ items, unsigned long long *maxbits) {
    const BatchItem &it = items[blockIdx.x];
    fx_range_part(it.pos, it.n_points, it.dim,
                  static_cast<int64_t>(blockIdx.y) * kBatchRangeThreads + threadIdx.x,
                  static_cast<int64_t>(kBatchRangeThreads) * kBatchRangeBlocks,
                  maxbits + 4 * blockIdx.x);
}

// Records of every item, one thread per mode (Fourier factor folded into z1,
// z2 first).
__global__ void batch_fx_table_kernel(const BatchItem *__restrict__ items,
                                      const int64_t *__restrict__ prefix, int64_t n_items,
                                      int64_t total, unsigned long long *maxbits,
                                      uint32_t *__restrict__ rec, int *range_flag) {
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
    double k[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < it.dim && d < 3; ++d) k[d] = it.cov[d * it.n_modes + j];
    fx_mode_entry(k, z1j, z2j, it.dim, it.incompr, maxbits + 4 * lo, maxbits + 4 * lo + 3,
                  rec + g * kFxRecWords, range_flag);
}

// Persistent batch kernel (see batch_plain_kernel in plain.cu).  SCALAR:
// an ensemble without incompressible items, whose kernel carries only the
// scalar variants (fewer registers, so R = 8 keeps 3 blocks per SM).
template <int R, bool SCALAR>
__global__ void __launch_bounds__(kFxThreads, R >= 8 ? (SCALAR ? 3 : 2) : 4)
batch_fx_kernel(const BatchItem *__restrict__ items, const BatchUnit *__restrict__ units,
                int64_t n_units, int *__restrict__ counter, const uint32_t *__restrict__ rec,
                const unsigned long long *__restrict__ maxbits) {
    __shared__ __align__(256) uint32_t srec[kFxTile * kFxRecWords];
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
        const uint32_t *rc = rec + it.mode_off * kFxRecWords;
        const unsigned long long *mb = maxbits + 4 * w.item;
        switch (it.dim * 2 + it.incompr) {
            case 2:
                fx_block<1, R, false, kFxTile>(it.pos, P, w.p_first, rc, w.jb, w.je, 0, dst, P,
                                              1, mb, srec);
                break;
            case 4:
                fx_block<2, R, false, kFxTile>(it.pos, P, w.p_first, rc, w.jb, w.je, 0, dst, P,
                                              1, mb, srec);
                break;
            case 5:
                if constexpr (!SCALAR)
                    fx_block<2, R, true, kFxTile>(it.pos, P, w.p_first, rc, w.jb, w.je, 0, dst, P,
                                                  1, mb, srec);
                break;
            case 6:
                fx_block<3, R, false, kFxTile>(it.pos, P, w.p_first, rc, w.jb, w.je, 0, dst, P,
                                              1, mb, srec);
                break;
            case 7:
                if constexpr (!SCALAR)
                    fx_block<3, R, true, kFxTile>(it.pos, P, w.p_first, rc, w.jb, w.je, 0, dst, P,
                                                  1, mb, srec);
                break;
            default:
                break;
        }
    }
}

using BatchFxFn = void (*)(const BatchItem *, const BatchUnit *, int64_t, int *, const uint32_t *,
                           const unsigned long long *);
BatchFxFn batch_fx_fn(int R, bool scalar) {
    if (R == 2) return scalar ? batch_fx_kernel<2, true> : batch_fx_kernel<2, false>;
    if (R == 4) return scalar ? batch_fx_kernel<4, true> : batch_fx_kernel<4, false>;
    if (R == 8) return scalar ? batch_fx_kernel<8, true> : batch_fx_kernel<8, false>;
    return nullptr;
}

}  // namespace

int mixed_fx_run(DeviceCtx &ctx, const PlainArgs &a, int *range_flag, cudaStream_t st) {
    const int64_t P = a.n_points, N = a.n_modes, dim = a.dim;
    if (P == 0) return GSC_OK;
    const int64_t nout = a.incompr ? dim : 1;
    if (dim < 1 || dim > 3 || (a.incompr && dim == 1))
        return set_error(GSC_ERR_DIM, "the mixed form supports dimensions 1, 2, 3 (incompressible: 2, 3)");
    constexpr int64_t kChunk = 1 << 20;   // modes per record build
    const int64_t chunk = std::min<int64_t>(N, kChunk);
    const int sms = fx_sm_count(ctx.device);

    // configuration: the tuned one for this shape bucket, else the default;
    // a miss is tuned on this call's data when the call is large (a single
    // record build, at least 2^26 point*modes; tuning costs about nine
    // calls once per shape bucket)
    const std::string key = device_name(ctx.device) + "|mixed|d" + std::to_string(dim) +
                            (a.incompr ? "i" : "s") + "|p" + std::to_string(tune_bucket(double(P))) +
                            "|n" + std::to_string(tune_bucket(double(N)));
    int tv[4] = {kFxR, kFxW, 0, 0};
    const int mode = tune_mode();
    bool tune = false;
    if (mode == 0 || !tune_get(key, tv)) {
        tv[0] = kFxR;
        tv[1] = kFxW;
        tune = mode == 2 && N <= kChunk && static_cast<double>(P) * N >= 67108864.0;
    }
    // blocks per SM targets, and one or two whole waves (W < 0)
    static const int kCandR[3] = {2, 4, 8}, kCandW[5] = {4, 8, 16, -1, -2};
    auto shape_of = [&](int r, int w) {
        return fx_shape(r, w, P, chunk, sms, w < 0 ? fx_occupancy(dim, a.incompr, r) : 4);
    };
    FxShape shp = shape_of(tv[0], tv[1]);
    if (shp.bx > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many points for one launch");
    int64_t S_max = shp.S;
    if (tune)
        for (int r : kCandR)
            for (int w : kCandW) S_max = std::max(S_max, shape_of(r, w).S);

    // range blocks: enough to stream the positions, at most four per SM
    const int64_t rb = std::max<int64_t>(
        1, std::min<int64_t>((P + kFxRangeThreads - 1) / kFxRangeThreads, 4 * static_cast<int64_t>(sms)));
    const size_t rec_bytes = static_cast<size_t>(chunk) * kFxRecBytesPerMode;
    const size_t part_bytes = S_max > 1 ? static_cast<size_t>(S_max) * nout * P * sizeof(double) : 0;
    const size_t off_mb = (rec_bytes + 255) / 256 * 256;
    const size_t off_rp = off_mb + 256;
    const size_t off_part = off_rp + (static_cast<size_t>(rb) * 3 * sizeof(unsigned long long) + 255) / 256 * 256;
    GSC_TRY(ensure_dev(ctx, ctx.scratch, off_part + part_bytes + 256));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    unsigned char *sbase = static_cast<unsigned char *>(ctx.scratch.ptr);
    uint32_t *rec = reinterpret_cast<uint32_t *>(sbase);
    unsigned long long *maxbits = reinterpret_cast<unsigned long long *>(sbase + off_mb);
    unsigned long long *range_part = reinterpret_cast<unsigned long long *>(sbase + off_rp);
    double *part = reinterpret_cast<double *>(sbase + off_part);

    {
        TimedLaunch tl(st);
        tl.begin(K_MIXED_MODES);
        fx_range_kernel<<<static_cast<unsigned>(rb), kFxRangeThreads, 0, st>>>(
            a.pos, P, static_cast<int>(dim), range_part, maxbits);
        tl.end();
        GSC_CUDA(cudaGetLastError());
    }
    auto build = [&](int64_t j0, int64_t nc) -> int {
        if (nc <= 0) return GSC_OK;
        TimedLaunch tl(st);
        tl.begin(K_MIXED_MODES);
        fx_mode_kernel<<<static_cast<unsigned>((nc + kFxModeThreads - 1) / kFxModeThreads),
                         kFxModeThreads, 0, st>>>(
            a.cov, a.z1, a.z2, static_cast<int>(dim), N, j0, nc, a.incompr ? 1 : 0, range_part,
            static_cast<int>(rb), maxbits, rec, range_flag);
        tl.end();
        GSC_CUDA(cudaGetLastError());
        return GSC_OK;
    };
    // the sums of modes [j0, j0 + nc) with records built, into the output
    // (first chunk) or added to it
    auto sums = [&](const FxShape &f, int64_t nc, bool first, bool timed) -> int {
        const bool split = f.S > 1;
        double *dst = split ? part : a.out;
        const int64_t sd = split ? P : a.out_sd, sp = split ? 1 : a.out_sp;
        const int64_t split_stride = split ? nout * P : 0;
        const int64_t mps_c = nc > 0 ? std::min<int64_t>(f.mps, nc) : 0;
        const dim3 g(static_cast<unsigned>(f.bx),
                     static_cast<unsigned>(nc > 0 ? std::min<int64_t>(f.S, (nc + mps_c - 1) / mps_c) : 1));
        TimedLaunch tl(st);
        if (timed) tl.begin(a.incompr ? K_MIXED_INCOMPR : K_MIXED_SCALAR);
        // splits write partials that split_reduce sums into the output; with
        // several record chunks they accumulate across chunks
        const int rc = dispatch_fx(f.R, dim, a.incompr, g, st, a.pos, P, rec, maxbits, nc, mps_c,
                                   first ? 0 : 1, dst, sd, sp, split_stride);
        if (timed) tl.end();
        return rc;
    };

    if (tune) {
        // every candidate on this call's data, timed by events; the winner
        // then computes the result
        GSC_TRY(build(0, chunk));
        cudaEvent_t e0, e1;
        GSC_CUDA(cudaEventCreate(&e0));
        GSC_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        int br = kFxR, bw = kFxW;
        int rc = GSC_OK;
        for (int r : kCandR)
            for (int w : kCandW) {
                const FxShape f = shape_of(r, w);
                if (rc == GSC_OK) rc = cuda_ok(cudaEventRecord(e0, st));
                if (rc == GSC_OK) rc = sums(f, chunk, true, false);
                if (rc == GSC_OK && f.S > 1)
                    rc = split_reduce(part, f.S, nout, P, a.out, a.out_sd, a.out_sp, st);
                if (rc == GSC_OK) rc = cuda_ok(cudaEventRecord(e1, st));
                if (rc == GSC_OK) rc = cuda_ok(cudaEventSynchronize(e1));
                float ms = 0.f;
                if (rc == GSC_OK) rc = cuda_ok(cudaEventElapsedTime(&ms, e0, e1));
                if (rc == GSC_OK && ms < best) {
                    best = ms;
                    br = r;
                    bw = w;
                }
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        GSC_TRY(rc);
        const int v[4] = {br, bw, 0, 0};
        tune_put(key, v);
        shp = shape_of(br, bw);
        GSC_TRY(sums(shp, chunk, true, true));
        if (shp.S > 1) GSC_TRY(split_reduce(part, shp.S, nout, P, a.out, a.out_sd, a.out_sp, st));
        GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
        return GSC_OK;
    }

    int64_t j0 = 0;
    bool first = true;
    do {
        const int64_t nc = std::min<int64_t>(N - j0, kChunk);
        GSC_TRY(build(j0, nc));
        GSC_TRY(sums(shp, nc, first, true));
        first = false;
        j0 += nc;
    } while (j0 < N);

    if (shp.S > 1) GSC_TRY(split_reduce(part, shp.S, nout, P, a.out, a.out_sd, a.out_sp, st));
    GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
    return GSC_OK;
}

// ---- batched ensembles ----------------------------------------------------------
int batch_fx_tables(const BatchItem *items, const int64_t *mode_prefix, int64_t n_items,
                    int64_t total_modes, uint32_t *rec, unsigned long long *maxbits,
                    int *range_flag, cudaStream_t st) {
    if (n_items == 0) return GSC_OK;
    TimedLaunch tl(st);
    tl.begin(K_BATCH_TABLES);
    GSC_CUDA(cudaMemsetAsync(maxbits, 0, static_cast<size_t>(n_items) * 4 * sizeof(unsigned long long),
                             st));
    batch_fx_range_kernel<<<dim3(static_cast<unsigned>(n_items), kBatchRangeBlocks),
                            kBatchRangeThreads, 0, st>>>(items, maxbits);
    if (total_modes > 0)
        batch_fx_table_kernel<<<static_cast<unsigned>((total_modes + 127) / 128), 128, 0, st>>>(
            items, mode_prefix, n_items, total_modes, maxbits, rec, range_flag);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

bool batch_fx_config_ok(int R) { return batch_fx_fn(R, false) != nullptr; }

int batch_fx_occupancy(int R, bool scalar) {
    BatchFxFn fn = batch_fx_fn(R, scalar);
    if (!fn) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kFxThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int batch_fx_launch(int R, bool scalar, int blocks, const BatchItem *items,
                    const BatchUnit *units, int64_t n_units, int *counter, const uint32_t *rec,
                    const unsigned long long *maxbits, cudaStream_t st) {
    BatchFxFn fn = batch_fx_fn(R, scalar);
    if (!fn) return set_error(GSC_ERR_INVALID, "unsupported batch configuration");
    TimedLaunch tl(st);
    tl.begin(K_BATCH_MIXED);
    fn<<<blocks, kFxThreads, 0, st>>>(items, units, n_units, counter, rec, maxbits);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    return GSC_OK;
}

}  // namespace gsc
