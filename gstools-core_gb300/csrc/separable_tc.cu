// separable_tc.cu -- the randomization-method summator on structured grids,
// as a complex contraction on tcgen05 tensor cores (sm_103a).
//
// On a structured grid x_p = (X_a, Y_b, Z_c) the phase factor separates:
//   z1 cos(k.x) + z2 sin(k.x) = Re[(z1 - i z2) e^{i kx X_a} e^{i ky Y_b} e^{i kz Z_c}]
// so the field (reference src/field.rs:37-65 evaluated on the flattened
// meshgrid) becomes, for every X_a,
//   u[a, b, c] = sum_j Re[ s_a[j] B[b, j] C[c, j] ],
//   s_a[j] = (z1_j - i z2_j) e^{i kx_j X_a},  B[b, j] = e^{i ky_j Y_b},
//   C[c, j] = e^{i kz_j Z_c} (times the projector weight p_i(k_j) for the
//   incompressible field, reference src/field.rs:138-152),
// i.e. one real GEMM per X_a with K = 2 * modes:
//   rows     F[b, 2j] = Re(s_a B),  F[b, 2j+1] = Im(s_a B)     (built on chip)
//   columns  G[c, 2j] = Re C,       G[c, 2j+1] = -Im C          (static table)
//   u[a, b, c] = sum_k F[b, k] G[c, k].
// In 2-D the same GEMM runs once with s = z1 - i z2 and (rows, columns) =
// (X, Y).
//
// Precision.  Both operands are split into two half-precision terms
// (hi + lo, 22 significant bits); the GEMM sums hi*hi + hi*lo + lo*hi
// ("f16x3"; "bf16x3" with bfloat16 terms) in FP32 tensor-memory
// accumulators.  FP32 accumulation over all 2N terms would round at the
// full field magnitude on every MMA instruction, so the K loop is cut into
// chunks of KC k-blocks: each chunk accumulates from zero in one TMEM
// region and the epilogue warps add it into a running total held in a
// second TMEM region while the next chunk is computed.
//
// Kernel structure (one CTA per output tile of 128 rows x 256 columns of
// one X_a; 10 warps):
//   warps 0-3  epilogue: drain chunk accumulators, final FP64 store
//   warps 4-7  producers: build the F tile (hi, lo) for each k-block in
//              the 128-byte-swizzled K-major layout the MMA reads
//   warp  8    TMA: loads the G tiles (hi, lo) of each k-block
//   warp  9    MMA issuer (one thread) and TMEM owner
// Two pipeline stages of 96 KB (F hi/lo 2 x 16 KB, G hi/lo 2 x 32 KB).
//
// The form chosen at the 1e-6 bar, "f16x5" (sep_x5_kernel below), keeps the
// same factorisation but sums its leading product exactly on an integer
// grid; its precision scheme, pipeline, tail split and epilogue are
// described with it, its FP32 factor tables with sep_x5_split_kernel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "dfturns.cuh"
#include "internal.h"
#include "sm100.cuh"

namespace gsc {
namespace {
using namespace sm100;

constexpr int BM = 128;                         // tile rows (TMEM lanes)
constexpr int BN = 256;                         // tile columns
constexpr int BK = 64;                          // K elements per k-block (32 modes)
constexpr int STAGES = 2;
constexpr int A_BYTES = BM * BK * 2;            // one F term of one stage
constexpr int G_BYTES = BN * BK * 2;            // one G term of one stage
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * G_BYTES;
constexpr int kThreadsTC = 320;
constexpr int kTmaWarp = 8;
constexpr int kMmaWarp = 9;
constexpr uint32_t kTmemCols = 512;             // acc [0, 256), total [256, 512)
constexpr size_t kSmemBytes = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;

// Both operands are scaled by 2^10 before the split so that the lo terms of
// values down to 2^-13 stay normal f16 numbers (the tensor core does not
// keep f16 subnormals); the epilogue multiplies by 2^-20, exactly.
constexpr float kOperandScale = 1024.0f;
constexpr float kProductUnscale = 1.0f / (1024.0f * 1024.0f);

constexpr double kTwoOverPi = 0.6366197723675814;
constexpr double kPio2Hi = 1.5707963267948966;      // fl(pi/2)
constexpr double kPio2Lo = 6.123233995736766e-17;   // fl(pi/2 - kPio2Hi)
constexpr double kRound = 6755399441055744.0;       // 1.5 * 2^52

// e^{i phi} to about one FP32 ulp: FP64 two-constant Cody-Waite reduction to
// |r| <= pi/4, FP32 sincos of r with a first-order correction for the FP32
// rounding of r, quadrant rotation.  |phi| beyond 1e13 uses FP64 sincos.
__device__ __forceinline__ float2 cis_f32(double phi) {
    if (!(fabs(phi) < 1.0e13)) {
        double s, c;
        sincos(phi, &s, &c);
        return make_float2(static_cast<float>(c), static_cast<float>(s));
    }
    const double t = fma(phi, kTwoOverPi, kRound);
    const double q = t - kRound;
    const int quad = __double2loint(t) & 3;
    double r = fma(-q, kPio2Hi, phi);
    r = fma(-q, kPio2Lo, r);
    const float rh = __double2float_rn(r);
    const float rl = __double2float_rn(r - static_cast<double>(rh));
    float sn, cs;
    sincosf(rh, &sn, &cs);
    const float s1 = fmaf(rl, cs, sn);
    const float c1 = fmaf(-rl, sn, cs);
    switch (quad) {
        case 0: return make_float2(c1, s1);
        case 1: return make_float2(-s1, c1);
        case 2: return make_float2(-c1, -s1);
        default: return make_float2(s1, -c1);
    }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// FP32 -> FP64 with integer operations only (GB300's FP64 pipe is 1/64 of
// FP32).  FP32 subnormals (< 1.2e-38) become signed zeros.
__device__ __forceinline__ double f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, man = u & 0x7FFFFFu;
    // selects, not branches, so that independent conversions interleave
    const uint32_t hi_norm = sign | ((e + 896u) << 20) | (man >> 3);
    const uint32_t hi_spec = sign | 0x7FF00000u | (man >> 3) | (man ? 0x80000u : 0u);
    uint32_t hi = e == 0xFFu ? hi_spec : hi_norm;
    hi = e == 0u ? sign : hi;
    const uint32_t lo = e == 0u ? 0u : man << 29;
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

// f32_to_f64(f * 2^k) for |k| small enough that no finite product leaves
// the normal FP64 range: the power of two is added to the exponent
// (ebias = (896 + k) << 20), so the scaling costs nothing and stays exact.
// FP32 zeros and subnormals give signed zeros, Inf and NaN stay Inf and NaN.
__device__ __forceinline__ double f32_to_f64_pow2(float f, uint32_t ebias) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t a = u & 0x7FFFFFFFu, sign = u & 0x80000000u;
    uint32_t hi = ((a >> 3) + ebias) | sign;
    hi = a >= 0x7F800000u ? (sign | 0x7FF00000u | ((a & 0x7FFFFFu) >> 3) | (a > 0x7F800000u ? 0x80000u : 0u))
                          : hi;
    const bool tiny = a < 0x00800000u;
    return __hiloint2double(static_cast<int>(tiny ? sign : hi), static_cast<int>(tiny ? 0u : u << 29));
}

// v * 2^q as FP64, exactly, with integer operations only: |v| < 2^31 has at
// most 31 significant bits; q keeps the result a normal FP64 number.  The
// sentinel v = -2^31 (a NaN sum) gives NaN.
__device__ __forceinline__ double i32_to_f64_pow2(int v, int q) {
    const uint32_t sign = static_cast<uint32_t>(v) & 0x80000000u;
    const uint32_t a = v < 0 ? 0u - static_cast<uint32_t>(v) : static_cast<uint32_t>(v);
    const int lz = __clz(a);                     // a in [2^k, 2^(k+1)), k = 31 - lz
    // a << (lz + 21) as a 64-bit value puts the leading 1 at bit 52; its
    // words by 32-bit funnel shifts
    const uint32_t sh = static_cast<uint32_t>(lz) + 21u;              // 21 .. 52
    const uint32_t mhi = sh >= 32u ? a << (sh - 32u) : __funnelshift_l(a, 0u, sh);
    const uint32_t mlo = sh >= 32u ? 0u : a << sh;
    const uint32_t hi = sign | (static_cast<uint32_t>(1023 + 31 - lz + q) << 20) | (mhi & 0xFFFFFu);
    const double d = __hiloint2double(static_cast<int>(a == 0u ? sign : hi), static_cast<int>(a == 0u ? 0u : mlo));
    return v == static_cast<int>(0x80000000u) ? __longlong_as_double(0x7ff8000000000000ll) : d;
}

template <bool BF16>
struct Split;
template <>
struct Split<false> {
    // v ~ hi + lo, both IEEE half, packed as (re, im) pairs
    __device__ __forceinline__ static void run(float re, float im, uint32_t &hi, uint32_t &lo) {
        const __half2 h = __floats2half2_rn(re, im);
        const float2 hf = __half22float2(h);
        const __half2 l = __floats2half2_rn(re - hf.x, im - hf.y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    }
};
template <>
struct Split<true> {
    __device__ __forceinline__ static void run(float re, float im, uint32_t &hi, uint32_t &lo) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(re, im);
        const float2 hf = __bfloat1622float2(h);
        const __nv_bfloat162 l = __floats2bfloat162_rn(re - hf.x, im - hf.y);
        hi = *reinterpret_cast<const uint32_t *>(&h);
        lo = *reinterpret_cast<const uint32_t *>(&l);
    }
};

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
struct TabArgs {
    const double *cov;          // (dim, n_modes) row-major
    const double *z1, *z2;
    int dim, n_modes;
    const double *ax_b;          // batch axis (X) for 3-D, unused in 2-D
    const double *ax_m;          // row axis
    const double *ax_n;          // column axis
    int kb_dim, km_dim, kn_dim;  // which k component goes with each axis
    int nb, nm, nn, ncomp, incompr;
    int k_pad;                   // K elements per G row (multiple of 64)
    int nm_ld;                   // B-table row length (nm rounded up to 16)
    int ncn_pad;                 // G rows (multiple of BN)
    float2 *svec;                // [nb][sv_stride]
    int64_t sv_stride;           // modes per svec row: n_modes, or (x5) kbt * 16 zero-padded
    float2 *btab;                // [n_modes][nm]
    uint32_t *ghi, *glo;         // [ncn_pad][k_pad/2] packed (re, -im) pairs
    float *wnorm;                // x5 form: {W, 1/W}, W = 2^ceil(log2 max|z1 - i z2|)
    int *bound_flag;             // x5 form: 1 when the exact main sum cannot be guaranteed
    int *bound_sticky;           // x5 form: set to 1 (never cleared here) in that case
    float *l1kb;                 // x5 form: per k-block bound of the leading products (counts)
    int kc;                      // x5 form: k-blocks per cross-accumulator chunk
    int kbt;                     // x5 form: k-blocks (16 modes each)
    int bn;                      // x5 form: G rows per stage block (tile width)
    // x5 form: FP32 inputs of the tables (sep_x5_split_kernel): per mode
    // kRecX5 floats, per axis point an (hi, lo) pair, axes b | m | n
    float *mrec;
    float2 *axs;
    int ax_off_m, ax_off_n;      // first m / n point in axs (b starts at 0)
};

// s_a[j] = (z1_j - i z2_j) e^{i k_x,j X_a} (3-D) or z1_j - i z2_j (2-D), times
// inv_w (1 unless the caller normalises here)
__device__ __forceinline__ void svec_entry(const TabArgs &t, int64_t i, double inv_w) {
    const int b = static_cast<int>(i / t.n_modes), j = static_cast<int>(i % t.n_modes);
    float2 w = make_float2(static_cast<float>(t.z1[j] * inv_w), static_cast<float>(-t.z2[j] * inv_w));
    if (t.dim == 3) {
        const float2 e = cis_f32(t.cov[t.kb_dim * t.n_modes + j] * t.ax_b[b]);
        // (z1 - i z2) e, formed in FP64 from the FP32 factor, rounded once
        const double re = (t.z1[j] * e.x + t.z2[j] * e.y) * inv_w;
        const double im = (t.z1[j] * e.y - t.z2[j] * e.x) * inv_w;
        w = make_float2(static_cast<float>(re), static_cast<float>(im));
    }
    t.svec[i] = w;
}

__global__ void sep_svec_kernel(TabArgs t) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.nb) * t.n_modes) return;
    svec_entry(t, i, t.wnorm ? static_cast<double>(t.wnorm[1]) : 1.0);
}

// B table [n_modes][nm_ld], columns nm .. nm_ld-1 zero (the f16x3 / bf16x3
// forms; the x5 form's tiled table is btab_x5_entry).
__device__ __forceinline__ void btab_entry(const TabArgs &t, int64_t i) {
    const int j = static_cast<int>(i / t.nm_ld);
    const int m = static_cast<int>(i % t.nm_ld);
    const float2 v = (m < t.nm && j < t.n_modes)
                         ? cis_f32(t.cov[t.km_dim * t.n_modes + j] * t.ax_m[m])
                         : make_float2(0.f, 0.f);
    t.btab[i] = v;
}

__global__ void sep_btab_kernel(TabArgs t) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.n_modes) * t.nm_ld) return;
    btab_entry(t, i);
}

template <bool BF16>
__global__ void sep_gtab_kernel(TabArgs t) {
    const int half_k = t.k_pad / 2;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.ncn_pad) * half_k) return;
    const int row = static_cast<int>(i / half_k), j = static_cast<int>(i % half_k);
    float re = 0.f, im = 0.f;
    if (row < t.ncomp * t.nn && j < t.n_modes) {
        const int c = row / t.nn, n = row - c * t.nn;
        float2 e = cis_f32(t.cov[t.kn_dim * t.n_modes + j] * t.ax_n[n]);
        double pw = 1.0;
        if (t.incompr) {
            // projector weight, as the reference forms it (src/field.rs:138-152)
            double kk = 0.0;
            for (int d = 0; d < t.dim; ++d) {
                const double kd = t.cov[d * t.n_modes + j];
                kk = __dadd_rn(kk, __dmul_rn(kd, kd));
            }
            const double k0 = t.cov[j];
            const double k_2 = __ddiv_rn(k0, kk);
            pw = (c == 0) ? __dadd_rn(1.0, -__dmul_rn(k0, k_2))
                          : -__dmul_rn(t.cov[c * t.n_modes + j], k_2);
        }
        re = static_cast<float>(pw * e.x) * kOperandScale;
        im = static_cast<float>(-(pw * e.y)) * kOperandScale;
    }
    uint32_t hi, lo;
    Split<BF16>::run(re, im, hi, lo);
    t.ghi[i] = hi;
    t.glo[i] = lo;
}

// ---------------------------------------------------------------------------
// GEMM kernel
// ---------------------------------------------------------------------------
struct TcParams {
    const float2 *svec;     // [nb][sv_stride]
    int64_t sv_stride;
    const float2 *btab;     // [n_modes][nm_ld]
    int n_modes, nm, nm_ld, nb, nn, ncn;   // ncn = ncomp * nn valid G rows
    int kb_total, kc;               // k-blocks, k-blocks per accumulation chunk
    int m_tiles, n_tiles;
    int64_t rows_total;             // x5: nb * nm rows, tiled across slices
    double *out;
    int64_t comp_stride, batch_stride, row_stride;
    int *status;
};

template <bool BF16>
__global__ void __launch_bounds__(kThreadsTC, 1)
sep_tc_kernel(const __grid_constant__ CUtensorMap map_ghi,
              const __grid_constant__ CUtensorMap map_glo, const TcParams p) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
    uint64_t *full_a = bars;                  // producers -> MMA   (128 arrivals)
    uint64_t *full_g = bars + STAGES;         // TMA -> MMA         (1 arrival + bytes)
    uint64_t *empty = bars + 2 * STAGES;      // MMA commit -> producers, TMA
    uint64_t *acc_full = bars + 3 * STAGES;   // MMA commit -> epilogue
    uint64_t *acc_empty = acc_full + 1;       // epilogue -> MMA    (128 arrivals)
    uint64_t *drain = acc_full + 2;           // MMA commit on abort
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int tile = blockIdx.x;
    const int nt = tile % p.n_tiles;
    tile /= p.n_tiles;
    const int mt = tile % p.m_tiles;
    const int b = tile / p.m_tiles;
    const int m0 = mt * BM, n0 = nt * BN;
    const int KB = p.kb_total, KC = p.kc;
    const int NC = (KB + KC - 1) / KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full_a[s], 128);
            mbar_init(&full_g[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, 128);
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    if (warp == kTmaWarp && lane == 0) {
        tma_prefetch_map(&map_ghi);
        tma_prefetch_map(&map_glo);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t t_acc = tmem, t_tot = tmem + 256;

    if (warp == kTmaWarp) {
        // ---- TMA: G tiles --------------------------------------------------
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < KB; ++kb) {
                const int s = kb % STAGES, n = kb / STAGES;
                if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1, abort_flag, p.status,
                                        kErrTimeoutEmpty))
                    break;
                unsigned char *st = smem + s * STAGE_BYTES;
                mbar_arrive_expect_tx(&full_g[s], 2 * G_BYTES);
                tma_load_2d(st + 2 * A_BYTES, &map_ghi, &full_g[s], kb * BK, n0);
                tma_load_2d(st + 2 * A_BYTES + G_BYTES, &map_glo, &full_g[s], kb * BK, n0);
                ++issued;
            }
            if (*abort_flag) {   // let the copies in flight land before the CTA exits
                for (int kb = issued > STAGES ? issued - STAGES : 0; kb < issued; ++kb)
                    mbar_wait_drain(&full_g[kb % STAGES], (kb / STAGES) & 1, p.status);
            }
        }
    } else if (warp == kMmaWarp) {
        // ---- MMA issue -------------------------------------------------------
        if (lane == 0) {
            const uint32_t idesc = idesc_f16(BM, BN, BF16);
            bool ok = true;
            for (int kb = 0; kb < KB; ++kb) {
                const int s = kb % STAGES, n = kb / STAGES;
                const int c = kb / KC;
                const bool first = (kb % KC) == 0;
                const bool last = (kb % KC) == KC - 1 || kb == KB - 1;
                if (first && c > 0)
                    ok = mbar_wait(acc_empty, (c - 1) & 1, abort_flag, p.status, kErrTimeoutAcc);
                if (ok) ok = mbar_wait(&full_a[s], n & 1, abort_flag, p.status, kErrTimeoutFull);
                if (ok) ok = mbar_wait(&full_g[s], n & 1, abort_flag, p.status, kErrTimeoutFull);
                if (!ok) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
                const uint32_t a_hi = sa, a_lo = sa + A_BYTES;
                const uint32_t g_hi = sa + 2 * A_BYTES, g_lo = g_hi + G_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const uint32_t off = kk * 32;   // 16 elements of 2 bytes
                    mma_f16_ss(t_acc, desc_k_sw128(a_hi + off), desc_k_sw128(g_hi + off), idesc,
                               (first && kk == 0) ? 0u : 1u);
                    mma_f16_ss(t_acc, desc_k_sw128(a_hi + off), desc_k_sw128(g_lo + off), idesc, 1u);
                    mma_f16_ss(t_acc, desc_k_sw128(a_lo + off), desc_k_sw128(g_hi + off), idesc, 1u);
                }
                mma_commit(&empty[s]);
                if (last) mma_commit(acc_full);
            }
            if (!ok) {   // wait for the MMAs already issued before TMEM is freed
                mma_commit(drain);
                mbar_wait_drain(drain, 0, p.status);
            }
        }
    } else if (warp >= 4) {
        // ---- producers: F tile rows ----------------------------------------------
        // Thread r builds row m0 + r.  The B-table values of k-block kb + 1
        // are loaded while k-block kb is converted, hiding the L2 latency.
        const int r = threadIdx.x - 128;
        const int m = m0 + r;
        const bool row_ok = m < p.nm;
        const float2 *sv = p.svec + static_cast<int64_t>(b) * p.sv_stride;
        const uint32_t row_off = (r >> 3) * 1024 + (r & 7) * 128;
        float2 cur[32];
        auto load_block = [&](int kb, float2 (&dst)[32]) {
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int j = kb * 32 + q;
                dst[q] = (row_ok && j < p.n_modes) ? __ldg(p.btab + static_cast<int64_t>(j) * p.nm_ld + m)
                                                   : make_float2(0.f, 0.f);
            }
        };
        load_block(0, cur);
        for (int kb = 0; kb < KB; ++kb) {
            const int s = kb % STAGES, n = kb / STAGES;
            float2 nxt[32];
            if (kb + 1 < KB) load_block(kb + 1, nxt);
            if (n > 0 &&
                !mbar_wait(&empty[s], (n - 1) & 1, abort_flag, p.status, kErrTimeoutEmpty))
                break;
            unsigned char *a_hi = smem + s * STAGE_BYTES;
            unsigned char *a_lo = a_hi + A_BYTES;
#pragma unroll
            for (int c = 0; c < 8; ++c) {   // 16-byte chunk c: modes 4c .. 4c+3
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int j = kb * 32 + c * 4 + q;
                    const float2 sj = j < p.n_modes ? __ldg(sv + j) : make_float2(0.f, 0.f);
                    const float2 v = cmulf(cur[c * 4 + q], sj);
                    Split<BF16>::run(v.x * kOperandScale, v.y * kOperandScale, hw[q], lw[q]);
                }
                const uint32_t phys = row_off + ((c ^ (r & 7)) << 4);
                *reinterpret_cast<uint4 *>(a_hi + phys) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(a_lo + phys) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            fence_proxy_async_smem();
            mbar_arrive(&full_a[s]);
#pragma unroll
            for (int q = 0; q < 32; ++q) cur[q] = nxt[q];
        }
    } else {
        // ---- epilogue: warps 0-3, TMEM lanes 32*warp .. +31 ----------------------
        const uint32_t lane_off = static_cast<uint32_t>(32 * warp) << 16;
        const int m = m0 + 32 * warp + lane;
        for (int c = 0; c < NC; ++c) {
            if (!mbar_wait(acc_full, c & 1, abort_flag, p.status, kErrTimeoutAcc)) break;
            tc_fence_after();
            if (c < NC - 1) {
                for (int g = 0; g < BN / 32; ++g) {
                    uint32_t a[32], t[32];
                    __syncwarp();
                    tmem_ld32(t_acc + lane_off + 32 * g, a);
                    if (c > 0) tmem_ld32(t_tot + lane_off + 32 * g, t);
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        t[i] = c > 0 ? __float_as_uint(__uint_as_float(t[i]) + __uint_as_float(a[i]))
                                     : a[i];
                    tmem_st32(t_tot + lane_off + 32 * g, t);
                }
                tmem_st_wait();
                tc_fence_before();
                mbar_arrive(acc_empty);
            } else {
                const bool row_ok = m < p.nm;
                double *orow = p.out + static_cast<int64_t>(b) * p.batch_stride +
                               static_cast<int64_t>(row_ok ? m : 0) * p.row_stride;
                for (int g = 0; g < BN / 32; ++g) {
                    uint32_t a[32], t[32];
                    __syncwarp();
                    tmem_ld32(t_acc + lane_off + 32 * g, a);
                    if (c > 0) tmem_ld32(t_tot + lane_off + 32 * g, t);
                    tmem_ld_wait();
                    const int gn0 = n0 + 32 * g;
                    if (row_ok && gn0 < p.ncn) {
#pragma unroll
                        for (int i = 0; i < 32; ++i) {
                            const int gn = gn0 + i;
                            if (gn < p.ncn) {
                                const float v = (c > 0 ? __uint_as_float(t[i]) + __uint_as_float(a[i])
                                                       : __uint_as_float(a[i])) * kProductUnscale;
                                const int comp = gn / p.nn;
                                orow[comp * p.comp_stride + (gn - comp * p.nn)] = f32_to_f64(v);
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kMmaWarp) tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------------------
// Exact-leading-term form ("f16x5").
//
// The f16x3 form above loses accuracy in the tensor core's FP32 accumulator,
// which truncates on every MMA instruction at the accumulator's magnitude.
// This form removes that error from the dominant product:
//   F (rows, |F| <= 1 after dividing s by W)  = F1 + F2 + F3
//   G (columns, |G| <= 1)                     = G1 + G2
// in units of 2^15:  F1 = 2^15 * rint(F * 2^(bF-1)) / 2^(bF-1)  (bF-bit integer grid),
//                    G1 = 2^15 * rint(G * 2^11) / 2^11           (12-bit integer grid),
// F2 = f16(F*2^15 - F1), F3 = f16(F*2^15 - F1 - F2), G2 = f16(G*2^15 - G1).
// Every product F1*G1 is an integer multiple of 2^(30-(bF-1)-11) ("counts");
// bF (3..9) is picked on the device (wnorm_block) so that six standard
// deviations of a random field stay below 2^23 counts; every partial sum of
// the "main" TMEM accumulator is then an FP32 integer and the accumulator
// adds them EXACTLY whatever the hardware rounding.  For any inputs this is
// checked as the sum runs: at every chunk boundary the main sum plus the
// most the next chunk's modes can add (the sum of |F1 G1| over them) must
// stay within 2^24 counts; inputs that break it (weights far from random,
// e.g. all in phase at a grid point) are flagged, and the caller recomputes
// them on the FP64 form or reports it.  The four cross products
// F2G1 + F1G2 + F2G2 + F3G1 (about 2^-bF of the field) go to a second TMEM
// accumulator that the workers drain every KC = 16 k-blocks (8 for the
// incompressible field) into FP32 totals held in registers, so their
// rounding never builds up at full magnitude.  The output is formed without
// any FP32 rounding at the field's magnitude: the exact main sum and the
// cross total are turned into one 32-bit integer of 1/64 counts (exact for
// the main sum) and that into FP64 with integer operations.  Representation: F to about 2^-(bF+22), G to 2^-24 relative
// (integers up to 2^11 are exact in f16, so 12 bits is the widest exact G
// grid; the exact main sum's budget fixes bF + bG, and G's single rest
// slice makes G the coarser factor); the product F3G2 (below 2^-28) is
// dropped.
//
// Warp roles (12 warps, 384 threads launched at 168 registers each, then
// re-split with setmaxnreg, X5Layout):
//   warps 0-7   workers: warp w builds the F1, F2, F3 slices of TMEM lanes
//               (rows) 32*(w%4).. for half the modes of each k-block, drains
//               columns HC*(w/4) .. +HC of the cross accumulator into
//               register totals, and writes the output in the epilogue
//   warp 8      bulk copies: G1, G2 and the tile's B rows per k-block
//   warp 9      MMA issuer and TMEM owner; warps 10-11 idle
// Stages: F1/F2/F3 3 x 8 KB + G1/G2 2 x BNX * 64 B + B rows 16 KB (72 KB
// for BNX = 256), three stages.
// ---------------------------------------------------------------------------
constexpr int X5_THREADS = 384;                 // 8 worker warps + 4 control warps
constexpr int X5_LAUNCH_REGS = 168;             // 65536 / 384, rounded down to 8
constexpr float kUnit = 32768.0f;            // 2^15
constexpr int kLeadBitsG = 12;               // G1 grid: 2^15 * rint(G * 2^11) / 2^11

// Sum over n modes of the largest leading product of each, in counts (see
// wnorm_block): leading grid 2^(bF-1), s1 = sum |w_j| / W over those modes.
__host__ __device__ __forceinline__ double x5_lead_bound(int bf, double s1, int64_t n) {
    return 2049.0 * (ldexp(1.0, bf - 1) * (1.0 + 0x1p-21) * s1 + 0.7072 * static_cast<double>(n));
}

// Normaliser and leading-grid width of the x5 form, one block of 256 threads:
//   W = 2^e > max |z1 - i z2|  (so |s / W| <= 1 and |F| <= 1),
//   the leading F grid 2^(bF-1) with bF (3..9) the largest for which six
//   standard deviations of the field, 6 sqrt(sum |w|^2 / 2) / W 2^(bF+10)
//   counts, stay below 2^23 counts (one bit under FP32's exact 2^24), and
//   no window of kc k-blocks can move a partial sum by more than 2^23 counts.
// Exactness for any inputs rests on a bound, checked while the sum runs:
// per mode j the leading product is at most
//     L(j) = 2049 (|w_j| / W (1 + 2^-21) 2^(bF-1) + 0.7072)  counts
// (|F| <= |w_j| up to FP32 rounding, |G| <= 1, each integer-grid rounding at
// most half a step per component), so a partial sum within a chunk of
// k-blocks moves at most by the chunk's sum of L(j).  l1kb[kb] holds that
// sum per k-block (rounded up); the kernel checks |main| + the next chunk's
// sum <= 2^24 at every chunk boundary and flags the call otherwise.  When
// even bF = 3 leaves a window above 2^23, bound_flag is set here and the
// GEMM skips its work; otherwise it is cleared (the GEMM may set it).
//   The s vector is stored unnormalised; the slicing constants absorb 1/W (a
//   power of two, so the slices are those of s / W bit for bit):
//   wnorm = {W, 1/W, 2^(bF-1) / W, 2^15 / 2^(bF-1), 2^15 / W, flag, 2^(bF-14), q},
//   an output value being (its 1/64-count integer) * 2^q, q = log2(W) - 16 - bF
__device__ void wnorm_block(const double *__restrict__ z1, const double *__restrict__ z2, int n,
                            int kbt, int kc, float *__restrict__ wnorm, float *__restrict__ l1kb,
                            int *__restrict__ bound_flag, int *__restrict__ bound_sticky) {
    __shared__ double red_max[256], red_sum[256];
    __shared__ float red_kb[256];
    __shared__ double s_W;
    __shared__ int s_bf;
    // one pass: largest |w|^2, sum of |w|^2, and per k-block the sum of |w|
    // rounded up (FP32, an upper bound), kept in l1kb until bF is known
    double m = 0.0, sum = 0.0;
    float mk = 0.f;
    for (int kb = threadIdx.x; kb < kbt; kb += blockDim.x) {
        float a1 = 0.f;
        for (int j = kb * 16; j < kb * 16 + 16 && j < n; ++j) {
            const double a = z1[j] * z1[j] + z2[j] * z2[j];
            m = fmax(m, a);
            sum += a;
            a1 = __fadd_ru(a1, __fsqrt_ru(__double2float_ru(a)));
        }
        l1kb[kb] = a1;
        mk = fmaxf(mk, a1);
    }
    red_max[threadIdx.x] = m;
    red_sum[threadIdx.x] = sum;
    red_kb[threadIdx.x] = mk;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red_max[threadIdx.x] = fmax(red_max[threadIdx.x], red_max[threadIdx.x + o]);
            red_sum[threadIdx.x] += red_sum[threadIdx.x + o];
            red_kb[threadIdx.x] = fmaxf(red_kb[threadIdx.x], red_kb[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int e = 0;
        const double mx = sqrt(red_max[0]);
        if (mx > 0.0 && isfinite(mx)) frexp(mx, &e);           // mx in [2^(e-1), 2^e)
        const double W = ldexp(1.0, e);
        s_W = W;
        const double typ = 6.0 * sqrt(fmax(red_sum[0], 1e-300) * 0.5) / W;
        // 2^(bF - 1 + kLeadBitsG - 1) * typ <= 2^23
        int bf = static_cast<int>(floor(23.0 + 2.0 - kLeadBitsG - log2(fmax(typ, 1.0))));
        bf = bf < 3 ? 3 : (bf > 9 ? 9 : bf);
        // no window of kc k-blocks may move a partial sum by more than 2^23 counts
        const double mkw = static_cast<double>(red_kb[0]) / W;
        auto window = [&](int b) { return kc * x5_lead_bound(b, mkw, 16); };
        while (bf > 3 && window(bf) > 8388608.0) --bf;
        const int over = (window(bf) > 8388608.0 || !isfinite(mkw)) ? 1 : 0;
        s_bf = bf;
        wnorm[0] = static_cast<float>(W);
        wnorm[1] = static_cast<float>(1.0 / W);
        wnorm[2] = static_cast<float>(ldexp(1.0, bf - 1) / W);      // lead scale of s
        wnorm[3] = kUnit / ldexpf(1.0f, bf - 1);                     // lead unit
        wnorm[4] = static_cast<float>(kUnit / W);                    // slice unit of s
        wnorm[5] = static_cast<float>(over);
        wnorm[6] = ldexpf(1.0f, bf - 14);                            // sum -> 1/64 counts
        wnorm[7] = static_cast<float>(e - 16 - bf);                  // 1/64 counts -> field: 2^q
        if (bound_flag) *bound_flag = over;
        if (bound_sticky && over) *bound_sticky = 1;
    }
    __syncthreads();
    const int bf = s_bf;
    const double W = s_W;
    for (int kb = threadIdx.x; kb < kbt; kb += blockDim.x) {
        const int cnt = min(16, n - kb * 16);
        // rounded up: the bound must not shrink in FP32
        l1kb[kb] = __double2float_ru(x5_lead_bound(bf, static_cast<double>(l1kb[kb]) / W, cnt) *
                                     (1.0 + 1e-6));
    }
}

// ---- FP32 factor tables of the x5 form ------------------------------------
// Per mode j (kRecX5 floats): kappa_d = k_d / 2 pi as hi, lo (d = 0..2), z1
// and z2 as hi, lo, the projector weights of the incompressible field
// (src/field.rs:138-152; 1 for the scalar field) as hi, lo.  Per axis point:
// x as hi, lo.  With these the tables need no FP64 arithmetic (cis_tab and
// compensated FP32 products), at the accuracy of the FP64 recipe.
constexpr int kRecX5 = 16;   // kh0-2 kl0-2 z1h z2h z1l z2l wh0-2 wl0-2

__global__ void __launch_bounds__(256) sep_x5_split_kernel(TabArgs t, int64_t n_ax) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < t.n_modes) {
        const int j = static_cast<int>(i);
        float *r = t.mrec + static_cast<int64_t>(j) * kRecX5;
        double k[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (d < t.dim) k[d] = t.cov[d * t.n_modes + j];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double kap = k[d] * kInv2Pi;
            const float hi = __double2float_rn(kap);
            r[d] = hi;
            r[3 + d] = __double2float_rn(kap - static_cast<double>(hi));
        }
        const double z1 = t.z1[j], z2 = t.z2[j];
        r[6] = __double2float_rn(z1);
        r[7] = __double2float_rn(z2);
        r[8] = __double2float_rn(z1 - static_cast<double>(r[6]));
        r[9] = __double2float_rn(z2 - static_cast<double>(r[7]));
        double w[3] = {1.0, 1.0, 1.0};
        if (t.incompr) {
            double kk = 0.0;
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (d < t.dim) kk = __dadd_rn(kk, __dmul_rn(k[d], k[d]));
            const double k_2 = __ddiv_rn(k[0], kk);
            w[0] = __dadd_rn(1.0, -__dmul_rn(k[0], k_2));
            w[1] = -__dmul_rn(k[1], k_2);
            w[2] = -__dmul_rn(k[2], k_2);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float h = __double2float_rn(w[c]);
            r[10 + c] = h;
            r[13 + c] = __double2float_rn(w[c] - static_cast<double>(h));
        }
        return;
    }
    const int64_t a = i - t.n_modes;
    if (a >= n_ax) return;
    double x;
    if (a < t.ax_off_m) x = t.ax_b[a];
    else if (a < t.ax_off_n) x = t.ax_m[a - t.ax_off_m];
    else x = t.ax_n[a - t.ax_off_n];
    const float hi = __double2float_rn(x);
    t.axs[a] = make_float2(hi, __double2float_rn(x - static_cast<double>(hi)));
}

// e^{i k x} for the mode component (kh, kl) (turns) and the axis point
// (xh, xl): FP32 pairs while |kappa x| < 2^22 turns, else the FP64
// reduction on k and x themselves.
__device__ __forceinline__ float2 cis_tab(float kh, float kl, float2 x, const double *k,
                                          const double *xd) {
    if (fabsf(kh * x.x) < 4194304.0f) return cis_turns_acc(kh, kl, x.x, x.y);
    return cis_f32(*k * *xd);
}

// a * b + c * d for FP32 pairs a, c (hi, lo) and FP32 b, d, to about half
// an FP32 ulp: exact products of the high parts, TwoSum, small terms added
__device__ __forceinline__ float dot2_pair(float ah, float al, float b, float ch, float cl, float d) {
    const float p1 = ah * b, e1 = fmaf(ah, b, -p1);
    const float p2 = ch * d, e2 = fmaf(ch, d, -p2);
    const float s = p1 + p2;
    const float bb = s - p1;
    const float es = (p1 - (s - bb)) + (p2 - bb);
    return s + (es + (e1 + e2) + fmaf(al, b, cl * d));
}

// s_a[j] = (z1_j - i z2_j) e^{i k_x,j X_a} (3-D) or z1_j - i z2_j (2-D), FP32;
// rows of sv_stride = 16 * k-blocks entries, zero past n_modes, so that the
// 16 modes of a k-block are one 128-byte block a bulk copy can move
__device__ __forceinline__ void svec_x5_entry(const TabArgs &t, int64_t i) {
    const int b = static_cast<int>(i / t.sv_stride), j = static_cast<int>(i % t.sv_stride);
    if (j >= t.n_modes) {
        t.svec[i] = make_float2(0.f, 0.f);
        return;
    }
    const float *r = t.mrec + static_cast<int64_t>(j) * kRecX5;
    float2 w = make_float2(__double2float_rn(t.z1[j]), __double2float_rn(-t.z2[j]));
    if (t.dim == 3) {
        const float2 e = cis_tab(r[0], r[3], t.axs[b], t.cov + j, t.ax_b + b);
        // (z1 - i z2) e with z1, z2 as FP32 pairs, rounded about once
        w = make_float2(dot2_pair(r[6], r[8], e.x, r[7], r[9], e.y),
                        dot2_pair(r[6], r[8], e.y, -r[7], -r[9], e.x));
    }
    t.svec[i] = w;
}

// B table of the x5 form: per k-block of 16 modes [nm rows][16 modes] float2,
// 128 bytes per row with the row's 16-byte chunk c (modes 2c, 2c+1) at
// position c ^ (m & 7): any run of consecutive rows is one contiguous block
// that a bulk copy moves into a stage unchanged, and eight consecutive rows
// read the same logical chunk from eight different bank groups.  i walks
// the stored layout (contiguous stores); modes past n_modes of the last
// k-block are zero.
__device__ __forceinline__ void btab_x5_entry(const TabArgs &t, int64_t i) {
    const int e = static_cast<int>(i & 15);
    const int64_t row = i >> 4;                      // kb * nm + m
    const int m = static_cast<int>(row % t.nm_ld);
    const int kb = static_cast<int>(row / t.nm_ld);
    const int j = kb * 16 + ((((e >> 1) ^ (m & 7)) << 1) | (e & 1));
    float2 v = make_float2(0.f, 0.f);
    if (m < t.nm && j < t.n_modes) {
        const float *r = t.mrec + static_cast<int64_t>(j) * kRecX5;
        v = cis_tab(r[t.km_dim], r[3 + t.km_dim], t.axs[t.ax_off_m + m],
                    t.cov + t.km_dim * t.n_modes + j, t.ax_m + m);
    }
    t.btab[i] = v;
}

// G table of the x5 form.  Element (component c, rows kGtabRows g .. of the
// column axis, mode j): the mode's record is read once for those rows.
// G1 on the 12-bit integer grid (units of 2^15 / 2^11 = 16), G2 the f16 rest;
// stored as contiguous stage blocks, one per (tile of t.bn rows, k-block of
// 16 modes), already in the 64-byte-swizzled K-major layout the MMA reads:
// row r at r * 64 bytes, 16-byte chunk c at c ^ ((r >> 1) & 3).
constexpr int kGtabRows = 2;
// groups of kGtabRows rows: ncomp * ceil(nn / kGtabRows) real ones, then the zero
// padding rows [ncomp * nn, ncn_pad)
__host__ __device__ __forceinline__ int64_t gtab_x5_groups(int ncomp, int nn, int ncn_pad) {
    const int64_t real = static_cast<int64_t>(ncomp) * ((nn + kGtabRows - 1) / kGtabRows);
    const int64_t pad = (ncn_pad - static_cast<int64_t>(ncomp) * nn + kGtabRows - 1) / kGtabRows;
    return real + (pad > 0 ? pad : 0);
}
__device__ __forceinline__ void gtab_x5_entry(const TabArgs &t, int64_t i) {
    const int half_k = t.k_pad / 2;
    const int ngrp = (t.nn + kGtabRows - 1) / kGtabRows;
    const int j = static_cast<int>(i % half_k);
    const int64_t gg = i / half_k;
    const int64_t nreal = static_cast<int64_t>(t.ncomp) * ngrp;
    int c, row0, nrows;
    if (gg < nreal) {
        c = static_cast<int>(gg / ngrp);
        const int n0 = static_cast<int>(gg % ngrp) * kGtabRows;
        row0 = c * t.nn + n0;
        nrows = min(kGtabRows, t.nn - n0);
    } else {
        c = t.ncomp;                                        // padding: zeros
        row0 = t.ncomp * t.nn + static_cast<int>(gg - nreal) * kGtabRows;
        nrows = min(kGtabRows, t.ncn_pad - row0);
    }
    const bool live = c < t.ncomp && j < t.n_modes;
    float pwh = 1.0f, pwl = 0.f, kh = 0.f, kl = 0.f;
    if (live) {
        const float *rec = t.mrec + static_cast<int64_t>(j) * kRecX5;
        if (t.incompr) {                       // projector weight (src/field.rs:138-152)
            pwh = rec[10 + c];
            pwl = rec[13 + c];
        }
        kh = rec[t.kn_dim];
        kl = rec[3 + t.kn_dim];
    }
    const float gs = static_cast<float>(1 << (kLeadBitsG - 1)), gu = kUnit / gs;
    const int kb = j / 16, jl = j % 16;
    for (int u = 0; u < nrows; ++u) {
        const int row = row0 + u;
        float re = 0.f, im = 0.f;
        if (live) {
            const int n = row - c * t.nn;
            const float2 e = cis_tab(kh, kl, t.axs[t.ax_off_n + n], t.cov + t.kn_dim * t.n_modes + j,
                                     t.ax_n + n);
            re = fmaf(pwh, e.x, pwl * e.x);
            im = -fmaf(pwh, e.y, pwl * e.y);
        }
        const float g1r = rintf(re * gs) * gu, g1i = rintf(im * gs) * gu;
        const __half2 h1 = __floats2half2_rn(g1r, g1i);
        const __half2 h2 = __floats2half2_rn(re * kUnit - g1r, im * kUnit - g1i);
        const int nt = row / t.bn, r = row % t.bn;
        const int64_t blk = (static_cast<int64_t>(nt) * t.kbt + kb) * (t.bn * 64);
        const int off = r * 64 + (((jl >> 2) ^ ((r >> 1) & 3)) << 4) + (jl & 3) * 4;
        const int64_t w = (blk + off) / 4;
        t.ghi[w] = *reinterpret_cast<const uint32_t *>(&h1);
        t.glo[w] = *reinterpret_cast<const uint32_t *>(&h2);
    }
}

// All tables of the x5 form in one launch: block 0 the normaliser, then
// blocks of G-table (several rows per thread: scheduled first), s-vector and
// B-table elements.
__global__ void __launch_bounds__(256)
sep_x5_tables_kernel(TabArgs t, int64_t n_svec, int64_t n_btab, int64_t n_gtab) {
    if (blockIdx.x == 0) {
        wnorm_block(t.z1, t.z2, t.n_modes, t.kbt, t.kc, t.wnorm, t.l1kb, t.bound_flag, t.bound_sticky);
        return;
    }
    int64_t i = static_cast<int64_t>(blockIdx.x - 1) * 256 + threadIdx.x;
    const int64_t b_gtab = (n_gtab + 255) / 256 * 256, b_svec = (n_svec + 255) / 256 * 256;
    if (i < b_gtab) {
        if (i < n_gtab) gtab_x5_entry(t, i);
        return;
    }
    i -= b_gtab;
    if (i < b_svec) {
        if (i < n_svec) svec_x5_entry(t, i);
        return;
    }
    i -= b_svec;
    if (i < n_btab) btab_x5_entry(t, i);
}

struct X5Params {
    TcParams base;
    const float *wnorm;      // see wnorm_block
    const float *l1kb;       // per k-block bound of the leading products, counts
    int *bound_flag;         // set to 1 when a partial sum could leave FP32's exact range
    int *bound_sticky;       // null, or set to 1 as well
    const unsigned char *g1, *g2, *bt;   // stage blocks (see the table kernels)
    // Tail split: tiles [0, full_tiles) run whole, one per CTA; each of the
    // n_split later tiles runs as ksplit CTAs (the launch's first n_split *
    // ksplit blocks) over consecutive parts of its k-blocks, whose
    // FP32 partials meet in `ws` ([slot][part][column][row]); the last part
    // to finish (counted in ws_cnt[slot]) adds them in part order and stores.
    int tile0;               // first tile of this launch (launches of wave-sized row ranges)
    int full_tiles, ksplit, n_split;
    float *ws;               // cross totals of the parts
    float *ws_main;          // exact main sums of the parts (same layout)
    int *ws_cnt;
    // 2 or 3: the output is written by tiled bulk stores through the kernel's
    // tensor map of that rank ((nn, rows) or (nn, rows, components));
    // 0: by plain stores
    int out_rank;
};

// Pipeline of the x5 kernel: k-blocks of 32 K elements (16 modes), three
// stages of 56 KB: F1 F2 F3 (128 rows x 64 B each) and G1 G2 (256 rows x
// 64 B, 64-byte swizzle), and a separate three-slot ring of B-table tiles
// (16 modes x 128 rows of float2, 16 KB), G and B moved by contiguous bulk
// copies from pre-tiled tables.  A B slot is refilled as soon as the workers
// have sliced it (three k-blocks ahead), not when the MMA releases the
// stage, so the slicing of a stage overlaps the copy of its G slices instead
// of following it.
//
// Warp roles (12 warps): warps 0-7 are "workers": worker warp w builds, for
// rows 32*(w%4) .. +31 of the F tile, the modes 8*(w/4) .. +7 of every
// k-block (two warps per SM sub-partition share the slicing work), and
// drains TMEM lanes 32*(w%4).., columns 128*(w/4) .. +128 of the cross
// accumulator into 128 FP32 registers; warp 8 issues the bulk copies,
// warp 9 the MMAs (and owns TMEM), warps 10-11 idle.  Workers drain a
// finished cross chunk whenever they find one, also while they wait for
// copies, so no wait of theirs can block the MMA that would release it.
constexpr int X5_BK = 32;
constexpr int X5_STAGES = 3;
constexpr int X5_BOX_OFF = 65536;   // epilogue: FP64 output boxes (2 x 8 warps x 2 x 4 KB)
constexpr int X5_F_BYTES = BM * X5_BK * 2;          // 8 KB
constexpr int X5_BT_BYTES = 16 * BM * 8;            // 16 KB
// s values staged beside each B tile: 16 modes (128 bytes) for each of the
// first X5_MAX_SL x-slices a tile's rows fall in
constexpr int X5_MAX_SL = 4;
constexpr int X5_BS_BYTES = X5_BT_BYTES + X5_MAX_SL * 128;   // one slot of the B ring
constexpr int X5_CHUNK = 16;                         // k-blocks per cross drain (256 modes)
// incompressible fields: the cross accumulator's truncation is the larger part
// of their error (the transverse components are small), so it is drained
// twice as often (about 3 % of the GEMM's time on 192^3 x 2048 modes)
constexpr int X5_CHUNK_INC = 8;
constexpr int kMaxSplit = 4;                         // most parts a tail tile is split into

// Stage layout for tiles of BNX output columns (256, or 192 where that pads
// the columns less, e.g. 3 x 192 components): every operand starts on a
// 1024-byte boundary, as the 64-byte swizzle and the bulk copies need.
template <int BNX>
struct X5Layout {
    static constexpr int G_BYTES = BNX * X5_BK * 2;      // 16 KB / 12 KB
    static constexpr int OFF_G1 = 3 * X5_F_BYTES;
    static constexpr int OFF_G2 = OFF_G1 + G_BYTES;
    static constexpr int STAGE = OFF_G2 + G_BYTES;       // 56 KB / 48 KB: F slices and G
    static constexpr int OFF_B = X5_STAGES * STAGE;      // the ring of B-table tiles and s
    static constexpr int DATA = OFF_B + X5_STAGES * X5_BS_BYTES;
    static constexpr size_t SMEM = DATA + 1024 + 256;
    static constexpr int HC = BNX / 2;                   // columns per worker half
    // setmaxnreg split: workers hold HC FP32 totals; the narrower tile leaves
    // the control warps room (chosen where ptxas reports no spills)
    static constexpr int WORK_REGS = BNX == 256 ? 216 : 200;
    static constexpr int CTRL_REGS = BNX == 256 ? 48 : 80;
    static_assert(4 * 32 * (2 * WORK_REGS + CTRL_REGS) <= X5_THREADS * X5_LAUNCH_REGS,
                  "setmaxnreg split exceeds the registers the block is launched with");
    static_assert(OFF_G2 % 1024 == 0 && OFF_B % 1024 == 0 && STAGE % 1024 == 0,
                  "stage operands must be 1024-byte aligned");
    static_assert(X5_BS_BYTES % 128 == 0 && DATA % 16 == 0, "B ring slots: 128-byte aligned");
    static_assert(DATA + 1024 + 256 <= 232448, "shared memory per block");
    static_assert(HC % 32 == 0 && BNX % 16 == 0 && BNX <= 256, "tile width");
    static_assert(8 * 32 * 33 * 4 <= X5_BOX_OFF && X5_BOX_OFF + 2 * 8 * 32 * 32 * 8 <= DATA,
                  "epilogue buffers must fit in the stage memory");
};
constexpr int kTmaWarpX5 = 8, kMmaWarpX5 = 9;

// three slices of a (re, im) pair in units of 2^15 (of v * ku / 2^15: the
// scales absorb the normaliser), packed as half2
__device__ __forceinline__ void slice3x2(float2 v, float ls, float lu, float ku, uint32_t &w1,
                                         uint32_t &w2, uint32_t &w3) {
    const float s1x = rintf(v.x * ls) * lu, s1y = rintf(v.y * ls) * lu;
    const float rx = fmaf(v.x, ku, -s1x), ry = fmaf(v.y, ku, -s1y);   // exact
    const __half2 h1 = __floats2half2_rn(s1x, s1y);
    const __half2 h2 = __floats2half2_rn(rx, ry);
    const float2 b2 = __half22float2(h2);
    const __half2 h3 = __floats2half2_rn(rx - b2.x, ry - b2.y);             // exact differences
    w1 = *reinterpret_cast<const uint32_t *>(&h1);
    w2 = *reinterpret_cast<const uint32_t *>(&h2);
    w3 = *reinterpret_cast<const uint32_t *>(&h3);
}

template <int BNX, bool SPLIT>
__global__ void __launch_bounds__(X5_THREADS, 1)
sep_x5_kernel(const __grid_constant__ CUtensorMap out_map, const X5Params xp) {
    using L = X5Layout<BNX>;
    const TcParams &p = xp.base;
    // inputs whose main sum could leave FP32's exact range are not computed
    // (the flag is the same for every CTA, so whole CTAs leave before any
    // barrier or TMEM allocation)
    if (xp.wnorm[5] != 0.f) return;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::DATA);
    uint64_t *full_t = bars;                    // [3] G copies -> MMA (1 arrival + bytes)
    uint64_t *full_a = bars + 3;                // [3] workers -> MMA (8 arrivals, one per warp)
    uint64_t *empty = bars + 6;                 // [3] MMA commit -> copy warp, workers
    uint64_t *cross_full = bars + 9;            // MMA commit -> workers (per chunk)
    uint64_t *cross_empty = bars + 10;          // workers -> MMA (8 arrivals)
    uint64_t *drain = bars + 11;
    uint64_t *main_read = bars + 12;            // workers -> MMA: main sum read (8 arrivals)
    uint64_t *b_full = bars + 13;               // [3] B copies -> workers (1 arrival + bytes)
    uint64_t *b_empty = bars + 16;              // [3] workers -> copy warp (8 arrivals)
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 19);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    volatile int *last_part = reinterpret_cast<volatile int *>(tmem_slot + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Rows are the nb * nm (x-slice, y) pairs taken in order, so a 128-row
    // tile may span two or more slices and no slice pads a partial tile.
    // a launch without split tiles compiles the split path out
    // the parts of split tiles come first, so that they finish early and the
    // SMs of the first wave do not all reach their epilogues at once
    const int u = static_cast<int>(blockIdx.x);
    const int n_parts = SPLIT ? xp.n_split * xp.ksplit : 0;
    const bool split = SPLIT && u < n_parts;
    const int tile = xp.tile0 + (split ? xp.full_tiles + u / xp.ksplit : u - n_parts);
    const int part = split ? u % xp.ksplit : 0;
    const int kbeg = split ? static_cast<int>(static_cast<int64_t>(part) * p.kb_total / xp.ksplit) : 0;
    const int KB = split ? static_cast<int>(static_cast<int64_t>(part + 1) * p.kb_total / xp.ksplit) - kbeg
                         : p.kb_total;          // k-blocks of this CTA
    const int nt = tile % p.n_tiles;
    const int64_t r0 = static_cast<int64_t>(tile / p.n_tiles) * BM;
    const int n0 = nt * BNX;
    const int rows_valid = static_cast<int>(min(static_cast<int64_t>(BM), p.rows_total - r0));
    const int KC = p.kc;
    const int NC = (KB + KC - 1) / KC;
    // Every tile walks the k-blocks from its own starting point, so the
    // CTAs of a wave do not all fetch the same table blocks at the same
    // moment; the sums do not depend on the order (the main sum is exact,
    // the rest is drained in chunks).
    const int rot = static_cast<int>((static_cast<int64_t>(blockIdx.x) * 97) % KB);
    auto kb_of = [&](int i) { const int t = i + rot; return kbeg + (t >= KB ? t - KB : t); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < X5_STAGES; ++s) {
            mbar_init(&full_t[s], 1);
            mbar_init(&full_a[s], 8);           // one arrival per worker warp
            mbar_init(&empty[s], 1);
            mbar_init(&b_full[s], 1);
            mbar_init(&b_empty[s], 8);
        }
        mbar_init(cross_full, 1);
        mbar_init(cross_empty, 8);
        mbar_init(drain, 1);
        mbar_init(main_read, 8);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarpX5) {
        tmem_alloc(tmem_slot, kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t t_main = tmem, t_cross = tmem + 256;

    if (warp >= 8) {
        regs_dec<L::CTRL_REGS>();
        if (warp == kTmaWarpX5 && lane == 0) {
            // ---- bulk copies: G1, G2, B-table block ----------------------------
            // the tile's runs of consecutive y rows (a run ends where the tile
            // crosses into the next x-slice) are the same for every k-block
            constexpr int kMaxRuns = 4;
            int run_r[kMaxRuns], run_m[kMaxRuns], run_len[kMaxRuns], n_runs = 0;
            {
                int r = 0, m = static_cast<int>(r0 % p.nm);
                while (r < rows_valid && n_runs < kMaxRuns) {
                    const int len = min(rows_valid - r, p.nm - m);
                    run_r[n_runs] = r;
                    run_m[n_runs] = m;
                    run_len[n_runs] = len;
                    ++n_runs;
                    r += len;
                    m = 0;
                }
                if (r < rows_valid) n_runs = -1;   // more runs (short y axis): computed per copy
            }
            // B rows of k-block i into ring slot i % X5_STAGES (one copy per
            // run), and after them the k-block's 16 s values of each of the
            // tile's first X5_MAX_SL x-slices (128-byte blocks of the padded
            // s rows)
            const int bs0 = static_cast<int>(r0 / p.nm);
            const int n_sl = min(X5_MAX_SL, static_cast<int>((r0 + rows_valid - 1) / p.nm) - bs0 + 1);
            auto copy_b = [&](int i) {
                const int sb = i % X5_STAGES, kb = kb_of(i);
                unsigned char *bd = smem + L::OFF_B + sb * X5_BS_BYTES;
                const unsigned char *bk = xp.bt + static_cast<int64_t>(kb) * p.nm * 128;
                mbar_arrive_expect_tx(&b_full[sb], rows_valid * 128 + n_sl * 128);
                for (int k = 0; k < n_sl; ++k)
                    bulk_copy_g2s(bd + X5_BT_BYTES + k * 128,
                                  p.svec + static_cast<int64_t>(bs0 + k) * p.sv_stride + kb * 16, 128,
                                  &b_full[sb]);
                if (n_runs >= 0) {
#pragma unroll
                    for (int k = 0; k < kMaxRuns; ++k)
                        if (k < n_runs)
                            bulk_copy_g2s(bd + run_r[k] * 128,
                                          bk + static_cast<int64_t>(run_m[k]) * 128,
                                          run_len[k] * 128, &b_full[sb]);
                } else {
                    for (int r = 0, m = static_cast<int>(r0 % p.nm); r < rows_valid; m = 0) {
                        const int len = min(rows_valid - r, p.nm - m);
                        bulk_copy_g2s(bd + r * 128, bk + static_cast<int64_t>(m) * 128, len * 128,
                                      &b_full[sb]);
                        r += len;
                    }
                }
            };
            int issued = 0, issued_b = 0;
            for (; issued_b < min(KB, X5_STAGES); ++issued_b) copy_b(issued_b);
            for (int i = 0; i < KB; ++i) {
                const int s = i % X5_STAGES, n = i / X5_STAGES, kb = kb_of(i);
                if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1, abort_flag, p.status,
                                        kErrTimeoutEmpty))
                    break;
                unsigned char *st = smem + s * L::STAGE;
                const int64_t gblk = (static_cast<int64_t>(nt) * p.kb_total + kb) * L::G_BYTES;
                mbar_arrive_expect_tx(&full_t[s], 2 * L::G_BYTES);
                bulk_copy_g2s(st + L::OFF_G1, xp.g1 + gblk, L::G_BYTES, &full_t[s]);
                bulk_copy_g2s(st + L::OFF_G2, xp.g2 + gblk, L::G_BYTES, &full_t[s]);
                ++issued;
                // B slot of k-block i, refilled with k-block i + 3 once the
                // workers have sliced k-block i
                if (issued_b < KB) {
                    if (!mbar_wait(&b_empty[s], n & 1, abort_flag, p.status, kErrTimeoutEmpty))
                        break;
                    copy_b(issued_b++);
                }
            }
            if (*abort_flag) {
                for (int i = issued > X5_STAGES ? issued - X5_STAGES : 0; i < issued; ++i)
                    mbar_wait_drain(&full_t[i % X5_STAGES], (i / X5_STAGES) & 1, p.status);
                for (int i = issued_b > X5_STAGES ? issued_b - X5_STAGES : 0; i < issued_b; ++i)
                    mbar_wait_drain(&b_full[i % X5_STAGES], (i / X5_STAGES) & 1, p.status);
            }
        } else if (warp == kMmaWarpX5 && lane == 0) {
            // ---- MMA ---------------------------------------------------------
            const uint32_t idesc = idesc_f16(BM, BNX, false);
            bool ok = true;
            for (int i = 0; i < KB; ++i) {
                const int s = i % X5_STAGES, n = i / X5_STAGES;
                const int c = i / KC;
                const bool first = (i % KC) == 0;
                const bool last = (i % KC) == KC - 1 || i == KB - 1;
                ok = mbar_wait(&full_t[s], n & 1, abort_flag, p.status, kErrTimeoutFull);
                if (ok) ok = mbar_wait(&full_a[s], n & 1, abort_flag, p.status, kErrTimeoutFull);
                if (!ok) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + s * L::STAGE);
                const uint32_t f1 = sa, f2 = sa + X5_F_BYTES, f3 = sa + 2 * X5_F_BYTES;
                const uint32_t g1 = sa + L::OFF_G1, g2 = sa + L::OFF_G2;
                // At a chunk boundary the cross MMAs go first, once the
                // workers have drained the last chunk; the main MMAs follow
                // once they have also read the main sum, a read that overlaps
                // those cross MMAs (other TMEM columns).
                const bool boundary = first && c > 0;
                if (boundary) {
                    ok = mbar_wait(cross_empty, (c - 1) & 1, abort_flag, p.status, kErrTimeoutAcc);
                    if (!ok) break;
                    tc_fence_after();
                }
#pragma unroll
                for (int kk = 0; kk < X5_BK / 16; ++kk) {
                    const uint32_t o = kk * 32;
                    mma_f16_ss(t_cross, desc_k_sw64(f2 + o), desc_k_sw64(g1 + o), idesc,
                               (first && kk == 0) ? 0u : 1u);
                    mma_f16_ss(t_cross, desc_k_sw64(f1 + o), desc_k_sw64(g2 + o), idesc, 1u);
                    mma_f16_ss(t_cross, desc_k_sw64(f2 + o), desc_k_sw64(g2 + o), idesc, 1u);
                    mma_f16_ss(t_cross, desc_k_sw64(f3 + o), desc_k_sw64(g1 + o), idesc, 1u);
                }
                if (boundary) {
                    ok = mbar_wait(main_read, (c - 1) & 1, abort_flag, p.status, kErrTimeoutAcc);
                    if (!ok) break;
                    tc_fence_after();
                }
#pragma unroll
                for (int kk = 0; kk < X5_BK / 16; ++kk) {
                    const uint32_t o = kk * 32;
                    mma_f16_ss(t_main, desc_k_sw64(f1 + o), desc_k_sw64(g1 + o), idesc,
                               (i > 0 || kk > 0) ? 1u : 0u);
                }
                mma_commit(&empty[s]);
                if (last) mma_commit(cross_full);
            }
            if (!ok) {
                mma_commit(drain);
                mbar_wait_drain(drain, 0, p.status);
            }
        }
    } else {
        regs_inc<L::WORK_REGS>();
        // ---- workers: F-tile slices, cross drains, final epilogue -----------------
        const int q = warp & 3, h = warp >> 2;
        const int r = 32 * q + lane;                            // F row and TMEM lane
        const uint32_t lane_off = static_cast<uint32_t>(32 * q) << 16;
        const bool row_ok = r < rows_valid;
        const int64_t grow = row_ok ? r0 + r : 0;               // (x-slice, y) of the row
        const int bsl = static_cast<int>(grow / p.nm), mrow = static_cast<int>(grow % p.nm);
        const float2 *sv = p.svec + static_cast<int64_t>(bsl) * p.sv_stride;
        // byte offsets, in this row's 128-byte B line, of the four 16-byte
        // chunks (modes 8h .. 8h+7) the thread reads: chunk c sits at c ^ (m & 7)
        const uint32_t bswz = static_cast<uint32_t>(mrow & 7);
        const uint32_t boff[4] = {((4 * h + 0) ^ bswz) << 4, ((4 * h + 1) ^ bswz) << 4,
                                  ((4 * h + 2) ^ bswz) << 4, ((4 * h + 3) ^ bswz) << 4};
        const uint32_t row_off = r * 64;                        // 64-byte rows
        const uint32_t swz = (r >> 1) & 3;                      // 64-byte swizzle phase
        const float ls = xp.wnorm[2], lu = xp.wnorm[3], ku = xp.wnorm[4];
        float tot[L::HC];
#pragma unroll
        for (int i = 0; i < L::HC; ++i) tot[i] = 0.f;
        int pend = 0;                                           // next cross chunk to drain
        // main-sum limit for the chunk after chunk c, in accumulator units:
        // 2^24 counts less the most that chunk's leading products can add
        const float cnt_unit = xp.wnorm[3] * 16.0f;             // 2^(20-bF)
        auto main_limit = [&](int c) -> float {
            float l1 = 0.f;
            const int i1 = min(KB, (c + 2) * KC);
#pragma unroll 1
            for (int i = (c + 1) * KC; i < i1; ++i) l1 = __fadd_ru(l1, __ldg(xp.l1kb + kb_of(i)));
            return (16777216.0f - l1) * cnt_unit;
        };
        auto drain_chunk = [&]() {
            tc_fence_after();
            // the cross chunk first (two loads in flight per wait): the next
            // chunk's cross MMAs start once every worker has drained it
#pragma unroll
            for (int g = 0; g < L::HC / 32; ++g) {
                uint32_t v[16], w[16];
                __syncwarp();
                tmem_ld16(t_cross + lane_off + L::HC * h + 32 * g, v);
                tmem_ld16(t_cross + lane_off + L::HC * h + 32 * g + 16, w);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    tot[32 * g + i] += __uint_as_float(v[i]);
                    tot[32 * g + 16 + i] += __uint_as_float(w[i]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(cross_empty);
            // then the main sums at the boundary, while those cross MMAs run:
            // the next chunk's main MMAs start once every worker has read them
            float mmax = 0.f;
#pragma unroll 1
            for (int g = 0; g < L::HC / 16; ++g) {
                uint32_t v[16];
                __syncwarp();
                tmem_ld16(t_main + lane_off + L::HC * h + 16 * g, v);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 16; ++i) mmax = fmaxf(mmax, fabsf(__uint_as_float(v[i])));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(main_read);
            // the main sum at this chunk boundary plus the next chunk's bound
            // must stay within 2^24 counts.  Rows past the grid are skipped
            // (their zero s factors meet stale B data, possibly NaN); a NaN
            // sum (NaN inputs) passes and leaves as NaN
            if (row_ok && mmax > main_limit(pend)) {
                *xp.bound_flag = 1;
                if (xp.bound_sticky) *xp.bound_sticky = 1;
            }
            ++pend;
        };
        // Decisions that lead to a warp-collective TMEM load are taken by the
        // whole warp: a barrier counts as passed once every lane has seen it.
        auto warp_passed = [&](uint64_t *bar, uint32_t parity) {
            return __all_sync(0xffffffffu, mbar_try_wait(bar, parity));
        };
        // drains every finished, not yet drained chunk except the last one
        // (a non-blocking probe: most polls find nothing to drain)
        auto poll_drain = [&]() {
            while (pend < NC - 1 && __all_sync(0xffffffffu, mbar_test_wait(cross_full, pend & 1)))
                drain_chunk();
        };
        // waits (bounded) for the chunk being drained next or the final commit
        auto wait_chunk = [&](int c) -> bool {
            const bool got = mbar_wait(cross_full, c & 1, abort_flag, p.status, kErrTimeoutAcc);
            return __all_sync(0xffffffffu, got);
        };
        // k-block i may be sliced once its B tile has arrived and the MMA has
        // released the F slices of stage s (k-block i - 3)
        auto stage_ready = [&](int s, int n) {
            return warp_passed(&b_full[s], n & 1) && (n == 0 || warp_passed(&empty[s], (n - 1) & 1));
        };
        // waits for stage s, draining chunks meanwhile; false on timeout/abort
        auto wait_stage = [&](int s, int n) -> bool {
            if (stage_ready(s, n)) return true;
            const uint64_t t0 = globaltimer_ns();
            for (uint32_t it = 1;; ++it) {
                poll_drain();
                if (stage_ready(s, n)) return true;
                if ((it & 63) == 0) {
                    int stop = *abort_flag ? 1 : (globaltimer_ns() - t0 > kWaitLimitNs ? 2 : 0);
                    stop = __shfl_sync(0xffffffffu, stop, 0);
                    if (stop == 2 && lane == 0) {
                        *abort_flag = 1;
                        atomicCAS(p.status, 0, kErrTimeoutFull);
                    }
                    if (stop) return false;
                }
            }
        };
        // this row's x-slice among the tile's staged ones; rows of a later
        // slice (y axes shorter than 32) read their s values from the table
        const int sl = bsl - static_cast<int>(r0 / p.nm);
        bool ok = true;
        for (int i = 0; i < KB; ++i) {
            const int s = i % X5_STAGES, n = i / X5_STAGES;
            if (!wait_stage(s, n)) {
                ok = false;
                break;
            }
            unsigned char *st = smem + s * L::STAGE;
            const unsigned char *bslot = smem + L::OFF_B + s * X5_BS_BYTES;
            const unsigned char *brow = bslot + r * 128;
            float2 sj[8];
            if (!row_ok) {
#pragma unroll
                for (int t = 0; t < 8; ++t) sj[t] = make_float2(0.f, 0.f);
            } else if (sl < X5_MAX_SL) {
                const float4 *sp = reinterpret_cast<const float4 *>(bslot + X5_BT_BYTES + sl * 128 + 64 * h);
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float4 v = sp[t];
                    sj[2 * t] = make_float2(v.x, v.y);
                    sj[2 * t + 1] = make_float2(v.z, v.w);
                }
            } else {
                const int j0 = kb_of(i) * 16 + 8 * h;      // padded rows: zero past n_modes
#pragma unroll
                for (int t = 0; t < 8; ++t) sj[t] = __ldg(sv + j0 + t);
            }
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {          // 16-byte chunks 2h, 2h+1: modes 4c .. 4c+3
                const int c = 2 * h + cc;
                uint32_t w1[4], w2[4], w3[4];
                // B modes 4c .. 4c+3 of this row: table chunks 2c and 2c+1
                const float4 b01 = *reinterpret_cast<const float4 *>(brow + boff[2 * cc]);
                const float4 b23 = *reinterpret_cast<const float4 *>(brow + boff[2 * cc + 1]);
                const float2 bv[4] = {make_float2(b01.x, b01.y), make_float2(b01.z, b01.w),
                                      make_float2(b23.x, b23.y), make_float2(b23.z, b23.w)};
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    // rows past the grid hold stale B data; their s factors are
                    // zero and their output rows are never stored
                    const float2 v = cmulf(bv[t], sj[4 * cc + t]);
                    slice3x2(v, ls, lu, ku, w1[t], w2[t], w3[t]);
                }
                const uint32_t phys = row_off + ((c ^ swz) << 4);
                *reinterpret_cast<uint4 *>(st + phys) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
                *reinterpret_cast<uint4 *>(st + X5_F_BYTES + phys) =
                    make_uint4(w2[0], w2[1], w2[2], w2[3]);
                *reinterpret_cast<uint4 *>(st + 2 * X5_F_BYTES + phys) =
                    make_uint4(w3[0], w3[1], w3[2], w3[3]);
            }
            // every thread's slices are visible to the MMA's async proxy,
            // then one lane per warp arrives for the warp
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&full_a[s]);
                mbar_arrive(&b_empty[s]);
            }
            poll_drain();
        }
        // remaining non-final chunks, then the final one (it follows every MMA)
        while (ok && pend < NC - 1) {
            ok = wait_chunk(pend);
            if (ok) drain_chunk();
        }
        if (ok) ok = wait_chunk(NC - 1);
        // ---- epilogue ------------------------------------------------------
        // Every MMA has completed, so the stage buffers are free.  A warp's
        // 32 rows x 32 columns of FP32 sums are converted to FP64 into
        // swizzled boxes in shared memory and written by tiled bulk stores;
        // where the output layout does not allow those, they are turned
        // around in shared memory and each lane stores one column.
        // Each output leaves as a 32-bit integer of 1/64 counts: the exact main
        // sum times 64 (below 2^30 by the leading-grid bound) plus the cross
        // total rounded to 1/64 count, summed as integers; it becomes FP64 by
        // integer operations (i32_to_f64_pow2) with the scale 2^q folded into
        // the exponent.  No FP32 rounding at the field's magnitude remains.
        const float to_t = xp.wnorm[6];
        const int qexp = static_cast<int>(xp.wnorm[7]);
        // a NaN or infinite sum (NaN inputs) leaves as the sentinel -2^31,
        // which no finite sum reaches (|main| < 2^30, the cross total far less)
        auto fixed = [&](float mainv, float crossv) -> float {
            const bool finite = fabsf(mainv) <= 3.0e38f && fabsf(crossv) <= 3.0e38f;
            return __int_as_float(finite ? __float2int_rn(mainv * to_t) + __float2int_rn(crossv * to_t)
                                         : static_cast<int>(0x80000000u));
        };
        auto to_f64 = [&](float bits) -> double { return i32_to_f64_pow2(__float_as_int(bits), qexp); };
        float *trf = reinterpret_cast<float *>(smem) + warp * (32 * 33);
        // output offset of row (warp's first row) + R; the warp's first row
        // is slice bs0, row ms0
        auto out_row = [&](int bs0, int ms0, int R) -> int64_t {
            int ms = ms0 + R, bs = bs0;
            while (ms >= p.nm) {
                ms -= p.nm;
                ++bs;
            }
            return static_cast<int64_t>(bs) * p.batch_stride + static_cast<int64_t>(ms) * p.row_stride;
        };
        // column group g: tot[32g .. 32g+31] += the cross accumulator's last
        // chunk, then each main sum with its cross total goes to `use` (in
        // halves of 16, to keep registers free)
        auto read_group = [&](int g, auto &&use) {
            uint32_t v[32];
            __syncwarp();
            tmem_ld32(t_cross + lane_off + L::HC * h + 32 * g, v);
            tmem_ld_wait();
#pragma unroll
            for (int t = 0; t < 32; ++t) tot[32 * g + t] += __uint_as_float(v[t]);
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                uint32_t mv[16];
                tmem_ld16(t_main + lane_off + L::HC * h + 32 * g + 16 * hf, mv);
                tmem_ld_wait();
#pragma unroll
                for (int t = 0; t < 16; ++t) use(32 * g + 16 * hf + t, __uint_as_float(mv[t]));
            }
        };
        auto store_group = [&](int g) {
            const int rows = max(0, min(32, rows_valid - 32 * q));
            const int64_t rq = r0 + 32 * q;
            const int gc = n0 + L::HC * h + 32 * g;              // first column of the group
            if (xp.out_rank > 0) {
                // Two boxes of 16 columns x 32 rows per warp and group, FP64,
                // in the 128-byte swizzled layout of the tensor map: this
                // thread's row is 128 bytes, its 16-byte pair c of columns
                // sits at chunk c ^ (row & 7), so a warp's 16-byte stores
                // meet no bank conflict.  Two buffers alternate by group;
                // rows and columns past the output are clipped by the copy.
                unsigned char *bx = smem + X5_BOX_OFF + (static_cast<size_t>(g & 1) * 8 + warp) * 8192;
                if (lane == 0) bulk_wait_read<1>();     // the buffer's previous stores have read it
                __syncwarp();
#pragma unroll
                for (int hb = 0; hb < 2; ++hb)
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const int t = 32 * g + 16 * hb + 2 * c;
                        *reinterpret_cast<double2 *>(bx + hb * 4096 + lane * 128 + ((c ^ (lane & 7)) << 4)) =
                            make_double2(to_f64(tot[t]), to_f64(tot[t + 1]));
                    }
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0 && rows > 0 && gc < p.ncn) {
                    const int comp = gc / p.nn;
                    const int32_t x = gc - comp * p.nn, y = static_cast<int32_t>(rq);
#pragma unroll
                    for (int hb = 0; hb < 2; ++hb) {
                        if (x + 16 * hb >= p.nn) break;
                        if (xp.out_rank == 3)
                            tma_store_3d(&out_map, bx + hb * 4096, x + 16 * hb, y, comp);
                        else
                            tma_store_2d(&out_map, bx + hb * 4096, x + 16 * hb, y);
                    }
                    bulk_commit();
                }
            } else {
                // transposed through shared memory (pitch 33 floats), one
                // column per lane: 256 contiguous bytes per row and store
                __syncwarp();
#pragma unroll
                for (int t = 0; t < 32; ++t) trf[lane * 33 + t] = tot[32 * g + t];
                __syncwarp();
                const int gn = gc + lane;
                const int bs0 = static_cast<int>(rq / p.nm), ms0 = static_cast<int>(rq % p.nm);
                if (gn < p.ncn) {
                    const int comp = gn / p.nn;
                    double *oc = p.out + comp * p.comp_stride + (gn - comp * p.nn);
                    for (int R = 0; R < rows; ++R) oc[out_row(bs0, ms0, R)] = to_f64(trf[R * 33 + lane]);
                }
            }
        };
        if (!split) {
            if (ok) {
                tc_fence_after();
#pragma unroll
                for (int g = 0; g < L::HC / 32; ++g) {
                    read_group(g, [&](int c, float mainv) { tot[c] = fixed(mainv, tot[c]); });
                    store_group(g);
                }
                __syncwarp();
            }
        } else if (SPLIT) {
            // a split tile: write this part's main sums and cross totals,
            // count the parts, and the last part adds all of them in part
            // order (the result does not depend on which part finishes
            // last; the main sums add exactly), then stores as above
            const int slot = tile - xp.tile0 - xp.full_tiles, ks = xp.ksplit;
            const int64_t slot_off = static_cast<int64_t>(slot) * ks * BNX * BM;
            // this thread's column c of part k sits at col0[(k * BNX + c) * BM]
            const int64_t c_off = static_cast<int64_t>(L::HC * h) * BM + r;
            float *col0 = xp.ws + slot_off + c_off;
            float *colm = xp.ws_main + slot_off + c_off;
            if (ok) {
                tc_fence_after();
                float *wm = colm + static_cast<int64_t>(part) * BNX * BM;
#pragma unroll
                for (int g = 0; g < L::HC / 32; ++g)
                    read_group(g, [&](int c, float mainv) { wm[c * BM] = mainv; });
                float *wp = col0 + static_cast<int64_t>(part) * BNX * BM;
#pragma unroll
                for (int c = 0; c < L::HC; ++c) wp[c * BM] = tot[c];
            }
            __threadfence();
            asm volatile("bar.sync 1, 256;" ::: "memory");      // the 256 worker threads
            if (threadIdx.x == 0)
                *last_part = (!*abort_flag && atomicAdd(xp.ws_cnt + slot, 1) == ks - 1) ? 1 : 0;
            asm volatile("bar.sync 1, 256;" ::: "memory");
            if (ok && *last_part) {
                __threadfence();
                if (threadIdx.x == 0) xp.ws_cnt[slot] = 0;          // ready for the next launch
                // every part (this one included) is read back from the
                // workspace, so the sums need no second register array; the
                // parts' main sums add exactly while the running total stays
                // within 2^24 counts
                const float lim = 16777216.0f * cnt_unit;
                bool over = false;
#pragma unroll
                for (int c = 0; c < L::HC; ++c) {
                    float a = __ldcg(col0 + c * BM), mm = __ldcg(colm + c * BM);
#pragma unroll
                    for (int k = 1; k < kMaxSplit; ++k)
                        if (k < ks) {
                            a += __ldcg(col0 + (k * BNX + c) * BM);
                            mm += __ldcg(colm + (k * BNX + c) * BM);
                            over = over || fabsf(mm) > lim;
                        }
                    tot[c] = fixed(mm, a);
                }
                if (over && row_ok) {
                    *xp.bound_flag = 1;
                    if (xp.bound_sticky) *xp.bound_sticky = 1;
                }
#pragma unroll
                for (int g = 0; g < L::HC / 32; ++g) store_group(g);
                __syncwarp();
            }
        }
    }

    // the tensor stores have read their boxes before shared memory is released
    if (xp.out_rank > 0 && warp < 8 && lane == 0) bulk_wait_read<0>();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kMmaWarpX5) tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiledFn *out) {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                               cudaEnableDefault, &q);
        if (err == cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    if (!fn) return set_error(GSC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    *out = fn;
    return GSC_OK;
}

// 2-D tiled tensor map: `inner` elements per row (contiguous), `rows` rows,
// box (box_inner, box_rows).
int make_map(CUtensorMap *map, void *base, CUtensorMapDataType dtype, int elem_bytes, int inner,
             int rows, int box_inner, int box_rows, CUtensorMapSwizzle swizzle) {
    EncodeTiledFn fn;
    GSC_TRY(encode_fn(&fn));
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(inner), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(inner) * elem_bytes};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_inner), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, dtype, 2, base, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GSC_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return GSC_OK;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

template <bool BF16>
int configure_tc() {
    return smem_attr(reinterpret_cast<const void *>(sep_tc_kernel<BF16>), kSmemBytes);
}

}  // namespace

namespace {
// Set-up of an x5 instantiation on the current device (once per device).
// The warps re-balance their registers with setmaxnreg; the increases can
// only be served from what the block was launched with, so a build that
// launches with fewer registers must not run.
template <int BNX, bool SPLIT>
int configure_x5() {
    int device = 0;
    GSC_CUDA(cudaGetDevice(&device));
    const void *fn = reinterpret_cast<const void *>(sep_x5_kernel<BNX, SPLIT>);
    return once_per_device(fn, device, [fn]() -> int {
        cudaFuncAttributes fa{};
        GSC_CUDA(cudaFuncGetAttributes(&fa, fn));
        if (fa.numRegs * X5_THREADS <
            4 * 32 * (2 * X5Layout<BNX>::WORK_REGS + X5Layout<BNX>::CTRL_REGS))
            return set_error(GSC_ERR_KERNEL, "x5 kernel built with too few registers per thread");
        GSC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(X5Layout<BNX>::SMEM)));
        return GSC_OK;
    });
}
}  // namespace

int sep_tc_run(DeviceCtx &ctx, const SepArgs &a, cudaStream_t st) {
    const bool x5 = a.form == GSC_FORM_SEP_F16X5;
    const bool bf16 = a.form == GSC_FORM_SEP_BF16X3;
    if (x5 && !a.bound_flag) return set_error(GSC_ERR_INVALID, "sep_f16x5 needs a bound flag word");
    const int dim = static_cast<int>(a.dim);
    const int N = static_cast<int>(a.n_modes);
    const int ncomp = a.incompr ? dim : 1;
    const int nb = dim == 3 ? static_cast<int>(a.n[0]) : 1;
    const int nm = static_cast<int>(dim == 3 ? a.n[1] : a.n[0]);
    const int nn = static_cast<int>(dim == 3 ? a.n[2] : a.n[1]);
    const int64_t P = static_cast<int64_t>(nb) * nm * nn;
    if (P == 0) return GSC_OK;
    const int bk = x5 ? X5_BK : BK;
    const int KB = std::max(1, (2 * N + bk - 1) / bk);
    const int k_pad = KB * bk;
    const int ncn = ncomp * nn;
    const int nm_ld = x5 ? nm : (nm + 15) / 16 * 16;
    // x5 tile width: 256 columns, or 192 where that pads the columns less
    // (e.g. three 192-point components: 576 columns in 3 tiles, not 768)
    const int bnx = (x5 && (ncn + 191) / 192 * 192 < (ncn + 255) / 256 * 256) ? 192 : BN;
    const int n_tiles = (ncn + bnx - 1) / bnx;
    const int ncn_pad = n_tiles * bnx;
    // x5 tiles the nb * nm (slice, row) pairs as one row range
    const int64_t rows_total = static_cast<int64_t>(nb) * nm;
    const int m_tiles = x5 ? static_cast<int>((rows_total + BM - 1) / BM) : (nm + BM - 1) / BM;

    // x5 launches: all row tiles at once, or (with a row hook) one launch per
    // wave of whole row tiles.  Tail split: the tiles of an incomplete last
    // wave run as ksplit CTAs each over a share of the k-blocks, when that
    // shortens the schedule.
    struct Launch {
        int64_t m0, m1, full_tiles, n_split;
        int ksplit;
    };
    std::vector<Launch> launches;
    int64_t n_split = 0;          // most split tiles of any launch
    int ksplit = 1;               // and their most parts
    if (x5) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device) != cudaSuccess ||
            sms <= 0) {
            cudaGetLastError();
            sms = 152;
        }
        const int64_t per = (a.on_rows && static_cast<int64_t>(m_tiles) * n_tiles > sms)
                                ? std::max<int64_t>(1, sms / n_tiles)
                                : m_tiles;
        for (int64_t m0 = 0; m0 < m_tiles; m0 += per) {
            Launch l;
            l.m0 = m0;
            l.m1 = std::min<int64_t>(m_tiles, m0 + per);
            const int64_t tiles = (l.m1 - l.m0) * n_tiles;
            l.full_tiles = tiles;
            l.n_split = 0;
            l.ksplit = 1;
            const int64_t waves = tiles / sms, rem = tiles % sms;
            double best = static_cast<double>(waves + (rem > 0 ? 1 : 0));
            for (int k = 2; k <= kMaxSplit && rem > 0 && KB / k >= 8; ++k) {
                // a part costs 1/k of a tile plus ~5 % for its partial traffic
                const double span = waves + std::ceil(static_cast<double>(rem * k) / sms) / k * 1.05;
                if (span < best - 1e-9) {
                    best = span;
                    l.ksplit = k;
                }
            }
            if (l.ksplit > 1) {
                l.full_tiles = tiles - rem;
                l.n_split = rem;
                n_split = std::max(n_split, rem);
                ksplit = std::max(ksplit, l.ksplit);
            }
            launches.push_back(l);
        }
    }

    // scratch: normaliser, svec, btab, G hi (G1), G lo (G2), split partials
    const size_t off_wn = 0;
    const size_t off_svec = 1024;
    const int64_t sv_stride = x5 ? static_cast<int64_t>(KB) * 16 : N;
    const size_t off_btab = align_up(off_svec + sizeof(float2) * nb * static_cast<size_t>(sv_stride), 1024);
    const size_t bt_modes = x5 ? static_cast<size_t>(KB) * 16 : static_cast<size_t>(N);
    const size_t off_ghi = align_up(off_btab + sizeof(float2) * bt_modes * nm_ld, 1024);
    const size_t g_bytes = static_cast<size_t>(ncn_pad) * k_pad * 2;
    const size_t off_glo = align_up(off_ghi + g_bytes, 1024);
    const size_t off_ws = align_up(off_glo + g_bytes, 1024);
    // cross totals and exact main sums of the split parts
    const size_t ws_half = static_cast<size_t>(n_split) * ksplit * bnx * BM * sizeof(float);
    const size_t ws_bytes = 2 * ws_half;
    const size_t off_cnt = align_up(off_ws + ws_bytes, 1024);
    // x5: FP32 mode records and axis splits for the tables
    const int ax_off_m = dim == 3 ? nb : 0, ax_off_n = ax_off_m + nm;
    const int64_t n_ax = static_cast<int64_t>(ax_off_n) + nn;
    const size_t off_l1 = align_up(off_cnt + static_cast<size_t>(n_split) * sizeof(int), 256);
    const size_t off_mrec = align_up(off_l1 + (x5 ? sizeof(float) * static_cast<size_t>(KB) : 0), 1024);
    const size_t off_axs = align_up(off_mrec + (x5 ? sizeof(float) * kRecX5 * static_cast<size_t>(N) : 0), 1024);
    const size_t total = off_axs + (x5 ? sizeof(float2) * static_cast<size_t>(n_ax) : 0) + 256;
    GSC_TRY(ensure_dev(ctx, ctx.scratch, total));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    unsigned char *base = static_cast<unsigned char *>(ctx.scratch.ptr);
    int *status = a.status;

    TabArgs t;
    t.cov = a.cov;
    t.z1 = a.z1;
    t.z2 = a.z2;
    t.dim = dim;
    t.n_modes = N;
    t.ax_b = dim == 3 ? a.axis[0] : nullptr;
    t.ax_m = dim == 3 ? a.axis[1] : a.axis[0];
    t.ax_n = dim == 3 ? a.axis[2] : a.axis[1];
    t.kb_dim = 0;
    t.km_dim = dim == 3 ? 1 : 0;
    t.kn_dim = dim == 3 ? 2 : 1;
    t.nb = nb;
    t.nm = nm;
    t.nn = nn;
    t.ncomp = ncomp;
    t.incompr = a.incompr ? 1 : 0;
    t.k_pad = k_pad;
    t.nm_ld = nm_ld;
    t.ncn_pad = ncn_pad;
    t.svec = reinterpret_cast<float2 *>(base + off_svec);
    t.sv_stride = sv_stride;
    t.btab = reinterpret_cast<float2 *>(base + off_btab);
    t.ghi = reinterpret_cast<uint32_t *>(base + off_ghi);
    t.glo = reinterpret_cast<uint32_t *>(base + off_glo);
    t.wnorm = x5 ? reinterpret_cast<float *>(base + off_wn) : nullptr;
    t.bound_flag = x5 ? a.bound_flag : nullptr;
    t.bound_sticky = x5 ? a.bound_sticky : nullptr;
    t.l1kb = x5 ? reinterpret_cast<float *>(base + off_l1) : nullptr;
    t.kc = a.chunk_kblocks > 0 ? a.chunk_kblocks : (a.incompr ? X5_CHUNK_INC : X5_CHUNK);
    t.kbt = KB;
    t.bn = bnx;
    t.mrec = reinterpret_cast<float *>(base + off_mrec);
    t.axs = reinterpret_cast<float2 *>(base + off_axs);
    t.ax_off_m = ax_off_m;
    t.ax_off_n = ax_off_n;

    {
        TimedLaunch tl(st);
        // one timing record per launch
        const int64_t n1 = static_cast<int64_t>(nb) * sv_stride, n2 = static_cast<int64_t>(bt_modes) * nm_ld;
        const int64_t n3 = static_cast<int64_t>(ncn_pad) * (k_pad / 2);
        if (x5) {
            const int64_t ng = gtab_x5_groups(ncomp, nn, ncn_pad) * (k_pad / 2);
            const int64_t blocks = 1 + (n1 + 255) / 256 + (n2 + 255) / 256 + (ng + 255) / 256;
            if (blocks > 0x7fffffff) return set_error(GSC_ERR_INVALID, "tables too large");
            const int64_t ns = N + n_ax;
            tl.begin(K_SEP_SPLIT);
            sep_x5_split_kernel<<<static_cast<unsigned>((ns + 255) / 256), 256, 0, st>>>(t, n_ax);
            tl.end();
            tl.begin(K_SEP_TABLES);
            sep_x5_tables_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(t, n1, n2, ng);
            tl.end();
        } else {
            if (n1 > 0) {
                tl.begin(K_SEP_TABLES);
                sep_svec_kernel<<<static_cast<unsigned>((n1 + 255) / 256), 256, 0, st>>>(t);
                tl.end();
            }
            if (n2 > 0) {
                tl.begin(K_SEP_TABLES);
                sep_btab_kernel<<<static_cast<unsigned>((n2 + 255) / 256), 256, 0, st>>>(t);
                tl.end();
            }
            tl.begin(K_SEP_TABLES);
            if (bf16)
                sep_gtab_kernel<true><<<static_cast<unsigned>((n3 + 255) / 256), 256, 0, st>>>(t);
            else
                sep_gtab_kernel<false><<<static_cast<unsigned>((n3 + 255) / 256), 256, 0, st>>>(t);
            tl.end();
        }
        GSC_CUDA(cudaGetLastError());
    }

    CUtensorMap mh, ml;
    if (!x5) {
        const CUtensorMapDataType gtype =
            bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
        GSC_TRY(make_map(&mh, t.ghi, gtype, 2, k_pad, ncn_pad, bk, BN, CU_TENSOR_MAP_SWIZZLE_128B));
        GSC_TRY(make_map(&ml, t.glo, gtype, 2, k_pad, ncn_pad, bk, BN, CU_TENSOR_MAP_SWIZZLE_128B));
    }

    TcParams p;
    p.svec = t.svec;
    p.sv_stride = sv_stride;
    p.btab = t.btab;
    p.n_modes = N;
    p.nm = nm;
    p.nm_ld = nm_ld;
    p.nb = nb;
    p.nn = nn;
    p.ncn = ncn;
    p.kb_total = KB;
    p.kc = x5 ? t.kc : (a.chunk_kblocks > 0 ? a.chunk_kblocks : 4);
    p.m_tiles = m_tiles;
    p.rows_total = rows_total;
    p.n_tiles = n_tiles;
    p.out = a.out;
    p.comp_stride = P;
    p.batch_stride = static_cast<int64_t>(nm) * nn;
    p.row_stride = nn;
    p.status = status;
    const int64_t grid = x5 ? static_cast<int64_t>(m_tiles) * n_tiles + n_split * ksplit
                            : static_cast<int64_t>(nb) * m_tiles * n_tiles;
    if (grid > 0x7fffffff) return set_error(GSC_ERR_INVALID, "grid too large");
    TimedLaunch tl(st);
    if (x5) {
        X5Params xp;
        xp.base = p;
        xp.wnorm = t.wnorm;
        xp.l1kb = t.l1kb;
        xp.bound_flag = a.bound_flag;
        xp.bound_sticky = a.bound_sticky;
        xp.g1 = reinterpret_cast<const unsigned char *>(t.ghi);
        xp.g2 = reinterpret_cast<const unsigned char *>(t.glo);
        xp.bt = reinterpret_cast<const unsigned char *>(t.btab);
        xp.ws = reinterpret_cast<float *>(base + off_ws);
        xp.ws_main = reinterpret_cast<float *>(base + off_ws + ws_half);
        xp.ws_cnt = reinterpret_cast<int *>(base + off_cnt);
        // The output (ncomp, rows, nn) is dense; tiled bulk stores write it
        // where its rows are 16-byte aligned and, for several components, no
        // 32-column group crosses from one component into the next.
        CUtensorMap om;
        memset(&om, 0, sizeof(om));
        xp.out_rank = 0;
        const bool tma_out = (reinterpret_cast<uintptr_t>(a.out) & 15) == 0 && nn % 2 == 0 &&
                             (ncomp == 1 || (nn % 32 == 0 && P % 2 == 0)) &&
                             rows_total < (int64_t(1) << 31);
        if (tma_out) {
            EncodeTiledFn fn;
            GSC_TRY(encode_fn(&fn));
            const cuuint64_t dims[3] = {static_cast<cuuint64_t>(nn), static_cast<cuuint64_t>(rows_total),
                                        static_cast<cuuint64_t>(ncomp)};
            const cuuint64_t strides[2] = {static_cast<cuuint64_t>(nn) * 8,
                                           static_cast<cuuint64_t>(P) * 8};
            const cuuint32_t box[3] = {16, 32, 1};            // 128-byte rows
            const cuuint32_t estr[3] = {1, 1, 1};
            const int rank = ncomp == 1 ? 2 : 3;
            const CUresult r = fn(&om, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, rank, a.out, dims, strides, box,
                                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return set_error(GSC_ERR_CUDA, "cuTensorMapEncodeTiled (output) failed");
            xp.out_rank = rank;
        }
        tl.begin(K_SEP_TC_F16X5);
        for (const Launch &l : launches) {
            xp.tile0 = static_cast<int>(l.m0 * n_tiles);
            xp.full_tiles = static_cast<int>(l.full_tiles);
            xp.ksplit = l.ksplit;
            xp.n_split = static_cast<int>(l.n_split);
            if (l.n_split > 0)
                GSC_CUDA(cudaMemsetAsync(xp.ws_cnt, 0, static_cast<size_t>(l.n_split) * sizeof(int), st));
            const unsigned g = static_cast<unsigned>(l.full_tiles + l.n_split * l.ksplit);
            if (bnx == 192 && l.n_split > 0) {
                GSC_TRY((configure_x5<192, true>()));
                sep_x5_kernel<192, true><<<g, X5_THREADS, X5Layout<192>::SMEM, st>>>(om, xp);
            } else if (bnx == 192) {
                GSC_TRY((configure_x5<192, false>()));
                sep_x5_kernel<192, false><<<g, X5_THREADS, X5Layout<192>::SMEM, st>>>(om, xp);
            } else if (l.n_split > 0) {
                GSC_TRY((configure_x5<256, true>()));
                sep_x5_kernel<256, true><<<g, X5_THREADS, X5Layout<256>::SMEM, st>>>(om, xp);
            } else {
                GSC_TRY((configure_x5<256, false>()));
                sep_x5_kernel<256, false><<<g, X5_THREADS, X5Layout<256>::SMEM, st>>>(om, xp);
            }
            GSC_CUDA(cudaGetLastError());
            if (a.on_rows)
                GSC_TRY((*a.on_rows)(l.m0 * BM, std::min<int64_t>(l.m1 * BM, rows_total)));
        }
    } else {
        tl.begin(bf16 ? K_SEP_TC_BF16 : K_SEP_TC_F16);
        if (bf16) {
            GSC_TRY(configure_tc<true>());
            sep_tc_kernel<true><<<static_cast<unsigned>(grid), kThreadsTC, kSmemBytes, st>>>(mh, ml, p);
        } else {
            GSC_TRY(configure_tc<false>());
            sep_tc_kernel<false><<<static_cast<unsigned>(grid), kThreadsTC, kSmemBytes, st>>>(mh, ml, p);
        }
    }
    tl.end();
    GSC_CUDA(cudaGetLastError());
    GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
    return GSC_OK;
}

}  // namespace gsc
