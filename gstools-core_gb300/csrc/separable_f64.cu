// separable_f64.cu -- the separable structured-grid contraction in FP64 on the
// double-precision MMA (mma.sync m8n8k4 f64), sm_103a.
//
// Same factorisation as separable_tc.cu (for each X_a one real GEMM with
// K = 2N: rows F[b, (2j, 2j+1)] = (Re, Im)(s_a[j] B[b, j]), columns
// G[c, (2j, 2j+1)] = (Re, -Im)(p_c C[c, j])), but every operand, product and
// sum is FP64, so the result agrees with the reference's summator
// (src/field.rs:37-65, :97-182 on the expanded grid) to FP64 round-off while
// doing 2 * points * 2N FLOPs instead of a sincos per point*mode.
//
// Tiles: one CTA per 64 x 64 output tile of one X_a, 4 warps of 32 x 32,
// K staged 32 at a time through shared memory (rows padded to 33 doubles to
// keep the fragment loads free of bank conflicts).  The F tile is formed in
// FP64 on the fly from the B table and s_a (4 FP64 operations per complex
// element, amortised over the 64 columns of the tile).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "internal.h"

namespace gsc {
namespace {

constexpr int TM = 64, TN = 64, TK = 32;     // tile rows, columns, K per stage
constexpr int LDS = TK + 1;                  // padded shared-memory row (doubles)
constexpr int kF64Threads = 128;

struct F64Tab {
    const double *cov, *z1, *z2;
    int dim, n_modes;
    const double *ax_b, *ax_m, *ax_n;
    int kb_dim, km_dim, kn_dim;
    int nb, nm, nn, ncomp, incompr;
    int k_pad, ncn_pad;
    double2 *svec;     // [nb][n_modes]
    double2 *btab;     // [n_modes][nm]
    double *g;         // [ncn_pad][k_pad]
    const int *run_if; // null, or a device word: the launch does nothing while it is 0
};

__global__ void f64_svec_kernel(F64Tab t) {
    if (t.run_if && *t.run_if == 0) return;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.nb) * t.n_modes) return;
    const int b = static_cast<int>(i / t.n_modes), j = static_cast<int>(i % t.n_modes);
    double re = t.z1[j], im = -t.z2[j];
    if (t.dim == 3) {
        double s, c;
        sincos(t.cov[t.kb_dim * t.n_modes + j] * t.ax_b[b], &s, &c);
        const double r2 = re * c - im * s;
        im = re * s + im * c;
        re = r2;
    }
    t.svec[i] = make_double2(re, im);
}

__global__ void f64_btab_kernel(F64Tab t) {
    if (t.run_if && *t.run_if == 0) return;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.n_modes) * t.nm) return;
    const int j = static_cast<int>(i / t.nm), m = static_cast<int>(i % t.nm);
    double s, c;
    sincos(t.cov[t.km_dim * t.n_modes + j] * t.ax_m[m], &s, &c);
    t.btab[i] = make_double2(c, s);
}

__global__ void f64_gtab_kernel(F64Tab t) {
    if (t.run_if && *t.run_if == 0) return;
    const int half_k = t.k_pad / 2;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<int64_t>(t.ncn_pad) * half_k) return;
    const int row = static_cast<int>(i / half_k), j = static_cast<int>(i % half_k);
    double re = 0.0, im = 0.0;
    if (row < t.ncomp * t.nn && j < t.n_modes) {
        const int c = row / t.nn, n = row - c * t.nn;
        double s, co;
        sincos(t.cov[t.kn_dim * t.n_modes + j] * t.ax_n[n], &s, &co);
        double pw = 1.0;
        if (t.incompr) {   // projector as the reference forms it (src/field.rs:138-152)
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
        re = pw * co;
        im = -(pw * s);
    }
    t.g[static_cast<int64_t>(row) * t.k_pad + 2 * j] = re;
    t.g[static_cast<int64_t>(row) * t.k_pad + 2 * j + 1] = im;
}

__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

struct F64Params {
    const double2 *svec, *btab;
    const double *g;
    int n_modes, nm, nn, ncn, k_pad;
    int m_tiles, n_tiles;
    double *out;
    int64_t comp_stride, batch_stride, row_stride;
    const int *run_if;   // as in F64Tab
};

__global__ void __launch_bounds__(kF64Threads)
sep_f64_kernel(const F64Params p) {
    if (p.run_if && *p.run_if == 0) return;
    __shared__ double As[TM * LDS];
    __shared__ double Bs[TN * LDS];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int tile = blockIdx.x;
    const int nt = tile % p.n_tiles;
    tile /= p.n_tiles;
    const int mt = tile % p.m_tiles;
    const int b = tile / p.m_tiles;
    const int m0 = mt * TM, n0 = nt * TN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;   // warp's 32 x 32 sub-tile
    const int grp = lane >> 2, tig = lane & 3;

    double acc[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    const double2 *sv = p.svec + static_cast<int64_t>(b) * p.n_modes;
    for (int k0 = 0; k0 < p.k_pad; k0 += TK) {
        __syncthreads();
        // F tile: 64 rows x 16 modes, (Re, Im) interleaved along K
        for (int e = tid; e < TM * (TK / 2); e += kF64Threads) {
            const int r = e % TM, jl = e / TM;
            const int j = k0 / 2 + jl, m = m0 + r;
            double re = 0.0, im = 0.0;
            if (m < p.nm && j < p.n_modes) {
                const double2 bt = p.btab[static_cast<int64_t>(j) * p.nm + m];
                const double2 s = sv[j];
                re = bt.x * s.x - bt.y * s.y;
                im = bt.x * s.y + bt.y * s.x;
            }
            As[r * LDS + 2 * jl] = re;
            As[r * LDS + 2 * jl + 1] = im;
        }
        // G tile: 64 rows x 32 K
        for (int e = tid; e < TN * TK; e += kF64Threads) {
            const int r = e / TK, k = e % TK;
            Bs[r * LDS + k] = p.g[static_cast<int64_t>(n0 + r) * p.k_pad + k0 + k];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; kk += 4) {
            double a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[(wm + 8 * i + grp) * LDS + kk + tig];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Bs[(wn + 8 * j + grp) * LDS + kk + tig];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j][0], acc[i][j][1], a[i], bb[j]);
        }
    }

    double *ob = p.out + static_cast<int64_t>(b) * p.batch_stride;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + wm + 8 * i + grp;
        if (m >= p.nm) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int gn = n0 + wn + 8 * j + 2 * tig + h;
                if (gn >= p.ncn) continue;
                const int comp = gn / p.nn;
                ob[static_cast<int64_t>(m) * p.row_stride + comp * p.comp_stride + (gn - comp * p.nn)] =
                    acc[i][j][h];
            }
    }
}

size_t up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

int sep_f64_run(DeviceCtx &ctx, const SepArgs &a, cudaStream_t st) {
    const int dim = static_cast<int>(a.dim);
    const int N = static_cast<int>(a.n_modes);
    const int ncomp = a.incompr ? dim : 1;
    const int nb = dim == 3 ? static_cast<int>(a.n[0]) : 1;
    const int nm = static_cast<int>(dim == 3 ? a.n[1] : a.n[0]);
    const int nn = static_cast<int>(dim == 3 ? a.n[2] : a.n[1]);
    const int64_t P = static_cast<int64_t>(nb) * nm * nn;
    if (P == 0) return GSC_OK;
    const int k_pad = std::max(TK, (2 * N + TK - 1) / TK * TK);
    const int ncn = ncomp * nn;
    const int n_tiles = (ncn + TN - 1) / TN, m_tiles = (nm + TM - 1) / TM;
    const int ncn_pad = n_tiles * TN;

    const size_t off_svec = 0;
    const size_t off_btab = up(off_svec + sizeof(double2) * nb * static_cast<size_t>(N), 256);
    const size_t off_g = up(off_btab + sizeof(double2) * static_cast<size_t>(N) * nm, 256);
    const size_t total = off_g + sizeof(double) * static_cast<size_t>(ncn_pad) * k_pad;
    GSC_TRY(ensure_dev(ctx, ctx.scratch, total));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx.scratch_ready, 0));
    unsigned char *base = static_cast<unsigned char *>(ctx.scratch.ptr);

    F64Tab t;
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
    t.ncn_pad = ncn_pad;
    t.svec = reinterpret_cast<double2 *>(base + off_svec);
    t.btab = reinterpret_cast<double2 *>(base + off_btab);
    t.g = reinterpret_cast<double *>(base + off_g);
    t.run_if = a.run_if;
    {
        TimedLaunch tl(st);
        tl.begin(K_SEP_TABLES);
        const int64_t n1 = static_cast<int64_t>(nb) * N, n2 = static_cast<int64_t>(N) * nm;
        const int64_t n3 = static_cast<int64_t>(ncn_pad) * (k_pad / 2);
        if (n1 > 0) f64_svec_kernel<<<static_cast<unsigned>((n1 + 255) / 256), 256, 0, st>>>(t);
        if (n2 > 0) f64_btab_kernel<<<static_cast<unsigned>((n2 + 255) / 256), 256, 0, st>>>(t);
        f64_gtab_kernel<<<static_cast<unsigned>((n3 + 255) / 256), 256, 0, st>>>(t);
        tl.end();
        GSC_CUDA(cudaGetLastError());
    }
    F64Params p;
    p.svec = t.svec;
    p.btab = t.btab;
    p.g = t.g;
    p.n_modes = N;
    p.nm = nm;
    p.nn = nn;
    p.ncn = ncn;
    p.k_pad = k_pad;
    p.m_tiles = m_tiles;
    p.n_tiles = n_tiles;
    p.out = a.out;
    p.comp_stride = P;
    p.batch_stride = static_cast<int64_t>(nm) * nn;
    p.row_stride = nn;
    p.run_if = a.run_if;
    const int64_t grid = static_cast<int64_t>(nb) * m_tiles * n_tiles;
    if (grid > 0x7fffffff) return set_error(GSC_ERR_INVALID, "grid too large");
    TimedLaunch tl(st);
    tl.begin(K_SEP_F64);
    sep_f64_kernel<<<static_cast<unsigned>(grid), kF64Threads, 0, st>>>(p);
    tl.end();
    GSC_CUDA(cudaGetLastError());
    GSC_CUDA(cudaEventRecord(ctx.scratch_ready, st));
    return GSC_OK;
}

}  // namespace gsc
