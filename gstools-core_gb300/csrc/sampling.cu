// sampling.cu -- on-device spectral sampling of the randomization method's
// inputs: wave vectors cov_samples (dim, N) drawn from a covariance model's
// spectral density and the weights z1, z2 ~ N(0, 1).
//
// GSTools draws these on the host (RandMeth / IncomprRandMeth) and passes
// them to summate; for Monte-Carlo ensembles of many realizations the
// host-side draws and their transfer dominate small realizations.  Here
// every value is a pure function of (seed, realization, mode, draw), so any
// subset of any realization can be regenerated anywhere without sharing
// generator state:
//
//  * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
//    easy as 1, 2, 3", SC'11): counter (mode lo, mode hi, realization, draw
//    block), key = the seed's two 32-bit halves, ten rounds with the
//    published multipliers and key increments;
//  * uniforms of 53 bits from two 32-bit words, normals by the Box-Muller
//    transform (u1 in (0, 1], u2 in [0, 1));
//  * spectra: Gaussian covariance -> k ~ N(0, 2 / l^2) per component;
//    exponential covariance -> multivariate Student-t with one degree of
//    freedom scaled by 1 / l: k = g / |n| / l, g ~ N(0, I), n ~ N(0, 1).
//
// Parity is in distribution (the reference has no sampler on this path):
// the tests check moments and Kolmogorov-Smirnov statistics, and the
// generator's words against a host restatement of Philox.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "internal.h"

namespace gsc {
namespace {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

__device__ __forceinline__ uint4 philox_round(uint4 c, uint32_t k0, uint32_t k1) {
    const uint32_t hi0 = __umulhi(kPhiloxM0, c.x), lo0 = kPhiloxM0 * c.x;
    const uint32_t hi1 = __umulhi(kPhiloxM1, c.z), lo1 = kPhiloxM1 * c.z;
    return make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += kPhiloxW0;
            k1 += kPhiloxW1;
        }
        c = philox_round(c, k0, k1);
    }
    return c;
}

// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double uniform53(uint32_t hi, uint32_t lo) {
    const uint64_t m = (static_cast<uint64_t>(hi >> 5) << 26) | (lo >> 6);
    return static_cast<double>(m) * 0x1.0p-53;
}

// two standard normals from one Philox output (Box-Muller)
__device__ __forceinline__ void normal_pair(uint4 w, double &a, double &b) {
    const double u1 = 1.0 - uniform53(w.x, w.y);     // (0, 1]
    const double u2 = uniform53(w.z, w.w);           // [0, 1)
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    a = r * c;
    b = r * s;
}

// One thread per mode of every item: six normals from three Philox blocks
// (draws 0, 1, 2): k components, the Student-t divisor, z1, z2.
__global__ void sample_kernel(const gsc_sample_item *__restrict__ items,
                              const int64_t *__restrict__ prefix, int64_t n_items,
                              int64_t total, uint32_t key0, uint32_t key1) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int64_t lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const gsc_sample_item &it = items[lo];
    const int64_t j = g - prefix[lo];
    const uint32_t jl = static_cast<uint32_t>(j), jh = static_cast<uint32_t>(j >> 32);
    const uint32_t rz = static_cast<uint32_t>(it.realization);
    double n[6];
    normal_pair(philox4x32_10(make_uint4(jl, jh, rz, 0u), key0, key1), n[0], n[1]);
    normal_pair(philox4x32_10(make_uint4(jl, jh, rz, 1u), key0, key1), n[2], n[3]);
    normal_pair(philox4x32_10(make_uint4(jl, jh, rz, 2u), key0, key1), n[4], n[5]);
    double scale;
    if (it.spectrum == GSC_SPECTRUM_GAUSSIAN) {
        scale = 1.4142135623730951 / it.len_scale;          // sqrt(2) / l
    } else {
        scale = 1.0 / (fabs(n[3]) * it.len_scale);          // Student-t, one degree of freedom
    }
    for (int d = 0; d < it.dim; ++d) it.cov[d * it.n_modes + j] = n[d] * scale;
    it.z1[j] = n[4];
    it.z2[j] = n[5];
}

}  // namespace
}  // namespace gsc

using namespace gsc;

extern "C" {

int gsc_sample_modes_batch_dev(const gsc_sample_item *items, int64_t count, uint64_t seed,
                               const gsc_opts *opts) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    if (count < 0 || (count > 0 && !items)) return set_error(GSC_ERR_INVALID, "bad item list");
    if (count == 0) return GSC_OK;
    std::vector<int64_t> prefix(static_cast<size_t>(count) + 1, 0);
    for (int64_t i = 0; i < count; ++i) {
        const gsc_sample_item &x = items[i];
        const std::string tag = "item " + std::to_string(i) + ": ";
        if (x.dim < 1 || x.dim > 3) return set_error(GSC_ERR_DIM, tag + "dimension must be 1, 2 or 3");
        if (x.n_modes < 0) return set_error(GSC_ERR_INVALID, tag + "negative mode count");
        if (x.spectrum != GSC_SPECTRUM_GAUSSIAN && x.spectrum != GSC_SPECTRUM_EXPONENTIAL)
            return set_error(GSC_ERR_INVALID, tag + "unknown spectrum");
        if (!(x.len_scale > 0.0)) return set_error(GSC_ERR_INVALID, tag + "len_scale must be > 0");
        if (x.n_modes > 0 && (!x.cov || !x.z1 || !x.z2))
            return set_error(GSC_ERR_INVALID, tag + "NULL output");
        prefix[static_cast<size_t>(i) + 1] = prefix[static_cast<size_t>(i)] + x.n_modes;
    }
    const int64_t total = prefix.back();
    if (total == 0) return GSC_OK;
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    for (int64_t i = 0; i < count; ++i) {
        GSC_TRY(check_device_ptr(items[i].cov, "cov"));
        GSC_TRY(check_device_ptr(items[i].z1, "z1"));
        GSC_TRY(check_device_ptr(items[i].z2, "z2"));
    }
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    cudaStream_t st = ro.stream;
    // item table and prefix: staged in a pinned buffer of the context (the
    // copy of the previous call from it has completed before it is reused),
    // copied asynchronously into the context's sampling buffer
    const size_t it_bytes = static_cast<size_t>(count) * sizeof(gsc_sample_item);
    const size_t pre_off = (it_bytes + 255) / 256 * 256;
    const size_t bytes = pre_off + prefix.size() * sizeof(int64_t);
    GSC_TRY(ensure_dev(*ctx, ctx->sampling, bytes));
    if (!ctx->sampling_ev) GSC_CUDA(cudaEventCreateWithFlags(&ctx->sampling_ev, cudaEventDisableTiming));
    GSC_CUDA(cudaEventSynchronize(ctx->sampling_ev));
    if (ctx->sampling_pinned_bytes < bytes) {
        if (ctx->sampling_pinned) GSC_CUDA(cudaFreeHost(ctx->sampling_pinned));
        ctx->sampling_pinned = nullptr;
        ctx->sampling_pinned_bytes = 0;
        GSC_TRY(alloc_pinned(&ctx->sampling_pinned, bytes, "cudaHostAlloc (sampling staging)"));
        ctx->sampling_pinned_bytes = bytes;
    }
    unsigned char *h = static_cast<unsigned char *>(ctx->sampling_pinned);
    memcpy(h, items, it_bytes);
    memcpy(h + pre_off, prefix.data(), prefix.size() * sizeof(int64_t));
    GSC_CUDA(cudaStreamWaitEvent(st, ctx->scratch_ready, 0));
    unsigned char *d = static_cast<unsigned char *>(ctx->sampling.ptr);
    GSC_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
    GSC_CUDA(cudaEventRecord(ctx->sampling_ev, st));
    TimedLaunch tl(st);
    tl.begin(K_SAMPLE_MODES);
    sample_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const gsc_sample_item *>(d), reinterpret_cast<const int64_t *>(d + pre_off),
        count, total, static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    tl.end();
    GSC_CUDA(cudaGetLastError());
    GSC_CUDA(cudaEventRecord(ctx->scratch_ready, st));
    return GSC_OK;
}

int gsc_sample_modes_dev(int32_t spectrum, int32_t dim, int64_t n_modes, double len_scale,
                         uint64_t seed, int64_t realization, double *cov, double *z1, double *z2,
                         const gsc_opts *opts) {
    gsc_sample_item it;
    it.spectrum = spectrum;
    it.dim = dim;
    it.n_modes = n_modes;
    it.len_scale = len_scale;
    it.realization = realization;
    it.cov = cov;
    it.z1 = z1;
    it.z2 = z2;
    return gsc_sample_modes_batch_dev(&it, 1, seed, opts);
}

int gsc_sample_modes_f64(int32_t spectrum, int32_t dim, int64_t n_modes, double len_scale,
                         uint64_t seed, int64_t realization, double *cov, double *z1, double *z2,
                         const gsc_opts *opts) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    if (n_modes < 0) return set_error(GSC_ERR_INVALID, "negative mode count");
    if (dim < 1 || dim > 3) return set_error(GSC_ERR_DIM, "dimension must be 1, 2 or 3");
    if (n_modes == 0) return GSC_OK;
    if (!cov || !z1 || !z2) return set_error(GSC_ERR_INVALID, "NULL output");
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    const size_t n = static_cast<size_t>(n_modes);
    double *d = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g;
        GSC_TRY(g.set(ctx->device));
        GSC_TRY(ensure_dev(*ctx, ctx->io, (dim + 2) * n * sizeof(double)));
        d = static_cast<double *>(ctx->io.ptr);
    }
    gsc_opts o{};
    o.struct_size = sizeof(gsc_opts);
    o.device = ctx->device;
    o.flags = ro.flags;
    o.stream = ctx->stream;
    GSC_TRY(gsc_sample_modes_dev(spectrum, dim, n_modes, len_scale, seed, realization, d,
                                 d + dim * n, d + (dim + 1) * n, &o));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    GSC_CUDA(cudaMemcpyAsync(cov, d, dim * n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GSC_CUDA(cudaMemcpyAsync(z1, d + dim * n, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GSC_CUDA(cudaMemcpyAsync(z2, d + (dim + 1) * n, n * sizeof(double), cudaMemcpyDeviceToHost,
                             ctx->stream));
    GSC_CUDA(cudaStreamSynchronize(ctx->stream));
    return GSC_OK;
}

}  // extern "C"
