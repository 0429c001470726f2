// selftest.cu -- exercises the failure path of the pipelined kernels on the
// GPU without faulting it: a CTA waits, with the same bounded wait the
// tensor-core kernels use, on an mbarrier that nothing ever completes.  The
// wait gives up after the given limit, records its code in the device status
// word, raises the CTA's abort flag (a second warp waiting on the same
// barrier sees it and leaves), and the kernel returns.  The host reads the
// status like after any other launch; the context stays usable.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "sm100.cuh"

namespace gsc {
namespace {

using namespace sm100;

__global__ void wait_timeout_probe_kernel(int *status, uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);            // one arrival expected; none ever comes
        abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        // warp 0 gives up first (its limit); warp 1 has the production limit
        // and leaves when it sees the abort flag
        mbar_wait(&bar, 0, &abort_flag, status, kErrTimeoutFull,
                  warp == 0 ? limit_ns : kWaitLimitNs);
    }
    __syncthreads();
}

// Issue-rate probes of the mixed kernel's instruction kinds: every thread
// runs kPipeChains independent chains of one kind (no chain waits on another
// thread), so the launch's time is the pipe's throughput for that kind.  At
// 16384 iterations a launch lasts about 1 ms (FP32) to 4 ms (high products).
constexpr int kPipeChains = 8, kPipeIters = 16384;

__global__ void pipe_imadhi_kernel(uint32_t *out, uint32_t a, uint32_t b) {
    uint32_t v[kPipeChains];
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) v[c] = threadIdx.x + c;
    for (int i = 0; i < kPipeIters; ++i)
#pragma unroll
        for (int c = 0; c < kPipeChains; ++c) v[c] = __umulhi(v[c], a) + b;
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) s ^= v[c];
    out[static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

__global__ void pipe_imad_kernel(uint32_t *out, uint32_t a, uint32_t b) {
    uint32_t v[kPipeChains];
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) v[c] = threadIdx.x + c;
    for (int i = 0; i < kPipeIters; ++i)
#pragma unroll
        for (int c = 0; c < kPipeChains; ++c) v[c] = v[c] * a + b;
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) s ^= v[c];
    out[static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

__global__ void pipe_ffma_kernel(uint32_t *out, float a, float b) {
    float v[kPipeChains];
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) v[c] = static_cast<float>(threadIdx.x + c);
    for (int i = 0; i < kPipeIters; ++i)
#pragma unroll
        for (int c = 0; c < kPipeChains; ++c) v[c] = fmaf(v[c], a, b);
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kPipeChains; ++c) s += v[c];
    out[static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x] = __float_as_uint(s);
}

}  // namespace
}  // namespace gsc

using namespace gsc;

extern "C" int gsc_selftest_pipe_rates(int32_t device, double *rates) {
    if (!rates) return set_error(GSC_ERR_INVALID, "rates is NULL");
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    cudaStream_t st = ctx->stream;
    int sms = 0;
    GSC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int blocks = 8 * sms, threads = 256;
    const double ops = static_cast<double>(blocks) * threads * kPipeIters * kPipeChains;
    uint32_t *out = nullptr;
    GSC_CUDA(cudaMalloc(reinterpret_cast<void **>(&out), sizeof(uint32_t) * blocks * threads));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = cuda_ok(cudaEventCreate(&e0));
    if (rc == GSC_OK) rc = cuda_ok(cudaEventCreate(&e1));
    // the first round is untimed (it brings the SM clock up from idle); the
    // kinds then alternate, so that a clock change between them shows in
    // every kind's samples alike, and each kind keeps its fastest launch
    float best[3] = {1e30f, 1e30f, 1e30f};
    for (int rep = 0; rep < 5 && rc == GSC_OK; ++rep) {
        for (int kind = 0; kind < 3 && rc == GSC_OK; ++kind) {
            rc = cuda_ok(cudaEventRecord(e0, st));
            if (kind == 0) pipe_imadhi_kernel<<<blocks, threads, 0, st>>>(out, 0x9E3779B9u, 7u);
            else if (kind == 1) pipe_imad_kernel<<<blocks, threads, 0, st>>>(out, 0x9E3779B9u, 7u);
            else pipe_ffma_kernel<<<blocks, threads, 0, st>>>(out, 0.999f, 1e-3f);
            if (rc == GSC_OK) rc = cuda_ok(cudaGetLastError());
            if (rc == GSC_OK) rc = cuda_ok(cudaEventRecord(e1, st));
            if (rc == GSC_OK) rc = cuda_ok(cudaEventSynchronize(e1));
            float ms = 0.f;
            if (rc == GSC_OK) rc = cuda_ok(cudaEventElapsedTime(&ms, e0, e1));
            if (rc == GSC_OK && rep > 0 && ms < best[kind]) best[kind] = ms;
        }
    }
    for (int kind = 0; kind < 3; ++kind)
        rates[kind] = rc == GSC_OK ? ops / (static_cast<double>(best[kind]) * 1e-3) : 0.0;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}

extern "C" int gsc_selftest_wait_timeout(int32_t device, int64_t limit_us) {
    if (limit_us < 1000 || limit_us > 2000000)
        return set_error(GSC_ERR_INVALID, "limit_us must lie in [1000, 2000000]");
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(device, &ctx));
    {
        // the context lock is released before gsc_device_status takes it
        std::lock_guard<std::mutex> lk(ctx->mu);
        DeviceGuard g;
        GSC_TRY(g.set(ctx->device));
        cudaStream_t st = ctx->stream;
        GSC_CUDA(cudaStreamWaitEvent(st, ctx->scratch_ready, 0));
        wait_timeout_probe_kernel<<<1, 64, 0, st>>>(ctx->status,
                                                    static_cast<uint64_t>(limit_us) * 1000);
        GSC_CUDA(cudaGetLastError());
        GSC_CUDA(cudaEventRecord(ctx->scratch_ready, st));
        GSC_CUDA(cudaStreamSynchronize(st));
    }
    return gsc_device_status(ctx->device);
}

// Per-device set-up registry under concurrent first calls (host only): the
// stand-in keys are addresses inside a static array, the stand-in device
// ordinals start far above any real one, so no real kernel's entry is hit.
extern "C" int gsc_selftest_once_per_device(int32_t n_devices, int32_t n_keys, int32_t n_threads,
                                            int64_t *setups) {
    if (n_devices < 1 || n_devices > 64 || n_keys < 1 || n_keys > 64 || n_threads < 1 ||
        n_threads > 64 || !setups)
        return set_error(GSC_ERR_INVALID, "n_devices, n_keys, n_threads must lie in [1, 64]");
    static char stand_in[64];
    static std::atomic<int> round{0};
    // each call gets fresh device ordinals, so the registry's entries from an
    // earlier call do not count
    const int dev0 = (1 << 20) + round.fetch_add(1) * 64;
    const int pairs = n_devices * n_keys;
    std::vector<std::atomic<int>> tries(pairs), ok(pairs);
    for (int i = 0; i < pairs; ++i) tries[i] = ok[i] = 0;
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t)
        th.emplace_back([&, t] {
            for (int v = 0; v < pairs; ++v) {
                const int i = (v * 7 + t * 13) % pairs;   // a different order per thread
                const int k = i % n_keys, d = i / n_keys;
                once_per_device(&stand_in[k], dev0 + d, [&, i]() -> int {
                    if (tries[i].fetch_add(1) == 0)
                        return set_error(GSC_ERR_CUDA, "stand-in set-up fails once");
                    ok[i].fetch_add(1);
                    return GSC_OK;
                });
            }
            // a second sweep: every pair is set up by now (its first sweep
            // retried a failure), so nothing runs again
            for (int i = 0; i < pairs; ++i)
                once_per_device(&stand_in[i % n_keys], dev0 + i / n_keys, [&, i]() -> int {
                    ok[i].fetch_add(1);
                    return GSC_OK;
                });
        });
    for (auto &x : th) x.join();
    int64_t total = 0;
    bool good = true;
    for (int i = 0; i < pairs; ++i) {
        total += ok[i];
        if (ok[i] != 1 || tries[i] > 2) good = false;
    }
    *setups = total;
    return good ? GSC_OK : set_error(GSC_ERR_KERNEL, "a pair was set up other than exactly once");
}
