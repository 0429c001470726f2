// selftest.cu -- exercises the failure path of the pipelined kernels on the
// GPU without faulting it: a CTA waits, with the same bounded wait the
// tensor-core kernels use, on an mbarrier that nothing ever completes.  The
// wait gives up after the given limit, records its code in the device status
// word, raises the CTA's abort flag (a second warp waiting on the same
// barrier sees it and leaves), and the kernel returns.  The host reads the
// status like after any other launch; the context stays usable.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

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

}  // namespace
}  // namespace gsc

using namespace gsc;

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
