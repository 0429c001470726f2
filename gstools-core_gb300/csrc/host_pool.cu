// host_pool.cu -- a cache of pinned host blocks for result arrays.
//
// A host-array call returns a fresh result array, as the reference does
// (src/lib.rs:47,64: into_pyarray_bound).  A fresh array of fresh pages
// costs a page fault per page on first touch, which for a 134 MB field takes
// several times longer than the GPU computing it.  The Python layer
// therefore allocates result arrays of 64 KiB and more from this pool: blocks
// of pinned (page-locked, always resident) host memory, rounded up to 64 KiB
// (2 MiB above 2 MiB),
// handed back to the pool when the last view of the array dies and reused by
// the next result of the same rounded size.  The device-to-host copy then
// runs at the link's speed with no fault on either side.
//
// The pool keeps at most `limit` bytes of free blocks (GSC_HOST_POOL_MB,
// default 2048 MiB, so that a shared host keeps its page-locked memory
// bounded; gsc_host_pool_trim releases every free block); a block freed
// beyond that is released.  Thread safe.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace gsc {
namespace {

constexpr size_t kGrain = size_t(2) << 20;        // blocks above 2 MiB: 2 MiB multiples
constexpr size_t kSmallGrain = size_t(64) << 10;  // up to 2 MiB: 64 KiB multiples

size_t round_block(size_t bytes) {
    const size_t g = bytes <= kGrain ? kSmallGrain : kGrain;
    return (bytes + g - 1) / g * g;
}

struct HostPool {
    std::mutex mu;
    std::map<size_t, std::vector<void *>> free_blocks;   // rounded size -> blocks
    std::map<void *, size_t> live;                        // handed out: block -> size
    size_t cached = 0;                                    // bytes in free_blocks
    size_t limit = 0;
    HostPool() {
        size_t mb = 2048;
        if (const char *e = getenv("GSC_HOST_POOL_MB")) {
            char *end = nullptr;
            const unsigned long long v = strtoull(e, &end, 10);
            if (end && end != e) mb = static_cast<size_t>(v);
        }
        limit = mb << 20;
    }
};

HostPool &pool() {
    static HostPool *p = new HostPool();   // never destroyed: blocks may outlive static teardown
    return *p;
}

}  // namespace

bool is_pinned_host(const void *p) {
    if (!p) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

}  // namespace gsc

using namespace gsc;

extern "C" {

int gsc_host_alloc(int64_t bytes, void **ptr) {
    if (!ptr) return set_error(GSC_ERR_INVALID, "ptr is NULL");
    *ptr = nullptr;
    if (bytes <= 0) return set_error(GSC_ERR_INVALID, "bytes must be positive");
    if (bytes > (int64_t(1) << 42)) return set_error(GSC_ERR_INVALID, "bytes too large");
    const size_t rounded = round_block(static_cast<size_t>(bytes));
    HostPool &hp = pool();
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        auto f = hp.free_blocks.find(rounded);
        if (f != hp.free_blocks.end() && !f->second.empty()) {
            void *p = f->second.back();
            f->second.pop_back();
            hp.cached -= rounded;
            hp.live[p] = rounded;
            *ptr = p;
            return GSC_OK;
        }
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return set_error(GSC_ERR_NO_DEVICE, "no usable CUDA device; this library has no CPU path");
    }
    void *p = nullptr;
    GSC_TRY(alloc_pinned(&p, rounded, "cudaHostAlloc (result pool)"));
    std::lock_guard<std::mutex> lk(hp.mu);
    hp.live[p] = rounded;
    *ptr = p;
    return GSC_OK;
}

int gsc_host_free(void *ptr) {
    if (!ptr) return GSC_OK;
    HostPool &hp = pool();
    size_t size = 0;
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        auto l = hp.live.find(ptr);
        if (l == hp.live.end())
            return set_error(GSC_ERR_INVALID, "pointer was not allocated by gsc_host_alloc");
        size = l->second;
        hp.live.erase(l);
        if (hp.cached + size <= hp.limit) {
            hp.free_blocks[size].push_back(ptr);
            hp.cached += size;
            return GSC_OK;
        }
    }
    GSC_CUDA(cudaFreeHost(ptr));
    return GSC_OK;
}

int gsc_host_pool_trim(void) {
    HostPool &hp = pool();
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        for (auto &kv : hp.free_blocks)
            for (void *p : kv.second) drop.push_back(p);
        hp.free_blocks.clear();
        hp.cached = 0;
    }
    int rc = GSC_OK;
    for (void *p : drop) {
        const cudaError_t e = cudaFreeHost(p);
        if (e != cudaSuccess && rc == GSC_OK) rc = cuda_fail(e, "cudaFreeHost (result pool)");
    }
    return rc;
}

int gsc_host_pool_stats(int64_t *live_bytes, int64_t *cached_bytes) {
    HostPool &hp = pool();
    std::lock_guard<std::mutex> lk(hp.mu);
    int64_t l = 0;
    for (auto &kv : hp.live) l += static_cast<int64_t>(kv.second);
    if (live_bytes) *live_bytes = l;
    if (cached_bytes) *cached_bytes = static_cast<int64_t>(hp.cached);
    return GSC_OK;
}

}  // extern "C"
