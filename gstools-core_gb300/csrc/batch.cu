// batch.cu -- Monte-Carlo ensembles of many realizations in one persistent
// launch, fed from a device work queue and replayable as a CUDA graph.
//
// A realization (item) is one call of the reference's summator,
// summator_incompr or summator_fourier (src/field.rs:37-65, :97-182,
// :219-249) with its own point and mode counts.  An ensemble of hundreds of
// them with point counts from 1e3 to 1e6 and mode counts from 256 to 8192
// would, as separate calls, leave the GPU idle between launches and run the
// small ones at a fraction of the machine.  Here one plan holds them all:
//
//  * the per-mode tables of every item are built by one launch;
//  * the work is cut into units -- one block of 128*R points of one item and
//    one range of its modes -- and sorted by cost, largest first;
//  * one persistent kernel (one block per resident slot) takes units from
//    the queue with an atomic counter until it is empty, so the long units
//    start first and the short ones fill the tail;
//  * items whose modes were split over several units write split partials,
//    summed in split order by one reduction launch (deterministic);
//  * the whole sequence is allocation-free and host-synchronisation-free,
//    so it is captured once into a CUDA graph and replayed.
//
// The autotuner picks the points per thread R, the modes per staged tile
// (FP64 form) and the work-unit granularity (how finely modes are split) by
// timing each candidate on an evenly spaced sample of the cost-sorted queue
// of this very ensemble, and caches the winner per ensemble shape.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"

namespace gsc {
namespace {

struct Cfg {
    int R = 4;          // points per thread
    int tile = 8;       // modes per staged tile (FP64 form)
    int upb = 8;        // target work units per resident block
};

int batch_sm_count(int device) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 152;
    }
    return n;
}

// out[e] = sum over s (ascending) of part[s][e] for every element of every
// split item; red_prefix holds the exclusive prefix of nout * n_points over
// the split items listed in red_items.
__global__ void batch_reduce_kernel(const BatchItem *__restrict__ items,
                                    const int32_t *__restrict__ red_items,
                                    const int64_t *__restrict__ red_prefix, int64_t n_red,
                                    int64_t total) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int64_t lo = 0, hi = n_red - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (red_prefix[mid] <= g) lo = mid; else hi = mid - 1;
    }
    const BatchItem &it = items[red_items[lo]];
    const int64_t e = g - red_prefix[lo];
    const int64_t slot = (it.incompr ? it.dim : 1) * it.n_points;
    double s = 0.0;
    for (int k = 0; k < it.splits; ++k) s += it.part[k * slot + e];
    it.out[e] = s;
}


}  // namespace
}  // namespace gsc

using namespace gsc;

struct gsc_batch {
    int device = -1;
    int form = GSC_FORM_PLAIN_F64;
    int flags = 0;
    std::vector<BatchItem> items;            // host copy; part pointers filled per config
    std::vector<int64_t> mode_prefix;
    int64_t total_modes = 0;
    double total_work = 0.0;                 // sum of n_points * n_modes (* components)
    // device memory
    BatchItem *d_items = nullptr;
    int64_t *d_prefix = nullptr;
    BatchUnit *d_units = nullptr;
    size_t units_cap = 0;
    int *d_counter = nullptr;
    void *d_tab = nullptr;                   // FP64 form: W tables (double2)
    double *d_rec = nullptr;                 // FP64 form: mode records
    float *d_frec = nullptr;                 // mixed forms: records
    double *d_rec64 = nullptr;
    unsigned long long *d_fxrange = nullptr; // mixed form: range words of every item
    int *range_flag = nullptr;               // mixed form: the device's sticky range word
    double *d_part = nullptr;
    size_t part_cap = 0;
    int32_t *d_red_items = nullptr;
    int64_t *d_red_prefix = nullptr;
    // chosen configuration
    Cfg cfg;
    int blocks = 0;
    int64_t n_units = 0;
    int max_splits = 1;
    int n_red = 0;
    int64_t red_total = 0;
    int tuned = 0;
    double tune_ms = 0.0;
    // CUDA graph of one run
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    ~gsc_batch() {
        int prev = -1;
        if (cudaGetDevice(&prev) == cudaSuccess && prev != device && device >= 0) cudaSetDevice(device);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap_stream) cudaStreamDestroy(cap_stream);
        for (void *p : {static_cast<void *>(d_items), static_cast<void *>(d_prefix),
                        static_cast<void *>(d_units), static_cast<void *>(d_counter), d_tab,
                        static_cast<void *>(d_rec), static_cast<void *>(d_frec),
                        static_cast<void *>(d_rec64), static_cast<void *>(d_fxrange),
                        static_cast<void *>(d_part),
                        static_cast<void *>(d_red_items), static_cast<void *>(d_red_prefix)})
            if (p) cudaFree(p);
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
    }
};

namespace gsc {
namespace {

int dmalloc(void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    return alloc_device(p, bytes, "cudaMalloc (batch plan)");
}

bool is_plain(const gsc_batch &b) { return b.form == GSC_FORM_PLAIN_F64; }
bool is_fx(const gsc_batch &b) { return b.form == GSC_FORM_MIXED; }
// modes per staged tile of the point-mixed kernels: mixed_fx.cu 64, mixed.cu 32
int mixed_tile(const gsc_batch &b) { return is_fx(b) ? 64 : 32; }
bool scalar_only(const gsc_batch &b) {
    for (const auto &it : b.items)
        if (it.incompr) return false;
    return true;
}

int occupancy(const gsc_batch &b, const Cfg &c) {
    if (is_fx(b)) return batch_fx_occupancy(c.R, scalar_only(b));
    return is_plain(b) ? batch_plain_occupancy(c.R, c.tile, b.device)
                       : batch_mixed_occupancy(c.R, true, b.device);
}

// Item table, mode prefix and total work of a plan from the caller's item
// descriptors, after their shapes, kinds and pointers are checked
// (pointers only when check_ptrs: the host-only queue check has none).
int fill_items(gsc_batch &b, const gsc_batch_item *items, int64_t count, bool check_ptrs) {
    b.items.resize(static_cast<size_t>(count));
    b.mode_prefix.assign(static_cast<size_t>(count) + 1, 0);
    for (int64_t i = 0; i < count; ++i) {
        const gsc_batch_item &x = items[i];
        const std::string tag = "item " + std::to_string(i) + ": ";
        if (x.n_modes < 0 || x.n_points < 0)
            return set_error(GSC_ERR_INVALID, tag + "negative mode or point count");
        if (x.n_modes > (int64_t(1) << 30) || x.n_points > (int64_t(1) << 40))
            return set_error(GSC_ERR_INVALID, tag + "too many modes or points");
        if (x.kind < GSC_BATCH_SCALAR || x.kind > GSC_BATCH_FOURIER)
            return set_error(GSC_ERR_INVALID, tag + "unknown kind");
        const bool inc = x.kind == GSC_BATCH_INCOMPR;
        if (x.dim < 1 || x.dim > 3 || (inc && x.dim == 1))
            return set_error(GSC_ERR_DIM, tag + (inc ? "Only two- and three-dimensional problems are supported."
                                                     : "batches support dimensions 1, 2 and 3"));
        const char *need[5] = {"cov", "z1", "z2", "pos", "out"};
        const void *ptrs[5] = {x.cov, x.z1, x.z2, x.pos, x.out};
        const bool needed[5] = {x.n_modes > 0, x.n_modes > 0, x.n_modes > 0, x.n_points > 0,
                                x.n_points > 0};
        for (int k = 0; k < 5; ++k) {
            if (!check_ptrs) continue;
            if (needed[k] && !ptrs[k]) return set_error(GSC_ERR_INVALID, tag + need[k] + " is NULL");
            GSC_TRY(check_device_ptr(ptrs[k], need[k]));
        }
        if (x.kind == GSC_BATCH_FOURIER && check_ptrs) {
            if (x.n_modes > 0 && !x.spectrum_factor)
                return set_error(GSC_ERR_INVALID, tag + "spectrum_factor is NULL");
            GSC_TRY(check_device_ptr(x.spectrum_factor, "spectrum_factor"));
        }
        BatchItem &it = b.items[static_cast<size_t>(i)];
        it.cov = x.cov;
        it.z1 = x.z1;
        it.z2 = x.z2;
        it.sf = x.kind == GSC_BATCH_FOURIER ? x.spectrum_factor : nullptr;
        it.pos = x.pos;
        it.out = x.out;
        it.part = nullptr;
        it.n_modes = x.n_modes;
        it.n_points = x.n_points;
        it.mode_off = b.mode_prefix[static_cast<size_t>(i)];
        it.dim = x.dim;
        it.incompr = inc ? 1 : 0;
        it.splits = 1;
        it.pad = 0;
        b.mode_prefix[static_cast<size_t>(i) + 1] = it.mode_off + x.n_modes;
        b.total_work += static_cast<double>(x.n_points) * static_cast<double>(x.n_modes) *
                         (inc ? x.dim : 1);
    }
    b.total_modes = b.mode_prefix.back();
    if (b.total_modes > 0x7fffffff) return set_error(GSC_ERR_INVALID, "too many modes in the batch");
    return GSC_OK;
}

// Work units of configuration c, cost-sorted (largest first), and the split
// counts they imply.  Fills b.items[*].splits.
int make_units(gsc_batch &b, const Cfg &c, int blocks, std::vector<BatchUnit> &units) {
    const int64_t ppb = static_cast<int64_t>(kBatchThreads) * c.R;
    const int tile = is_plain(b) ? c.tile : mixed_tile(b);
    const double target = std::max(1.0, b.total_work / (static_cast<double>(blocks) * c.upb));
    units.clear();
    std::vector<double> cost;
    for (size_t i = 0; i < b.items.size(); ++i) {
        BatchItem &it = b.items[i];
        const int64_t P = it.n_points, N = it.n_modes;
        const int64_t nblk = (P + ppb - 1) / ppb;
        int64_t S = 1;
        if (N > 0) {
            const double block_cost = static_cast<double>(std::min(P, ppb)) * N;
            S = static_cast<int64_t>(std::ceil(block_cost / target));
            S = std::min<int64_t>(S, std::max<int64_t>(1, N / (2 * tile)));
            S = std::max<int64_t>(1, std::min<int64_t>(S, 64));
        }
        int64_t mps = N > 0 ? (N + S - 1) / S : 0;
        mps = (mps + tile - 1) / tile * tile;
        if (mps > 0) S = std::max<int64_t>(1, (N + mps - 1) / mps);
        it.splits = static_cast<int32_t>(S);
        for (int64_t blk = 0; blk < nblk; ++blk) {
            const int64_t p_first = blk * ppb;
            const int64_t np = std::min(ppb, P - p_first);
            for (int64_t s = 0; s < S; ++s) {
                BatchUnit u;
                u.item = static_cast<int32_t>(i);
                u.split = static_cast<int32_t>(s);
                u.p_first = p_first;
                u.jb = std::min(N, s * mps);
                u.je = std::min(N, (s + 1) * mps);
                units.push_back(u);
                cost.push_back(static_cast<double>(np) * static_cast<double>(u.je - u.jb + 1));
            }
        }
    }
    std::vector<size_t> order(units.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t x, size_t y) { return cost[x] > cost[y]; });
    std::vector<BatchUnit> sorted(units.size());
    for (size_t k = 0; k < order.size(); ++k) sorted[k] = units[order[k]];
    units.swap(sorted);
    return GSC_OK;
}

// Validates a work queue before it is uploaded: every unit names an item and
// a split that exist, starts on a point-block boundary inside its item and
// covers a mode range inside it; every (point block, split) of every item
// appears exactly once, and the splits of a block tile [0, n_modes) in order.
// A queue that fails would make the persistent kernels skip or double-count
// points, so the plan refuses it.
int check_units(const std::vector<BatchItem> &items, int64_t ppb,
                const std::vector<BatchUnit> &units) {
    std::vector<int64_t> first(items.size() + 1, 0);
    for (size_t i = 0; i < items.size(); ++i) {
        const int64_t nblk = (items[i].n_points + ppb - 1) / ppb;
        first[i + 1] = first[i] + nblk * std::max<int32_t>(1, items[i].splits);
    }
    const int64_t n_slots = first.back();
    auto bad = [](size_t k, const std::string &why) {
        return set_error(GSC_ERR_INVALID, "corrupt batch work queue: unit " + std::to_string(k) +
                                              " " + why);
    };
    if (static_cast<int64_t>(units.size()) != n_slots)
        return set_error(GSC_ERR_INVALID, "corrupt batch work queue: " +
                                              std::to_string(units.size()) + " units for " +
                                              std::to_string(n_slots) + " (point block, split) pairs");
    std::vector<int64_t> jb(static_cast<size_t>(n_slots), -1), je(static_cast<size_t>(n_slots), -1);
    for (size_t k = 0; k < units.size(); ++k) {
        const BatchUnit &u = units[k];
        if (u.item < 0 || static_cast<size_t>(u.item) >= items.size())
            return bad(k, "names item " + std::to_string(u.item));
        const BatchItem &it = items[static_cast<size_t>(u.item)];
        if (u.split < 0 || u.split >= std::max<int32_t>(1, it.splits))
            return bad(k, "names split " + std::to_string(u.split));
        if (u.p_first < 0 || u.p_first >= it.n_points || u.p_first % ppb != 0)
            return bad(k, "starts at point " + std::to_string(u.p_first));
        if (u.jb < 0 || u.jb > u.je || u.je > it.n_modes)
            return bad(k, "covers modes [" + std::to_string(u.jb) + ", " + std::to_string(u.je) + ")");
        const size_t slot = static_cast<size_t>(first[static_cast<size_t>(u.item)] +
                                                u.p_first / ppb * std::max<int32_t>(1, it.splits) +
                                                u.split);
        if (jb[slot] >= 0) return bad(k, "repeats an earlier unit");
        jb[slot] = u.jb;
        je[slot] = u.je;
    }
    for (size_t i = 0; i < items.size(); ++i) {
        const int64_t S = std::max<int32_t>(1, items[i].splits);
        for (int64_t q = first[i]; q < first[i + 1]; q += S) {
            int64_t at = 0;
            for (int64_t s = 0; s < S; ++s) {
                if (jb[static_cast<size_t>(q + s)] != at)
                    return set_error(GSC_ERR_INVALID,
                                     "corrupt batch work queue: item " + std::to_string(i) +
                                         ": split " + std::to_string(s) + " of point block " +
                                         std::to_string((q - first[i]) / S) +
                                         " does not start where the previous split ends");
                at = je[static_cast<size_t>(q + s)];
            }
            if (at != items[i].n_modes)
                return set_error(GSC_ERR_INVALID, "corrupt batch work queue: item " +
                                                      std::to_string(i) +
                                                      ": the splits do not reach the last mode");
        }
    }
    return GSC_OK;
}

// Device buffers for the split partials of the current split counts, and the
// reduction list; uploads the item table.
int prepare_items(gsc_batch &b) {
    size_t need = 0;
    std::vector<int32_t> red;
    std::vector<int64_t> red_prefix;
    int64_t acc = 0;
    b.max_splits = 1;
    for (size_t i = 0; i < b.items.size(); ++i) {
        const BatchItem &it = b.items[i];
        b.max_splits = std::max<int>(b.max_splits, it.splits);
        if (it.splits > 1) {
            const int64_t slot = (it.incompr ? it.dim : 1) * it.n_points;
            need += static_cast<size_t>(it.splits) * slot;
            red.push_back(static_cast<int32_t>(i));
            red_prefix.push_back(acc);
            acc += slot;
        }
    }
    if (need > b.part_cap) {
        if (b.d_part) cudaFree(b.d_part);
        b.d_part = nullptr;
        b.part_cap = 0;
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b.d_part), need * sizeof(double)));
        b.part_cap = need;
    }
    size_t off = 0;
    for (auto &it : b.items) {
        if (it.splits > 1) {
            it.part = b.d_part + off;
            off += static_cast<size_t>(it.splits) * (it.incompr ? it.dim : 1) * it.n_points;
        } else {
            it.part = nullptr;
        }
    }
    GSC_CUDA(cudaMemcpy(b.d_items, b.items.data(), b.items.size() * sizeof(BatchItem),
                        cudaMemcpyHostToDevice));
    if (b.d_red_items) cudaFree(b.d_red_items);
    if (b.d_red_prefix) cudaFree(b.d_red_prefix);
    b.d_red_items = nullptr;
    b.d_red_prefix = nullptr;
    b.n_red = static_cast<int>(red.size());
    b.red_total = acc;
    if (!red.empty()) {
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b.d_red_items), red.size() * sizeof(int32_t)));
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b.d_red_prefix), red_prefix.size() * sizeof(int64_t)));
        GSC_CUDA(cudaMemcpy(b.d_red_items, red.data(), red.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        GSC_CUDA(cudaMemcpy(b.d_red_prefix, red_prefix.data(), red_prefix.size() * sizeof(int64_t),
                            cudaMemcpyHostToDevice));
    }
    return GSC_OK;
}

int upload_units(gsc_batch &b, const std::vector<BatchUnit> &units) {
    if (units.size() > b.units_cap) {
        if (b.d_units) cudaFree(b.d_units);
        b.d_units = nullptr;
        b.units_cap = 0;
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b.d_units), units.size() * sizeof(BatchUnit)));
        b.units_cap = units.size();
    }
    if (!units.empty())
        GSC_CUDA(cudaMemcpy(b.d_units, units.data(), units.size() * sizeof(BatchUnit),
                            cudaMemcpyHostToDevice));
    return GSC_OK;
}

int enqueue_tables(gsc_batch &b, cudaStream_t st) {
    if (is_fx(b))
        return batch_fx_tables(b.d_items, b.d_prefix, static_cast<int64_t>(b.items.size()),
                               b.total_modes, reinterpret_cast<uint32_t *>(b.d_frec), b.d_fxrange,
                               b.range_flag, st);
    if (is_plain(b))
        return batch_plain_tables(b.d_items, b.d_prefix, static_cast<int64_t>(b.items.size()),
                                  b.total_modes, b.d_tab, b.d_rec, st);
    return batch_mixed_tables(b.d_items, b.d_prefix, static_cast<int64_t>(b.items.size()),
                              b.total_modes, b.d_frec, b.d_rec64, st);
}

int enqueue_sum(gsc_batch &b, const Cfg &c, int blocks, int64_t n_units, cudaStream_t st) {
    GSC_CUDA(cudaMemsetAsync(b.d_counter, 0, sizeof(int), st));
    if (n_units == 0) return GSC_OK;
    if (is_fx(b))
        return batch_fx_launch(c.R, scalar_only(b), blocks, b.d_items, b.d_units, n_units,
                               b.d_counter, reinterpret_cast<const uint32_t *>(b.d_frec),
                               b.d_fxrange, st);
    if (is_plain(b))
        return batch_plain_launch(c.R, c.tile, blocks, b.d_items, b.d_units, n_units, b.d_counter,
                                  b.d_tab, b.d_rec, st);
    return batch_mixed_launch(c.R, b.form == GSC_FORM_MIXED_F64PHASE, blocks, b.d_items, b.d_units,
                              n_units, b.d_counter, b.d_frec, b.d_rec64, st);
}

int enqueue_run(gsc_batch &b, cudaStream_t st) {
    GSC_TRY(enqueue_tables(b, st));
    GSC_TRY(enqueue_sum(b, b.cfg, b.blocks, b.n_units, st));
    if (b.n_red > 0) {
        batch_reduce_kernel<<<static_cast<unsigned>((b.red_total + 255) / 256), 256, 0, st>>>(
            b.d_items, b.d_red_items, b.d_red_prefix, b.n_red, b.red_total);
        GSC_CUDA(cudaGetLastError());
    }
    return GSC_OK;
}

// Adopts configuration c: units, split partials, device tables.
int apply_config(gsc_batch &b, const Cfg &c) {
    const int occ = occupancy(b, c);
    if (occ <= 0) return set_error(GSC_ERR_INVALID, "batch configuration cannot be launched");
    const int blocks = occ * batch_sm_count(b.device);
    std::vector<BatchUnit> units;
    GSC_TRY(make_units(b, c, blocks, units));
    if (units.size() > 0x7fffffff)   // the queue counter is a 32-bit integer
        return set_error(GSC_ERR_INVALID, "batch too large: more than 2^31 work units");
    GSC_TRY(check_units(b.items, static_cast<int64_t>(kBatchThreads) * c.R, units));
    GSC_TRY(prepare_items(b));
    GSC_TRY(upload_units(b, units));
    b.cfg = c;
    b.blocks = blocks;
    b.n_units = static_cast<int64_t>(units.size());
    return GSC_OK;
}

std::vector<Cfg> candidates(const gsc_batch &b) {
    std::vector<Cfg> out;
    const int upbs[2] = {4, 16};
    if (is_plain(b)) {
        const int rt[4][2] = {{2, 8}, {4, 8}, {4, 16}, {8, 8}};
        for (auto &x : rt)
            for (int u : upbs) out.push_back(Cfg{x[0], x[1], u});
    } else {
        // 8 points per thread is left out: its samples timed faster than 4 on
        // parts of C5, but whole runs with it were slower (220 against 215 ms
        // end to end)
        const int rs[2] = {2, 4};
        for (int r : rs)
            for (int u : upbs) out.push_back(Cfg{r, 32, u});
    }
    return out;
}

// Times every candidate on an evenly spaced sample of its own cost-sorted
// queue (at least 8 units per resident block and 1/32 of the queue, the
// faster of two timed passes) and keeps the fastest per point*mode.
int autotune(gsc_batch &b, cudaStream_t st) {
    cudaEvent_t e0, e1;
    GSC_CUDA(cudaEventCreate(&e0));
    GSC_CUDA(cudaEventCreate(&e1));
    double best_rate = -1.0;
    Cfg best = b.cfg;
    int rc = GSC_OK;
    GSC_TRY(enqueue_tables(b, st));
    for (const Cfg &c : candidates(b)) {
        const int occ = occupancy(b, c);
        if (occ <= 0) continue;
        const int blocks = occ * batch_sm_count(b.device);
        std::vector<BatchUnit> units;
        if ((rc = make_units(b, c, blocks, units)) != GSC_OK) break;
        if ((rc = prepare_items(b)) != GSC_OK) break;
        // at least 8 units per block: with fewer, the time is that of the
        // largest sampled unit, which favours small units
        const size_t want = std::max<size_t>(8 * static_cast<size_t>(blocks), units.size() / 32);
        const size_t step = std::max<size_t>(1, units.size() / std::max<size_t>(1, want));
        std::vector<BatchUnit> sample;
        double work = 0.0;
        const int64_t ppb = static_cast<int64_t>(kBatchThreads) * c.R;
        for (size_t k = 0; k < units.size(); k += step) {
            const BatchUnit &u = units[k];
            const BatchItem &it = b.items[u.item];
            const int64_t np = std::min(ppb, it.n_points - u.p_first);
            work += static_cast<double>(np) * static_cast<double>(u.je - u.jb) *
                    (it.incompr ? it.dim : 1);
            sample.push_back(u);
        }
        if (sample.empty() || work <= 0.0) continue;
        if ((rc = upload_units(b, sample)) != GSC_OK) break;
        const int64_t ns = static_cast<int64_t>(sample.size());
        // one untimed pass (first launch of the instantiation), then the
        // faster of two timed ones
        if ((rc = enqueue_sum(b, c, blocks, ns, st)) != GSC_OK) break;
        float ms = 1e30f;
        for (int t = 0; t < 2 && rc == GSC_OK; ++t) {
            GSC_CUDA(cudaEventRecord(e0, st));
            if ((rc = enqueue_sum(b, c, blocks, ns, st)) != GSC_OK) break;
            GSC_CUDA(cudaEventRecord(e1, st));
            GSC_CUDA(cudaEventSynchronize(e1));
            float m = 0.f;
            GSC_CUDA(cudaEventElapsedTime(&m, e0, e1));
            b.tune_ms += m;
            ms = std::min(ms, m);
        }
        if (rc != GSC_OK) break;
        const double rate = work / std::max(1e-6, static_cast<double>(ms));
        if (rate > best_rate) {
            best_rate = rate;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != GSC_OK) return rc;
    b.cfg = best;
    return GSC_OK;
}

}  // namespace
}  // namespace gsc

extern "C" {

int gsc_batch_create(const gsc_batch_item *items, int64_t count, const gsc_opts *opts,
                     const gsc_batch_config *config, gsc_batch **out) {
    if (!out) return set_error(GSC_ERR_INVALID, "out is NULL");
    *out = nullptr;
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    if (count < 0 || (count > 0 && !items)) return set_error(GSC_ERR_INVALID, "bad item list");
    if (count > (int64_t(1) << 30)) return set_error(GSC_ERR_INVALID, "too many items");
    if (config && config->struct_size < static_cast<int32_t>(sizeof(gsc_batch_config)))
        return set_error(GSC_ERR_INVALID, "gsc_batch_config.struct_size is too small");
    int form = ro.form;
    if (form == GSC_FORM_AUTO) form = ro.tolerance >= 1e-6 ? GSC_FORM_MIXED : GSC_FORM_PLAIN_F64;
    if (form != GSC_FORM_PLAIN_F64 && form != GSC_FORM_MIXED && form != GSC_FORM_MIXED_F64PHASE)
        return set_error(GSC_ERR_INVALID,
                         "batches run the point forms: AUTO, PLAIN_F64, MIXED or MIXED_F64PHASE");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(GSC_ERR_NO_DEVICE, "no usable CUDA device; this library has no CPU path");
    }
    int device = ro.device;
    if (device < 0) GSC_CUDA(cudaGetDevice(&device));
    if (device >= ndev) return set_error(GSC_ERR_INVALID, "device ordinal out of range");
    DeviceGuard g;
    GSC_TRY(g.set(device));

    std::unique_ptr<gsc_batch> b(new gsc_batch);
    b->device = device;
    b->form = form;
    b->flags = ro.flags;
    GSC_TRY(fill_items(*b, items, count, true));

    // device memory of the plan
    GSC_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    const size_t nit = std::max<size_t>(1, b->items.size());
    GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_items), nit * sizeof(BatchItem)));
    GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_prefix), b->mode_prefix.size() * sizeof(int64_t)));
    GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_counter), sizeof(int)));
    GSC_CUDA(cudaMemcpy(b->d_prefix, b->mode_prefix.data(), b->mode_prefix.size() * sizeof(int64_t),
                        cudaMemcpyHostToDevice));
    const size_t M = static_cast<size_t>(b->total_modes);
    if (is_plain(*b)) {
        GSC_TRY(dmalloc(&b->d_tab, M * kPlainTableBytesPerMode));
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_rec), M * kPlainRecBytesPerMode));
    } else if (is_fx(*b)) {
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_frec), M * kFxRecBytesPerMode));
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_fxrange), nit * 4 * sizeof(unsigned long long)));
        DeviceCtx *ctx = nullptr;
        GSC_TRY(get_ctx(b->device, &ctx));
        b->range_flag = ctx->status + 4;        // the sticky range word gsc_device_status reads
    } else {
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_frec), M * kMixedRecBytesPerMode));
        GSC_TRY(dmalloc(reinterpret_cast<void **>(&b->d_rec64), M * kMixedRec64BytesPerMode));
    }
    GSC_CUDA(cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(BatchItem),
                        cudaMemcpyHostToDevice));

    // configuration: given, cached, or tuned on this ensemble
    Cfg c;
    const bool given = config && config->points_per_thread > 0 && config->units_per_block > 0 &&
                       (!is_plain(*b) || config->tile_modes > 0);
    if (given) {
        c.R = config->points_per_thread;
        c.tile = is_plain(*b) ? config->tile_modes : mixed_tile(*b);
        c.upb = config->units_per_block;
        const bool ok = is_plain(*b) ? batch_plain_config_ok(c.R, c.tile)
                         : is_fx(*b) ? batch_fx_config_ok(c.R) : batch_mixed_config_ok(c.R);
        if (!ok)
            return set_error(GSC_ERR_INVALID,
                             "unsupported batch configuration (points per thread 2, 4, 8; tile "
                             "modes 8 or 16 with 2 or 4 points per thread)");
    } else {
        int64_t pts = 0;
        for (auto &it : b->items) pts += it.n_points;
        // the autotuner's cache (tuner.cu): device, form, item count and the
        // buckets of the total work and point count
        const std::string key = device_name(device) + "|batch|f" + std::to_string(form) + "|c" +
                                std::to_string(count) + "|w" +
                                std::to_string(tune_bucket(b->total_work)) + "|p" +
                                std::to_string(tune_bucket(static_cast<double>(pts)));
        int v[4] = {0, 0, 0, 0};
        const int mode = tune_mode();
        if (mode != 0 && tune_get(key, v)) {
            c.R = v[0];
            c.tile = v[1];
            c.upb = v[2];
            const bool ok = c.upb > 0 && (is_plain(*b) ? batch_plain_config_ok(c.R, c.tile)
                                          : is_fx(*b) ? batch_fx_config_ok(c.R)
                                                      : batch_mixed_config_ok(c.R));
            if (!ok) c = Cfg{};                  // an entry from an older build
        } else if (mode == 2) {
            // the tuner reads the inputs: let pending work on them finish
            GSC_CUDA(cudaDeviceSynchronize());
            timing_reset(false);
            GSC_TRY(autotune(*b, b->cap_stream));
            GSC_CUDA(cudaStreamSynchronize(b->cap_stream));
            c = b->cfg;
            b->tuned = 1;
            const int nv[4] = {c.R, c.tile, c.upb, 0};
            tune_put(key, nv);
        }
        if (!is_plain(*b)) c.tile = mixed_tile(*b);   // the mixed forms' staged tiles
    }
    GSC_TRY(apply_config(*b, c));
    GSC_CUDA(cudaStreamSynchronize(b->cap_stream));
    *out = b.release();
    return GSC_OK;
}

int gsc_batch_run(gsc_batch *b, void *stream) {
    if (!b) return set_error(GSC_ERR_INVALID, "batch is NULL");
    DeviceGuard g;
    GSC_TRY(g.set(b->device));
    timing_reset(b->flags & GSC_FLAG_TIMING);
    return enqueue_run(*b, static_cast<cudaStream_t>(stream));
}

int gsc_batch_run_graph(gsc_batch *b, void *stream) {
    if (!b) return set_error(GSC_ERR_INVALID, "batch is NULL");
    DeviceGuard g;
    GSC_TRY(g.set(b->device));
    if (!b->exec) {
        timing_reset(false);   // no timing events inside the graph
        GSC_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_run(*b, b->cap_stream);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->cap_stream, &graph);
        if (rc != GSC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (batch)");
        b->graph = graph;
        GSC_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    GSC_CUDA(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
    return GSC_OK;
}

int gsc_batch_get_config(const gsc_batch *b, gsc_batch_config *cfg) {
    if (!b || !cfg) return set_error(GSC_ERR_INVALID, "batch or config is NULL");
    if (cfg->struct_size < static_cast<int32_t>(sizeof(gsc_batch_config)))
        return set_error(GSC_ERR_INVALID, "gsc_batch_config.struct_size is too small");
    cfg->points_per_thread = b->cfg.R;
    cfg->tile_modes = is_plain(*b) ? b->cfg.tile : mixed_tile(*b);
    cfg->units_per_block = b->cfg.upb;
    cfg->form = b->form;
    cfg->blocks = b->blocks;
    cfg->units = b->n_units;
    cfg->max_splits = b->max_splits;
    cfg->tuned = b->tuned;
    cfg->tune_ms = b->tune_ms;
    cfg->work = b->total_work;
    return GSC_OK;
}

int gsc_batch_destroy(gsc_batch *b) {
    delete b;
    return GSC_OK;
}

// The host-array ensemble call under the device context's lock.  *range_hit
// is set when a mixed-form item met a wave number past its integer phase
// range (its output is then invalid).
static int summate_batch_host(const gsc_batch_item *items, int64_t count, const Resolved &ro,
                              const gsc_batch_config *config, bool *range_hit) {
    *range_hit = false;
    if (count < 0 || (count > 0 && !items)) return set_error(GSC_ERR_INVALID, "bad item list");
    // host-side validation (the plan re-checks shapes and forms)
    size_t n_in = 0, n_out = 0;
    double total_work = 0.0;
    std::vector<double> work(static_cast<size_t>(count));
    for (int64_t i = 0; i < count; ++i) {
        const gsc_batch_item &x = items[i];
        if (x.n_modes < 0 || x.n_points < 0 || x.dim < 1 || x.dim > 3)
            return set_error(x.dim < 1 || x.dim > 3 ? GSC_ERR_DIM : GSC_ERR_INVALID,
                             "item " + std::to_string(i) + ": bad dimension, mode or point count");
        const bool f = x.kind == GSC_BATCH_FOURIER;
        if ((x.n_modes > 0 && (!x.cov || !x.z1 || !x.z2 || (f && !x.spectrum_factor))) ||
            (x.n_points > 0 && (!x.pos || !x.out)))
            return set_error(GSC_ERR_INVALID, "item " + std::to_string(i) + ": NULL array");
        const int64_t nout = x.kind == GSC_BATCH_INCOMPR ? x.dim : 1;
        n_in += static_cast<size_t>(x.dim * x.n_modes + 2 * x.n_modes + (f ? x.n_modes : 0) +
                                    x.dim * x.n_points);
        n_out += static_cast<size_t>(nout * x.n_points);
        work[static_cast<size_t>(i)] = static_cast<double>(x.n_points) * x.n_modes * nout;
        total_work += work[static_cast<size_t>(i)];
    }
    // Large ensembles run as a few groups of consecutive items, each its own
    // plan: the inputs of one group are packed and copied
    // (copy stream) while the previous group computes, and the results of a
    // group are copied back while the next one computes.  Groups alternate
    // between two compute streams, so that a group's persistent kernel takes
    // the SMs that the previous group's last units leave idle.
    // The first and the last group are small (1/(4G) of the work each): the
    // first group's input copy and the last group's result copy are the ones
    // that nothing hides.  The others share the rest equally; their inputs
    // copy (about 5 times faster than they compute) within the previous
    // group, and their results while the next one computes.
    const int G = (total_work >= 4.0e10 && count >= 16) ? 8
                  : (total_work >= 4.0e9 && count >= 8) ? 4 : 1;
    auto group_end = [G](int g) {          // fraction of the work in groups [0, g]
        const double edge = 1.0 / (4.0 * G);
        return g >= G - 1 ? 1.0 : edge + (1.0 - 2.0 * edge) * g / (G - 2);
    };
    std::vector<int64_t> gstart(static_cast<size_t>(G) + 1, count);
    gstart[0] = 0;
    {
        double acc = 0.0;
        int g = 1;
        for (int64_t i = 0; i < count && g < G; ++i) {
            acc += work[static_cast<size_t>(i)];
            while (g < G && acc >= total_work * group_end(g - 1)) gstart[static_cast<size_t>(g++)] = i + 1;
        }
        for (; g < G; ++g) gstart[static_cast<size_t>(g)] = count;
    }
    timing_reset(ro.flags & GSC_FLAG_TIMING);
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(ro.device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g;
    GSC_TRY(g.set(ctx->device));
    cudaStream_t st = ctx->stream;
    if (!ctx->copy_stream)
        GSC_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    cudaStream_t cs = ctx->copy_stream;
    if (G > 1 && !ctx->stream2)
        GSC_CUDA(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
    GSC_TRY(ensure_pinned(*ctx, std::max(n_in, n_out) * sizeof(double) + 64));
    GSC_TRY(ensure_dev(*ctx, ctx->io, (n_in + n_out) * sizeof(double) + 256));
    double *h = static_cast<double *>(ctx->pinned);
    double *d = static_cast<double *>(ctx->io.ptr);
    double *dout = d + n_in;
    std::vector<gsc_batch_item> dev(static_cast<size_t>(count));
    // Every input is packed back to back into the pinned staging and moved
    // in 64 MiB chunks (h2d_packed): one pageable copy per array would pay
    // the driver's fixed cost hundreds of times.
    std::vector<std::vector<HostSrc>> in_segs(static_cast<size_t>(G));
    size_t off = 0, oo = 0;
    for (int gi = 0; gi < G; ++gi) {
        auto &segs = in_segs[static_cast<size_t>(gi)];
        auto put = [&](const double *src, int64_t n) -> const double * {
            if (n <= 0) return nullptr;
            const double *r = d + off;
            segs.push_back(HostSrc{src, off * sizeof(double), static_cast<size_t>(n) * sizeof(double)});
            off += static_cast<size_t>(n);
            return r;
        };
        for (int64_t i = gstart[static_cast<size_t>(gi)]; i < gstart[static_cast<size_t>(gi) + 1]; ++i) {
            const gsc_batch_item &x = items[i];
            gsc_batch_item &y = dev[static_cast<size_t>(i)];
            y = x;
            y.cov = put(x.cov, x.dim * x.n_modes);
            y.z1 = put(x.z1, x.n_modes);
            y.z2 = put(x.z2, x.n_modes);
            y.spectrum_factor =
                x.kind == GSC_BATCH_FOURIER ? put(x.spectrum_factor, x.n_modes) : nullptr;
            y.pos = put(x.pos, x.dim * x.n_points);
            y.out = x.n_points > 0 ? dout + oo : nullptr;
            oo += static_cast<size_t>((x.kind == GSC_BATCH_INCOMPR ? x.dim : 1) * x.n_points);
        }
    }
    // fault in pageable output pages on host threads while the GPU works
    std::vector<HostSeg> osegs;
    for (int64_t i = 0; i < count; ++i) {
        const gsc_batch_item &x = items[i];
        const size_t n = static_cast<size_t>((x.kind == GSC_BATCH_INCOMPR ? x.dim : 1) * x.n_points);
        osegs.push_back(HostSeg{is_pinned_host(x.out) ? nullptr : x.out, n * sizeof(double)});
    }
    Prefault pf;
    pf.start_many(osegs);
    std::vector<cudaEvent_t> ev(static_cast<size_t>(2 * G), nullptr);
    auto destroy_events = [&] {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    };
    int rc = GSC_OK;
    for (auto &e : ev)
        if (rc == GSC_OK) rc = cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // Launch choices of the groups: the caller's, else one set for the whole
    // ensemble -- from the autotuner's cache under the ensemble's key, or
    // tuned on the group with the most work and stored there -- so that a
    // small group's noisy timing does not choose for the rest.  Groups
    // created before that one run on the defaults (4 points per thread, 16
    // units per block).
    // (a config whose fields are zero asks the autotuner, as for one plan)
    const bool cfg_given = config && config->points_per_thread > 0 && config->units_per_block > 0;
    gsc_batch_config gcfg{};
    gcfg.struct_size = sizeof(gsc_batch_config);
    bool have_cfg = cfg_given;
    if (cfg_given) gcfg = *config;
    int gmax = 0;
    std::string gkey;
    if (G > 1 && !cfg_given) {
        std::vector<double> gw(static_cast<size_t>(G), 0.0);
        double pts = 0.0;
        for (int gi = 0; gi < G; ++gi)
            for (int64_t i = gstart[static_cast<size_t>(gi)]; i < gstart[static_cast<size_t>(gi) + 1]; ++i) {
                gw[static_cast<size_t>(gi)] += work[static_cast<size_t>(i)];
                pts += static_cast<double>(items[i].n_points);
            }
        for (int gi = 1; gi < G; ++gi)
            if (gw[static_cast<size_t>(gi)] > gw[static_cast<size_t>(gmax)]) gmax = gi;
        gkey = device_name(ctx->device) + "|batchg|f" + std::to_string(ro.form) + "|t" +
               std::to_string(static_cast<int64_t>(ro.tolerance * 1e15)) + "|c" +
               std::to_string(count) + "|w" + std::to_string(tune_bucket(total_work)) + "|p" +
               std::to_string(tune_bucket(pts));
        int v[4] = {0, 0, 0, 0};
        if (tune_mode() != 0 && tune_get(gkey, v) && v[0] > 0 && v[2] > 0) {
            gcfg.points_per_thread = v[0];
            gcfg.tile_modes = v[1];
            gcfg.units_per_block = v[2];
            have_cfg = true;
        }
    }
    if (ctx->batch.size() != static_cast<size_t>(G)) {
        for (gsc_batch *b : ctx->batch) {
            if (rc == GSC_OK) rc = cuda_ok(cudaStreamSynchronize(st));
            gsc_batch_destroy(b);
        }
        ctx->batch.assign(static_cast<size_t>(G), nullptr);
        ctx->batch_sig.assign(static_cast<size_t>(G), {});
    }
    // the range word of this call's plans (device calls keep the sticky word)
    int *range_word = ctx->status + 7;
    if (rc == GSC_OK) rc = cuda_ok(cudaMemsetAsync(range_word, 0, sizeof(int), st));
    // the second compute stream starts after the work queued before this call
    if (rc == GSC_OK && G > 1) {
        cudaEvent_t e0 = ev[static_cast<size_t>(2 * G - 1)];
        rc = cuda_ok(cudaEventRecord(e0, st));
        if (rc == GSC_OK) rc = cuda_ok(cudaStreamWaitEvent(ctx->stream2, e0, 0));
    }
    for (int gi = 0; gi < G && rc == GSC_OK; ++gi) {
        const int64_t i0 = gstart[static_cast<size_t>(gi)], i1 = gstart[static_cast<size_t>(gi) + 1];
        cudaStream_t gs = (gi & 1) ? ctx->stream2 : st;
        // the copies are timed here only when the plan is reused (a new
        // plan's creation starts the call's timing afresh)
        TimedLaunch tc(cs);
        tc.begin(K_COPY_H2D);
        rc = h2d_packed(cs, d, h, in_segs[static_cast<size_t>(gi)]);
        tc.end();
        if (rc == GSC_OK) rc = cuda_ok(cudaEventRecord(ev[static_cast<size_t>(gi)], cs));
        if (rc == GSC_OK) rc = cuda_ok(cudaStreamWaitEvent(gs, ev[static_cast<size_t>(gi)], 0));
        if (rc != GSC_OK) break;
        if (i1 == i0) {            // an empty group (a few items hold most of the work)
            rc = cuda_ok(cudaEventRecord(ev[static_cast<size_t>(G + gi)], gs));
            continue;
        }
        // the group's plan of the previous call is reused when the shapes match
        std::vector<int64_t> sig = {reinterpret_cast<int64_t>(ctx->io.ptr), ro.form,
                                    static_cast<int64_t>(ro.tolerance * 1e15), i1 - i0, gi};
        if (config)
            sig.insert(sig.end(),
                       {config->points_per_thread, config->tile_modes, config->units_per_block});
        for (int64_t i = i0; i < i1; ++i) {
            const auto &y = dev[static_cast<size_t>(i)];
            // the device addresses too: they move with the earlier groups' sizes
            sig.insert(sig.end(), {y.dim, y.kind, y.n_modes, y.n_points,
                                   reinterpret_cast<int64_t>(y.cov), reinterpret_cast<int64_t>(y.pos),
                                   reinterpret_cast<int64_t>(y.out)});
        }
        gsc_batch *&plan = ctx->batch[static_cast<size_t>(gi)];
        if (!plan || sig != ctx->batch_sig[static_cast<size_t>(gi)]) {
            // the old plan's runs and this group's inputs must be done (the
            // new plan's tuner reads the inputs)
            rc = cuda_ok(cudaStreamSynchronize(gs));
            if (rc == GSC_OK) rc = cuda_ok(cudaStreamSynchronize(cs));
            if (plan) {
                gsc_batch_destroy(plan);
                plan = nullptr;
            }
            gsc_opts o{};
            o.struct_size = sizeof(gsc_opts);
            o.form = ro.form;
            o.device = ctx->device;
            o.flags = ro.flags;
            o.stream = nullptr;
            o.tolerance = ro.tolerance;
            const gsc_batch_config *pc = config;
            gsc_batch_config dflt = gcfg;
            if (G > 1 && !cfg_given) {
                if (have_cfg) {
                    pc = &gcfg;
                } else if (gi != gmax) {
                    dflt.points_per_thread = 4;
                    dflt.tile_modes = 8;
                    dflt.units_per_block = 16;
                    pc = &dflt;
                }                   // the largest group: the autotuner chooses
            }
            if (rc == GSC_OK) rc = gsc_batch_create(dev.data() + i0, i1 - i0, &o, pc, &plan);
            if (rc != GSC_OK) break;
            if (G > 1 && !cfg_given && !have_cfg && gi == gmax) {
                gsc_batch_config c{};
                c.struct_size = sizeof(gsc_batch_config);
                rc = gsc_batch_get_config(plan, &c);
                if (rc != GSC_OK) break;
                gcfg.points_per_thread = c.points_per_thread;
                gcfg.tile_modes = c.tile_modes;
                gcfg.units_per_block = c.units_per_block;
                have_cfg = true;
                if (tune_mode() == 2) {
                    const int v[4] = {c.points_per_thread, c.tile_modes, c.units_per_block, 0};
                    tune_put(gkey, v);
                }
            }
            plan->range_flag = range_word;
            ctx->batch_sig[static_cast<size_t>(gi)] = sig;
            timing_reset(ro.flags & GSC_FLAG_TIMING);
        }
        plan->flags = ro.flags;                       // this call's timing request
        rc = enqueue_run(*plan, gs);                  // (gsc_batch_run would restart the timing records)
        if (rc == GSC_OK) rc = cuda_ok(cudaEventRecord(ev[static_cast<size_t>(G + gi)], gs));
    }
    pf.join();
    // each group's results, once it is done, straight into the callers' arrays
    oo = 0;
    for (int gi = 0; gi < G && rc == GSC_OK; ++gi) {
        rc = cuda_ok(cudaStreamWaitEvent(cs, ev[static_cast<size_t>(G + gi)], 0));
        TimedLaunch tc(cs);
        tc.begin(K_COPY_D2H);
        for (int64_t i = gstart[static_cast<size_t>(gi)];
             i < gstart[static_cast<size_t>(gi) + 1] && rc == GSC_OK; ++i) {
            const size_t n = osegs[static_cast<size_t>(i)].bytes;
            if (n > 0)
                rc = cuda_ok(cudaMemcpyAsync(items[i].out, dout + oo, n, cudaMemcpyDeviceToHost, cs));
            oo += n / sizeof(double);
        }
        tc.end();
    }
    // on an error, let the queued work on the buffers finish before returning
    int rs = cuda_ok(cudaStreamSynchronize(st));
    if (G > 1) {
        const int r2 = cuda_ok(cudaStreamSynchronize(ctx->stream2));
        if (rs == GSC_OK) rs = r2;
    }
    const int rcs = cuda_ok(cudaStreamSynchronize(cs));
    destroy_events();
    GSC_TRY(rc);
    GSC_TRY(rs);
    GSC_TRY(rcs);
    int hit = 0;
    GSC_CUDA(cudaMemcpy(&hit, range_word, sizeof(int), cudaMemcpyDeviceToHost));
    *range_hit = hit != 0;
    return GSC_OK;
}

int gsc_summate_batch_f64(const gsc_batch_item *items, int64_t count, const gsc_opts *opts,
                          const gsc_batch_config *config) {
    Resolved ro;
    GSC_TRY(resolve_opts(opts, &ro));
    bool range_hit = false;
    GSC_TRY(summate_batch_host(items, count, ro, config, &range_hit));
    if (!range_hit) return GSC_OK;
    // a wave number past the mixed form's integer phase range: AUTO recomputes
    // the ensemble on the plain FP64 form, an explicit mixed form reports it
    if (ro.form != GSC_FORM_AUTO)
        return set_error(GSC_ERR_KERNEL,
                         "mixed: a wave number times the largest coordinate of its item exceeds "
                         "2^30 turns, past the range of its integer phase; the outputs are "
                         "invalid.  Use form AUTO (which recomputes such ensembles on the plain "
                         "FP64 form) or plain");
    Resolved rp = ro;
    rp.form = GSC_FORM_PLAIN_F64;
    return summate_batch_host(items, count, rp, nullptr, &range_hit);
}

int gsc_selftest_batch_queue(const gsc_batch_item *items, int64_t count, int32_t form,
                             const gsc_batch_config *config, int32_t blocks, int32_t corruption) {
    if (count < 0 || (count > 0 && !items)) return set_error(GSC_ERR_INVALID, "bad item list");
    if (count > (int64_t(1) << 20)) return set_error(GSC_ERR_INVALID, "too many items");
    if (!config || config->struct_size < static_cast<int32_t>(sizeof(gsc_batch_config)))
        return set_error(GSC_ERR_INVALID, "config is NULL or its struct_size is too small");
    if (form != GSC_FORM_PLAIN_F64 && form != GSC_FORM_MIXED && form != GSC_FORM_MIXED_F64PHASE)
        return set_error(GSC_ERR_INVALID, "batches run the point forms PLAIN_F64, MIXED or MIXED_F64PHASE");
    if (blocks < 1 || blocks > (1 << 20)) return set_error(GSC_ERR_INVALID, "blocks out of range");
    if (corruption < 0 || corruption > 6) return set_error(GSC_ERR_INVALID, "unknown corruption");
    gsc_batch b;   // host fields only: no device memory is made
    b.form = form;
    GSC_TRY(fill_items(b, items, count, false));
    Cfg c;
    c.R = config->points_per_thread;
    c.tile = is_plain(b) ? config->tile_modes : mixed_tile(b);
    c.upb = config->units_per_block;
    const bool ok = c.upb > 0 && (is_plain(b) ? batch_plain_config_ok(c.R, c.tile)
                                  : is_fx(b)  ? batch_fx_config_ok(c.R)
                                              : batch_mixed_config_ok(c.R));
    if (!ok) return set_error(GSC_ERR_INVALID, "unsupported batch configuration");
    std::vector<BatchUnit> units;
    GSC_TRY(make_units(b, c, blocks, units));
    if (units.size() > (size_t(1) << 26)) return set_error(GSC_ERR_INVALID, "queue too large for the check");
    if (corruption > 0) {
        if (units.empty()) return set_error(GSC_ERR_INVALID, "no units to corrupt");
        const size_t k = units.size() / 2;
        switch (corruption) {
        case 1: units.erase(units.begin() + static_cast<std::ptrdiff_t>(k)); break;
        case 2:
            if (units.size() > 1) units[(k + 1) % units.size()] = units[k];
            else units.push_back(units[k]);
            break;
        case 3: units[k].item = static_cast<int32_t>(count); break;
        case 4: units[k].jb += 1; break;
        case 5: units[k].p_first += 1; break;
        case 6: units[k].split = b.items[static_cast<size_t>(units[k].item)].splits; break;
        }
    }
    return check_units(b.items, static_cast<int64_t>(kBatchThreads) * c.R, units);
}

int gsc_last_batch_config(int32_t device, gsc_batch_config *config) {
    DeviceCtx *ctx = nullptr;
    GSC_TRY(get_ctx(device, &ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->batch.empty() || !ctx->batch[0])
        return set_error(GSC_ERR_INVALID, "no batch has run on this device");
    // a call split into groups reports the first group's launch choices and
    // the totals of all groups
    GSC_TRY(gsc_batch_get_config(ctx->batch[0], config));
    for (size_t i = 1; i < ctx->batch.size(); ++i) {
        gsc_batch_config c = *config;
        if (!ctx->batch[i]) continue;
        GSC_TRY(gsc_batch_get_config(ctx->batch[i], &c));
        config->units += c.units;
        config->work += c.work;
        config->tune_ms += c.tune_ms;
        config->tuned = config->tuned || c.tuned;
        config->max_splits = std::max(config->max_splits, c.max_splits);
    }
    return GSC_OK;
}

}  // extern "C"
