// tuner.cu -- the autotuner's cache of launch configurations.
//
// Kernels with choices that depend on the shape of a call (points per
// thread, how finely modes are split over blocks, the batch planner's unit
// granularity) time their candidates on the call's own data the first time a
// shape bucket is seen (tune mode 2, the default) and keep the winner here,
// keyed by text: the device's name, the kernel family and the shape buckets.
// With a cache file (gsc_tune_cache_open, or the path in GSC_TUNE_CACHE on
// first use) the entries persist across processes:
//
//     # gstools-core-gb300 autotuner cache v1
//     <key> TAB <v0> <v1> <v2> <v3>
//     ...
//     #checksum <FNV-1a 64 of every byte above, 16 hex digits>
//
// A file whose header, lines or checksum do not match is refused as a whole
// (gsc_tune_cache_open returns GSC_ERR_INVALID) and then neither read nor
// overwritten.  The file is rewritten (to a temporary name, then renamed)
// after every new entry.  Thread safe.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "internal.h"

namespace gsc {
namespace {

constexpr const char *kHeader = "# gstools-core-gb300 autotuner cache v1\n";

struct TuneCache {
    std::mutex mu;
    std::map<std::string, std::array<int, 4>> entries;
    std::string path;          // persistence file, empty = memory only
    bool env_checked = false;
    int mode = -1;             // -1: not read from the environment yet
};

TuneCache &cache() {
    static TuneCache *c = new TuneCache();   // never destroyed: used until exit
    return *c;
}

uint64_t fnv1a(const std::string &s) {
    uint64_t h = 1469598103934665603ull;
    for (unsigned char ch : s) {
        h ^= ch;
        h *= 1099511628211ull;
    }
    return h;
}

std::string serialise(const std::map<std::string, std::array<int, 4>> &e) {
    std::string body = kHeader;
    for (const auto &kv : e) {
        char buf[96];
        snprintf(buf, sizeof(buf), "\t%d %d %d %d\n", kv.second[0], kv.second[1], kv.second[2],
                 kv.second[3]);
        body += kv.first + buf;
    }
    char tail[48];
    snprintf(tail, sizeof(tail), "#checksum %016llx\n",
             static_cast<unsigned long long>(fnv1a(body)));
    return body + tail;
}

// Parses a whole file; false (with the reason) for anything out of shape.
bool parse(const std::string &text, std::map<std::string, std::array<int, 4>> &out,
           std::string &why) {
    const size_t hl = strlen(kHeader);
    if (text.compare(0, hl, kHeader) != 0) {
        why = "unknown header";
        return false;
    }
    const size_t cpos = text.rfind("#checksum ");
    if (cpos == std::string::npos || cpos < hl) {
        why = "no checksum line";
        return false;
    }
    const std::string body = text.substr(0, cpos);
    char hex[17] = {0};
    if (sscanf(text.c_str() + cpos, "#checksum %16[0-9a-f]", hex) != 1 || strlen(hex) != 16 ||
        text.size() != cpos + 27) {
        why = "malformed checksum line";
        return false;
    }
    if (strtoull(hex, nullptr, 16) != fnv1a(body)) {
        why = "checksum mismatch";
        return false;
    }
    std::istringstream in(body.substr(hl));
    std::string line;
    while (std::getline(in, line)) {
        const size_t tab = line.find('\t');
        std::array<int, 4> v{};
        if (tab == std::string::npos || tab == 0 ||
            sscanf(line.c_str() + tab + 1, "%d %d %d %d", &v[0], &v[1], &v[2], &v[3]) != 4) {
            why = "malformed entry";
            return false;
        }
        out[line.substr(0, tab)] = v;
    }
    return true;
}

int open_locked(TuneCache &c, const char *path) {
    c.path.clear();
    if (!path || !*path) return GSC_OK;
    FILE *f = fopen(path, "rb");
    if (f) {
        std::string text;
        char buf[4096];
        size_t n;
        while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
        fclose(f);
        std::map<std::string, std::array<int, 4>> loaded;
        std::string why;
        if (!parse(text, loaded, why))
            return set_error(GSC_ERR_INVALID, std::string("autotuner cache ") + path +
                                                  " refused (" + why +
                                                  "); it is neither read nor overwritten");
        for (auto &kv : loaded) c.entries[kv.first] = kv.second;
    }
    c.path = path;
    return GSC_OK;
}

void env_once(TuneCache &c) {
    if (c.env_checked) return;
    c.env_checked = true;
    if (c.mode < 0) {
        const char *m = getenv("GSC_TUNE");
        c.mode = (m && (m[0] == '0' || m[0] == '1') && !m[1]) ? m[0] - '0' : 2;
    }
    if (const char *p = getenv("GSC_TUNE_CACHE")) open_locked(c, p);
}

void save_locked(TuneCache &c) {
    if (c.path.empty()) return;
    const std::string text = serialise(c.entries);
    const std::string tmp = c.path + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return;
    const bool ok = fwrite(text.data(), 1, text.size(), f) == text.size();
    fclose(f);
    if (ok) rename(tmp.c_str(), c.path.c_str());
    else remove(tmp.c_str());
}

}  // namespace

bool tune_get(const std::string &key, int v[4]) {
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_once(c);
    auto f = c.entries.find(key);
    if (f == c.entries.end()) return false;
    for (int i = 0; i < 4; ++i) v[i] = f->second[i];
    return true;
}

void tune_put(const std::string &key, const int v[4]) {
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_once(c);
    c.entries[key] = {v[0], v[1], v[2], v[3]};
    save_locked(c);
}

int tune_mode() {
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_once(c);
    return c.mode;
}

std::string device_name(int device) {
    cudaDeviceProp p{};
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        cudaGetLastError();
        return "device" + std::to_string(device);
    }
    std::string s = p.name;
    for (char &ch : s)
        if (ch == '\t' || ch == '\n' || ch == '|') ch = ' ';
    return s;
}

int tune_bucket(double v) {
    int e = 0;
    if (v >= 1.0) frexp(v, &e);
    return e;
}

}  // namespace gsc

using namespace gsc;

extern "C" {

int gsc_tune_cache_open(const char *path) {
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.env_checked = true;            // an explicit path overrides GSC_TUNE_CACHE
    if (c.mode < 0) {
        const char *m = getenv("GSC_TUNE");
        c.mode = (m && (m[0] == '0' || m[0] == '1') && !m[1]) ? m[0] - '0' : 2;
    }
    return open_locked(c, path);
}

int gsc_tune_cache_size(int64_t *entries) {
    if (!entries) return set_error(GSC_ERR_INVALID, "entries is NULL");
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_once(c);
    *entries = static_cast<int64_t>(c.entries.size());
    return GSC_OK;
}

int gsc_tune_cache_get(const char *key, int32_t *values) {
    if (!key || !values) return set_error(GSC_ERR_INVALID, "key or values is NULL");
    int v[4];
    if (!tune_get(key, v)) return set_error(GSC_ERR_INVALID, std::string("no entry ") + key);
    for (int i = 0; i < 4; ++i) values[i] = v[i];
    return GSC_OK;
}

int gsc_tune_cache_put(const char *key, const int32_t *values) {
    if (!key || !values || !*key) return set_error(GSC_ERR_INVALID, "key or values is NULL");
    for (const char *p = key; *p; ++p)
        if (*p == '\t' || *p == '\n') return set_error(GSC_ERR_INVALID, "key holds a tab or newline");
    const int v[4] = {values[0], values[1], values[2], values[3]};
    tune_put(key, v);
    return GSC_OK;
}

int gsc_tune_cache_clear(void) {
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.entries.clear();
    return GSC_OK;
}

int gsc_tune_set_mode(int32_t mode) {
    if (mode < 0 || mode > 2) return set_error(GSC_ERR_INVALID, "tune mode must be 0, 1 or 2");
    TuneCache &c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_once(c);
    c.mode = mode;
    return GSC_OK;
}

}  // extern "C"
