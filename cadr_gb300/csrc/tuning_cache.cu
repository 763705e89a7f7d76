// tuning_cache.cu - the batched form's autotuner search and its persistent
// cache (host code only).
//
// The search walks every supported (block threads, items per thread, CTAs
// per SM) combination and keeps the fastest, as timed by a caller-supplied
// function.  Before it times anything it looks the key up in a cache file;
// after a search it stores the pick under the key.  cadr_autotune_batched
// supplies a CUDA-event timer and a key made of the batch's shape, the GPU
// and its driver; the search itself needs no GPU, so it is tested on the
// CPU with a stand-in timer.
//
// Cache file: JSON, one entry per line under "entries", written whole to a
// temporary file and renamed over the old one, so a reader never sees a
// torn file (with several writers the last rename wins):
//   {
//    "version": 2,
//    "entries": {
//     "<key>": {"block_threads": 256, "items_per_thread": 8, "ctas_per_sm": 4, "form": 0, "ms": 0.7712},
//     ...
//    }
//   }
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace cadr;

namespace cadr {
namespace {

struct Entry {
    cadr_tuning tuning;
    float ms;
};

std::mutex g_cache_mu;

// Keys are written between double quotes: they may not contain quotes,
// backslashes or line breaks.
bool key_ok(const char* key)
{
    if (!key || !*key) return false;
    for (const char* p = key; *p; p++)
        if (*p == '"' || *p == '\\' || *p == '\n' || *p == '\r') return false;
    return true;
}

// Entries of a cache file; a missing or unreadable file has none.
std::map<std::string, Entry> read_cache(const char* path)
{
    std::map<std::string, Entry> out;
    FILE* f = std::fopen(path, "r");
    if (!f) return out;
    char line[4096];
    while (std::fgets(line, sizeof line, f)) {
        const char* q0 = std::strchr(line, '"');
        if (!q0) continue;
        const char* q1 = std::strchr(q0 + 1, '"');
        if (!q1) continue;
        const char* body = std::strstr(q1, "\"block_threads\"");
        if (!body) continue;
        Entry e{};
        if (std::sscanf(body,
                        "\"block_threads\": %u, \"items_per_thread\": %u, \"ctas_per_sm\": %u, \"form\": %u, "
                        "\"ms\": %f",
                        &e.tuning.block_threads, &e.tuning.items_per_thread, &e.tuning.ctas_per_sm, &e.tuning.form,
                        &e.ms) == 5)
            out[std::string(q0 + 1, q1)] = e;
    }
    std::fclose(f);
    return out;
}

bool write_cache(const char* path, const std::map<std::string, Entry>& entries)
{
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "{\n \"version\": 2,\n \"entries\": {\n");
    size_t k = 0;
    for (const auto& kv : entries) {
        const cadr_tuning& t = kv.second.tuning;
        std::fprintf(f,
                     "  \"%s\": {\"block_threads\": %u, \"items_per_thread\": %u, \"ctas_per_sm\": %u, "
                     "\"form\": %u, \"ms\": %.6f}%s\n",
                     kv.first.c_str(), t.block_threads, t.items_per_thread, t.ctas_per_sm, t.form, kv.second.ms,
                     ++k < entries.size() ? "," : "");
    }
    std::fprintf(f, " }\n}\n");
    const bool ok = std::fclose(f) == 0;
    return ok && std::rename(tmp.c_str(), path) == 0;
}

}  // namespace

// The combinations the autotuner tries, in search order: every persistent
// shape whose threads an SM holds, then the three-launch form.
std::vector<cadr_tuning> tuning_candidates()
{
    std::vector<cadr_tuning> out;
    for (uint32_t th : {128u, 256u, 512u})
        for (uint32_t ipt : {4u, 8u, 16u})
            for (uint32_t c : {2u, 4u, 8u})
                if (th * c <= 2048) out.push_back(cadr_tuning{th, ipt, c, CADR_BATCHED_PERSISTENT});
    out.push_back(cadr_tuning{256u, 8u, 4u, CADR_BATCHED_THREE_LAUNCH});
    return out;
}

}  // namespace cadr

extern "C" {

CADR_API cadr_status cadr_tuning_cache_lookup(const char* path, const char* key, cadr_tuning* out, float* ms)
{
    if (!path || !out || !key_ok(key)) return fail(CADR_ERR_INVALID_ARG, "tuning_cache_lookup: bad argument");
    std::lock_guard<std::mutex> lk(g_cache_mu);
    const auto entries = read_cache(path);
    const auto it = entries.find(key);
    if (it == entries.end()) return CADR_ERR_NOT_READY;
    *out = it->second.tuning;
    if (ms) *ms = it->second.ms;
    return CADR_OK;
}

CADR_API cadr_status cadr_tuning_cache_store(const char* path, const char* key, const cadr_tuning* tuning, float ms)
{
    if (!path || !tuning || !key_ok(key)) return fail(CADR_ERR_INVALID_ARG, "tuning_cache_store: bad argument");
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto entries = read_cache(path);
    entries[key] = Entry{*tuning, ms};
    if (!write_cache(path, entries)) return fail(CADR_ERR_INVALID_ARG, "tuning_cache_store: cannot write %s", path);
    return CADR_OK;
}

CADR_API cadr_status cadr_autotune_with(const char* cache_path, const char* key, cadr_time_tuning_fn time_fn,
                                        void* user, cadr_tuning* best, float* best_ms, int* from_cache)
{
    if (!time_fn || !best || (cache_path && !key_ok(key)))
        return fail(CADR_ERR_INVALID_ARG, "autotune_with: bad argument");
    if (from_cache) *from_cache = 0;
    if (cache_path) {
        float ms = 0;
        if (cadr_tuning_cache_lookup(cache_path, key, best, &ms) == CADR_OK) {
            if (best_ms) *best_ms = ms;
            if (from_cache) *from_cache = 1;
            return CADR_OK;
        }
    }
    float best_t = 0;
    bool have = false;
    for (const cadr_tuning& tu : tuning_candidates()) {
        float ms = 0;
        const cadr_status st = time_fn(&tu, user, &ms);
        if (st != CADR_OK) return st;
        if (!have || ms < best_t) {
            best_t = ms;
            *best = tu;
            have = true;
        }
    }
    if (best_ms) *best_ms = best_t;
    if (cache_path) return cadr_tuning_cache_store(cache_path, key, best, best_t);
    return CADR_OK;
}

}  // extern "C"
