// tune_cache.cpp — the autotune cache: the winner of solrt_batch_autotune
// for a batch's shape, kept in a text file of JSON lines so that a later
// process with the same batch on the same GPU skips the timing.
//
//   {"key": "gpu=NVIDIA_GB300|sm=152|kind=0|cap=134217728|flags=1|jobs=256|h=9c0f...",
//    "block_size": 128, "smem_stack": 32, "pass_paths": 0, "best_ms": 428.1}
//
// (one object per line). The key names the GPU, the BVH kind, the path
// capacity, the batch flags and a 64-bit FNV-1a hash of every job's shape
// (size, spp, bounces, modes, integrator, triangle count): what changes the
// best launch shape, not the cameras or frames. No counterpart in the
// reference (its launch shape is the driver's).
#include <cuda_runtime.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct solrt_context : solrt::Context {};
struct solrt_batch : solrt::Batch {};

namespace solrt {

namespace {

struct Entry {
    std::string key;
    TuneConfig cfg;
    float best_ms = 0.0f;
};

void fnv(uint64_t& h, uint32_t v) {
    for (int i = 0; i < 4; ++i) {
        h ^= (v >> (8 * i)) & 0xffu;
        h *= 1099511628211ull;
    }
}

// Value after `"name":` in a line, or nullptr.
const char* field(const std::string& line, const char* name) {
    const std::string pat = std::string("\"") + name + "\"";
    size_t at = line.find(pat);
    if (at == std::string::npos) return nullptr;
    at += pat.size();
    while (at < line.size() && isspace((unsigned char)line[at])) ++at;
    if (at >= line.size() || line[at] != ':') return nullptr;
    ++at;
    while (at < line.size() && isspace((unsigned char)line[at])) ++at;
    return line.c_str() + at;
}

bool parse_uint(const std::string& line, const char* name, uint32_t& out) {
    const char* v = field(line, name);
    if (!v || !isdigit((unsigned char)*v)) return false;
    char* end = nullptr;
    const unsigned long long x = strtoull(v, &end, 10);
    if (end == v || x > 0xffffffffull) return false;
    out = (uint32_t)x;
    return true;
}

bool parse_line(const std::string& line, Entry& e) {
    const char* k = field(line, "key");
    if (!k || *k != '"') return false;
    const char* close = strchr(k + 1, '"');
    if (!close) return false;
    e.key.assign(k + 1, close);
    if (!parse_uint(line, "block_size", e.cfg.block) || !parse_uint(line, "smem_stack", e.cfg.smem) ||
        !parse_uint(line, "pass_paths", e.cfg.pass_paths))
        return false;
    if (!extend_variant_ok(e.cfg.block, e.cfg.smem)) return false;
    const char* b = field(line, "best_ms");
    e.best_ms = b ? strtof(b, nullptr) : 0.0f;
    return true;
}

// Every parsable entry of the file (none when it cannot be read).
std::vector<Entry> read_all(const char* path) {
    std::vector<Entry> out;
    FILE* f = fopen(path, "r");
    if (!f) return out;
    std::string line;
    char buf[1024];
    while (fgets(buf, sizeof(buf), f)) {
        line += buf;
        if (line.empty() || line.back() != '\n') {
            if (!feof(f)) continue;  // a line longer than the buffer: keep reading it
        }
        Entry e;
        if (parse_line(line, e)) out.push_back(e);
        line.clear();
    }
    fclose(f);
    return out;
}

bool key_ok(const char* key) {
    if (!key || !*key) return false;
    const size_t n = strlen(key);
    if (n >= SOLRT_TUNE_KEY_MAX) return false;
    for (size_t i = 0; i < n; ++i) {
        const unsigned char c = (unsigned char)key[i];
        if (c < 0x20 || c == '"' || c == '\\' || c == 0x7f) return false;
    }
    return true;
}

solrt_status write_all(const char* path, const std::vector<Entry>& es) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) {
        set_error("cannot write %s", tmp.c_str());
        return SOLRT_ERR_INVALID;
    }
    bool ok = true;
    for (const Entry& e : es)
        ok = ok && fprintf(f, "{\"key\": \"%s\", \"block_size\": %u, \"smem_stack\": %u, \"pass_paths\": %u, "
                              "\"best_ms\": %.3f}\n",
                           e.key.c_str(), e.cfg.block, e.cfg.smem, e.cfg.pass_paths, (double)e.best_ms) > 0;
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        set_error("cannot write %s", path);
        return SOLRT_ERR_INVALID;
    }
    return SOLRT_OK;
}

std::string batch_key(const Batch& b) {
    const Context& ctx = *b.ctx;
    cudaDeviceProp prop{};
    std::string gpu = "unknown";
    if (cudaGetDeviceProperties(&prop, ctx.device) == cudaSuccess) {
        gpu.clear();
        for (const char* c = prop.name; *c && gpu.size() < 64; ++c)
            gpu += (isalnum((unsigned char)*c) || *c == '-' || *c == '.') ? *c : '_';
    } else {
        cudaGetLastError();
    }
    uint64_t h = 14695981039346656037ull;
    for (const DevJob& J : b.jobs) {
        fnv(h, J.width);
        fnv(h, J.height);
        fnv(h, J.spp);
        fnv(h, J.max_bounces);
        fnv(h, J.rng_mode);
        fnv(h, J.accum_mode);
        fnv(h, J.material_mode);
        fnv(h, J.miss_mode);
        fnv(h, J.integrator);
        fnv(h, J.sc.tri_count);
    }
    char buf[SOLRT_TUNE_KEY_MAX];
    snprintf(buf, sizeof(buf), "gpu=%s|sm=%d|kind=%u|cap=%u|flags=%u|jobs=%zu|h=%016llx", gpu.c_str(), ctx.sm_count,
             b.kind, ctx.capacity, b.flags, b.jobs.size(), (unsigned long long)h);
    return buf;
}

}  // namespace

}  // namespace solrt

using namespace solrt;

extern "C" {

solrt_status solrt_batch_tune_key(solrt_batch* batch, char* key, size_t key_bytes) {
    if (!batch || !key) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    const std::string k = batch_key(*batch);
    if (k.size() + 1 > key_bytes) {
        set_error("key needs %zu bytes", k.size() + 1);
        return SOLRT_ERR_INVALID;
    }
    memcpy(key, k.c_str(), k.size() + 1);
    return SOLRT_OK;
}

solrt_status solrt_tune_cache_lookup(const char* path, const char* key, solrt_tune_config* cfg, float* best_ms) {
    if (!path || !cfg || !key_ok(key)) {
        set_error("null path or output, or a key with quotes, backslashes or control characters");
        return SOLRT_ERR_INVALID;
    }
    const std::vector<Entry> es = read_all(path);
    for (size_t i = es.size(); i-- > 0;) {  // the last entry of a key wins
        if (es[i].key == key) {
            cfg->block_size = es[i].cfg.block;
            cfg->smem_stack = es[i].cfg.smem;
            cfg->pass_paths = es[i].cfg.pass_paths;
            cfg->reserved = 0;
            if (best_ms) *best_ms = es[i].best_ms;
            return SOLRT_OK;
        }
    }
    set_error("no tune cache entry for %s in %s", key, path);
    return SOLRT_ERR_NOT_FOUND;
}

solrt_status solrt_tune_cache_store(const char* path, const char* key, const solrt_tune_config* cfg, float best_ms) {
    if (!path || !cfg || !key_ok(key)) {
        set_error("null path or configuration, or a key with quotes, backslashes or control characters");
        return SOLRT_ERR_INVALID;
    }
    if (!extend_variant_ok(cfg->block_size, cfg->smem_stack)) {
        set_error("block_size must be 64, 128 or 256 and smem_stack 16 or 32");
        return SOLRT_ERR_INVALID;
    }
    std::vector<Entry> es = read_all(path);
    Entry e;
    e.key = key;
    e.cfg.block = cfg->block_size;
    e.cfg.smem = cfg->smem_stack;
    e.cfg.pass_paths = cfg->pass_paths;
    e.best_ms = best_ms;
    bool replaced = false;
    for (Entry& x : es) {
        if (x.key == e.key) {
            x = e;
            replaced = true;
        }
    }
    if (!replaced) es.push_back(e);
    return write_all(path, es);
}

solrt_status solrt_batch_autotune_cached(solrt_batch* batch, const char* path, solrt_tune_result* out,
                                         uint32_t* hit) {
    if (!batch || !path) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    if (cudaSetDevice(batch->ctx->device) != cudaSuccess) {
        set_error("cudaSetDevice failed");
        return SOLRT_ERR_DEVICE;
    }
    const std::string key = batch_key(*batch);
    solrt_tune_config cfg{};
    float best_ms = 0.0f;
    if (solrt_tune_cache_lookup(path, key.c_str(), &cfg, &best_ms) == SOLRT_OK &&
        cfg.pass_paths <= batch->ctx->capacity) {
        TuneConfig t;
        t.block = cfg.block_size;
        t.smem = cfg.smem_stack;
        t.pass_paths = cfg.pass_paths;
        SOLRT_TRY(batch_apply_tune(*batch, t));
        if (out) {
            out->best = cfg;
            out->best_ms = best_ms;
            out->initial_ms = 0.0f;
            out->candidates = 0;
            out->reserved = 0;
        }
        if (hit) *hit = 1;
        return SOLRT_OK;
    }
    solrt_tune_result r{};
    SOLRT_TRY(batch_autotune(*batch, &r));
    if (out) *out = r;
    if (hit) *hit = 0;
    return solrt_tune_cache_store(path, key.c_str(), &r.best, r.best_ms);
}

}  // extern "C"
