// Launch-shape cache of the engine's autotuner (include/foort_gpu.h, foort_tune_*).
//
// One process-wide table maps a tuning key -- the GPU's SM count, the kernel variant
// (metric, integrator, precision, decision and strong-field options) and the launch-size
// bucket floor(log2 n) -- to the launch shape measured fastest for it. The search itself
// (foort_gpu_autotune, engine.cu) times candidate shapes on the GPU; this file only keeps
// and persists its results, so it needs no GPU. The reference has no counterpart: its
// round loop is an OpenMP for with the static schedule (Main.cpp:348).
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../include/foort_gpu.h"

namespace {

std::mutex g_mu;
std::map<std::string, foort_launch_shape> g_cache;

bool valid_shape(const foort_launch_shape& s) {
    return s.block_size >= 32 && s.block_size <= 128 && s.block_size % 32 == 0 && (s.lanes == 1 || s.lanes == 2) &&
           s.refill_steps >= 1 && s.poll_steps >= 1;
}

bool valid_key(const char* key) {
    if (!key || !*key) return false;
    for (const char* p = key; *p; ++p)
        if (*p == ' ' || *p == '\n' || *p == '\t') return false;
    return std::strlen(key) < 128;
}

}  // namespace

extern "C" {

uint32_t foort_tune_bucket(uint64_t n) {
    uint32_t b = 0;
    while (n > 1) {
        n >>= 1;
        ++b;
    }
    return b;
}

int foort_tune_key(const foort_run_desc* d, int32_t num_sms, uint64_t n, char* buf, uint64_t cap) {
    if (!d || !buf || cap == 0 || num_sms <= 0) return FOORT_E_BADARG;
    const int region = ((d->mixed_options & FOORT_MIXED_FP64_NEAR_HORIZON) && d->mixed_fp64_margin > 0.0 ? 1 : 0) |
                       ((d->mixed_options & FOORT_MIXED_FP64_TURNING_POINTS) ? 2 : 0);
    const int decide64 = (d->mixed_options & FOORT_MIXED_FP64_DECISIONS) != 0;
    const int w = std::snprintf(buf, cap, "sm%d:m%d:i%d:p%d:r%d:d%d:f%d:b%u", num_sms, d->metric_id,
                                d->integrator_id, d->precision, d->rlog ? 1 : 0, decide64, region,
                                foort_tune_bucket(n));
    return (w > 0 && static_cast<uint64_t>(w) < cap) ? FOORT_OK : FOORT_E_BADARG;
}

int foort_tune_put(const char* key, const foort_launch_shape* shape) {
    if (!valid_key(key) || !shape || !valid_shape(*shape)) return FOORT_E_BADARG;
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[key] = *shape;
    return FOORT_OK;
}

int foort_tune_get(const char* key, foort_launch_shape* shape) {
    if (!key || !shape) return FOORT_E_BADARG;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) return FOORT_E_BADARG;
    *shape = it->second;
    return FOORT_OK;
}

uint64_t foort_tune_count(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_cache.size();
}

void foort_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache.clear();
}

// One line per entry: key block_size blocks_per_sm lanes refill_steps poll_steps ms.
int foort_tune_save(const char* path) {
    if (!path) return FOORT_E_BADARG;
    std::lock_guard<std::mutex> lk(g_mu);
    FILE* f = std::fopen(path, "w");
    if (!f) return FOORT_E_IO;
    bool ok = std::fprintf(f, "# foort launch-shape cache v1\n") > 0;
    for (const auto& kv : g_cache) {
        const foort_launch_shape& s = kv.second;
        ok = ok && std::fprintf(f, "%s %u %u %u %u %u %.17g\n", kv.first.c_str(), s.block_size, s.blocks_per_sm,
                                s.lanes, s.refill_steps, s.poll_steps, s.ms) > 0;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FOORT_OK : FOORT_E_IO;
}

// Entries of the file are added to (and replace) the table's; a malformed line fails the
// whole load and leaves the table as it was.
int foort_tune_load(const char* path) {
    if (!path) return FOORT_E_BADARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return FOORT_E_IO;
    std::map<std::string, foort_launch_shape> got;
    char line[512];
    int rc = FOORT_OK;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        char key[256];
        foort_launch_shape s{};
        if (std::sscanf(line, "%255s %u %u %u %u %u %lf", key, &s.block_size, &s.blocks_per_sm, &s.lanes,
                        &s.refill_steps, &s.poll_steps, &s.ms) != 7 ||
            !valid_key(key) || !valid_shape(s)) {
            rc = FOORT_E_BADARG;
            break;
        }
        got[key] = s;
    }
    std::fclose(f);
    if (rc != FOORT_OK) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    for (const auto& kv : got) g_cache[kv.first] = kv.second;
    return FOORT_OK;
}

}  // extern "C"
