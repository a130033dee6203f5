// options.cpp -- process-wide launch options (accspmm_set_option).
//
// Each option starts from its environment variable, read once, at the first
// call that needs an option (the launch paths read the cached values, not the
// environment); accspmm_set_option changes it for every thread from the next
// call on.  Options change speed only, never an element's arithmetic (the
// window block size moves the partial-window boundaries; see the header).
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "accspmm.h"
#include "common.hpp"
#include "options.hpp"

namespace accspmm {

namespace {

constexpr int kNumOptions = ACCSPMM_OPT_KERNEL + 1;
std::atomic<int> g_opt[kNumOptions];
std::once_flag g_opt_once;

int env_or(const char* name, int dflt) {
    const char* e = std::getenv(name);
    return e && *e ? std::atoi(e) : dflt;
}

int kernel_from_env() {
    const char* e = std::getenv("ACCSPMM_KERNEL");
    if (!e || !*e) return ACCSPMM_KERNEL_DIRECT;
    if (!std::strcmp(e, "pipe")) return ACCSPMM_KERNEL_PIPE;
    if (!std::strcmp(e, "bulk")) return ACCSPMM_KERNEL_BULK;
    if (!std::strcmp(e, "lean")) return ACCSPMM_KERNEL_LEAN;
    if (!std::strcmp(e, "db")) return ACCSPMM_KERNEL_DB;
    if (!std::strcmp(e, "tma")) return ACCSPMM_KERNEL_TMA;
    if (!std::strcmp(e, "staged")) return ACCSPMM_KERNEL_STAGED;
    return ACCSPMM_KERNEL_DIRECT;
}

bool valid(int option, int v) {
    switch (option) {
        case ACCSPMM_OPT_PACK:
        case ACCSPMM_OPT_PREFETCH: return v >= -1 && v <= 1;
        case ACCSPMM_OPT_SCHEDULE:
        case ACCSPMM_OPT_HOST_DIRECT_C: return v == 0 || v == 1;
        case ACCSPMM_OPT_SLICE_WIDTH:
        case ACCSPMM_OPT_HOST_SLICE_WIDTH: return v == 0 || v == 32 || v == 64 || v == 128;
        case ACCSPMM_OPT_CTAS_PER_SM: return v == 0 || v == 2 || v == 3;
        case ACCSPMM_OPT_TILE_RING: return v >= -1 && v <= 1;
        case ACCSPMM_OPT_WINDOWS_PER_CTA: return v >= 0 && v <= 1024;
        case ACCSPMM_OPT_KERNEL:
#ifdef ACCSPMM_LAB
            return v >= ACCSPMM_KERNEL_DIRECT && v <= ACCSPMM_KERNEL_STAGED;
#else
            return v == ACCSPMM_KERNEL_DIRECT;
#endif
        default: return false;
    }
}

void init_from_env() {
    // ACCSPMM_PACK: 0 never pack, 2 pack wherever the shape allows, else the rule
    const int pk = env_or("ACCSPMM_PACK", -1);
    g_opt[ACCSPMM_OPT_PACK] = pk == 0 ? 0 : pk == 2 ? 1 : -1;
    // ACCSPMM_PREFETCH: 0 never, 1 always, else the rule
    const int pf = env_or("ACCSPMM_PREFETCH", -1);
    g_opt[ACCSPMM_OPT_PREFETCH] = pf == 0 ? 0 : pf == 1 ? 1 : -1;
    g_opt[ACCSPMM_OPT_SCHEDULE] = env_or("ACCSPMM_SCHEDULE", 1) ? 1 : 0;
    g_opt[ACCSPMM_OPT_HOST_DIRECT_C] = env_or("ACCSPMM_HOST_DIRECT", 1) ? 1 : 0;
    const struct {
        int option;
        const char* name;
        int dflt;
    } ints[] = {{ACCSPMM_OPT_SLICE_WIDTH, "ACCSPMM_FS", 0},
                {ACCSPMM_OPT_HOST_SLICE_WIDTH, "ACCSPMM_HOST_FS", 0},
                {ACCSPMM_OPT_CTAS_PER_SM, "ACCSPMM_OCC", 0},
                {ACCSPMM_OPT_TILE_RING, "ACCSPMM_ROLL", -1},
                {ACCSPMM_OPT_WINDOWS_PER_CTA, "ACCSPMM_WB", 0}};
    for (const auto& o : ints) {
        const int v = env_or(o.name, o.dflt);
        g_opt[o.option] = valid(o.option, v) ? v : o.dflt;  // out-of-range values keep the default
    }
    const int k = kernel_from_env();
    g_opt[ACCSPMM_OPT_KERNEL] = valid(ACCSPMM_OPT_KERNEL, k) ? k : int(ACCSPMM_KERNEL_DIRECT);
}

}  // namespace

int option(int id) {
    std::call_once(g_opt_once, init_from_env);
    return g_opt[id].load(std::memory_order_relaxed);
}

int set_option(int id, int value) {
    if (id < 0 || id >= kNumOptions) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown option %d", id);
    std::call_once(g_opt_once, init_from_env);
    if (!valid(id, value)) {
        if (id == ACCSPMM_OPT_KERNEL && value >= ACCSPMM_KERNEL_PIPE && value <= ACCSPMM_KERNEL_STAGED)
            ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED,
                     "kernel %d is a measurement variant, built into libaccspmm_lab.so only", value);
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "value %d is not valid for option %d", value, id);
    }
    g_opt[id].store(value, std::memory_order_relaxed);
    return ACCSPMM_SUCCESS;
}

int lab_env(const char* name, int dflt) {
    // measurement-build knobs (shape details of the variant kernels), read
    // once per name: the lab build's kernels call this while choosing a shape
    static std::mutex mu;
    static std::vector<std::pair<std::string, int>> cache;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& kv : cache)
        if (kv.first == name) return kv.second;
    const int v = env_or(name, dflt);
    cache.emplace_back(name, v);
    return v;
}

}  // namespace accspmm
