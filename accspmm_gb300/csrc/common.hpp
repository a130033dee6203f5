// common.hpp -- internal helpers shared by the library's translation units.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "accspmm.h"

namespace accspmm {

// Row-window and tile geometry of METCF: ROW_WINDOW = COL_WINDOW = 8,
// include/common.hpp:48-50.
constexpr uint32_t kWin = 8;
constexpr uint32_t kPad = 0xFFFFFFFFu;  // sparseA2B padding, format.hpp:28

// Per-thread message of the last failure (accspmm_last_error).
void set_error(const char* fmt, ...);
void clear_error();
const char* last_error();

// Fail with a status and a message.
#define ACC_FAIL(code, ...)                  \
    do {                                     \
        ::accspmm::set_error(__VA_ARGS__);   \
        return (code);                       \
    } while (0)

#define ACC_CHECK_ARG(cond, ...)                                          \
    do {                                                                  \
        if (!(cond)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, __VA_ARGS__);  \
    } while (0)

// Number of host worker threads (hardware concurrency, overridable with
// ACCSPMM_HOST_THREADS).
unsigned host_threads();

// Runs f(begin, end) over [0, n) split into contiguous chunks on the host
// worker threads; chunk boundaries are deterministic for a given n.
template <class F>
void parallel_chunks(size_t n, F&& f, size_t min_chunk = 4096) {
    unsigned p = host_threads();
    if (n < 2 * min_chunk || p <= 1) {
        f(size_t(0), n, 0u);
        return;
    }
    size_t chunks = std::min<size_t>(p, (n + min_chunk - 1) / min_chunk);
    std::vector<std::thread> ts;
    ts.reserve(chunks);
    for (size_t c = 0; c < chunks; ++c) {
        size_t b = n * c / chunks, e = n * (c + 1) / chunks;
        ts.emplace_back([&f, b, e, c] { f(b, e, unsigned(c)); });
    }
    for (auto& t : ts) t.join();
}

inline size_t num_chunks_for(size_t n, size_t min_chunk = 4096) {
    unsigned p = host_threads();
    if (n < 2 * min_chunk || p <= 1) return 1;
    return std::min<size_t>(p, (n + min_chunk - 1) / min_chunk);
}

}  // namespace accspmm
