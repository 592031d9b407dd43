// Internal helpers shared by the host-side translation units.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>
#include <atomic>

#include "siml_gb300.h"

namespace siml {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

inline int host_threads() {
    unsigned n = std::thread::hardware_concurrency();
    if (n == 0) n = 1;
    if (n > 64) n = 64;
    return (int)n;
}

// Static block partition of [0, n) over the host's cores.
template <class F>
void parallel_for(int64_t n, F&& fn, int64_t min_per_thread = 256) {
    if (n <= 0) return;
    int nt = host_threads();
    int64_t want = (n + min_per_thread - 1) / min_per_thread;
    if (want < nt) nt = (int)want;
    if (nt <= 1) {
        for (int64_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)nt);
    for (int t = 0; t < nt; t++) {
        int64_t b = n * t / nt, e = n * (t + 1) / nt;
        th.emplace_back([b, e, &fn]() {
            for (int64_t i = b; i < e; i++) fn(i);
        });
    }
    for (auto& x : th) x.join();
}

}  // namespace siml
