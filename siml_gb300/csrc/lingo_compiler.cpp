// SMILES -> LINGO multiset compiler (host side, multithreaded).  The
// preprocessing and window rules are in lingo_compile_core.h, shared with the
// GPU compiler.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "lingo_compile_core.h"
#include "siml_internal.h"

namespace {

using siml::lingo::ascii_window;
using siml::lingo::preprocess;
using siml::lingo::tail_window;
using siml::lingo::window_code;

struct Bag {
    std::vector<int32_t> codes;   // scratch: all windows, then unique codes
    std::vector<int32_t> counts;
    std::vector<unsigned char> proc;
    int32_t n = 0;
    int32_t mag = 0;

    void build(const unsigned char* in, int64_t inlen) {
        proc.resize((size_t)inlen + 8);
        const int32_t len = preprocess(in, inlen, proc.data());
        n = 0;
        mag = 0;
        if (len - 3 < 1) return;
        const unsigned char* s = proc.data();
        codes.resize((size_t)len + 8);
        int32_t m = 0;
        bool ascii = true;
        for (int32_t q = 0; q < len; q++) ascii &= s[q] < 0x80u;
        if (ascii) {
            for (int32_t p = 0; p + 3 < len; p++) codes[(size_t)m++] = ascii_window(s, p);
        } else {
            for (int32_t p = 0; p + 3 < len; p++) codes[(size_t)m++] = window_code(s, len, p / 4, p % 4);
            for (int k = 1; k <= 3; k++) {
                int32_t c;
                if (tail_window(s, len, k, &c)) codes[(size_t)m++] = c;
            }
        }
        std::sort(codes.begin(), codes.begin() + m);
        counts.resize((size_t)m);
        for (int32_t t = 0; t < m; t++) {
            if (n > 0 && codes[(size_t)n - 1] == codes[(size_t)t]) {
                counts[(size_t)n - 1]++;
            } else {
                codes[(size_t)n] = codes[(size_t)t];
                counts[(size_t)n] = 1;
                n++;
            }
        }
        mag = len - 3;
    }
};

bool check_args(const char* buf, const int64_t* offsets, int64_t n) {
    if (n < 0 || (n > 0 && (!buf || !offsets))) return false;
    for (int64_t s = 0; s < n; s++)
        if (offsets[s + 1] < offsets[s]) return false;
    return true;
}

// Strings per task: large batches in 1,024-string tasks; small ones (a
// request of a few hundred SMILES) split over a few threads, each with at
// least 128 strings so thread start-up stays small against the work.
int64_t chunk_of(int64_t n) {
    const int64_t per = (n + 2 * siml::host_threads() - 1) / (2 * siml::host_threads());
    return std::max<int64_t>(128, std::min<int64_t>(1024, per));
}

}  // namespace

extern "C" {

int64_t siml_compile_width(const char* buf, const int64_t* offsets, int64_t n) {
    siml::clear_error();
    if (!check_args(buf, offsets, n)) return -siml::fail(SIML_ERR_INVALID, "siml_compile_width: bad offsets");
    // chunked so each thread keeps one Bag
    const int64_t chunk = chunk_of(n);
    const int64_t nchunks = (n + chunk - 1) / chunk;
    std::vector<int64_t> chunk_max((size_t)nchunks, 0);
    siml::parallel_for(nchunks, [&](int64_t c) {
        Bag bag;
        int64_t mx = 0;
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t s = c * chunk; s < e; s++) {
            bag.build((const unsigned char*)buf + offsets[s], offsets[s + 1] - offsets[s]);
            mx = std::max<int64_t>(mx, bag.n);
        }
        chunk_max[(size_t)c] = mx;
    }, 1);
    int64_t w = 0;
    for (auto v : chunk_max) w = std::max(w, v);
    return w;
}

int siml_compile_smiles(const char* buf, const int64_t* offsets, int64_t n,
                        int32_t* lingos, int32_t* counts, int32_t* lengths,
                        int32_t* mags, int64_t width) {
    siml::clear_error();
    if (!check_args(buf, offsets, n) || width < 0 ||
        (n > 0 && (!lingos || !counts || !lengths || !mags)))
        return siml::fail(SIML_ERR_INVALID, "siml_compile_smiles: bad arguments");
    const int64_t chunk = chunk_of(n);
    const int64_t nchunks = (n + chunk - 1) / chunk;
    std::atomic<int> overflow{0};
    siml::parallel_for(nchunks, [&](int64_t c) {
        Bag bag;
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t s = c * chunk; s < e; s++) {
            bag.build((const unsigned char*)buf + offsets[s], offsets[s + 1] - offsets[s]);
            int32_t* lr = lingos + s * width;
            int32_t* cr = counts + s * width;
            if (bag.n > width) { overflow = 1; continue; }
            if (bag.n) {
                std::memcpy(lr, bag.codes.data(), (size_t)bag.n * sizeof(int32_t));
                std::memcpy(cr, bag.counts.data(), (size_t)bag.n * sizeof(int32_t));
            }
            if (width > bag.n) {
                std::memset(lr + bag.n, 0, (size_t)(width - bag.n) * sizeof(int32_t));
                std::memset(cr + bag.n, 0, (size_t)(width - bag.n) * sizeof(int32_t));
            }
            lengths[s] = bag.n;
            mags[s] = bag.mag;
        }
    }, 1);
    if (overflow) return siml::fail(SIML_ERR_INVALID, "siml_compile_smiles: width smaller than a string's unique LINGO count");
    return SIML_OK;
}

// One-pass form: every string compiled once into staging (its unique codes
// and counts at [offsets[s], offsets[s] + lengths[s]), within its own byte
// stretch since a string has at most as many unique windows as bytes), then
// scattered into zero-padded rows.
int64_t siml_compile_stage(const char* buf, const int64_t* offsets, int64_t n, int32_t* stage_codes,
                           int32_t* stage_counts, int32_t* lengths, int32_t* mags) {
    siml::clear_error();
    if (!check_args(buf, offsets, n) || (n > 0 && (!stage_codes || !stage_counts || !lengths || !mags)))
        return -siml::fail(SIML_ERR_INVALID, "siml_compile_stage: bad arguments");
    const int64_t chunk = chunk_of(n);
    const int64_t nchunks = (n + chunk - 1) / chunk;
    std::vector<int64_t> chunk_max((size_t)nchunks, 0);
    siml::parallel_for(nchunks, [&](int64_t c) {
        Bag bag;
        int64_t mx = 0;
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t s = c * chunk; s < e; s++) {
            bag.build((const unsigned char*)buf + offsets[s], offsets[s + 1] - offsets[s]);
            if (bag.n) {
                std::memcpy(stage_codes + offsets[s], bag.codes.data(), (size_t)bag.n * sizeof(int32_t));
                std::memcpy(stage_counts + offsets[s], bag.counts.data(), (size_t)bag.n * sizeof(int32_t));
            }
            lengths[s] = bag.n;
            mags[s] = bag.mag;
            mx = std::max<int64_t>(mx, bag.n);
        }
        chunk_max[(size_t)c] = mx;
    }, 1);
    int64_t w = 0;
    for (auto v : chunk_max) w = std::max(w, v);
    return w;
}

int siml_compile_scatter(const int64_t* offsets, int64_t n, const int32_t* stage_codes,
                         const int32_t* stage_counts, const int32_t* lengths, int32_t* lingos, int32_t* counts,
                         int64_t width) {
    siml::clear_error();
    if (n < 0 || width < 0 || (n > 0 && (!offsets || !stage_codes || !stage_counts || !lengths ||
                                         (width > 0 && (!lingos || !counts)))))
        return siml::fail(SIML_ERR_INVALID, "siml_compile_scatter: bad arguments");
    const int64_t chunk = chunk_of(n);
    const int64_t nchunks = (n + chunk - 1) / chunk;
    std::atomic<int> overflow{0};
    siml::parallel_for(nchunks, [&](int64_t c) {
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t s = c * chunk; s < e; s++) {
            // a count is bounded by the string's stretch, so no read leaves it
            const int64_t nu = std::min<int64_t>(std::max(lengths[s], 0), offsets[s + 1] - offsets[s]);
            if (nu > width) { overflow = 1; continue; }
            int32_t* lr = lingos + s * width;
            int32_t* cr = counts + s * width;
            if (nu) {
                std::memcpy(lr, stage_codes + offsets[s], (size_t)nu * sizeof(int32_t));
                std::memcpy(cr, stage_counts + offsets[s], (size_t)nu * sizeof(int32_t));
            }
            if (width > nu) {
                std::memset(lr + nu, 0, (size_t)(width - nu) * sizeof(int32_t));
                std::memset(cr + nu, 0, (size_t)(width - nu) * sizeof(int32_t));
            }
        }
    }, 1);
    if (overflow) return siml::fail(SIML_ERR_INVALID, "siml_compile_scatter: width smaller than a string's unique LINGO count");
    return SIML_OK;
}

}  // extern "C"
