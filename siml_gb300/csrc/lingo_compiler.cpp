// SMILES -> LINGO multiset compiler (host side, multithreaded).
//
// Produces exactly what the reference's C compiler produces
// (pysiml/_ccompiler.cpp:276-381, wrapped by pysiml/compiler.py:53-82):
// per string, the sorted (signed int32) unique little-endian-packed 4-byte
// windows of the preprocessed string, their counts, the number of unique
// codes and the magnitude smilen-3 (0 and no codes when smilen < 4).
//
// Preprocessing follows the reference's state machine
// (pysiml/_ccompiler.cpp:178-264): digits become '0' except directly after
// '+', '-', 'H' or '[' (those digits are copied until a non-digit, which is
// copied without being re-examined); "%" copies and swallows the next
// character; a space, '\n' or '\r' ends the string (the name is dropped).
//
// Windows are formed directly from the processed bytes instead of by the
// reference's shift-the-whole-buffer loop (:119-150).  That loop shifts
// signed int32 words, so a byte >= 0x80 that reaches the top byte of its
// 4-byte block makes every byte shifted in after it (within that block) read
// 0xFF.  The closed form used here: window p = 4i + k (block i, shift k) has
// byte j = s[p+j] if k+j <= 3, else 0xFF when any of s[4i+3 .. p+j-1] is
// >= 0x80, else s[p+j].  For k in 1..3 the first window that runs past the
// end of the string is still emitted when that rule turns its top byte into
// 0xFF (the reference's scan only stops at a zero top byte).
#include <algorithm>
#include <cstring>
#include <vector>

#include "siml_internal.h"

namespace {

inline bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }

// Returns the processed length; out needs inlen + 1 bytes.
int32_t preprocess(const unsigned char* in, int64_t inlen, unsigned char* out) {
    enum State { kNormal, kSwallow, kAfterDigit, kVerbatimDigits };
    State st = kNormal;
    int32_t n = 0;
    for (int64_t ip = 0; ip < inlen; ip++) {
        const unsigned char ch = in[ip];
        if (ch == 0) break;
        if (st == kSwallow) { st = kAfterDigit; continue; }
        if (st == kVerbatimDigits) {
            out[n++] = ch;
            if (!is_digit(ch)) st = kNormal;
            continue;
        }
        // kNormal and kAfterDigit share everything but the '+-H[' rule
        if (ch == ' ' || ch == '\n' || ch == '\r') break;
        if (is_digit(ch)) { out[n++] = '0'; st = kAfterDigit; continue; }
        if (ch == '%') { out[n++] = ch; st = kSwallow; continue; }
        if (st == kNormal && (ch == '+' || ch == '-' || ch == 'H' || ch == '[')) {
            out[n++] = ch;
            st = kVerbatimDigits;
            continue;
        }
        out[n++] = ch;
        st = kNormal;
    }
    return n;
}

inline uint32_t byte_at(const unsigned char* s, int32_t len, int64_t q) { return q < len ? s[q] : 0u; }

// Code of window (block i, shift k) under the sign-fill rule above.
inline int32_t window_code(const unsigned char* s, int32_t len, int64_t i, int k) {
    const int64_t p = 4 * i + k;
    uint32_t v = 0;
    bool filled = false;
    for (int j = 0; j < 4; j++) {
        const int64_t q = p + j;
        uint32_t b;
        if (k + j <= 3) {
            b = byte_at(s, len, q);
        } else {
            // bytes entering from the next block: 0xFF once a high byte has
            // passed through the top of this block
            if (!filled) filled = byte_at(s, len, q - 1) >= 0x80u;
            b = filled ? 0xFFu : byte_at(s, len, q);
        }
        v |= b << (8 * j);
    }
    return (int32_t)v;
}

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
            for (int32_t p = 0; p + 3 < len; p++) {
                codes[(size_t)m++] = (int32_t)((uint32_t)s[p] | ((uint32_t)s[p + 1] << 8) |
                                               ((uint32_t)s[p + 2] << 16) | ((uint32_t)s[p + 3] << 24));
            }
        } else {
            for (int32_t p = 0; p + 3 < len; p++) codes[(size_t)m++] = window_code(s, len, p / 4, p % 4);
            const int64_t nblocks = len / 4 + 1;
            for (int k = 1; k <= 3; k++) {
                // first block whose shift-k window reaches past the end
                const int64_t need = (int64_t)len - k - 3;
                const int64_t i = need <= 0 ? 0 : (need + 3) / 4;
                if (i >= nblocks) continue;
                const int32_t c = window_code(s, len, i, k);
                if (((uint32_t)c >> 24) != 0u) codes[(size_t)m++] = c;
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

}  // namespace

extern "C" {

int64_t siml_compile_width(const char* buf, const int64_t* offsets, int64_t n) {
    siml::clear_error();
    if (!check_args(buf, offsets, n)) return -siml::fail(SIML_ERR_INVALID, "siml_compile_width: bad offsets");
    // chunked so each thread keeps one Bag
    const int64_t chunk = 1024;
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
    const int64_t chunk = 1024;
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

}  // extern "C"
