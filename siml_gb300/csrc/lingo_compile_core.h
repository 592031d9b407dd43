// SMILES -> LINGO rules shared by the host compiler (lingo_compiler.cpp) and
// the GPU compiler (compile_gpu.cu), so both produce the same bytes.
//
// The output is what the reference's C compiler produces
// (pysiml/_ccompiler.cpp:276-381, wrapped by pysiml/compiler.py:53-82): per
// string, the sorted (signed int32) unique little-endian-packed 4-byte
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
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SIML_CHD __host__ __device__ __forceinline__
#else
#define SIML_CHD inline
#endif

namespace siml {
namespace lingo {

SIML_CHD bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }

// Bytes that make preprocessing depend on state: the '+', '-', 'H', '['
// and '%' rules and the terminators.  A string with none of them is
// preprocessed by mapping each digit to '0' and keeping every other byte.
SIML_CHD bool stateful_byte(unsigned char c) {
    return c == '+' || c == '-' || c == 'H' || c == '[' || c == '%' || c == ' ' || c == '\n' || c == '\r' ||
           c == 0;
}

// Returns the processed length; out needs inlen bytes.
SIML_CHD int32_t preprocess(const unsigned char* in, int64_t inlen, unsigned char* out) {
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

SIML_CHD uint32_t byte_at(const unsigned char* s, int32_t len, int64_t q) { return q < len ? s[q] : 0u; }

// Code of window (block i, shift k) under the sign-fill rule above.
SIML_CHD int32_t window_code(const unsigned char* s, int32_t len, int64_t i, int k) {
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

// Window p of an all-ASCII string (no byte >= 0x80): the four bytes at p.
SIML_CHD int32_t ascii_window(const unsigned char* s, int32_t p) {
    return (int32_t)((uint32_t)s[p] | ((uint32_t)s[p + 1] << 8) | ((uint32_t)s[p + 2] << 16) |
                     ((uint32_t)s[p + 3] << 24));
}

// The shift-k window (k = 1..3) that runs past the end of a string holding
// a byte >= 0x80: true (and its code) when the reference emits it.
SIML_CHD bool tail_window(const unsigned char* s, int32_t len, int k, int32_t* code) {
    const int64_t nblocks = len / 4 + 1;
    const int64_t need = (int64_t)len - k - 3;
    const int64_t i = need <= 0 ? 0 : (need + 3) / 4;   // first block whose window reaches past the end
    if (i >= nblocks) return false;
    const int32_t c = window_code(s, len, i, k);
    if (((uint32_t)c >> 24) == 0u) return false;
    *code = c;
    return true;
}

}  // namespace lingo
}  // namespace siml
