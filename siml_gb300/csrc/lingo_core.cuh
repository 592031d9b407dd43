// Core arithmetic of the LINGO multiset-Tanimoto kernels, shared by the CUDA
// kernels and by host-side unit tests (every function is __host__ __device__).
//
// Intersection counting.  For two LINGO multisets A and B the reference sums
// min(countA, countB) over shared codes (pysiml/_CPULingo.c:53-71,
// pysiml/kernels.py:162-199).  Here min(a, c) is written as
// sum_{k>=1} [a >= k][c >= k]: a database code with count c is stored as c
// "entries" (code, level 1..c), each with its own virtual id (vid), and a CTA
// holds a shared-memory table T[vid] whose bit r is set when row r of its
// 32-row group has that code with count >= level.  The intersection of row r
// with a database molecule is then the number of the molecule's entries whose
// T word has bit r set: 32 rows are counted at once by adding the 32-bit
// words into a bit-sliced counter (bit r of plane p = bit p of row r's count).
//
// The counter uses carry-save adders (Harley-Seal style): eight masks are
// reduced with seven full adders into the ones/twos/fours planes and one
// weight-8 carry, which ripples into the higher planes.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SIML_HD __host__ __device__ __forceinline__
#else
#define SIML_HD inline
#endif

namespace siml {

// Full adder over 32 independent bit lanes: a + b + c = lo + 2*hi.
SIML_HD void full_add(uint32_t& hi, uint32_t& lo, uint32_t a, uint32_t b, uint32_t c) {
    const uint32_t u = a ^ b;
    lo = u ^ c;
    hi = (a & b) | (u & c);
}

// Bit-sliced counter for 32 rows with NP planes (counts up to 2^NP - 1).
// plane[0] = ones, plane[1] = twos, plane[2] = fours, plane[3..] = the
// weight-8 counter.
template <int NP>
struct SlicedCounter {
    uint32_t plane[NP];

    SIML_HD void clear() {
#pragma unroll
        for (int p = 0; p < NP; p++) plane[p] = 0u;
    }

    // add a weight-8 carry word into plane[3..]
    SIML_HD void add_eights(uint32_t carry) {
#pragma unroll
        for (int p = 3; p < NP; p++) {
            const uint32_t t = plane[p] & carry;
            plane[p] ^= carry;
            carry = t;
        }
    }

    // add one 32-row mask
    SIML_HD void add1(uint32_t m) {
#pragma unroll
        for (int p = 0; p < NP; p++) {
            const uint32_t t = plane[p] & m;
            plane[p] ^= m;
            m = t;
        }
    }

    // eight masks into planes 0..2; returns their weight-8 carry, not yet
    // added (add_eights or add_eights2 adds it)
    SIML_HD uint32_t add8_open(uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3,
                               uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7) {
        uint32_t twos_a, twos_b, fours_a, fours_b, eights;
        full_add(twos_a, plane[0], plane[0], m0, m1);
        full_add(twos_b, plane[0], plane[0], m2, m3);
        full_add(fours_a, plane[1], plane[1], twos_a, twos_b);
        full_add(twos_a, plane[0], plane[0], m4, m5);
        full_add(twos_b, plane[0], plane[0], m6, m7);
        full_add(fours_b, plane[1], plane[1], twos_a, twos_b);
        full_add(eights, plane[2], plane[2], fours_a, fours_b);
        return eights;
    }

    // two weight-8 carries at once: plane 3 absorbs them as a carry-save
    // accumulator and one weight-16 carry ripples on (9 operations where two
    // add_eights take 18)
    SIML_HD void add_eights2(uint32_t ea, uint32_t eb) {
        uint32_t carry;
        full_add(carry, plane[3], plane[3], ea, eb);
#pragma unroll
        for (int p = 4; p < NP; p++) {
            const uint32_t t = plane[p] & carry;
            plane[p] ^= carry;
            carry = t;
        }
    }

    // add eight 32-row masks (each contributes 1 to every row whose bit is set)
    SIML_HD void add8(uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3,
                      uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7) {
        uint32_t twos_a, twos_b, fours_a, fours_b, eights;
        full_add(twos_a, plane[0], plane[0], m0, m1);
        full_add(twos_b, plane[0], plane[0], m2, m3);
        full_add(fours_a, plane[1], plane[1], twos_a, twos_b);
        full_add(twos_a, plane[0], plane[0], m4, m5);
        full_add(twos_b, plane[0], plane[0], m6, m7);
        full_add(fours_b, plane[1], plane[1], twos_a, twos_b);
        full_add(eights, plane[2], plane[2], fours_a, fours_b);
        add_eights(eights);
    }
};

// In-place 8x8 bit-matrix transposes of the four byte lanes of eight words:
// on entry bit (8b + j) of w[k] is bit k of the count of row 8b + j; on exit
// byte b of w[k] is the count (bits 0..7) of row 8b + k.  Recursive block
// exchange (swap 4x4, then 2x2, then 1x1 sub-blocks), 3 rounds x 4 pairs.
SIML_HD void transpose_planes8(uint32_t w[8]) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t t = ((w[k] >> 4) ^ w[k + 4]) & 0x0F0F0F0Fu;
        w[k + 4] ^= t;
        w[k] ^= t << 4;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int k = (q & 1) + ((q >> 1) << 2);  // 0, 1, 4, 5
        const uint32_t t = ((w[k] >> 2) ^ w[k + 2]) & 0x33333333u;
        w[k + 2] ^= t;
        w[k] ^= t << 2;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int k = 2 * q;  // 0, 2, 4, 6
        const uint32_t t = ((w[k] >> 1) ^ w[k + 1]) & 0x55555555u;
        w[k + 1] ^= t;
        w[k] ^= t << 1;
    }
}

// Row counts out of a sliced counter.  After counts_from_planes, the count of
// row r is extracted by row_count(cnt, r).
template <int NP>
struct RowCounts {
    uint32_t lo[8];   // planes 0..7 transposed: byte b of lo[k] = low byte of row 8b+k
    uint32_t hi[8];   // planes 8..15 transposed (NP == 16 only)
};

template <int NP>
SIML_HD void counts_from_planes(const SlicedCounter<NP>& c, RowCounts<NP>& out) {
    static_assert(NP == 8 || NP == 16, "8 or 16 planes");
#pragma unroll
    for (int k = 0; k < 8; k++) out.lo[k] = c.plane[k];
    transpose_planes8(out.lo);
    if (NP == 16) {
#pragma unroll
        for (int k = 0; k < 8; k++) out.hi[k] = c.plane[(k + 8) % NP];
        transpose_planes8(out.hi);
    }
}

template <int NP>
SIML_HD uint32_t row_count(const RowCounts<NP>& rc, int r) {
    uint32_t v = (rc.lo[r & 7] >> (8 * (r >> 3))) & 0xFFu;
    if (NP == 16) v |= ((rc.hi[r & 7] >> (8 * (r >> 3))) & 0xFFu) << 8;
    return v;
}

// Row count for a row index known only at run time (a byte extract per word).
template <int NP>
SIML_HD uint32_t row_count_dyn(const RowCounts<NP>& rc, int r) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if ((r & 7) == k) {
            lo = rc.lo[k];
            if (NP == 16) hi = rc.hi[k];
        }
    }
    const int sh = 8 * (r >> 3);
    uint32_t v = (lo >> sh) & 0xFFu;
    if (NP == 16) v |= ((hi >> sh) & 0xFFu) << 8;
    return v;
}

// Histogram bins, identical to the oracle's rules:
// 101 bins: (unsigned)(t*100) clamped to 100, below zero / NaN to 0
// (pysiml/_cpuutil.cpp:64-66, pysiml/kernels.py:660-661);
// 1000 bins: min((unsigned)(t*1000.0f), 999), below zero / NaN to 0.
SIML_HD uint32_t bin_of(float s, uint32_t top) {
    if (!(s >= 0.0f)) return 0u;
    if (s >= 4294967040.0f) return top;
    const uint32_t b = (uint32_t)s;
    return b < top ? b : top;
}

#if defined(__CUDACC__)
// Correctly rounded quotient a / b of two integers for 0 <= a <= 2^24 and
// 1 <= b <= 2^16, by Markstein's correction of a reciprocal estimate
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990): q0 = a*y, r = a - q0*b
// (exact with one fused multiply-add), q = q0 + r*y rounded once.  With y the
// hardware reciprocal estimate (relative error < 2^-22) the unrounded q is
// within about 2^-21 ulp of a/b, while a/b (b not a power of two) lies at
// least 1/(b * 2^25) relative, i.e. > 2^-18 ulp, from any rounding midpoint,
// so the single rounding lands on RN(a/b); for b a power of two every step is
// exact.  tests/native/division_test.cu checks all a <= b <= 2^14 against
// __fdiv_rn on the GPU.
__device__ __forceinline__ float div_small(float af, float bf) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(bf));
    const float q0 = __fmul_rn(af, y);
    const float r = __fmaf_rn(-q0, bf, af);
    return __fmaf_rn(r, y, q0);
}
__device__ __forceinline__ float div_small_int(int a, int b) {
    return div_small(__int2float_rn(a), __int2float_rn(b));
}
// Exact fp32 value of an integer 0 <= i < 2^23 with full-rate integer and
// fp32 adds: the bit pattern 0x4B000000 | i is the float 2^23 + i.
__device__ __forceinline__ float small_int_to_float(uint32_t i) {
    return __fsub_rn(__uint_as_float(0x4B000000u | i), 8388608.0f);
}
#endif

}  // namespace siml
