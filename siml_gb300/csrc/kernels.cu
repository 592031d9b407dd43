// Similarity kernels (sm_103a).
//
// Table kernels (k_rows, k_nbr): one CTA per (32-row group, database slice).
//   1. The CTA clears a shared-memory table T[vid] (one 32-bit word per
//      database (code, level) pair) and sets bit r of T[vid] for every entry
//      of its row r.  Rows are the reference's SIML-ref rows.
//   2. Each warp streams a contiguous range of database chunks (32 molecules,
//      one per lane).  Consecutive chunks are contiguous in memory, so the
//      entry loads (16 bytes per lane, 512 contiguous bytes per warp) are
//      prefetched two steps ahead straight across chunk boundaries, and the
//      per-lane metadata one chunk ahead.  Eight T words per step go into a
//      bit-sliced counter: 32 row intersections advance per table read.
//   3. At the end of a chunk an epilogue consumes the counter:
//      k_rows transposes it into 32 row counts and stores 32 Tanimotos;
//      k_nbr compares all 32 counts against a conservative per-lane integer
//      threshold in bit-sliced form (~40 instructions for 32 pairs) and runs
//      the reference's exact neighbour test only for the rows that pass.
// k_nbr_finish puts each row's neighbours in ascending order, or recomputes
// a row with the reference's ordered wave scan when it overflowed.
// k_rows_merge is the reference's per-pair sorted merge, used only when the
// table would not fit in shared memory or counts exceed 16 bits.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "engine.h"
#include "lingo_core.cuh"
#include "table_core.cuh"

namespace siml {

namespace {

constexpr int kNbrSortMax = 2048;   // rows with more hits are recomputed in order

// First chunk c in [lo, hi] whose first entry group is at or past `target`
// (the chunk offsets are non-decreasing).
__device__ __forceinline__ int64_t chunk_at_volume(const int64_t* __restrict__ off, int64_t lo, int64_t hi,
                                                   int64_t target) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) < target) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Splits chunks [cb, ce) among the CTA's warps by entry volume, so warps with
// chunks of long molecules (the sorted layout orders sizes inside a window)
// get fewer of them.
__device__ __forceinline__ void warp_split(const int64_t* __restrict__ off, int64_t cb, int64_t ce,
                                           int64_t& wb, int64_t& we) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int64_t g0 = __ldg(off + cb), g1 = __ldg(off + ce);
    wb = warp == 0 ? cb : chunk_at_volume(off, cb, ce, g0 + (g1 - g0) * warp / nwarps);
    we = warp == nwarps - 1 ? ce : chunk_at_volume(off, cb, ce, g0 + (g1 - g0) * (warp + 1) / nwarps);
}

// Chunks [wb, we) of this warp: the CTA's slice split by volume.
__device__ __forceinline__ void warp_range(const GroupParams& p, int64_t& wb, int64_t& we) {
    const int64_t n = p.chunk_end - p.chunk_begin;
    const int64_t cb = p.chunk_begin + n * blockIdx.y / gridDim.y;
    const int64_t ce = p.chunk_begin + n * (blockIdx.y + 1) / gridDim.y;
    warp_split(p.off, cb, ce, wb, we);
}

// Entry types of the database layout: 2-byte vids, 4-byte vids, or 4-byte
// byte offsets into the table (off32_t: the lookup needs no index arithmetic).
struct off32_t {
    uint32_t v;
};
template <typename ET>
__device__ __forceinline__ uint32_t tload(const uint32_t* T, uint32_t w) {
    if constexpr (sizeof(ET) == 4 && !std::is_same<ET, uint32_t>::value)
        return *reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(T) + w);
    else
        return T[w];
}

// Streams the entries of chunks [wb, we) through the bit-sliced counter and
// calls epi(chunk, meta, counter) at the end of each chunk.  All lanes of the
// warp are in the same chunk at the same time.
template <int NP, typename ET, bool RARE = false, class Epi>
__device__ __forceinline__ void stream_chunks(const uint32_t* __restrict__ T, const GroupParams& p,
                                              int64_t wb, int64_t we, Epi& epi) {
    if (wb >= we) return;
    constexpr int SPG = sizeof(ET) == 2 ? 1 : 2;  // 16-byte groups per 8-entry step
    const int lane = threadIdx.x & 31;
    const uint4* E = reinterpret_cast<const uint4*>(p.entries) + lane;
    const int64_t gend = p.off[we];
    int64_t g = p.off[wb];
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    uint4 n0 = zero, n1 = zero, m0 = zero, m1 = zero;
    if (g < gend) { n0 = __ldg(E + g); if (SPG == 2) n1 = __ldg(E + g + 32); }
    if (g + 32 * SPG < gend) { m0 = __ldg(E + g + 32 * SPG); if (SPG == 2) m1 = __ldg(E + g + 32 * SPG + 32); }
    int64_t c = wb;
    int4 meta = __ldg(p.meta + c * 32 + lane);
    int ng_cur = p.ng[c];
    int steps = ng_cur / SPG;
    int4 meta_next = make_int4(-1, 0, 0, 0);
    int ng_next = 0;
    if (c + 1 < we) { meta_next = __ldg(p.meta + (c + 1) * 32 + lane); ng_next = p.ng[c + 1]; }
    // the entry block of the next chunk is pulled into L2 one chunk ahead, so
    // the two-step register prefetch only has to cover L2 latency
    const char* Eb = reinterpret_cast<const char*>(p.entries);
    int64_t next_off = g + (int64_t)ng_cur * 32;   // first group of chunk c + 1
    if (lane == 0) {
        prefetch_l2(Eb + g * 16, (uint32_t)ng_cur * 512u);
        if (c + 1 < we) prefetch_l2(Eb + next_off * 16, (uint32_t)ng_next * 512u);
    }
    SlicedCounter<NP> acc;
    acc.clear();
    for (;;) {
        while (steps == 0) {
            if constexpr (RARE) rare_add<NP>(T, p, c * 32 + lane, acc);
            epi(c, meta, acc);
            acc.clear();
            if (++c >= we) return;
            meta = meta_next;
            steps = ng_next / SPG;
            next_off += (int64_t)ng_next * 32;            // first group of chunk c + 1
            if (c + 1 < we) {
                meta_next = __ldg(p.meta + (c + 1) * 32 + lane);
                ng_next = p.ng[c + 1];
                if (lane == 0) prefetch_l2(Eb + next_off * 16, (uint32_t)ng_next * 512u);
            }
        }
        const uint4 c0 = n0, c1 = n1;
        n0 = m0;
        n1 = m1;
        g += 32 * SPG;
        const int64_t gn = g + 32 * SPG;
        if (gn < gend) { m0 = __ldg(E + gn); if (SPG == 2) m1 = __ldg(E + gn + 32); }
        else { m0 = zero; m1 = zero; }
        if (SPG == 1)
            acc.add8(T[c0.x & 0xFFFFu], T[c0.x >> 16], T[c0.y & 0xFFFFu], T[c0.y >> 16],
                     T[c0.z & 0xFFFFu], T[c0.z >> 16], T[c0.w & 0xFFFFu], T[c0.w >> 16]);
        else
            acc.add8(tload<ET>(T, c0.x), tload<ET>(T, c0.y), tload<ET>(T, c0.z), tload<ET>(T, c0.w),
                     tload<ET>(T, c1.x), tload<ET>(T, c1.y), tload<ET>(T, c1.z), tload<ET>(T, c1.w));
        steps--;
    }
}

// True when no pair of a chunk (magnitudes [r.x, r.y]) and the group's rows
// (magnitudes [amin, amax]) can reach lo: t <= min(ma, mb) / max(ma, mb), and
// the largest such bound over the two ranges sits at their nearest ends.  The
// fp32 quotient is the reference's pre-filter (pysiml/kernels.py:437-448) and
// rounding is monotone, so the corner value is the exact maximum.
__device__ __forceinline__ bool chunk_out_of_reach(int2 r, int amin, int amax, float lo) {
    if (r.x > r.y) return true;   // padding only
    float b;
    if (r.y < amin) b = __fdiv_rn(__int2float_rn(r.y), __int2float_rn(amin));
    else if (r.x > amax) b = __fdiv_rn(__int2float_rn(amax), __int2float_rn(r.x));
    else return false;
    return !(b >= lo);
}

// stream_chunks over the chunks of [wb, we) that can hold a pair with
// t >= lo for some row of the group (lo <= 0 or NaN: every chunk).  Chunks
// are tested warp-uniformly; runs of reachable chunks are streamed whole.
// Returns the number of chunks streamed.
template <int NP, typename ET, bool RARE = false, class Epi>
__device__ __forceinline__ int64_t stream_chunks_within(const uint32_t* __restrict__ T, const GroupParams& p,
                                                        const RowSmem& rs, int64_t wb, int64_t we, float lo,
                                                        Epi& epi) {
    if (!(lo > 0.0f) || p.crange == nullptr || rs.max_amag < 0) {
        stream_chunks<NP, ET, RARE>(T, p, wb, we, epi);
        return we > wb ? we - wb : 0;
    }
    const int amin = rs.min_amag, amax = rs.max_amag;
    int64_t c = wb, streamed = 0;
    while (c < we) {
        while (c < we && chunk_out_of_reach(p.crange[c], amin, amax, lo)) c++;
        int64_t e = c;
        while (e < we && !chunk_out_of_reach(p.crange[e], amin, amax, lo)) e++;
        if (e > c) stream_chunks<NP, ET, RARE>(T, p, c, e, epi);
        streamed += e - c;
        c = e;
    }
    return streamed;
}

// The CTA's chunk slice [cb, ce) of this launch (blockIdx.y of gridDim.y).
__device__ __forceinline__ void cta_range(const GroupParams& p, int64_t& cb, int64_t& ce) {
    const int64_t n = p.chunk_end - p.chunk_begin;
    cb = p.chunk_begin + n * blockIdx.y / gridDim.y;
    ce = p.chunk_begin + n * (blockIdx.y + 1) / gridDim.y;
}

// Warps take the CTA's chunks from a shared counter, kGrab at a time, so a
// warp slowed by candidates or skipped chunks does not hold the CTA back.
// `next` starts at the slice's first chunk (set before the table build's
// barrier).
// Near the end of the range (fewer than kGrabTail chunks left, read without
// synchronization as a hint) warps take one chunk at a time, so they reach
// the CTA's next barrier at nearly the same time.
constexpr int kGrab = 4;
constexpr long long kGrabTail = kGrab * (kThreads / 32);
template <int NP, typename ET, bool RARE = false, class Epi>
__device__ __forceinline__ void stream_dynamic(const uint32_t* __restrict__ T, const GroupParams& p,
                                               const RowSmem& rs, long long* next, int64_t ce, float lo, int nr,
                                               Epi& epi) {
    const int lane = threadIdx.x & 31;
    int64_t streamed = 0;
    for (;;) {
        long long c0 = 0, g = kGrab;
        if (lane == 0) {
            g = ce - *reinterpret_cast<volatile long long*>(next) > kGrabTail ? kGrab : 1;
            c0 = atomicAdd(reinterpret_cast<unsigned long long*>(next), (unsigned long long)g);
        }
        c0 = __shfl_sync(0xFFFFFFFFu, c0, 0);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
        if (c0 >= ce) break;
        streamed += stream_chunks_within<NP, ET, RARE>(T, p, rs, c0, c0 + g < ce ? c0 + g : ce, lo, epi);
    }
    if (p.eval && lane == 0 && streamed > 0)
        atomicAdd(p.eval, (unsigned long long)streamed * 32ull * (unsigned long long)(nr > 0 ? nr : 0));
}

// ------------------------------------------------------------- k_rows ----
// Largest row stride for which 31 rows of fp32 stay within 32-bit byte offsets.
constexpr int64_t kFullGroupLdo = (int64_t)(0xFFFFFFFFull / (31ull * 4ull));

template <int NP>
struct RowsEpi {
    const RowSmem& rs;
    int nr;
    int mode;
    float* out;     // first row of this group
    int64_t ldo;

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int32_t m = meta.x;
        if (m < 0) return;
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
        const int32_t bmag = mode == kModeSingle ? meta.z : meta.y;
        float* o = out + m;
        if (rs.allfast && fast_mag(bmag, meta.z)) {
            // union = ((float)amag + bmag) - isct, all exact: the reference's order
            const float bf = small_int_to_float((uint32_t)bmag);
            const float4* am4 = reinterpret_cast<const float4*>(rs.amagf);
            if (NP == 8 && nr == 32 && ldo < kFullGroupLdo) {
                // full group: no row predicate; one byte permute forms the
                // float 2^23 + count straight from the transposed planes; rows
                // advance by 32-bit byte offsets from the lane's column
                char* ob = reinterpret_cast<char*>(o);
                const uint32_t step = (uint32_t)ldo * 4u;
#pragma unroll
                for (int r4 = 0; r4 < 8; r4++) {
                    const float4 a4 = am4[r4];
                    const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const int r = 4 * r4 + k;
                        const uint32_t bits = __byte_perm(rc.lo[r & 7], 0x4B000000u, 0x7440u | (uint32_t)(r >> 3));
                        const float isf = __fsub_rn(__uint_as_float(bits), 8388608.0f);
                        const float u = __fsub_rn(__fadd_rn(av[k], bf), isf);
                        *reinterpret_cast<float*>(ob + (uint32_t)r * step) = div_small(isf, u);
                    }
                }
                return;
            }
#pragma unroll
            for (int r4 = 0; r4 < 8; r4++) {
                const float4 a4 = am4[r4];
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int r = 4 * r4 + k;
                    if (r < nr) {
                        const float isf = small_int_to_float(row_count<NP>(rc, r));
                        const float u = __fsub_rn(__fadd_rn(av[k], bf), isf);
                        o[(int64_t)r * ldo] = div_small(isf, u);
                    }
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < 32; r++) {
                if (r < nr) {
                    const int is = (int)row_count<NP>(rc, r);
                    const float t = mode == kModeSingle ? tanimoto_single(is, rs.amag[r], bmag, rs.alen[r], meta.w)
                                                        : tanimoto_rows(is, rs.amag[r], bmag);
                    o[(int64_t)r * ldo] = t;
                }
            }
        }
    }
};

template <int NP, typename ET, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_rows(const GroupParams p, float* out, int64_t ldo) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    const int nr = build_table(T, rs, p);
    int64_t wb, we;
    warp_range(p, wb, we);
    RowsEpi<NP> epi{rs, nr, p.mode, out + (int64_t)blockIdx.x * 32 * ldo, ldo};
    stream_chunks<NP, ET, RARE>(T, p, wb, we, epi);
}

// -------------------------------------------------------------- k_nbr ----
struct NbrArgs {
    float lo, hi;
    float thr_scale;   // conservative lo / (1 + lo)
    int thr_mode;      // 0: threshold test, 1: every row is a candidate, 2: nothing can match
    int64_t pitch;
    int32_t* idx;      // [rows, pitch]
    float* sims;       // [rows, pitch] or null
    int32_t* counts;   // [rows], zeroed before the launch
    int32_t col_begin, col_end;   // database columns searched
    const int4* rowinfo;          // per output row {ref row, col_begin, col_end, 0}; null: rowbase + row, [col_begin, col_end)
};

NbrArgs nbr_args(float lo, float hi, int64_t pitch, int32_t* idx, float* sims, int32_t* counts,
                 int64_t col_begin, int64_t col_end) {
    NbrArgs a;
    a.lo = lo;
    a.hi = hi;
    a.pitch = pitch;
    a.idx = idx;
    a.sims = sims;
    a.counts = counts;
    a.col_begin = (int32_t)col_begin;
    a.col_end = (int32_t)col_end;
    a.rowinfo = nullptr;
    if (std::isnan(lo)) a.thr_mode = 2;
    else if (lo <= 0.0f) a.thr_mode = 1;
    else a.thr_mode = 0;
    a.thr_scale = a.thr_mode == 0 ? bound_coef(lo) : 0.0f;
    return a;
}

// Bit r of the result is set when the count of row r (bit-sliced in planes)
// is >= th.  MSB-first compare: eq tracks rows equal so far, gt rows greater.
template <int NP>
__device__ __forceinline__ uint32_t sliced_ge(const SlicedCounter<NP>& acc, uint32_t th) {
    if (th >= (1u << NP)) return 0u;
    uint32_t gt = 0u, eq = 0xFFFFFFFFu;
#pragma unroll
    for (int p = NP - 1; p >= 0; p--) {
        const uint32_t tb = 0u - ((th >> p) & 1u);   // all ones where the threshold bit is 1
        gt |= eq & acc.plane[p] & ~tb;
        eq &= ~(acc.plane[p] ^ tb);
    }
    return gt | eq;
}

// The same with a threshold per row, bit-sliced like the counts (bit r of
// tp[p] = bit p of row r's threshold).
template <int NP>
__device__ __forceinline__ uint32_t sliced_ge_rows(const SlicedCounter<NP>& acc, const uint32_t (&tp)[NP]) {
    uint32_t gt = 0u, eq = 0xFFFFFFFFu;
#pragma unroll
    for (int p = NP - 1; p >= 0; p--) {
        gt |= eq & acc.plane[p] & ~tp[p];
        eq &= ~(acc.plane[p] ^ tp[p]);
    }
    return gt | eq;
}

template <int NP>
__device__ __forceinline__ int sliced_row(const SlicedCounter<NP>& acc, int r) {
    int v = 0;
#pragma unroll
    for (int p = 0; p < NP; p++) v |= (int)((acc.plane[p] >> r) & 1u) << p;
    return v;
}

// getNeighbors' per-pair test (pysiml/kernels.py:437-448): fp32 magnitude
// bound min/max >= lo, then lo <= t < hi.
__device__ __forceinline__ bool neighbor_test(int isct, int ma, int mb, float lo, float hi, float& t) {
    const float bound = __fdiv_rn(__int2float_rn(min(ma, mb)), __int2float_rn(max(ma, mb)));
    if (!(bound >= lo)) return false;
    t = tanimoto_rows(isct, ma, mb);
    return t >= lo && t < hi;
}

template <int NP>
struct NbrEpi {
    const RowSmem& rs;
    int nr;
    int64_t row0;      // first output row of this group
    NbrArgs a;

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int32_t m = meta.x;
        const bool valid = m >= a.col_begin && m < a.col_end;
        const int32_t mb = meta.y;
        uint32_t cand;
        if (!valid || a.thr_mode == 2) {
            return;
        } else if (a.thr_mode == 1) {
            cand = 0xFFFFFFFFu;
        } else {
            // exact t >= lo > 0 implies isct >= lo/(1+lo) * (ma + mb) >= th
            const float s = (float)rs.min_amag + (float)mb;
            const float thf = floorf(a.thr_scale * s);
            const uint32_t th = thf <= 0.0f ? 0u : (thf >= 4.0e9f ? 0xFFFFFFFFu : (uint32_t)thf);
            cand = sliced_ge<NP>(acc, th);
        }
        if (nr < 32) cand &= (1u << nr) - 1u;
        while (cand) {
            const int r = __ffs(cand) - 1;
            cand &= cand - 1u;
            const int is = sliced_row<NP>(acc, r);
            float t;
            if (!neighbor_test(is, rs.amag[r], mb, a.lo, a.hi, t)) continue;
            const int64_t row = rs.orow[r];
            const int pos = atomicAdd(a.counts + row, 1);
            if (pos < a.pitch) {
                a.idx[row * a.pitch + pos] = m;
                if (a.sims) a.sims[row * a.pitch + pos] = t;
            }
        }
    }
};

template <int NP, typename ET, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_nbr(const GroupParams p, const NbrArgs a) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ long long next;
    if ((int64_t)blockIdx.x * 32 >= live_rows(p)) return;   // uniform over the CTA
    int64_t cb, ce;
    cta_range(p, cb, ce);
    if (threadIdx.x == 0) next = cb;
    const int nr = build_table(T, rs, p);   // synchronizes the block
    NbrEpi<NP> epi{rs, nr, (int64_t)blockIdx.x * 32, a};
    stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ce, a.thr_mode == 0 ? a.lo : 0.0f, nr, epi);
}

// ---------------------------------------------------------- k_rows_bal ----
// Full-matrix rows over the balanced layout.  A chunk's 8-entry steps are
// dealt to its 32 lanes in runs of L (the layout's ng / SPG), so lane j
// streams steps [j L, (j + 1) L) of the chunk's molecules laid end to end and
// a molecule may span several lanes.  Each lane flushes a partial counter
// whenever a molecule ends inside its run (and at the end of its run) into
// piece slot j + m of its warp's shared buffer; the slots of one warp are
// distinct because runs are ordered.  Lane l then owns molecule l: it adds
// the pieces of slots [first lane + l, last lane + l] with a bit-sliced
// ripple adder and runs the padded kernel's epilogue, so stores stay one
// 128-byte line per row.
//
// MODE >= 1 (layouts whose runs are all at most 32 steps: every chunk of a
// database whose molecules hold fewer than about 256 entries): lanes know
// their flush steps before streaming.  The owner of each molecule sets bit
// (end % L) of lane end / L's mask, and a lane's next molecule after a flush
// is the next set bit of the warp's ballot of non-empty molecules, so a step
// costs one bit test besides the flush itself.  MODE 0: lanes walk the
// prefix array.  MODE 2 (runs of at most 15 steps, with 8-plane counts): a
// run holds at most 120 entries, so the lane's running counter and its
// pieces need 7 planes; the ripple of each step's weight-8 carry is one
// plane shorter and a flush stores one word less.  The molecule's counter,
// made of the pieces, keeps NP planes.
constexpr int kPieceSlots = 64;
constexpr int kPrefixWords = 34;
constexpr int kRowsBalThreads = 1024;   // threads of a k_rows_bal CTA (one CTA per SM beside the table)

__host__ __device__ constexpr size_t rows_bal_extra_smem(int np, int warps) {
    return (size_t)warps * ((size_t)np * kPieceSlots + kPrefixWords) * 4;
}

template <int NPR>
__device__ __forceinline__ void piece_store(uint32_t* pc, int slot, const SlicedCounter<NPR>& acc) {
#pragma unroll
    for (int q = 0; q < NPR; q++) pc[q * kPieceSlots + slot] = acc.plane[q];
}

// Adds an NPR-plane piece into an NP-plane counter (NPR <= NP).
template <int NP, int NPR>
__device__ __forceinline__ void piece_add(SlicedCounter<NP>& acc, const uint32_t* pc, int slot) {
    uint32_t carry = 0u;
#pragma unroll
    for (int q = 0; q < NPR; q++) {
        const uint32_t a = acc.plane[q], b = pc[q * kPieceSlots + slot];
        acc.plane[q] = a ^ b ^ carry;
        carry = (a & b) | (carry & (a ^ b));
    }
#pragma unroll
    for (int q = NPR; q < NP; q++) {
        const uint32_t a = acc.plane[q];
        acc.plane[q] = a ^ carry;
        carry = a & carry;
    }
}

// floor(x / L) for 0 <= x <= 64 L and 1 <= L <= 1024, from rl ~ 1 / L (the
// hardware reciprocal estimate, relative error below 2^-22): (x + 0.5) / L
// lies at least 0.5 / L from an integer, far beyond the product's error.
__device__ __forceinline__ int div_run(int x, float rl) {
    return (int)__fmul_rz(__int2float_rn(x) + 0.5f, rl);
}

template <int NP, typename ET, bool RARE, int MODE>
__global__ void __launch_bounds__(kRowsBalThreads, 1) k_rows_bal(const GroupParams p, float* out, int64_t ldo) {
    constexpr bool MASKED = MODE >= 1;
    constexpr int NPR = (MODE == 2 && NP == 8) ? 7 : NP;   // planes of a lane's running counter
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    const int nr = build_table(T, rs, p);   // synchronizes the block
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    uint32_t* pc = T + p.tab_words + (size_t)warp * NP * kPieceSlots;
    int* pre = reinterpret_cast<int*>(T + p.tab_words + (size_t)nwarps * NP * kPieceSlots) + warp * kPrefixWords;
    int64_t wb, we;
    warp_range(p, wb, we);
    constexpr int SPG = sizeof(ET) == 2 ? 1 : 2;
    const uint4* E = reinterpret_cast<const uint4*>(p.entries) + lane;
    const char* Eb = reinterpret_cast<const char*>(p.entries);
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    RowsEpi<NP> epi{rs, nr, p.mode, out + (int64_t)blockIdx.x * 32 * ldo, ldo};
    if (lane == 0 && wb < we) prefetch_l2(Eb + __ldg(p.off + wb) * 16, (uint32_t)__ldg(p.ng + wb) * 512u);
    for (int64_t c = wb; c < we; c++) {
        const int4 meta = __ldg(p.meta + c * 32 + lane);
        const int64_t base = __ldg(p.off + c);
        const int L = __ldg(p.ng + c) / SPG;   // steps per lane
        if (lane == 0 && c + 1 < we)
            prefetch_l2(Eb + __ldg(p.off + c + 1) * 16, (uint32_t)__ldg(p.ng + c + 1) * 512u);
        int es = meta.z;   // streamed entries: all, or the common ones (split vocabulary)
        if constexpr (RARE) {
            if (meta.x >= 0) es -= (int)(__ldg(p.rare_off + c * 32 + lane + 1) - __ldg(p.rare_off + c * 32 + lane));
        }
        const int g = meta.x >= 0 ? (es + 7) >> 3 : 0;
        int incl = g;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        const int P = incl - g;
        const int G = __shfl_sync(0xFFFFFFFFu, incl, 31);
        float rl = 0.0f;
        if constexpr (MASKED) {
            asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rl) : "f"(__int2float_rn(max(L, 1))));
            pc[lane] = 0u;   // flush masks, in the piece buffer until the first flush
        }
        pre[lane] = P;
        if (lane == 31) pre[32] = G;
        __syncwarp();
        uint32_t fmask = 0u;
        if constexpr (MASKED) {
            if (g > 0) {
                const int e = incl - 1;   // the molecule's last step
                const int j = div_run(e, rl);
                atomicOr(pc + j, 1u << (e - j * L));
            }
            __syncwarp();
            fmask = pc[lane];
        }
        const int seg0 = lane * L, seg1 = min(G, seg0 + L);
        // molecule holding step seg0: the largest m with pre[m] <= seg0
        int m = 0;
#pragma unroll
        for (int q = 16; q > 0; q >>= 1)
            if (m + q <= 31 && pre[m + q] <= seg0) m += q;
        SlicedCounter<NPR> acc;
        acc.clear();
        uint4 a0 = zero, b0 = zero, a1 = zero, b1 = zero;
        const uint4* Ec = E + base;
        if (0 < L) { a0 = __ldg(Ec); if (SPG == 2) b0 = __ldg(Ec + 32); }
        if (1 < L) { a1 = __ldg(Ec + SPG * 32); if (SPG == 2) b1 = __ldg(Ec + SPG * 32 + 32); }
        auto step = [&](int s) {
            const uint4 x = a0, y = b0;
            a0 = a1;
            b0 = b1;
            if (s + 2 < L) {
                a1 = __ldg(Ec + (s + 2) * SPG * 32);
                if (SPG == 2) b1 = __ldg(Ec + (s + 2) * SPG * 32 + 32);
            }
            if (SPG == 1)
                acc.add8(T[x.x & 0xFFFFu], T[x.x >> 16], T[x.y & 0xFFFFu], T[x.y >> 16],
                         T[x.z & 0xFFFFu], T[x.z >> 16], T[x.w & 0xFFFFu], T[x.w >> 16]);
            else
                acc.add8(T[x.x], T[x.y], T[x.z], T[x.w], T[y.x], T[y.y], T[y.z], T[y.w]);
        };
        if constexpr (MASKED) {
            const uint32_t nz = __ballot_sync(0xFFFFFFFFu, g > 0);
            // the run ends inside a molecule (its last step ends none)
            const bool open_end = seg1 > seg0 && !((fmask >> (seg1 - seg0 - 1)) & 1u);
            __syncwarp();   // every mask is read before pieces overwrite them
            uint32_t f = fmask;
            for (int s = 0; s < L; s++) {
                step(s);
                if (f & 1u) {   // molecule m ends at this step
                    piece_store<NPR>(pc, lane + m, acc);
                    acc.clear();
                    m = __ffs(nz & (0xFFFFFFFEu << m)) - 1;   // next molecule with entries
                }
                f >>= 1;
            }
            if (open_end) piece_store<NPR>(pc, lane + m, acc);
        } else {
            int endm = pre[m + 1];
            bool pending = false;
            for (int s = 0; s < L; s++) {
                step(s);
                const int gs = seg0 + s + 1;
                if (gs <= seg1) pending = true;   // a step of the run (past it: zero padding)
                if (gs == endm && gs <= seg1) {   // molecule m ends inside this lane's run
                    piece_store<NPR>(pc, lane + m, acc);
                    acc.clear();
                    pending = false;
                    do { m++; } while (m < 32 && pre[m + 1] == pre[m]);   // skip molecules with no entries
                    endm = m < 32 ? pre[m + 1] : 0x7FFFFFFF;
                }
            }
            if (pending && m < 32) piece_store<NPR>(pc, lane + m, acc);   // run ended inside molecule m
        }
        __syncwarp();
        SlicedCounter<NP> own;
        own.clear();
        if (g > 0) {
            int fl, ll;
            if constexpr (MASKED) {
                asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rl) : "f"(__int2float_rn(L)));
                fl = div_run(P, rl);
                ll = div_run(P + g - 1, rl);
            } else {
                fl = P / L;
                ll = (P + g - 1) / L;
            }
            for (int j = fl; j <= ll; j++) piece_add<NP, NPR>(own, pc, j + lane);
        }
        if constexpr (RARE) rare_add<NP>(T, p, c * 32 + lane, own);
        epi(c, meta, own);
        __syncwarp();   // pieces and prefix are rewritten for the next chunk
    }
}

// ---------------------------------------------------------- k_collect ----
// Top-k candidate collection: every pair with t >= its row's bound
// (GroupParams.row_lo).  Lane r forms row r's integer threshold at the
// chunk's smallest magnitude (valid for every lane of the chunk: the bound
// grows with the magnitude) and ballots slice the 32 thresholds into
// planes, so the bit-sliced compare is per row.  Positions come from
// shared-memory counters: each (row, database split) owns a segment of
// seg_cap entries of the candidate buffer [rows][splits][seg_cap], and the
// per-segment counts (which may exceed seg_cap) go to seg_counts[rows][splits]
// when the CTA ends.  No magnitude pre-filter here: a row or molecule with
// no LINGOs scores 0 and still ranks.
struct CollectArgs {
    int64_t seg_cap;
    int32_t* cand_i;
    float* cand_t;
    int32_t* seg_counts;
};

template <int NP>
struct CollectEpi {
    const RowSmem& rs;
    int nr;
    int* scount;        // shared, per group row
    int32_t* cand_i;    // this CTA's segment of row 0: + row * splits * seg_cap
    float* cand_t;
    int64_t row_stride; // splits * seg_cap
    int64_t seg_cap;

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int32_t m = meta.x, mb = meta.y;
        const bool valid = m >= 0;
        int mbm = valid ? mb : 0x7FFFFFFF;
        for (int o = 16; o > 0; o >>= 1) mbm = min(mbm, __shfl_xor_sync(0xFFFFFFFFu, mbm, o));
        if (mbm == 0x7FFFFFFF) return;   // padding-only chunk (uniform)
        const int lane = threadIdx.x & 31;
        const float thf = floorf(rs.coef[lane] * (rs.amagf[lane] + (float)mbm));
        const bool never = lane >= nr || thf >= (float)(1u << NP);
        const uint32_t thr = never || thf <= 0.0f ? 0u : (uint32_t)thf;
        uint32_t tp[NP];
#pragma unroll
        for (int q = 0; q < NP; q++) tp[q] = __ballot_sync(0xFFFFFFFFu, (thr >> q) & 1u);
        const uint32_t never_m = __ballot_sync(0xFFFFFFFFu, never);
        if (!valid) return;
        uint32_t cand = sliced_ge_rows<NP>(acc, tp) & ~never_m;
        while (cand) {
            const int r = __ffs(cand) - 1;
            cand &= cand - 1u;
            const int is = sliced_row<NP>(acc, r);
            // the lane's own integer bound first, the exact similarity after
            if ((float)is < floorf(rs.coef[r] * (rs.amagf[r] + (float)mb))) continue;
            const float t = tanimoto_rows(is, rs.amag[r], mb);
            if (!(t >= rs.lo[r])) continue;
            const int pos = atomicAdd(scount + r, 1);
            if (pos < seg_cap) {
                const int64_t o = (int64_t)rs.orow[r] * row_stride + pos;
                cand_i[o] = m;
                cand_t[o] = t;
            }
        }
    }
};

template <int NP, typename ET, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_collect(const GroupParams p, const CollectArgs c) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ int scount[32];
    __shared__ long long next;
    if ((int64_t)blockIdx.x * 32 >= live_rows(p)) return;   // uniform over the CTA
    if (threadIdx.x < 32) scount[threadIdx.x] = 0;
    int64_t cb, ce;
    cta_range(p, cb, ce);
    if (threadIdx.x == 0) next = cb;
    const int nr = build_table(T, rs, p);   // synchronizes the block
    const int64_t row_stride = (int64_t)gridDim.y * c.seg_cap;
    CollectEpi<NP> epi{rs, nr, scount, c.cand_i + blockIdx.y * c.seg_cap, c.cand_t + blockIdx.y * c.seg_cap,
                       row_stride, c.seg_cap};
    stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ce, rs.min_lo, nr, epi);
    __syncthreads();
    if (threadIdx.x < nr) c.seg_counts[(int64_t)rs.orow[threadIdx.x] * gridDim.y + blockIdx.y] = scount[threadIdx.x];
}

// ------------------------------------------------------------- k_hist ----
// Histograms of all pairs of a row block: per row, 101 bins of
// (unsigned)(t*100) (getMultipleHistogrammedRows, pysiml/kernels.py:606-666),
// or one 1000-bin histogram of min((unsigned)(t*1000), 999) for the block.
// Counts go to shared memory and are flushed with one atomic per bin per CTA.
constexpr int kBins101 = 101;
constexpr int kBins1000 = 1000;

// bin of a similarity: (unsigned)(t * scale) clamped to top; the product is
// one fp32 multiply as in the reference, truncated by a round-toward-zero add
// of 2^23 (exact floor for 0 <= s < 2^23).
__device__ __forceinline__ uint32_t bin_fast(float t, float scale, uint32_t top) {
    const float s = __fmul_rn(t, scale);
    const uint32_t b = __float_as_uint(__fadd_rz(s, 8388608.0f)) - 0x4B000000u;
    return b < top ? b : top;
}

template <int NP, bool GLOBAL>
struct HistEpi {
    const RowSmem& rs;
    int nr;
    uint32_t* H;   // shared: [32][101] or [1000]

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        if (meta.x < 0) return;
        const int32_t bmag = meta.y;
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
        const float scale = GLOBAL ? 1000.0f : 100.0f;
        const uint32_t top = GLOBAL ? 999u : 100u;
        if (rs.allfast && fast_mag(bmag, meta.z)) {
            const float bf = small_int_to_float((uint32_t)bmag);
            if (NP == 8 && nr == 32) {   // full group: as the fp32 block epilogue
#pragma unroll
                for (int r = 0; r < 32; r++) {
                    const uint32_t bits = __byte_perm(rc.lo[r & 7], 0x4B000000u, 0x7440u | (uint32_t)(r >> 3));
                    const float isf = __fsub_rn(__uint_as_float(bits), 8388608.0f);
                    const float t = div_small(isf, __fsub_rn(__fadd_rn(rs.amagf[r], bf), isf));
                    const uint32_t b = bin_fast(t, scale, top);
                    atomicAdd(H + (GLOBAL ? b : r * kBins101 + b), 1u);
                }
                return;
            }
#pragma unroll
            for (int r = 0; r < 32; r++) {
                if (r < nr) {
                    const float isf = small_int_to_float(row_count<NP>(rc, r));
                    const float t = div_small(isf, __fsub_rn(__fadd_rn(rs.amagf[r], bf), isf));
                    const uint32_t b = bin_fast(t, scale, top);
                    atomicAdd(H + (GLOBAL ? b : r * kBins101 + b), 1u);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < 32; r++) {
                if (r < nr) {
                    const float t = tanimoto_rows((int)row_count<NP>(rc, r), rs.amag[r], bmag);
                    const uint32_t b = bin_of(__fmul_rn(t, scale), top);
                    atomicAdd(H + (GLOBAL ? b : r * kBins101 + b), 1u);
                }
            }
        }
    }
};

// out: GLOBAL ? uint64 [1000] (accumulated) : int32 [rows, ldo] (zeroed first)
template <int NP, typename ET, bool GLOBAL, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_hist(const GroupParams p, void* out, int64_t ldo) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ uint32_t H[GLOBAL ? kBins1000 : 32 * kBins101];
    __shared__ long long next;
    for (int i = threadIdx.x; i < (GLOBAL ? kBins1000 : 32 * kBins101); i += blockDim.x) H[i] = 0u;
    int64_t cb, ce;
    cta_range(p, cb, ce);
    if (threadIdx.x == 0) next = cb;
    const int nr = build_table(T, rs, p);   // synchronizes the block
    HistEpi<NP, GLOBAL> epi{rs, nr, H};
    stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ce, 0.0f, nr, epi);
    __syncthreads();
    if (GLOBAL) {
        unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
        for (int i = threadIdx.x; i < kBins1000; i += blockDim.x)
            if (H[i]) atomicAdd(o + i, (unsigned long long)H[i]);
    } else {
        int32_t* o = reinterpret_cast<int32_t*>(out);
        for (int i = threadIdx.x; i < nr * kBins101; i += blockDim.x) {
            const int r = i / kBins101, b = i - r * kBins101;
            if (H[i]) atomicAdd(o + (int64_t)rs.orow[r] * ldo + b, (int)H[i]);
        }
    }
}

// ------------------------------------------------------------ k_loghist ----
// Per-row histogram for the sample pass of top-k.  Bins follow the bits of
// t: 64 per octave over [2^-8, 1), one below 2^-8 and one for t = 1, so every
// bin is about 1.6% wide and its lower edge is an exact float.  Counts are
// 16-bit halves of shared words; the launcher keeps each CTA's molecules per
// row under 65,536 so no half carries into its neighbour.
constexpr int kLogBins = 514;
constexpr int kLogWords = (kLogBins + 1) / 2;

__device__ __forceinline__ int log_bin(float t) {
    if (!(t >= 0.00390625f)) return 0;
    if (t >= 1.0f) return kLogBins - 1;
    const uint32_t u = __float_as_uint(t);
    const int e = (int)(u >> 23) - 127;   // -8 .. -1
    return 1 + (e + 8) * 64 + (int)((u >> 17) & 63u);
}

// Lower edge of bin b: every t of bins >= b is >= it (-1 for bin 0).
__device__ __forceinline__ float log_bin_floor(int b) {
    if (b <= 0) return -1.0f;
    if (b >= kLogBins - 1) return 1.0f;
    const uint32_t e = (uint32_t)((b - 1) / 64 - 8 + 127), m = (uint32_t)((b - 1) % 64);
    return __uint_as_float((e << 23) | (m << 17));
}

template <int NP>
struct LogHistEpi {
    const RowSmem& rs;
    int nr;
    uint32_t* H;   // shared: [32][kLogWords]

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        if (meta.x < 0) return;
        const int32_t bmag = meta.y;
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
        const bool fast = rs.allfast && fast_mag(bmag, meta.z);
        const float bf = small_int_to_float((uint32_t)(bmag > 0 ? bmag : 0));
        if (NP == 8 && fast && nr == 32) {   // full group: as the fp32 block epilogue
#pragma unroll
            for (int r = 0; r < 32; r++) {
                const uint32_t bits = __byte_perm(rc.lo[r & 7], 0x4B000000u, 0x7440u | (uint32_t)(r >> 3));
                const float isf = __fsub_rn(__uint_as_float(bits), 8388608.0f);
                const float t = div_small(isf, __fsub_rn(__fadd_rn(rs.amagf[r], bf), isf));
                const int b = log_bin(t);
                atomicAdd(H + r * kLogWords + (b >> 1), 1u << ((b & 1) * 16));
            }
            return;
        }
#pragma unroll
        for (int r = 0; r < 32; r++) {
            if (r < nr) {
                float t;
                if (fast) {
                    const float isf = small_int_to_float(row_count<NP>(rc, r));
                    t = div_small(isf, __fsub_rn(__fadd_rn(rs.amagf[r], bf), isf));
                } else {
                    t = tanimoto_rows((int)row_count<NP>(rc, r), rs.amag[r], bmag);
                }
                const int b = log_bin(t);
                atomicAdd(H + r * kLogWords + (b >> 1), 1u << ((b & 1) * 16));
            }
        }
    }
};

// The same histogram restricted to pairs with t >= the row's floor
// (GroupParams.row_lo).  Pairs below the floor cost only CollectEpi's
// pre-filter: per-row integer bounds at the chunk's smallest magnitude,
// compared bit-sliced for all 32 rows at once.
template <int NP>
struct LogHistFloorEpi {
    const RowSmem& rs;
    int nr;
    uint32_t* H;   // shared: [32][kLogWords]

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int32_t m = meta.x, mb = meta.y;
        const bool valid = m >= 0;
        int mbm = valid ? mb : 0x7FFFFFFF;
        for (int o = 16; o > 0; o >>= 1) mbm = min(mbm, __shfl_xor_sync(0xFFFFFFFFu, mbm, o));
        if (mbm == 0x7FFFFFFF) return;   // padding-only chunk (uniform)
        const int lane = threadIdx.x & 31;
        const float thf = floorf(rs.coef[lane] * (rs.amagf[lane] + (float)mbm));
        const bool never = lane >= nr || thf >= (float)(1u << NP);
        const uint32_t thr = never || thf <= 0.0f ? 0u : (uint32_t)thf;
        uint32_t tp[NP];
#pragma unroll
        for (int q = 0; q < NP; q++) tp[q] = __ballot_sync(0xFFFFFFFFu, (thr >> q) & 1u);
        const uint32_t never_m = __ballot_sync(0xFFFFFFFFu, never);
        if (!valid) return;
        uint32_t cand = sliced_ge_rows<NP>(acc, tp) & ~never_m;
        while (cand) {
            const int r = __ffs(cand) - 1;
            cand &= cand - 1u;
            const int is = sliced_row<NP>(acc, r);
            if ((float)is < floorf(rs.coef[r] * (rs.amagf[r] + (float)mb))) continue;
            const float t = tanimoto_rows(is, rs.amag[r], mb);
            if (!(t >= rs.lo[r])) continue;
            const int b = log_bin(t);
            atomicAdd(H + r * kLogWords + (b >> 1), 1u << ((b & 1) * 16));
        }
    }
};

// out: int32 [rows, kLogBins], accumulated (zeroed by the caller).  FLOOR:
// only pairs at or above the rows' floors (LogHistFloorEpi).
template <int NP, typename ET, bool FLOOR, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_loghist(const GroupParams p, int32_t* out) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ uint32_t H[32 * kLogWords];
    __shared__ long long next;
    for (int i = threadIdx.x; i < 32 * kLogWords; i += blockDim.x) H[i] = 0u;
    int64_t cb, ce;
    cta_range(p, cb, ce);
    if (threadIdx.x == 0) next = cb;
    const int nr = build_table(T, rs, p);   // synchronizes the block
    if constexpr (FLOOR) {
        LogHistFloorEpi<NP> epi{rs, nr, H};
        stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ce, rs.min_lo, nr, epi);
    } else {
        LogHistEpi<NP> epi{rs, nr, H};
        stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ce, 0.0f, nr, epi);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nr * kLogBins; i += blockDim.x) {
        const int r = i / kLogBins, b = i - r * kLogBins;
        const uint32_t v = (H[r * kLogWords + (b >> 1)] >> ((b & 1) * 16)) & 0xFFFFu;
        if (v) atomicAdd(out + (int64_t)rs.orow[r] * kLogBins + b, (int)v);
    }
}

// Merge-path fallback: one thread per pair, global atomics.
template <bool GLOBAL>
__global__ void k_hist_merge(const struct RawArgs ra, void* out, int64_t ldo);

// ------------------------------------------------------------- k_topk ----
// Per-row top-k (k <= kTopkMax): the k largest similarities of each row,
// ties to the lower query index.  Each CTA keeps, per row, a heap of the k
// best (t, index) pairs of its database slice, worst first, so the root is
// the row's current k-th best; the root's (t, index) is also published as one
// 64-bit word (never torn, only rising) with the coefficient of a
// conservative integer test.  Warp 0 first fills the heaps from the slice's
// first chunks with no locks (lane r owns row r, values reach it through a
// shared-memory transpose); then every warp streams the rest, tests each pair
// against its own row's threshold, computes the exact similarity only for
// pairs that pass, and inserts under a per-row lock whose spin is bounded (on
// expiry the CTA sets an error word instead of waiting).  Heaps go to a
// scratch buffer [rows][splits][k] that k_topk_merge reduces per row.
constexpr int kTopkMax = 256;
constexpr int kTopkSpinLimit = 1 << 22;

struct TopkSmem {
    int lock[32];
    int size[32];
    unsigned long long root[32];   // (float bits of t) << 32 | index of the k-th best, 0 until full
    float coef[32];                 // t >= root.t implies isct >= coef * (magA + magB)
    int coef_min_bits;              // float bits of the lowest coef once every heap is full
    float stage_t[32][33];          // warm-up transpose: [lane][row]
    int err;
};

// a is worse than b: lower similarity, or equal similarity and higher index
__device__ __forceinline__ bool worse(float ta, int ia, float tb, int ib) {
    return ta < tb || (ta == tb && ia > ib);
}

__device__ void heap_sift_up(float* ht, int* hi, int i) {
    while (i > 0) {
        const int par = (i - 1) >> 1;
        if (!worse(ht[i], hi[i], ht[par], hi[par])) return;
        const float tt = ht[i]; ht[i] = ht[par]; ht[par] = tt;
        const int ti = hi[i]; hi[i] = hi[par]; hi[par] = ti;
        i = par;
    }
}

__device__ void heap_sift_down(float* ht, int* hi, int n) {
    int i = 0;
    for (;;) {
        const int l = 2 * i + 1, r = l + 1;
        int w = i;
        if (l < n && worse(ht[l], hi[l], ht[w], hi[w])) w = l;
        if (r < n && worse(ht[r], hi[r], ht[w], hi[w])) w = r;
        if (w == i) return;
        const float tt = ht[i]; ht[i] = ht[w]; ht[w] = tt;
        const int ti = hi[i]; hi[i] = hi[w]; hi[w] = ti;
        i = w;
    }
}

// Inserts (t, m) into row r's heap; caller holds row r (lock or ownership).
// Publishes the new k-th best when the heap is full.
__device__ __forceinline__ void heap_offer(TopkSmem& ts, float* ht, int* hi, int k, int r, float t, int m) {
    float* rt = ht + r * k;
    int* ri = hi + r * k;
    int n = ts.size[r];
    if (n < k) {
        rt[n] = t; ri[n] = m;
        heap_sift_up(rt, ri, n);
        ts.size[r] = ++n;
    } else if (worse(rt[0], ri[0], t, m)) {
        rt[0] = t; ri[0] = m;
        heap_sift_down(rt, ri, k);
    } else {
        return;
    }
    if (n == k) {
        const float th = rt[0];
        ts.coef[r] = th > 0.0f ? th / (1.0f + th) * (1.0f - 1.0f / 4096.0f) : 0.0f;
        __threadfence_block();
        *(volatile unsigned long long*)&ts.root[r] =
            ((unsigned long long)__float_as_uint(th) << 32) | (unsigned long long)(uint32_t)ri[0];
    }
}

// Raises the lowest-coefficient word from the rows' current coefficients
// (0 while a heap is not full).  Coefficients only rise, so racing updates
// leave a valid lower bound.
__device__ __forceinline__ void update_coef_min(TopkSmem& ts, int nr) {
    float mn = 3.0e38f;
    for (int q = 0; q < nr; q++) {
        const float cq = *(volatile unsigned long long*)&ts.root[q] == 0ull ? 0.0f : *(volatile float*)&ts.coef[q];
        mn = fminf(mn, cq);
    }
    if (mn > 0.0f) atomicMax(&ts.coef_min_bits, __float_as_int(mn));
}

__device__ __forceinline__ bool beats_root(unsigned long long root, float t, int m) {
    if (root == 0ull) return true;   // heap not full yet
    return worse(__uint_as_float((uint32_t)(root >> 32)), (int)(uint32_t)root, t, m);
}

// Warm-up: every pair of a chunk, inserted by the lane that owns the row.
template <int NP>
struct TopkWarmEpi {
    const RowSmem& rs;
    TopkSmem& ts;
    float* ht;
    int* hi;
    int nr, k;

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int lane = threadIdx.x & 31;
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
#pragma unroll
        for (int r = 0; r < 32; r++)
            ts.stage_t[lane][r] = meta.x >= 0 && r < nr ? tanimoto_rows((int)row_count<NP>(rc, r), rs.amag[r], meta.y)
                                                        : 0.0f;
        __syncwarp();
        for (int s = 0; s < 32; s++) {
            const int m = __shfl_sync(0xFFFFFFFFu, meta.x, s);
            if (m >= 0 && lane < nr) heap_offer(ts, ht, hi, k, lane, ts.stage_t[s][lane], m);
        }
        __syncwarp();
    }
};

// Main phase.  A lane first compares all 32 counts, bit-sliced, against
// the threshold implied by the lowest row coefficient, then each remaining
// row against its own bound and k-th best, giving a per-lane row mask; the
// warp skips the chunk when no lane has a candidate.  Rows with candidates
// are visited in an order rotated by warp id (so warps do not queue on the
// same lock); per row one lane takes the lock for the whole warp and the
// passing lanes insert in turn.
template <int NP>
struct TopkEpi {
    const RowSmem& rs;
    TopkSmem& ts;
    float* ht;
    int* hi;
    int nr, k;

    __device__ __forceinline__ void operator()(int64_t, const int4& meta, const SlicedCounter<NP>& acc) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int32_t m = meta.x;
        const int32_t mb = meta.y;
        const float mbf = (float)mb;
        uint32_t th = 0u;
        const float cmin = __int_as_float(*(volatile int*)&ts.coef_min_bits);
        if (cmin > 0.0f) {
            const float thf = floorf(cmin * ((float)rs.min_amag + mbf));
            th = thf <= 0.0f ? 0u : (thf >= 4.0e9f ? 0xFFFFFFFFu : (uint32_t)thf);
        }
        uint32_t cand = m >= 0 ? sliced_ge<NP>(acc, th) : 0u;
        if (nr < 32) cand &= (1u << nr) - 1u;
        if (!__any_sync(0xFFFFFFFFu, cand != 0u)) return;
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
        uint32_t pm = 0u;   // rows whose pair may enter the heap
#pragma unroll
        for (int r = 0; r < 32; r++) {
            if ((cand >> r) & 1u) {
                const uint32_t is = row_count<NP>(rc, r);
                const float coef = *(volatile float*)&ts.coef[r];
                if (!((float)is < coef * (rs.amagf[r] + mbf))) {
                    const float t = tanimoto_rows((int)is, rs.amag[r], mb);
                    if (beats_root(*(volatile unsigned long long*)&ts.root[r], t, m)) pm |= 1u << r;
                }
            }
        }
        const uint32_t rows_any = __reduce_or_sync(0xFFFFFFFFu, pm);
        if (rows_any == 0u) return;
        const uint32_t rot = (rows_any >> (warp & 31)) | (warp & 31 ? rows_any << (32 - (warp & 31)) : 0u);
        uint32_t left = rot;
        bool changed = false;
        while (left) {
            const int j = __ffs(left) - 1;
            left &= left - 1u;
            const int r = (j + warp) & 31;
            const bool pass = (pm >> r) & 1u;
            float t = 0.0f;
            if (pass) t = tanimoto_rows((int)row_count_dyn<NP>(rc, r), rs.amag[r], mb);
            const unsigned b = __ballot_sync(0xFFFFFFFFu, pass);
            const int leader = __ffs(b) - 1;
            int got = 1;
            if (lane == leader) {
                int spins = 0;
                while (atomicCAS(&ts.lock[r], 0, 1) != 0) {
                    if (++spins > kTopkSpinLimit) { got = 0; break; }
                }
                if (!got) atomicOr(&ts.err, 1);
                __threadfence_block();
            }
            got = __shfl_sync(0xFFFFFFFFu, got, leader);
            if (got) {
                unsigned rest = b;
                while (rest) {
                    const int L = __ffs(rest) - 1;
                    rest &= rest - 1u;
                    if (lane == L) heap_offer(ts, ht, hi, k, r, t, m);
                    __syncwarp();
                }
                if (lane == leader) {
                    __threadfence_block();
                    atomicExch(&ts.lock[r], 0);
                }
                changed = true;
            }
        }
        if (changed && lane == 0) update_coef_min(ts, nr);
    }
};

// scratch: float t[rows][splits][k] followed by int idx[rows][splits][k]
template <int NP, typename ET, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_topk(const GroupParams p, int k, float* part_t, int* part_i,
                                                      int* err) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ TopkSmem ts;
    float* ht = reinterpret_cast<float*>(T + p.tab_words);
    int* hi = reinterpret_cast<int*>(ht + 32 * k);
    if (threadIdx.x < 32) {
        ts.lock[threadIdx.x] = 0;
        ts.size[threadIdx.x] = 0;
        ts.root[threadIdx.x] = 0ull;
        ts.coef[threadIdx.x] = 0.0f;
    }
    if (threadIdx.x == 0) {
        ts.err = 0;
        ts.coef_min_bits = 0;
    }
    const int nr = build_table(T, rs, p);   // synchronizes the block
    const int64_t cb = p.chunk_begin + (p.chunk_end - p.chunk_begin) * blockIdx.y / gridDim.y;
    const int64_t ce = p.chunk_begin + (p.chunk_end - p.chunk_begin) * (blockIdx.y + 1) / gridDim.y;
    const int64_t want_warm = (k + 31) / 32 + 8;
    const int64_t warm = (ce - cb) < want_warm ? (ce - cb) : want_warm;
    if ((threadIdx.x >> 5) == 0) {
        TopkWarmEpi<NP> we{rs, ts, ht, hi, nr, k};
        stream_chunks<NP, ET, RARE>(T, p, cb, cb + warm, we);
        __syncwarp();
        if (threadIdx.x == 0) update_coef_min(ts, nr);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int64_t rb = cb + warm;
    const int64_t wb = rb + (ce - rb) * warp / nwarps, wend = rb + (ce - rb) * (warp + 1) / nwarps;
    TopkEpi<NP> epi{rs, ts, ht, hi, nr, k};
    stream_chunks<NP, ET, RARE>(T, p, wb, wend, epi);
    __syncthreads();
    const int splits = gridDim.y;
    for (int i = threadIdx.x; i < nr * k; i += blockDim.x) {
        const int r = i / k, j = i - r * k;
        const int64_t row = rs.orow[r];
        const int64_t o = (row * splits + blockIdx.y) * k + j;
        const bool ok = j < ts.size[r];
        part_t[o] = ok ? ht[r * k + j] : -3.0e38f;
        part_i[o] = ok ? hi[r * k + j] : -1;
    }
    if (threadIdx.x == 0 && ts.err) atomicOr(err, 1);
}

// One CTA per row: bitonic sort of the row's splits x k partial entries by
// (similarity descending, index ascending) and the first k written out.
constexpr int kTopkMergeMax = 8192;
__global__ void __launch_bounds__(512) k_topk_merge(const float* part_t, const int* part_i, int splits, int k,
                                                    int32_t* idx, float* sims) {
    extern __shared__ __align__(16) uint32_t sm[];
    const int n = splits * k;
    int N = 1;
    while (N < n) N <<= 1;
    float* st = reinterpret_cast<float*>(sm);
    int* si = reinterpret_cast<int*>(st + N);
    const int64_t row = blockIdx.x;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        st[i] = i < n ? part_t[row * n + i] : -3.0e38f;
        si[i] = i < n ? part_i[row * n + i] : -1;
    }
    __syncthreads();
    for (int kk = 2; kk <= N; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool asc = (i & kk) == 0;
                    const bool vi = si[i] >= 0, vj = si[ixj] >= 0;
                    // ji: element ixj ranks before element i (invalid entries, index -1, last)
                    bool ji;
                    if (vi != vj) ji = vj;
                    else if (!vi) ji = false;
                    else ji = worse(st[i], si[i], st[ixj], si[ixj]);
                    if (ji == asc) {
                        const float tt = st[i]; st[i] = st[ixj]; st[ixj] = tt;
                        const int ti = si[i]; si[i] = si[ixj]; si[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        const bool ok = j < n && si[j] >= 0;
        idx[row * k + j] = ok ? si[j] : -1;
        sims[row * k + j] = ok ? st[j] : -1.0f;
    }
}

// Fallback (no table or k > kTopkMax): one CTA per row scans every column
// with the sorted merge and keeps a k-heap in shared memory under the same
// bounded lock, then sorts it.
__global__ void __launch_bounds__(256) k_topk_rowscan(const struct RawArgs ra, int k, int32_t* idx, float* sims,
                                                      int* err, const int* list, const int* list_count);

// ---------------------------------------------- threshold-and-collect top-k ----
// Exact top-k in three steps, for tables that fit in shared memory:
//  1. per-row histograms of a sample (a prefix of the database's chunks,
//     k_loghist) give each row a bound theta: the lower edge of the highest
//     bin at which the sample already holds k molecules.  At least k database
//     molecules reach theta, so the row's true k-th best is >= theta.  The
//     sample's histogram is taken above floors from a smaller prefix (the
//     same rule on 1/8 of the sample), which skips most of its pairs with
//     the bit-sliced integer compare and leaves theta unchanged;
//  2. k_collect gathers every pair with t >= theta into per-(row, split)
//     segments of a candidate buffer;
//  3. k_topk_select sorts each row's candidates by (similarity descending,
//     index ascending) and writes the first k.  A row whose segments
//     overflowed takes the k-th best of the candidates kept as its new bound
//     (still at least k molecules above it) and goes on a device list for
//     another collection pass; rows that overflow again are scanned by
//     k_topk_rowscan.  No host synchronization is needed between the steps.
constexpr int kSelectMax = 8192;

// One warp per row: walks the bins from the top, 32 at a time, to the
// highest bin at which k molecules have been seen.
__global__ void k_topk_theta(const int32_t* hist, int k, int64_t rows, float* row_lo, int* list_counts) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        list_counts[0] = 0;
        list_counts[1] = 0;
    }
    if (i >= rows) return;   // uniform over the warp
    const int32_t* h = hist + i * kLogBins;
    int64_t acc = 0;
    int found = 0;   // bin index, 0 when fewer than k above bin 0
    for (int top = kLogBins - 1; top > 0 && !found; top -= 32) {
        const int b = top - lane;                       // lane 0 holds the highest bin of the slice
        const int64_t v = b > 0 ? h[b] : 0;
        int64_t incl = v;                               // inclusive prefix over lanes = count of bins >= b in slice
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        const unsigned hit = __ballot_sync(0xFFFFFFFFu, b > 0 && acc + incl >= k);
        if (hit) found = top - (__ffs(hit) - 1);
        acc += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) row_lo[i] = log_bin_floor(found);   // bin 0: collect all
}

// One CTA per row (listed rows: absolute row ids, rowbase subtracted).
// Candidates of row r: segments s = 0..splits-1 of seg_cap entries at
// cand + (r * splits + s) * seg_cap, holding min(count, seg_cap) entries.
__global__ void __launch_bounds__(512) k_topk_select(const int32_t* cand_i, const float* cand_t,
                                                     const int32_t* seg_counts, int splits, int64_t seg_cap, int k,
                                                     int64_t rowbase, const int* list, const int* list_count,
                                                     float* row_lo, int* next, int* next_count, int32_t* idx,
                                                     float* sims) {
    extern __shared__ __align__(16) uint32_t sm[];
    __shared__ int seg_off[1025];
    __shared__ int s_over;
    int64_t row;
    if (list) {
        if ((int)blockIdx.x >= *list_count) return;   // uniform over the CTA
        row = list[blockIdx.x] - rowbase;
    } else {
        row = blockIdx.x;
    }
    if (threadIdx.x == 0) {
        int acc = 0, over = 0;
        for (int q = 0; q < splits; q++) {
            const int c = seg_counts[row * splits + q];
            seg_off[q] = acc;
            acc += c < seg_cap ? c : (int)seg_cap;
            over |= c > seg_cap;
        }
        seg_off[splits] = acc;
        s_over = over;
    }
    __syncthreads();
    const int n = seg_off[splits];
    const bool over = s_over != 0;
    int N = 1;
    while (N < n) N <<= 1;
    float* st = reinterpret_cast<float*>(sm);
    int* si = reinterpret_cast<int*>(st + N);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        st[i] = -3.0e38f;
        si[i] = -1;
    }
    __syncthreads();
    for (int q = 0; q < splits; q++) {
        const int c = seg_off[q + 1] - seg_off[q];
        const int64_t base = (row * splits + q) * seg_cap;
        for (int i = threadIdx.x; i < c; i += blockDim.x) {
            st[seg_off[q] + i] = cand_t[base + i];
            si[seg_off[q] + i] = cand_i[base + i];
        }
    }
    __syncthreads();
    for (int kk = 2; kk <= N; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool asc = (i & kk) == 0;
                    const bool vi = si[i] >= 0, vj = si[ixj] >= 0;
                    bool ji;
                    if (vi != vj) ji = vj;
                    else if (!vi) ji = false;
                    else ji = worse(st[i], si[i], st[ixj], si[ixj]);
                    if (ji == asc) {
                        const float tt = st[i]; st[i] = st[ixj]; st[ixj] = tt;
                        const int ti = si[i]; si[i] = si[ixj]; si[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
    if (over) {
        if (threadIdx.x == 0) {
            row_lo[row] = st[k - 1];
            next[atomicAdd(next_count, 1)] = (int)(row + rowbase);
        }
        return;
    }
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        const bool ok = j < n;
        idx[row * k + j] = ok ? si[j] : -1;
        sims[row * k + j] = ok ? st[j] : -1.0f;
    }
}

// -------------------------------------------------------- k_batch_nbr ----
// Persistent batched neighbour search over ragged jobs (a job = a range of
// ref rows against a range of database columns).  The plan orders each
// job's rows by magnitude (GroupParams.row_order holds the ordered ref rows
// of all jobs) and splits every job into work items of at most 32 of those
// rows x a chunk range; one CTA per SM pulls items from a device queue head.
// The shared table is updated incrementally: an item whose rows differ from
// the CTA's current rows first clears the current rows' bits (their vid
// lists, not the whole table) and then sets its own.  Lanes outside the
// job's columns are masked in the epilogue; chunks whose magnitudes cannot
// reach the bound against the item's rows are skipped.
// Item layout: two int4 {first order position, rows, output row - ref row,
// col_begin}, {col_end, c0, c1, 0}.
//
// Every item is checked against the plan's extents before it is used (its
// order positions, chunk range, ref rows and output rows); an item that
// fails sets bit 2 of the engine's asynchronous error word and is skipped,
// so a damaged or stale plan cannot make the kernel touch memory outside
// its buffers.
struct BatchLimits {
    int64_t order_len;   // entries of row_order
    int64_t rows_out;    // output rows
    int64_t nref;        // ref rows
    int* err;            // asynchronous error word (bit 2: bad item)
};

__device__ __forceinline__ void set_rows(uint32_t* T, RowSmem& rs, const GroupParams& p, int64_t pos0, int nr,
                                         int64_t bias) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    if (warp == 0) {
        const int r = lane;
        const int64_t gr = p.row_order[pos0 + (r < nr ? r : 0)];
        const int am = r < nr ? p.row_mag[gr] : 0;
        rs.orow[r] = (int)(gr + bias);
        rs.amag[r] = am;
        rs.amagf[r] = (float)am;
        rs.alen[r] = r < nr ? p.row_len[gr] : 0;
        const bool f = r >= nr || fast_mag(am, p.row_cmag[gr]);
        const unsigned all = __ballot_sync(0xFFFFFFFFu, f);
        int mn = r < nr ? am : 0x7FFFFFFF, mxa = r < nr ? am : -1;
        for (int o = 16; o > 0; o >>= 1) {
            mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o));
            mxa = max(mxa, __shfl_xor_sync(0xFFFFFFFFu, mxa, o));
        }
        if (r == 0) {
            rs.allfast = all == 0xFFFFFFFFu;
            rs.min_amag = mn;
            rs.max_amag = mxa;
        }
    }
    for (int r = warp; r < nr; r += nwarps) {
        const uint32_t* rv = p.row_vid + (int64_t)p.row_order[pos0 + r] * p.row_stride;
        for (int64_t e = lane; e < p.row_stride; e += 32) table_set(T, p, rv[e], 1u << r);
    }
}

__device__ __forceinline__ void clear_rows(uint32_t* T, const GroupParams& p, int64_t pos0, int nr) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nwarps) {
        const uint32_t* rv = p.row_vid + (int64_t)p.row_order[pos0 + r] * p.row_stride;
        for (int64_t e = lane; e < p.row_stride; e += 32) {
            const uint32_t v = rv[e];
            if (v && (int64_t)v <= p.ncommon) T[v] = 0u;
        }
    }
    // the rare-vid hash is cleared whole
    for (int i = p.vt_words + threadIdx.x * 4; i < p.tab_words; i += blockDim.x * 4)
        *reinterpret_cast<uint4*>(T + i) = make_uint4(0u, 0u, 0u, 0u);
}

template <int NP, typename ET, bool RARE = false>
__global__ void __launch_bounds__(kThreads, 1) k_batch_nbr(const GroupParams p, const int4* __restrict__ items,
                                                           int64_t nitems, unsigned int* head, NbrArgs a,
                                                           const BatchLimits lim) {
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RowSmem rs;
    __shared__ long long s_item;
    __shared__ long long cur_pos, cur_bias;
    __shared__ int cur_nr;
    __shared__ long long next;
    for (int i = threadIdx.x * 4; i < p.tab_words; i += blockDim.x * 4)
        *reinterpret_cast<uint4*>(T + i) = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) { cur_pos = -1; cur_bias = 0; cur_nr = 0; }
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = (long long)atomicAdd(head, 1u);
            if (s_item < nitems) next = items[2 * s_item + 1].y;   // the item's first chunk
        }
        __syncthreads();
        const long long w = s_item;
        if (w >= nitems) break;
        const int4 ia = items[2 * w], ib = items[2 * w + 1];
        const int64_t pos0 = ia.x, bias = ia.z;
        const int nr = ia.y;
        if (nr < 1 || nr > 32 || pos0 < 0 || pos0 + nr > lim.order_len || ib.y < 0 || ib.y > ib.z ||
            ib.z > p.nchunks) {   // uniform: skip the item
            if (threadIdx.x == 0) atomicOr(lim.err, 2);
            __syncthreads();   // every thread has read s_item
            continue;
        }
        if (pos0 != cur_pos || nr != cur_nr || bias != cur_bias) {
            // the item's rows are checked when they enter the table
            bool bad = false;
            if (threadIdx.x < nr) {
                const int64_t gr = p.row_order[pos0 + threadIdx.x];
                bad = gr < 0 || gr >= lim.nref || gr + bias < 0 || gr + bias >= lim.rows_out;
            }
            if (__syncthreads_or(bad)) {   // uniform: skip the item, keep the current rows
                if (threadIdx.x == 0) atomicOr(lim.err, 2);
                continue;
            }
            if (cur_nr > 0) clear_rows(T, p, cur_pos, cur_nr);
            __syncthreads();
            set_rows(T, rs, p, pos0, nr, bias);
            if (threadIdx.x == 0) { cur_pos = pos0; cur_nr = nr; cur_bias = bias; }
            __syncthreads();
        }
        NbrArgs ai = a;
        ai.col_begin = ia.w;
        ai.col_end = ib.x;
        NbrEpi<NP> epi{rs, nr, 0, ai};
        stream_dynamic<NP, ET, RARE>(T, p, rs, &next, ib.z, ai.thr_mode == 0 ? ai.lo : 0.0f, nr, epi);
        __syncthreads();
    }
}

// ------------------------------------------------------- k_nbr_finish ----
struct RawArgs {
    const int32_t *rl, *rc, *rlen, *rmag, *rcmag;
    int64_t rw;
    const int32_t *ql, *qc, *qlen, *qmag, *qcmag;
    int64_t qw, nq;
    int64_t rowbase;
};

__device__ __forceinline__ int merge_isct(const int32_t* a, const int32_t* as, int32_t alen,
                                          const int32_t* b, const int32_t* bs, int32_t blen) {
    int32_t i = 0, j = 0, isct = 0;
    while (i < alen && j < blen) {
        const int32_t x = a[i], y = b[j];
        if (x == y) { isct += min(as[i], bs[j]); i++; j++; }
        else if (x < y) i++;
        else j++;
    }
    return isct;
}

// One CTA (128 threads) per output row.  Rows whose hits fit and number at
// most kNbrSortMax are sorted by column; the others (or all rows when
// force_ordered) are recomputed with the reference's ordered scan: waves of
// 128 columns, hits written in column order while they fit in pitch, the
// count growing by whole waves, stopping after the first wave that takes it
// above pitch (pysiml/kernels.py:433-474).
__global__ void __launch_bounds__(128) k_nbr_finish(const RawArgs ra, const NbrArgs a, int force_ordered) {
    __shared__ int skey[kNbrSortMax];
    __shared__ float sval[kNbrSortMax];
    __shared__ int wcount[4];
    const int64_t row = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int64_t ref_row = ra.rowbase + row;
    int64_t col0 = a.col_begin, col1 = a.col_end;
    if (a.rowinfo) {
        const int4 ri = a.rowinfo[row];
        if (ri.x < 0) return;   // output row not covered by any job
        ref_row = ri.x;
        col0 = ri.y;
        col1 = ri.z;
        if (ri.w) force_ordered = 1;   // a job the plan gives to the per-pair merge
    }
    int32_t* idx = a.idx + row * a.pitch;
    float* sims = a.sims ? a.sims + row * a.pitch : nullptr;
    const int n = force_ordered ? 0x7FFFFFFF : a.counts[row];
    if (!force_ordered && n <= a.pitch && n <= kNbrSortMax) {
        if (n <= 1) return;
        int N = 1;
        while (N < n) N <<= 1;
        for (int i = tid; i < N; i += blockDim.x) {
            skey[i] = i < n ? idx[i] : 0x7FFFFFFF;
            sval[i] = (i < n && sims) ? sims[i] : 0.0f;
        }
        __syncthreads();
        for (int k = 2; k <= N; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < N; i += blockDim.x) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const bool asc = (i & k) == 0;
                        if ((skey[i] > skey[ixj]) == asc) {
                            const int tk = skey[i]; skey[i] = skey[ixj]; skey[ixj] = tk;
                            const float tv = sval[i]; sval[i] = sval[ixj]; sval[ixj] = tv;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = tid; i < n; i += blockDim.x) {
            idx[i] = skey[i];
            if (sims) sims[i] = sval[i];
        }
        return;
    }
    // ordered recompute over [col0, col1), waves of 128 from col0
    const int64_t r = ref_row;
    const int32_t* ar = ra.rl + r * ra.rw;
    const int32_t* acnt = ra.rc + r * ra.rw;
    const int32_t alen = ra.rlen[r], ma = ra.rmag[r];
    int64_t count = 0;
    for (int64_t base = col0; base < col1; base += 128) {
        const int64_t col = base + tid;
        bool flag = false;
        float t = 0.0f;
        if (col < col1) {
            const int32_t mb = ra.qmag[col];
            const float bound = __fdiv_rn(__int2float_rn(min(ma, mb)), __int2float_rn(max(ma, mb)));
            if (bound >= a.lo) {
                const int is = merge_isct(ar, acnt, alen, ra.ql + col * ra.qw, ra.qc + col * ra.qw, ra.qlen[col]);
                t = tanimoto_rows(is, ma, mb);
                flag = t >= a.lo && t < a.hi;
            }
        }
        const unsigned b = __ballot_sync(0xFFFFFFFFu, flag);
        if (lane == 0) wcount[warp] = __popc(b);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < 4; w++) {
            const int cw = wcount[w];
            if (w < warp) before += cw;
            total += cw;
        }
        const int64_t pos = count + before + __popc(b & ((1u << lane) - 1u));
        if (flag && pos < a.pitch) {
            idx[pos] = (int32_t)col;
            if (sims) sims[pos] = t;
        }
        count += total;
        __syncthreads();
        if (count > a.pitch) break;
    }
    if (tid == 0) a.counts[row] = (int32_t)(count < 0x7FFFFFFF ? count : 0x7FFFFFFF);
}

// ------------------------------------------------------ k_rows_merge ----
// Sorted merge per pair (pysiml/_CPULingo.c:53-71, pysiml/kernels.py:162-199).
__global__ void k_rows_merge(const RawArgs ra, float* out, int64_t ldo, int mode) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t r = ra.rowbase + blockIdx.y;
    if (col >= ra.nq) return;
    const int32_t alen = ra.rlen[r], blen = ra.qlen[col];
    const int isct = merge_isct(ra.rl + r * ra.rw, ra.rc + r * ra.rw, alen,
                                ra.ql + col * ra.qw, ra.qc + col * ra.qw, blen);
    const float t = mode == kModeSingle ? tanimoto_single(isct, ra.rcmag[r], ra.qcmag[col], alen, blen)
                                        : tanimoto_rows(isct, ra.rmag[r], ra.qmag[col]);
    out[(int64_t)blockIdx.y * ldo + col] = t;
}

__global__ void __launch_bounds__(256) k_topk_rowscan(const RawArgs ra, int k, int32_t* idx, float* sims,
                                                      int* err, const int* list, const int* list_count) {
    extern __shared__ __align__(16) uint32_t sm[];
    float* ht = reinterpret_cast<float*>(sm);
    int* hi = reinterpret_cast<int*>(ht + k);
    __shared__ int lock, size, err_s;
    __shared__ unsigned long long root;   // published k-th best, 0 until the heap is full
    if (list && (int)blockIdx.x >= *list_count) return;   // uniform over the CTA
    if (threadIdx.x == 0) { lock = 0; size = 0; err_s = 0; root = 0ull; }
    __syncthreads();
    const int64_t r = list ? (int64_t)list[blockIdx.x] : ra.rowbase + blockIdx.x;   // absolute row
    const int64_t orow = r - ra.rowbase;
    const int32_t* a = ra.rl + r * ra.rw;
    const int32_t* as = ra.rc + r * ra.rw;
    const int32_t alen = ra.rlen[r], ma = ra.rmag[r];
    for (int64_t col = threadIdx.x; col < ra.nq; col += blockDim.x) {
        const int is = merge_isct(a, as, alen, ra.ql + col * ra.qw, ra.qc + col * ra.qw, ra.qlen[col]);
        const float t = tanimoto_rows(is, ma, ra.qmag[col]);
        const int m = (int)col;
        if (!beats_root(*(volatile unsigned long long*)&root, t, m)) continue;
        int spins = 0;
        bool got = true;
        while (atomicCAS(&lock, 0, 1) != 0) {
            if (++spins > kTopkSpinLimit) { got = false; break; }
            __nanosleep(32);
        }
        if (!got) { atomicOr(&err_s, 1); continue; }
        __threadfence_block();
        int n = size;
        bool changed = true;
        if (n < k) {
            ht[n] = t; hi[n] = m;
            heap_sift_up(ht, hi, n);
            size = ++n;
        } else if (worse(ht[0], hi[0], t, m)) {
            ht[0] = t; hi[0] = m;
            heap_sift_down(ht, hi, k);
        } else {
            changed = false;
        }
        if (changed && n == k)
            *(volatile unsigned long long*)&root =
                ((unsigned long long)__float_as_uint(ht[0]) << 32) | (unsigned long long)(uint32_t)hi[0];
        __threadfence_block();
        atomicExch(&lock, 0);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // heap sort into best-first order
        const int n = size;
        for (int end = n - 1; end > 0; end--) {
            const float tt = ht[0]; ht[0] = ht[end]; ht[end] = tt;
            const int ti = hi[0]; hi[0] = hi[end]; hi[end] = ti;
            heap_sift_down(ht, hi, end);
        }
        if (err_s) atomicOr(err, 1);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        const bool ok = j < size;
        idx[orow * k + j] = ok ? hi[j] : -1;
        sims[orow * k + j] = ok ? ht[j] : -1.0f;
    }
}

template <bool GLOBAL>
__global__ void k_hist_merge(const RawArgs ra, void* out, int64_t ldo) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t r = ra.rowbase + blockIdx.y;
    if (col >= ra.nq) return;
    const int isct = merge_isct(ra.rl + r * ra.rw, ra.rc + r * ra.rw, ra.rlen[r],
                                ra.ql + col * ra.qw, ra.qc + col * ra.qw, ra.qlen[col]);
    const float t = tanimoto_rows(isct, ra.rmag[r], ra.qmag[col]);
    if (GLOBAL) atomicAdd(reinterpret_cast<unsigned long long*>(out) + bin_of(__fmul_rn(t, 1000.0f), 999u), 1ull);
    else atomicAdd(reinterpret_cast<int32_t*>(out) + (int64_t)blockIdx.y * ldo + bin_of(__fmul_rn(t, 100.0f), 100u), 1);
}

// rowHistogram101 (pysiml/_cpuutil.cpp:52-72): one CTA per row of a dense
// matrix, 101 shared bins, bin = (unsigned)(x*100) clamped to 100 (the
// product in the input's precision), values below zero and NaN to bin 0.
template <typename F>
__global__ void k_row_hist101(const F* __restrict__ data, int64_t cols, int64_t ld, uint32_t* __restrict__ hist) {
    __shared__ uint32_t H[kBins101];
    for (int i = threadIdx.x; i < kBins101; i += blockDim.x) H[i] = 0u;
    __syncthreads();
    const F* row = data + (int64_t)blockIdx.x * ld;
    for (int64_t c = threadIdx.x; c < cols; c += blockDim.x) {
        uint32_t b;
        if (sizeof(F) == 4) {
            b = bin_of(__fmul_rn((float)row[c], 100.0f), 100u);
        } else {
            const double s = __dmul_rn((double)row[c], 100.0);
            b = !(s >= 0.0) ? 0u : (s >= 100.0 ? 100u : (uint32_t)s);
        }
        atomicAdd(H + b, 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins101; i += blockDim.x) hist[(int64_t)blockIdx.x * kBins101 + i] = H[i];
}

// ---------------------------------------------------------- launchers ----
RawArgs raw_args(siml_engine* h, int64_t rowbase) {
    RawArgs m;
    m.rl = h->ref.lingos; m.rc = h->ref.counts; m.rlen = h->ref.len; m.rmag = h->ref.mag; m.rcmag = h->ref.cmag;
    m.rw = h->ref.width;
    m.ql = h->qry.lingos; m.qc = h->qry.counts; m.qlen = h->qry.len; m.qmag = h->qry.mag; m.qcmag = h->qry.cmag;
    m.qw = h->qry.width; m.nq = h->qry.n;
    m.rowbase = rowbase;
    return m;
}

template <int NP, typename ET>
int launch_rows_bal_t(siml_engine* h, const GroupParams& p, size_t smem, float* out, int64_t ldo, int64_t max_ng) {
    const int64_t groups = (p.rows + 31) / 32;
    const size_t sm = smem + rows_bal_extra_smem(NP, kRowsBalThreads / 32);
    constexpr int SPG = sizeof(ET) == 2 ? 1 : 2;
    const int64_t run = max_ng / SPG;   // longest run of steps of a lane
    // 1: every run fits a 32-bit flush mask; 2: and its counts fit 7 planes
    const int mode = run > 32 ? 0 : (NP == 8 && run * 8 <= 127 ? 2 : 1);
    auto kern = mode == 0 ? k_rows_bal<NP, ET, false, 0> : k_rows_bal<NP, ET, false, 1>;
    if constexpr (NP == 8) {
        if (mode == 2) kern = k_rows_bal<NP, ET, false, 2>;
    }
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) {
            kern = mode == 0 ? k_rows_bal<NP, ET, true, 0> : k_rows_bal<NP, ET, true, 1>;
            if constexpr (NP == 8) {
                if (mode == 2) kern = k_rows_bal<NP, ET, true, 2>;
            }
        } else {
            return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
        }
    }
    int rc = set_smem(kern, sm);
    if (rc) return rc;
    const int s = choose_splits(groups, p.nchunks, h->num_sms, kRowsBalThreads / 32);
    dim3 grid((unsigned)groups, (unsigned)s);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kRowsBalThreads, sm, h->stream>>>(p, out, ldo);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

template <int NP, typename ET>
int launch_rows_t(siml_engine* h, const GroupParams& p, size_t smem, float* out, int64_t ldo) {
    const int64_t groups = (p.rows + 31) / 32;
    auto kern = k_rows<NP, ET, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_rows<NP, ET, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    const int s = choose_splits(groups, p.nchunks, h->num_sms, kThreads / 32);
    dim3 grid((unsigned)groups, (unsigned)s);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kThreads, smem, h->stream>>>(p, out, ldo);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

template <int NP, typename ET>
int launch_nbr_t(siml_engine* h, const GroupParams& p, size_t smem, const NbrArgs& a) {
    const int64_t groups = (p.rows + 31) / 32;
    auto kern = k_nbr<NP, ET, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_nbr<NP, ET, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    const int s = choose_splits(groups, p.chunk_end - p.chunk_begin, h->num_sms, kThreads / 32);
    dim3 grid((unsigned)groups, (unsigned)s);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kThreads, smem, h->stream>>>(p, a);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

template <int NP, typename ET, bool GLOBAL>
int launch_hist_t(siml_engine* h, const GroupParams& p, size_t smem, void* out, int64_t ldo) {
    const int64_t groups = (p.rows + 31) / 32;
    auto kern = k_hist<NP, ET, GLOBAL, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_hist<NP, ET, GLOBAL, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    const int s = choose_splits(groups, p.nchunks, h->num_sms, kThreads / 32);
    dim3 grid((unsigned)groups, (unsigned)s);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kThreads, smem, h->stream>>>(p, out, ldo);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

template <int NP, typename ET>
int launch_topk_t(siml_engine* h, const GroupParams& p, size_t smem, int k, int splits, float* pt, int* pi) {
    const int64_t groups = (p.rows + 31) / 32;
    auto kern = k_topk<NP, ET, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_topk<NP, ET, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    dim3 grid((unsigned)groups, (unsigned)splits);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kThreads, smem, h->stream>>>(p, k, pt, pi, h->d_async_err);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

template <int NP, typename ET>
int launch_batch_t(siml_engine* h, const GroupParams& p, size_t smem, const int4* items, int64_t nitems,
                   unsigned int* head, const NbrArgs& a, const BatchLimits& lim, cudaStream_t st) {
    auto kern = k_batch_nbr<NP, ET, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_batch_nbr<NP, ET, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    kern<<<(unsigned)h->num_sms, kThreads, smem, st>>>(p, items, nitems, head, a, lim);
    SIML_CUDA(cudaGetLastError());
    return SIML_OK;
}

}  // namespace

bool direct_table_fits(siml_engine* h, int64_t nvid) {
    return (size_t)((nvid + 1 + 3) / 4 * 4) * 4 + sizeof(RowSmem) + 64 <= h->smem_optin;
}

int64_t split_table_capacity(siml_engine* h) {
    // room for the rare-vid hash and the largest per-kernel extra (the
    // sample histogram of top-k), with a margin for static shared memory
    const int64_t extra = (int64_t)kRareSlots * 8 + 32 * kLogWords * 4 + (int64_t)sizeof(RowSmem) + 2048;
    const int64_t words = ((int64_t)h->smem_optin - extra) / 4;
    return std::max<int64_t>(0, words / 4 * 4 - 4);   // (ncommon + 1) rounded up to 4 stays <= words
}

int64_t split_balanced_capacity(siml_engine* h) {
    const int64_t extra = (int64_t)kRareSlots * 8 + (int64_t)rows_bal_extra_smem(8, kRowsBalThreads / 32) +
                          (int64_t)sizeof(RowSmem) + 2048;
    const int64_t words = ((int64_t)h->smem_optin - extra) / 4;
    return std::max<int64_t>(0, words / 4 * 4 - 4);
}

bool rows_balanced_fits(siml_engine* h) {
    if (h->vocab.split) {   // 8 planes only; the layout keeps split_balanced_capacity common vids
        const int np = planes_needed(std::min(h->ref.max_entries, h->qry.max_entries));
        return np <= 8 && split_balanced_capacity(h) > 0;
    }
    const int vt_words = (int)((h->vocab.ncommon + 1 + 3) / 4 * 4);
    const int np = planes_needed(std::min(h->ref.max_entries, h->qry.max_entries)) <= 8 ? 8 : 16;
    return (size_t)vt_words * 4 + rows_bal_extra_smem(np, kRowsBalThreads / 32) + sizeof(RowSmem) + 64 <= h->smem_optin;
}

int batch_nbr_usable(siml_engine* h, const DbLayout* d) {
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    return table_params(h, d, 0, 1, kModeRows, p, smem, np) ? 1 : 0;
}

int launch_batch_neighbors(siml_engine* h, const DbLayout* d, const int4* items, int64_t nitems, unsigned int* head,
                           const int32_t* order, int64_t order_len, const int4* rowinfo, int64_t rows_out, float lo,
                           float hi, int64_t pitch, int32_t* idx, float* sims, int32_t* counts, cudaStream_t st) {
    NbrArgs a = nbr_args(lo, hi, pitch, idx, sims, counts, 0, 0);
    a.rowinfo = rowinfo;
    const BatchLimits lim{order_len, rows_out, h->ref.n, h->d_async_err};
    SIML_CUDA(cudaMemsetAsync(counts, 0, rows_out * sizeof(int32_t), st));
    SIML_CUDA(cudaMemsetAsync(head, 0, sizeof(unsigned int), st));
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    int force_ordered = 1;
    int rc;
    if (nitems > 0 && table_params(h, d, 0, 1, kModeRows, p, smem, np)) {
        force_ordered = 0;
        p.row_order = order;
        if (np == 8)
            rc = d->entry_bytes == 2 ? launch_batch_t<8, uint16_t>(h, p, smem, items, nitems, head, a, lim, st)
                                     : launch_batch_t<8, uint32_t>(h, p, smem, items, nitems, head, a, lim, st);
        else
            rc = d->entry_bytes == 2 ? launch_batch_t<16, uint16_t>(h, p, smem, items, nitems, head, a, lim, st)
                                     : launch_batch_t<16, uint32_t>(h, p, smem, items, nitems, head, a, lim, st);
        if (rc) return rc;
        h->launches++;
    }
    if (rows_out > 0) {
        k_nbr_finish<<<(unsigned)rows_out, 128, 0, st>>>(raw_args(h, 0), a, force_ordered);
        SIML_CUDA(cudaGetLastError());
        h->launches++;
    }
    return SIML_OK;
}


int topk_plan(siml_engine* h, const DbLayout* d, int64_t rowbase, int64_t rowlimit, int k, TopkPlan& plan) {
    const int64_t rows = rowlimit - rowbase;
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    plan.splits = 0;
    plan.partial_entries = 0;
    const size_t heap_bytes = (size_t)32 * k * 8;
    if (k <= kTopkMax && table_params(h, d, rowbase, rows, kModeRows, p, smem, np) &&
        smem + heap_bytes + sizeof(RowSmem) + sizeof(TopkSmem) + 64 <= h->smem_optin) {
        const int64_t groups = (rows + 31) / 32;
        int splits = choose_splits(groups, p.nchunks, h->num_sms, kThreads / 32);
        while (splits > 1 && (int64_t)splits * k > kTopkMergeMax) splits--;
        plan.splits = splits;
        plan.partial_entries = (size_t)rows * splits * k;
    } else if ((size_t)k * 8 + 64 > h->smem_optin) {
        return fail(SIML_ERR_UNSUPPORTED, "top-k: k = %d too large", k);
    }
    return SIML_OK;
}

int launch_topk_core(siml_engine* h, const DbLayout* d, int64_t rowbase, int64_t rowlimit, int k,
                     const TopkPlan& plan, const int32_t* order, float* part_t, int* part_i, int32_t* idx,
                     float* sims) {
    const int64_t rows = rowlimit - rowbase;
    int rc;
    if (plan.splits > 0) {
        GroupParams p;
        size_t smem = 0;
        int np = 0;
        table_params(h, d, rowbase, rows, kModeRows, p, smem, np);
        p.row_order = order;
        const size_t sm = smem + (size_t)32 * k * 8;
        const bool u16 = d->entry_bytes == 2;
        if (np == 8) rc = u16 ? launch_topk_t<8, uint16_t>(h, p, sm, k, plan.splits, part_t, part_i) : launch_topk_t<8, uint32_t>(h, p, sm, k, plan.splits, part_t, part_i);
        else rc = u16 ? launch_topk_t<16, uint16_t>(h, p, sm, k, plan.splits, part_t, part_i) : launch_topk_t<16, uint32_t>(h, p, sm, k, plan.splits, part_t, part_i);
        if (rc) return rc;
        int N = 1;
        while (N < plan.splits * k) N <<= 1;
        const size_t msm = (size_t)N * 8;
        if ((rc = set_smem(k_topk_merge, msm))) return rc;
        k_topk_merge<<<(unsigned)rows, 512, msm, h->stream>>>(part_t, part_i, plan.splits, k, idx, sims);
        SIML_CUDA(cudaGetLastError());
        h->launches++;
        return SIML_OK;
    }
    const size_t sm = (size_t)k * 8;
    if ((rc = set_smem(k_topk_rowscan, sm))) return rc;
    SIML_CUDA(mark(h, h->ev0));
    k_topk_rowscan<<<(unsigned)rows, 256, sm, h->stream>>>(raw_args(h, rowbase), k, idx, sims, h->d_async_err, nullptr,
                                                           nullptr);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

namespace {

constexpr int64_t kTopkBlockRows = 8192;   // rows per pass of the threshold-and-collect path

// The sample histogram kernel fits next to the table.
bool smem_hist_ok(siml_engine* h, const DbLayout* d) {
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    return table_params(h, d, 0, 1, kModeRows, p, smem, np) &&
           smem + 32 * kLogWords * 4 + sizeof(RowSmem) + 64 <= h->smem_optin;
}
constexpr int64_t kSampleFraction = 8;     // the sample is 1/8 of the database's chunks

// Holds the engine's per-launch timing so a multi-kernel call brackets all
// of its launches with one event pair.
struct TimingHold {
    siml_engine* h;
    explicit TimingHold(siml_engine* e) : h(e) { h->hold_timing = true; }
    ~TimingHold() { h->hold_timing = false; }
};

template <int NP, typename ET>
int launch_collect_t(siml_engine* h, const GroupParams& p, size_t smem, int splits, const CollectArgs& c) {
    auto kern = k_collect<NP, ET, false>;
    if (p.rare_slots) {
        if constexpr (std::is_same<ET, uint16_t>::value) kern = k_collect<NP, ET, true>;
        else return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
    }
    int rc = set_smem(kern, smem);
    if (rc) return rc;
    dim3 grid((unsigned)((p.rows + 31) / 32), (unsigned)splits);
    kern<<<grid, kThreads, smem, h->stream>>>(p, c);
    SIML_CUDA(cudaGetLastError());
    h->launches++;
    return SIML_OK;
}

// Database splits of the collection pass and the candidate segment size:
// splits * seg_cap <= kSelectMax entries per row, seg_cap >= k.
void collect_shape(siml_engine* h, const DbLayout* d, int64_t rows, int k, int& splits, int64_t& seg_cap) {
    const int64_t groups = (rows + 31) / 32;
    splits = choose_splits(groups, d->nchunks, h->num_sms, kThreads / 32);
    while (splits > 1 && (int64_t)kSelectMax / splits < std::max<int64_t>(k, 64)) splits--;
    seg_cap = kSelectMax / splits;
}

size_t topk_collect_bytes(int64_t rows, int splits, int64_t seg_cap) {
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    return up((size_t)rows * kLogBins * 4) + up((size_t)rows * 4) + 2 * up((size_t)rows * splits * seg_cap * 4) +
           up((size_t)rows * splits * 4) + 2 * up((size_t)rows * 4) + up(16);
}

template <int NP, typename ET>
int topk_collect_block(siml_engine* h, const DbLayout* d, int64_t r0, int64_t rows, int k, int64_t sample,
                       size_t smem, const int32_t* order, char* buf, int32_t* idx, float* sims) {
    int splits = 1;
    int64_t seg_cap = 0;
    collect_shape(h, d, rows, k, splits, seg_cap);
    auto carve = [&](size_t bytes) {
        char* q = buf;
        buf += (bytes + 255) / 256 * 256;
        return q;
    };
    int32_t* hist = reinterpret_cast<int32_t*>(carve((size_t)rows * kLogBins * 4));
    float* row_lo = reinterpret_cast<float*>(carve((size_t)rows * 4));
    float* cand_t = reinterpret_cast<float*>(carve((size_t)rows * splits * seg_cap * 4));
    int32_t* cand_i = reinterpret_cast<int32_t*>(carve((size_t)rows * splits * seg_cap * 4));
    int32_t* seg_counts = reinterpret_cast<int32_t*>(carve((size_t)rows * splits * 4));
    int* list_a = reinterpret_cast<int*>(carve((size_t)rows * 4));
    int* list_b = reinterpret_cast<int*>(carve((size_t)rows * 4));
    int* list_n = reinterpret_cast<int*>(carve(16));
    int rc;
    // 1. per-row histograms of the sample (chunks [0, sample)) and the bounds.
    // With a large enough sample this takes two stages: the first 1/8 of the
    // sample gives floors (its k-th largest similarity or less, so the whole
    // sample holds at least k pairs at or above them), and the sample's
    // histogram is then taken above those floors only.  Its bins from the
    // floor up are complete, so the bound equals the one-stage bound.
    GroupParams ps;
    size_t sm0 = 0;
    int np = 0;
    table_params(h, d, r0, rows, kModeRows, ps, sm0, np);
    ps.row_order = order;
    auto sample_bounds = [&](const GroupParams& g, int64_t nch, bool floor) -> int {
        SIML_CUDA(cudaMemsetAsync(hist, 0, (size_t)rows * kLogBins * 4, h->stream));
        const int64_t groups = (rows + 31) / 32;
        int hs = choose_splits(groups, nch, h->num_sms, kThreads / 32);
        hs = (int)std::max<int64_t>(hs, (nch * 32 + 65534) / 65535);   // <= 65,535 molecules per CTA
        dim3 grid((unsigned)groups, (unsigned)hs);
        auto kern = floor ? k_loghist<NP, ET, true, false> : k_loghist<NP, ET, false, false>;
        if (g.rare_slots) {
            if constexpr (std::is_same<ET, uint16_t>::value)
                kern = floor ? k_loghist<NP, ET, true, true> : k_loghist<NP, ET, false, true>;
            else
                return fail(SIML_ERR_UNSUPPORTED, "a split vocabulary needs 16-bit entries");
        }
        int rc2;
        if ((rc2 = set_smem(kern, smem))) return rc2;
        kern<<<grid, kThreads, smem, h->stream>>>(g, hist);
        SIML_CUDA(cudaGetLastError());
        k_topk_theta<<<(unsigned)((rows + 7) / 8), 256, 0, h->stream>>>(hist, k, rows, row_lo, list_n);
        SIML_CUDA(cudaGetLastError());
        h->launches += 2;
        return SIML_OK;
    };
    const int64_t sample1 = sample / kSampleFraction;
    if (sample1 * 32 >= 4 * (int64_t)k) {
        GroupParams p1 = ps;
        p1.chunk_end = sample1;
        if ((rc = sample_bounds(p1, sample1, false))) return rc;
        GroupParams p2 = ps;
        p2.chunk_end = sample;
        p2.row_lo = row_lo;   // read when each CTA starts, rewritten by the bound kernel after it
        if ((rc = sample_bounds(p2, sample, true))) return rc;
    } else {
        GroupParams p1 = ps;
        p1.chunk_end = sample;
        if ((rc = sample_bounds(p1, sample, false))) return rc;
    }
    // 2. collect every pair at or above its row's bound
    GroupParams pc = ps;
    pc.chunk_begin = 0;
    pc.chunk_end = d->nchunks;
    pc.row_lo = row_lo;
    const CollectArgs ca{seg_cap, cand_i, cand_t, seg_counts};
    if ((rc = launch_collect_t<NP, ET>(h, pc, smem, splits, ca))) return rc;
    // 3. select; rows whose segments overflowed go to list a with a higher bound
    const size_t ssm = (size_t)kSelectMax * 8;
    if ((rc = set_smem(k_topk_select, ssm))) return rc;
    k_topk_select<<<(unsigned)rows, 512, ssm, h->stream>>>(cand_i, cand_t, seg_counts, splits, seg_cap, k, r0,
                                                          nullptr, nullptr, row_lo, list_a, list_n, idx, sims);
    SIML_CUDA(cudaGetLastError());
    // one more collection and selection for the listed rows
    GroupParams pl = pc;
    pl.row_order = list_a;
    pl.rows_dev = list_n;
    if ((rc = launch_collect_t<NP, ET>(h, pl, smem, splits, ca))) return rc;
    k_topk_select<<<(unsigned)rows, 512, ssm, h->stream>>>(cand_i, cand_t, seg_counts, splits, seg_cap, k, r0,
                                                          list_a, list_n, row_lo, list_b, list_n + 1, idx, sims);
    SIML_CUDA(cudaGetLastError());
    // rows that overflowed twice: exact scan
    if ((rc = set_smem(k_topk_rowscan, (size_t)k * 8))) return rc;
    k_topk_rowscan<<<(unsigned)rows, 256, (size_t)k * 8, h->stream>>>(raw_args(h, r0), k, idx, sims, h->d_async_err,
                                                                     list_b, list_n + 1);
    SIML_CUDA(cudaGetLastError());
    h->launches += 3;
    return SIML_OK;
}

}  // namespace

int launch_topk(siml_engine* h, int64_t rowbase, int64_t rowlimit, int k, int32_t* idx, float* sims) {
    const DbLayout* d = nullptr;
    int rc = ensure_layout(h, true, &d);
    if (rc) return rc;
    TopkPlan plan;
    if ((rc = topk_plan(h, d, rowbase, rowlimit, k, plan))) return rc;
    const int64_t sample = std::max<int64_t>(d->nchunks / kSampleFraction, (4 * (int64_t)k + 31) / 32);
    if (plan.splits > 0 && 32 * (int64_t)k <= kSelectMax && 2 * sample <= d->nchunks && smem_hist_ok(h, d)) {
        GroupParams p;
        size_t smem = 0;
        int np = 0;
        table_params(h, d, rowbase, 1, kModeRows, p, smem, np);
        TimingHold hold(h);
        SIML_CUDA(cudaEventRecord(h->ev0, h->stream));
        for (int64_t r0 = rowbase; r0 < rowlimit; r0 += kTopkBlockRows) {
            const int64_t r1 = std::min(rowlimit, r0 + kTopkBlockRows), rows = r1 - r0;
            const int32_t* order = nullptr;
            if ((rc = row_order_by_magnitude(h, r0, r1, &order))) return rc;
            int splits = 1;
            int64_t seg_cap = 0;
            collect_shape(h, d, rows, k, splits, seg_cap);
            void* buf = nullptr;
            if ((rc = scratch_reserve(h, topk_collect_bytes(rows, splits, seg_cap), &buf, kSlotPartial))) return rc;
            int32_t* oi = idx + (r0 - rowbase) * k;
            float* os = sims + (r0 - rowbase) * k;
            char* b = reinterpret_cast<char*>(buf);
            const bool u16 = d->entry_bytes == 2;
            if (np == 8)
                rc = u16 ? topk_collect_block<8, uint16_t>(h, d, r0, rows, k, sample, smem, order, b, oi, os)
                         : topk_collect_block<8, uint32_t>(h, d, r0, rows, k, sample, smem, order, b, oi, os);
            else
                rc = u16 ? topk_collect_block<16, uint16_t>(h, d, r0, rows, k, sample, smem, order, b, oi, os)
                         : topk_collect_block<16, uint32_t>(h, d, r0, rows, k, sample, smem, order, b, oi, os);
            if (rc) return rc;
        }
        SIML_CUDA(cudaEventRecord(h->ev1, h->stream));
        h->timed = true;
        return SIML_OK;
    }
    const int32_t* order = nullptr;
    float* pt = nullptr;
    int* pi = nullptr;
    if (plan.splits > 0) {
        if ((rc = row_order_by_magnitude(h, rowbase, rowlimit, &order))) return rc;
        void* buf = nullptr;
        if ((rc = scratch_reserve(h, plan.partial_entries * 8, &buf, kSlotPartial))) return rc;
        pt = reinterpret_cast<float*>(buf);
        pi = reinterpret_cast<int*>(pt + plan.partial_entries);
    }
    return launch_topk_core(h, d, rowbase, rowlimit, k, plan, order, pt, pi, idx, sims);
}

int launch_hist(siml_engine* h, int64_t rowbase, int64_t rowlimit, bool global, void* out, int64_t ldo) {
    const DbLayout* d = nullptr;
    int rc = ensure_layout(h, true, &d);
    if (rc) return rc;
    const int64_t rows = rowlimit - rowbase;
    if (!global) SIML_CUDA(cudaMemset2DAsync(out, ldo * 4, 0, kBins101 * 4, rows, h->stream));
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    if (table_params(h, d, rowbase, rows, kModeRows, p, smem, np) &&
        smem + (global ? kBins1000 : 32 * kBins101) * 4 + sizeof(RowSmem) + 64 <= h->smem_optin) {
        if ((rc = row_order_by_magnitude(h, rowbase, rowlimit, &p.row_order))) return rc;
        const bool u16 = d->entry_bytes == 2;
        if (global) {
            if (np == 8) return u16 ? launch_hist_t<8, uint16_t, true>(h, p, smem, out, ldo) : launch_hist_t<8, uint32_t, true>(h, p, smem, out, ldo);
            return u16 ? launch_hist_t<16, uint16_t, true>(h, p, smem, out, ldo) : launch_hist_t<16, uint32_t, true>(h, p, smem, out, ldo);
        }
        if (np == 8) return u16 ? launch_hist_t<8, uint16_t, false>(h, p, smem, out, ldo) : launch_hist_t<8, uint32_t, false>(h, p, smem, out, ldo);
        return u16 ? launch_hist_t<16, uint16_t, false>(h, p, smem, out, ldo) : launch_hist_t<16, uint32_t, false>(h, p, smem, out, ldo);
    }
    if (rows > 65535) return fail(SIML_ERR_UNSUPPORTED, "merge path: more than 65535 rows per call");
    dim3 grid((unsigned)((h->qry.n + 255) / 256), (unsigned)rows);
    SIML_CUDA(mark(h, h->ev0));
    if (global) k_hist_merge<true><<<grid, 256, 0, h->stream>>>(raw_args(h, rowbase), out, ldo);
    else k_hist_merge<false><<<grid, 256, 0, h->stream>>>(raw_args(h, rowbase), out, ldo);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

int launch_row_hist101(siml_engine* h, const void* data, bool f64, int64_t rows, int64_t cols, int64_t ld,
                       uint32_t* hist) {
    if (rows == 0) return SIML_OK;
    if (rows > 0x7FFFFFFF) return fail(SIML_ERR_UNSUPPORTED, "rowHistogram101: too many rows");
    if (f64) k_row_hist101<double><<<(unsigned)rows, 256, 0, h->stream>>>((const double*)data, cols, ld, hist);
    else k_row_hist101<float><<<(unsigned)rows, 256, 0, h->stream>>>((const float*)data, cols, ld, hist);
    SIML_CUDA(cudaGetLastError());
    h->launches++;
    return SIML_OK;
}

int launch_rows(siml_engine* h, const RowsArgs& a) {
    bool done = false;
    int rc = launch_rows_sched(h, a, &done);   // the scheduled kernel where it applies
    if (rc || done) return rc;
    const DbLayout* d = nullptr;
    rc = ensure_layout(h, false, &d);
    if (rc) return rc;
    const int64_t rows = a.rowlimit - a.rowbase;
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    if (table_params(h, d, a.rowbase, rows, a.mode, p, smem, np)) {
        if (d->balanced && !d->offsets) {
            if (np == 8)
                return d->entry_bytes == 2 ? launch_rows_bal_t<8, uint16_t>(h, p, smem, a.out, a.ldo, d->max_ng)
                                           : launch_rows_bal_t<8, uint32_t>(h, p, smem, a.out, a.ldo, d->max_ng);
            return d->entry_bytes == 2 ? launch_rows_bal_t<16, uint16_t>(h, p, smem, a.out, a.ldo, d->max_ng)
                                       : launch_rows_bal_t<16, uint32_t>(h, p, smem, a.out, a.ldo, d->max_ng);
        }
        if (d->offsets)
            return np == 8 ? launch_rows_t<8, off32_t>(h, p, smem, a.out, a.ldo)
                           : launch_rows_t<16, off32_t>(h, p, smem, a.out, a.ldo);
        if (np == 8)
            return d->entry_bytes == 2 ? launch_rows_t<8, uint16_t>(h, p, smem, a.out, a.ldo)
                                       : launch_rows_t<8, uint32_t>(h, p, smem, a.out, a.ldo);
        return d->entry_bytes == 2 ? launch_rows_t<16, uint16_t>(h, p, smem, a.out, a.ldo)
                                   : launch_rows_t<16, uint32_t>(h, p, smem, a.out, a.ldo);
    }
    if (rows > 65535) return fail(SIML_ERR_UNSUPPORTED, "merge path: more than 65535 rows per call");
    dim3 grid((unsigned)((h->qry.n + 255) / 256), (unsigned)rows);
    SIML_CUDA(mark(h, h->ev0));
    k_rows_merge<<<grid, 256, 0, h->stream>>>(raw_args(h, a.rowbase), a.out, a.ldo, a.mode);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

void sorted_chunk_range(const DbLayout* d, int64_t c0, int64_t c1, int64_t& chunk_begin, int64_t& chunk_end) {
    const int64_t W = d->window, per_window = W / kChunk;
    chunk_begin = (c0 / W) * per_window;
    chunk_end = std::min<int64_t>(d->nchunks, ((c1 + W - 1) / W) * per_window);
    if (c1 <= c0) chunk_end = chunk_begin;
}


int launch_neighbors(siml_engine* h, const NbrCall& c) {
    const DbLayout* d = nullptr;
    int rc = ensure_layout(h, true, &d);
    if (rc) return rc;
    const int64_t rows = c.rowlimit - c.rowbase;
    NbrArgs a = nbr_args(c.lo, c.hi, c.pitch, c.idx, c.sims, c.counts, c.col_begin, c.col_end);
    SIML_CUDA(cudaMemsetAsync(c.counts, 0, rows * sizeof(int32_t), h->stream));
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    int force_ordered = 1;
    if (c.col_end > c.col_begin && table_params(h, d, c.rowbase, rows, kModeRows, p, smem, np)) {
        force_ordered = 0;
        sorted_chunk_range(d, c.col_begin, c.col_end, p.chunk_begin, p.chunk_end);
        if ((rc = row_order_by_magnitude(h, c.rowbase, c.rowlimit, &p.row_order))) return rc;
        if (np == 8)
            rc = d->entry_bytes == 2 ? launch_nbr_t<8, uint16_t>(h, p, smem, a) : launch_nbr_t<8, uint32_t>(h, p, smem, a);
        else
            rc = d->entry_bytes == 2 ? launch_nbr_t<16, uint16_t>(h, p, smem, a) : launch_nbr_t<16, uint32_t>(h, p, smem, a);
        if (rc) return rc;
    }
    if (rows > 0x7FFFFFFF) return fail(SIML_ERR_UNSUPPORTED, "too many rows");
    k_nbr_finish<<<(unsigned)rows, 128, 0, h->stream>>>(raw_args(h, c.rowbase), a, force_ordered);
    SIML_CUDA(cudaGetLastError());
    h->launches++;
    return SIML_OK;
}

}  // namespace siml
