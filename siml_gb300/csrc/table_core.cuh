// Device-side pieces shared by the table kernels of kernels.cu and
// rows_sched.cu: the ref-row group parameters, the shared-memory table of a
// 32-row group and its build, the rare-vid hash of split vocabularies, the
// reference's fp32 Tanimoto expression, and the launch helpers that fill
// the parameters.  Everything is in an anonymous namespace, so each
// translation unit has its own copy.
#pragma once
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "engine.h"
#include "lingo_core.cuh"

namespace siml {
namespace {

constexpr int kThreads = 1024;

// getMultipleRows: _CPULingo.c:53-71 order — ((float)amag + bmag) - isct in
// fp32, then isct / union with IEEE round-to-nearest; 0 when a magnitude is 0.
__device__ __forceinline__ float tanimoto_rows(int isct, int amag, int bmag) {
    if (amag == 0 || bmag == 0) return 0.0f;
    const float u = __fsub_rn(__fadd_rn(__int2float_rn(amag), __int2float_rn(bmag)), __int2float_rn(isct));
    return __fdiv_rn(__int2float_rn(isct), u);
}

// getTanimotoRow: pysiml/kernels.py:122-159 — zero when either molecule has
// no LINGOs, union formed in int32 from the count sums, then converted.
__device__ __forceinline__ float tanimoto_single(int isct, int amag, int bmag, int alen, int blen) {
    if (alen == 0 || blen == 0) return 0.0f;
    const int u = (int)((unsigned)amag + (unsigned)bmag - (unsigned)isct);
    return __fdiv_rn(__int2float_rn(isct), __int2float_rn(u));
}

// A molecule's magnitude admits the fast epilogue when 1 <= mag <= 32768 and
// mag >= its count sum: then for any pair isct <= min(magA, magB), the union
// magA + magB - isct lies in [1, 65536] and the fp32 sum order of the
// reference is exact, so isct / union can use div_small.
__device__ __forceinline__ bool fast_mag(int mag, int cmag) { return mag >= 1 && mag <= 32768 && mag >= cmag; }

struct GroupParams {
    // ref rows
    const uint32_t* row_vid;
    int64_t row_stride;
    const int32_t* row_mag;
    const int32_t* row_cmag;
    const int32_t* row_len;
    int64_t rowbase;
    int rows;
    const int32_t* row_order;   // absolute row of group position i, or null for rowbase + i
    // database layout
    const void* entries;
    const int64_t* off;
    const int32_t* ng;
    const int4* meta;
    int64_t nchunks;
    int64_t chunk_begin, chunk_end;   // chunks this launch covers (a column range)
    int vt_words;             // words of the direct table (vids 0..ncommon)
    int tab_words;            // vt_words + the rare-vid hash (2 * rare_slots words)
    int64_t ncommon;          // vids above it are rare (split vocabulary)
    int rare_slots;           // 0, or kRareSlots with a split vocabulary
    const int64_t* rare_off;  // split vocabulary: slot s's rare vids are rare_vid[rare_off[s] ..
    const uint32_t* rare_vid; //   rare_off[s + 1])
    int mode;
    const float* row_lo;      // per output row lower bound (per-row threshold search) or null
    const int* rows_dev;      // device row count bounding `rows` (row lists built on the device) or null
    const int2* crange;       // per chunk {smallest, largest} magnitude (the layout's), for chunk skipping
    unsigned long long* eval; // counts the pairs of streamed (not skipped) chunks, or null
    int* err;                 // asynchronous error word: bit 3 when a ref row's vid fits neither the
                              // table nor the rare-vid hash (the entry is not used)
    int rare_fixup;           // rare vids are counted by a later pass (k_rare_fix): the table skips them
};

// Bit of the asynchronous error word set when a table build meets a vid it
// cannot hold: a vid above the layout's common set without a rare-vid hash,
// or a rare-vid hash with no free slot.  Neither happens for row lists built
// from the database's vocabulary; the bit reports a damaged list instead of
// dropping the entry unseen.
constexpr int kErrBadRowVid = 4;

struct RowSmem {
    int amag[32];
    int alen[32];
    int orow[32];            // output row (relative to rowbase) of group row r
    __align__(16) float amagf[32];
    int allfast;
    int min_amag;
    int max_amag;
    float min_lo;            // lowest per-row bound of the group
    float lo[32];            // per-row lower bound (GroupParams.row_lo)
    float coef[32];          // its integer-test coefficient (bound_coef)
    float min_coef;          // lowest integer-test coefficient of the group's bounds
};

// Coefficient of the conservative integer test for a bound lo > 0:
// t >= lo implies isct >= lo / (1 + lo) * (magA + magB); the factor
// (1 - 2^-12) absorbs fp32 rounding of the test itself.
__host__ __device__ __forceinline__ float bound_coef(float lo) {
    return lo > 0.0f ? (float)((double)lo / (1.0 + (double)lo) * (1.0 - 1.0 / 4096.0)) : 0.0f;
}

// Rows this launch really has: p.rows, or fewer when a device counter says so.
__device__ __forceinline__ int live_rows(const GroupParams& p) {
    return p.rows_dev ? min(p.rows, *p.rows_dev) : p.rows;
}

// Rare-vid hash of a row group (split vocabulary): kRareSlots keys (0 =
// empty) after the direct table, then their 32-row masks.  Linear probing;
// at most 32 x kRareRowMax keys, so it is never more than 3/4 full and every
// probe sequence ends.
__device__ __forceinline__ uint32_t rare_hash(uint32_t v) { return (v * 0x9E3779B1u) >> (32 - kRareSlotsLog2); }

__device__ __forceinline__ void rare_insert(uint32_t* keys, uint32_t v, uint32_t bit, int* err) {
    uint32_t h = rare_hash(v);
    for (int probe = 0; probe < kRareSlots; probe++) {
        const uint32_t prev = atomicCAS(&keys[h], 0u, v);
        if (prev == 0u || prev == v) {
            atomicOr(&keys[kRareSlots + h], bit);
            return;
        }
        h = (h + 1) & (kRareSlots - 1);
    }
    if (err) atomicOr(err, kErrBadRowVid);   // no free slot: the entry is not used
}

__device__ __forceinline__ uint32_t rare_lookup(const uint32_t* keys, uint32_t v) {
    uint32_t h = rare_hash(v);
    for (int probe = 0; probe < kRareSlots; probe++) {
        const uint32_t k = keys[h];
        if (k == v) return keys[kRareSlots + h];
        if (k == 0u) return 0u;
        h = (h + 1) & (kRareSlots - 1);
    }
    return 0u;
}

// Sets a row's bit for one of its vids: the direct table, or the rare hash.
__device__ __forceinline__ void table_set(uint32_t* T, const GroupParams& p, uint32_t v, uint32_t bit) {
    if (v == 0u) return;
    if ((int64_t)v <= p.ncommon) atomicOr(&T[v], bit);
    else if (p.rare_slots) rare_insert(T + p.vt_words, v, bit, p.err);
    else if (p.err && !p.rare_fixup) atomicOr(p.err, kErrBadRowVid);
}

// Adds the rare entries of layout slot `slot` (split vocabulary) to acc.
template <int NP>
__device__ __forceinline__ void rare_add(const uint32_t* T, const GroupParams& p, int64_t slot,
                                         SlicedCounter<NP>& acc) {
    const int64_t b = __ldg(p.rare_off + slot), e = __ldg(p.rare_off + slot + 1);
    const uint32_t* keys = T + p.vt_words;
    for (int64_t i = b; i < e; i++) {
        const uint32_t m = rare_lookup(keys, __ldg(p.rare_vid + i));
        if (m) acc.add1(m);
    }
}

// Clears T, sets bit r of T[vid] for the entries of row r, fills RowSmem.
// Returns the number of rows of the group.
__device__ __forceinline__ int build_table(uint32_t* T, RowSmem& rs, const GroupParams& p) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * 32;
    const int nr = min(32, live_rows(p) - (int)row0);
    for (int i = threadIdx.x * 4; i < p.tab_words; i += blockDim.x * 4)
        *reinterpret_cast<uint4*>(T + i) = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        const int r = lane;
        const int64_t gr = r < nr ? (p.row_order ? (int64_t)p.row_order[row0 + r] : p.rowbase + row0 + r) : p.rowbase;
        rs.orow[r] = (int)(gr - p.rowbase);
        const int am = r < nr ? (p.mode == kModeSingle ? p.row_cmag[gr] : p.row_mag[gr]) : 0;
        rs.amag[r] = am;
        rs.amagf[r] = (float)am;
        rs.alen[r] = r < nr ? p.row_len[gr] : 0;
        const bool f = r >= nr || (p.mode == kModeRows && fast_mag(am, p.row_cmag[gr]));
        const unsigned all = __ballot_sync(0xFFFFFFFFu, f);
        int mn = r < nr ? am : 0x7FFFFFFF, mxa = r < nr ? am : -1;
        for (int o = 16; o > 0; o >>= 1) {
            mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o));
            mxa = max(mxa, __shfl_xor_sync(0xFFFFFFFFu, mxa, o));
        }
        if (p.row_lo) {
            const float lo = r < nr ? p.row_lo[gr - p.rowbase] : 3.0e38f;
            rs.lo[r] = lo;
            float c = r < nr ? bound_coef(lo) : 3.0e38f;
            rs.coef[r] = r < nr ? c : 0.0f;
            float ml = lo;
            for (int o = 16; o > 0; o >>= 1) {
                c = fminf(c, __shfl_xor_sync(0xFFFFFFFFu, c, o));
                ml = fminf(ml, __shfl_xor_sync(0xFFFFFFFFu, ml, o));
            }
            if (r == 0) {
                rs.min_coef = c;
                rs.min_lo = ml;
            }
        }
        if (r == 0) {
            rs.allfast = all == 0xFFFFFFFFu;
            rs.min_amag = mn;
            rs.max_amag = mxa;
        }
    }
    __syncthreads();
    for (int r = warp; r < nr; r += nwarps) {
        const uint32_t* rv = p.row_vid + (int64_t)(p.rowbase + rs.orow[r]) * p.row_stride;
        for (int64_t e = lane; e < p.row_stride; e += 32) table_set(T, p, rv[e], 1u << r);
    }
    __syncthreads();
    return nr;
}

// Hint: bring [p, p + bytes) into L2 with one bulk prefetch (no completion
// to wait for).  p and bytes are multiples of 16.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    if (bytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

int planes_needed(int64_t max_count) {
    int b = 0;
    while (b < 62 && (1ll << b) <= max_count) b++;
    return b;
}

// Splits of the database per row group so that groups x splits fills whole
// waves of one CTA per SM and every warp still has several chunks.
int choose_splits(int64_t groups, int64_t nchunks, int num_sms, int nwarps) {
    int best = 1;
    double best_cost = 1e300;
    const int64_t max_s = std::max<int64_t>(1, std::min<int64_t>(1024, nchunks / (4 * nwarps)));
    for (int64_t s = 1; s <= max_s; s++) {
        const int64_t ctas = groups * s;
        const int64_t waves = (ctas + num_sms - 1) / num_sms;
        const double cost = (double)waves * (1.0 / (double)s + 0.004);
        if (cost < best_cost * 0.999) { best_cost = cost; best = (int)s; }
    }
    return best;
}

// Table kernels are usable when T (and, with a split vocabulary, the rare-vid
// hash) fits in shared memory, no ref row holds more rare entries than the
// hash allows, and 16-bit counters suffice; fills p and the dynamic
// shared-memory size.
bool table_params(siml_engine* h, const DbLayout* d, int64_t rowbase, int64_t rows, int mode,
                  GroupParams& p, size_t& smem, int& np) {
    const bool split = d->ncommon < h->vocab.nvid;
    const int64_t max_rare = d->ncommon >= h->vocab.ncommon ? h->rows.max_rare
                             : (d->scheduled ? h->rows.max_rare_sched : h->rows.max_rare_bal);
    if (split && (max_rare > kRareRowMax || !d->rare_off)) return false;
    const int vt_words = (int)((d->ncommon + 1 + 3) / 4 * 4);
    const int rare_slots = split ? kRareSlots : 0;
    const int tab_words = vt_words + 2 * rare_slots;
    smem = (size_t)tab_words * 4;
    np = planes_needed(std::min(h->ref.max_entries, h->qry.max_entries));
    if (smem + sizeof(RowSmem) + 64 > h->smem_optin || np > 16) return false;
    np = np <= 8 ? 8 : 16;
    p.row_vid = h->rows.vid;
    p.row_stride = h->rows.stride;
    p.row_mag = h->ref.mag;
    p.row_cmag = h->ref.cmag;
    p.row_len = h->ref.len;
    p.rowbase = rowbase;
    p.rows = (int)rows;
    p.row_order = nullptr;
    p.entries = d->entries;
    p.off = d->off;
    p.ng = d->ng;
    p.meta = d->meta;
    p.nchunks = d->nchunks;
    p.chunk_begin = 0;
    p.chunk_end = d->nchunks;
    p.vt_words = vt_words;
    p.tab_words = tab_words;
    p.ncommon = d->ncommon;
    p.rare_slots = rare_slots;
    p.rare_off = split ? d->rare_off : nullptr;
    p.rare_vid = split ? d->rare_vid : nullptr;
    p.mode = mode;
    p.row_lo = nullptr;
    p.rows_dev = nullptr;
    p.crange = d->crange;
    p.eval = h->d_eval;
    p.err = h->d_async_err;
    p.rare_fixup = 0;
    return true;
}

// Records a timing event on the engine's stream unless a multi-kernel call
// holds the timing to bracket all of its launches itself.
cudaError_t mark(siml_engine* h, cudaEvent_t ev) {
    return h->hold_timing ? cudaSuccess : cudaEventRecord(ev, h->stream);
}

template <class K>
int set_smem(K kernel, size_t smem) {
    return raise_smem_limit(reinterpret_cast<const void*>(kernel), smem);
}

}  // namespace
}  // namespace siml
