// getMultipleRows over the scheduled layout (sm_103a).
//
// A CTA holds the shared-memory table of 32 ref rows and splits its 32 warps
// into G independent groups of P = 32 / G warps.  Each group writes the
// group's 32 rows x one window of W = 2048 / G database columns at a time,
// and the groups work on different windows, synchronised only among
// themselves (named barriers), so one group's stream phase runs beside
// another's store phase and the table is shared by all.
//
// The layout sorts database molecules by entry count inside windows of W, so
// the 32 molecules of a chunk (one per lane) have nearly equal lists and a
// warp streams whole molecules, with no partial counters to merge.  Work is
// balanced at layout build, not at run time: each window's chunks, longest
// first, are dealt to the group's P warps in equal shares, where an item (a
// chunk, or a range of a chunk's 8-entry steps) costs its steps plus a fixed
// overhead for its epilogue, and the share is the smallest for which the
// wrap-around fill fits P warps (found by bisection).  A chunk whose steps
// straddle two shares is split into items that add into the same counts.
// Each (window, warp) run of items is stored contiguously, so a warp's loads
// stream one array, two steps ahead, with no bounds tests (the array carries
// two steps of padding), and the run of the group's next window is pulled
// into L2 while the current one streams.
//
// Phase 1 (per window): the group's warps stream their items through the
// bit-sliced counter (lingo_core.cuh); at the end of an item the 8 planes
// are transposed into 32 byte counts and stored, 8 words per molecule, into
// the group's staging area at the molecule's natural position in the window
// (a split item adds its words atomically; bytes cannot carry, the counts of
// a whole molecule being below 256).
// Phase 2 (per window, after the group's barrier): each thread takes 4
// consecutive columns and 4 rows per staging word and forms the reference's
// fp32 Tanimoto, ((float)amag + bmag) - isct and isct / union, with
// Markstein's correction of the reciprocal estimate (exact for the integer
// ranges fast_mag admits; other pairs take the IEEE division), then writes
// 16 bytes per row: a warp's store covers 512 contiguous bytes of one row.
// A full group whose pairs all admit the fast division takes a
// straight-line path in scalar fp32 (no row or column predicates); scalar
// code issues faster here than the packed f32x2 form, which the partial
// path keeps.  The staging words are zeroed as they are read.
#include <vector>

#include "table_core.cuh"

namespace siml {
namespace {

constexpr int kSThreads = 1024;
constexpr int kSWarpsAll = kSThreads / 32;
// Columns in flight per CTA (G windows of kSColsAll / G).  The staging holds
// a byte count per row and column, so 64-row groups keep half the columns.
template <int ROWS>
constexpr int kSColsAll = ROWS == 32 ? kSchedColumns32 : kSchedColumns64;
// An item's flush and record loads, in 8-entry steps, for the schedule: a
// higher cost makes fewer split items at some cost in balance.  Measured
// best: 2 for 32-row groups, 6 for 64-row groups (two counters to flush,
// windows half as long; 3, 4 and 8 were slower).
constexpr double item_cost(int rows) { return rows == 64 ? 6.0 : 2.0; }
constexpr int kItemStepsMask = 0xFFFF;
constexpr int kItemSplit = 1 << 16;   // the chunk has several items: add counts atomically
constexpr int kItemFirst = 1 << 17;   // the item holds the chunk's first step: column data, rare entries
constexpr int kItemLast = 1 << 18;    // the last item of its (window, warp) run
constexpr int kItemEmpty = 1 << 19;   // a placeholder for a run with no items (no steps, no lanes)
// L2 prefetch distance of the entry stream, in 8-entry steps ahead of a
// warp's read position: about one to three windows of 64-row groups ahead
// (measured best of 4-12 ... 24-56)
constexpr int kPrefetchFrom = 8, kPrefetchTo = 24;
constexpr int kPadSteps = 2;          // steps of zero padding after the entries (loads run two steps ahead)
// Largest row stride for which ROWS - 1 rows of fp32 stay within 32-bit byte offsets.
template <int ROWS>
constexpr int64_t kFullGroupLdo = (int64_t)(0xFFFFFFFFull / ((ROWS - 1ull) * 4ull));
// staging (ROWS / 4 count words per column) + column magnitudes, over all groups
template <int ROWS>
constexpr size_t kSchedExtraSmem = (size_t)(ROWS / 4 + 1) * kSColsAll<ROWS> * 4;
// The 64-row kernel's rare-pair hash: kRare64Slots keys, then a 64-bit row
// mask per slot.  At most 64 x kRare64RowMax keys: never more than 3/4 full.
constexpr int kRare64SlotsLog2 = 11;
constexpr int kRare64Slots = 1 << kRare64SlotsLog2;
constexpr int kRare64RowMax = 24;

struct SchedArgs {
    const int2* items;     // work items, with two padding records after the last
    const int* lanes;      // [items + 2][32] per lane: window position << 16 | fast column magnitude (0 for
                           // the IEEE path), or -1 for no molecule
    const int2* rare;      // split vocabulary: [items + 2][32] per lane {first rare entry, count}, counted once
                           // per molecule (items holding the chunk's first step), else null
    const int2* wrun;      // [nwin * P] {first item, end item} of (window, warp of the group)
    const int64_t* grun;   // [nwin * P][2] first and end 16-byte group of (window, warp of the group)
    const int32_t* qmag;   // database magnitudes in natural order (IEEE-division path)
    int64_t nq;
    int64_t nwin;
    float* out;            // row rowbase of the block
    int64_t ldo;
    int64_t ngroups;       // 16-byte groups of the entry array, padding included (prefetch bound)
};

// ---- packed fp32 pairs (two IEEE round-to-nearest operations each)
__device__ __forceinline__ uint64_t f2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unf2(uint64_t v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ float rcp_est(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Two Tanimotos i / (s - i) at once, each as div_small (lingo_core.cuh) with
// the reference's union order: u = s - i, q0 = i * y, r = fma(q0, -u, i)
// (the same value as fma(-q0, u, i)), q = fma(r, y, q0).
__device__ __forceinline__ uint64_t tanimoto2(uint64_t I, uint64_t S) {
    const uint64_t U = sub2(S, I), NU = sub2(I, S);
    float u0, u1;
    unf2(U, u0, u1);
    const uint64_t Y = f2(rcp_est(u0), rcp_est(u1));
    const uint64_t Q0 = mul2(I, Y);
    const uint64_t R = fma2(Q0, NU, I);
    return fma2(R, Y, Q0);
}

// ---- 64-row groups: one 8-byte table word per pair (bits 0-31: rows 0-31,
// bits 32-63: rows 32-63), read with one 8-byte shared load, so the vid
// extraction, the lookups, the loop and the entry stream serve 64 rows.
struct RowSmem64 {
    int amag[64];
    __align__(16) float amagf[64];
    int allfast;
};

__device__ __forceinline__ uint32_t rare64_hash(uint32_t v) { return (v * 0x9E3779B1u) >> (32 - kRare64SlotsLog2); }

// Sets bit `bit` of half `half` of vid v's mask in the rare-pair hash.
__device__ __forceinline__ void rare64_insert(uint32_t* keys, uint32_t v, int half, uint32_t bit, int* err) {
    uint32_t h = rare64_hash(v);
    for (int probe = 0; probe < kRare64Slots; probe++) {
        const uint32_t prev = atomicCAS(&keys[h], 0u, v);
        if (prev == 0u || prev == v) {
            atomicOr(&keys[kRare64Slots + 2 * h + half], bit);
            return;
        }
        h = (h + 1) & (kRare64Slots - 1);
    }
    if (err) atomicOr(err, kErrBadRowVid);   // no free slot: the entry is not used
}

__device__ __forceinline__ uint2 rare64_lookup(const uint32_t* keys, uint32_t v) {
    uint32_t h = rare64_hash(v);
    for (int probe = 0; probe < kRare64Slots; probe++) {
        const uint32_t k = keys[h];
        if (k == v) return *reinterpret_cast<const uint2*>(keys + kRare64Slots + 2 * h);
        if (k == 0u) return make_uint2(0u, 0u);
        h = (h + 1) & (kRare64Slots - 1);
    }
    return make_uint2(0u, 0u);
}

// Clears the 64-row table (p.vt_words words: 2 per vid) and its rare hash,
// sets the bits of the group's rows, fills rs.  Full-matrix mode only (the
// scheduled layout serves getMultipleRows).  Returns the group's rows.
__device__ __forceinline__ int build_table64(uint32_t* T, RowSmem64& rs, const GroupParams& p) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * 64;
    const int nr = min(64, live_rows(p) - (int)row0);
    for (int i = threadIdx.x * 4; i < p.tab_words; i += blockDim.x * 4)
        *reinterpret_cast<uint4*>(T + i) = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) {
        bool all = true;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int r = 32 * h + lane;
            const int64_t gr = r < nr ? p.rowbase + row0 + r : p.rowbase;
            const int am = r < nr ? p.row_mag[gr] : 0;
            rs.amag[r] = am;
            rs.amagf[r] = (float)am;
            all = __all_sync(0xFFFFFFFFu, r >= nr || fast_mag(am, p.row_cmag[gr])) && all;
        }
        if (lane == 0) rs.allfast = all;
    }
    __syncthreads();
    uint32_t* keys = T + p.vt_words;
    for (int r = warp; r < nr; r += nwarps) {
        const uint32_t* rv = p.row_vid + (p.rowbase + row0 + r) * p.row_stride;
        const int half = r >> 5;
        const uint32_t bit = 1u << (r & 31);
        for (int64_t e = lane; e < p.row_stride; e += 32) {
            const uint32_t v = rv[e];
            if (v == 0u) continue;
            if ((int64_t)v <= p.ncommon) atomicOr(&T[2 * v + half], bit);
            else if (p.rare_slots) rare64_insert(keys, v, half, bit, p.err);
            else if (p.err && !p.rare_fixup) atomicOr(p.err, kErrBadRowVid);
        }
    }
    __syncthreads();
    return nr;
}

// The bit-sliced counters of a ROWS-row group: one 8-plane counter per 32 rows.
template <int ROWS>
struct GroupCounter {
    SlicedCounter<8> c[ROWS / 32];

    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int h = 0; h < ROWS / 32; h++) c[h].clear();
    }

    // one 8-entry step (vids ix, see step_vids) into planes 0..2, its
    // weight-8 carries returned in e (close1 or close2 adds them)
    __device__ __forceinline__ void step_open(const uint32_t* T, const uint32_t (&ix)[8], uint32_t (&e)[ROWS / 32]) {
        if constexpr (ROWS == 32) {
            e[0] = c[0].add8_open(T[ix[0]], T[ix[1]], T[ix[2]], T[ix[3]], T[ix[4]], T[ix[5]], T[ix[6]], T[ix[7]]);
        } else {
            const uint2* T2 = reinterpret_cast<const uint2*>(T);
            const uint2 m0 = T2[ix[0]], m1 = T2[ix[1]], m2 = T2[ix[2]], m3 = T2[ix[3]];
            const uint2 m4 = T2[ix[4]], m5 = T2[ix[5]], m6 = T2[ix[6]], m7 = T2[ix[7]];
            e[0] = c[0].add8_open(m0.x, m1.x, m2.x, m3.x, m4.x, m5.x, m6.x, m7.x);
            e[1] = c[1].add8_open(m0.y, m1.y, m2.y, m3.y, m4.y, m5.y, m6.y, m7.y);
        }
    }
    __device__ __forceinline__ void close1(const uint32_t (&e)[ROWS / 32]) {
#pragma unroll
        for (int h = 0; h < ROWS / 32; h++) c[h].add_eights(e[h]);
    }
    __device__ __forceinline__ void close2(const uint32_t (&ea)[ROWS / 32], const uint32_t (&eb)[ROWS / 32]) {
#pragma unroll
        for (int h = 0; h < ROWS / 32; h++) c[h].add_eights2(ea[h], eb[h]);
    }

    // adds one rare entry (split vocabulary) through the group's hash
    __device__ __forceinline__ void add_rare_vid(const uint32_t* T, const GroupParams& p, uint32_t v) {
        if constexpr (ROWS == 32) {
            const uint32_t m = rare_lookup(T + p.vt_words, v);
            if (m) c[0].add1(m);
        } else {
            const uint2 m = rare64_lookup(T + p.vt_words, v);
            if (m.x) c[0].add1(m.x);
            if (m.y) c[1].add1(m.y);
        }
    }

    // a molecule's rare entries: rr = {first, count} in p.rare_vid, the first
    // two loaded ahead into v0, v1 (when the item started)
    __device__ __forceinline__ void add_rare(const uint32_t* T, const GroupParams& p, int2 rr, uint32_t v0,
                                             uint32_t v1) {
        if (rr.y <= 0) return;
        add_rare_vid(T, p, v0);
        if (rr.y <= 1) return;
        add_rare_vid(T, p, v1);
        for (int i = 2; i < rr.y; i++) add_rare_vid(T, p, __ldg(p.rare_vid + rr.x + i));
    }
};

// The 8 vids of a step's 16-byte entry group.  The empty asm makes them
// complete before the caller's next statement, which reloads the register
// that held the group with the step two ahead: the load then writes the
// registers the group held instead of others that a move must bring back
// at the end of the loop.
__device__ __forceinline__ void step_vids(const uint4 q, uint32_t (&ix)[8]) {
    ix[0] = q.x & 0xFFFFu;
    ix[1] = q.x >> 16;
    ix[2] = q.y & 0xFFFFu;
    ix[3] = q.y >> 16;
    ix[4] = q.z & 0xFFFFu;
    ix[5] = q.z >> 16;
    ix[6] = q.w & 0xFFFFu;
    ix[7] = q.w >> 16;
    asm volatile("" : "+r"(ix[0]), "+r"(ix[1]), "+r"(ix[2]), "+r"(ix[3]), "+r"(ix[4]), "+r"(ix[5]), "+r"(ix[6]),
                 "+r"(ix[7]));
}

// The first two rare entries of an item's molecule, loaded when the item
// starts so that they arrive while it streams.
__device__ __forceinline__ void rare_prefetch(const GroupParams& p, int2 rr, uint32_t& v0, uint32_t& v1) {
    v0 = rr.y > 0 ? __ldg(p.rare_vid + rr.x) : 0u;
    v1 = rr.y > 1 ? __ldg(p.rare_vid + rr.x + 1) : 0u;
}

// End of an item: each 32-row counter's planes become 32 byte counts, stored
// at the molecule's window position: staging word 8 h + k holds rows
// 32 h + k, + 8, + 16, + 24.
template <int WIN, int ROWS>
__device__ __forceinline__ void flush_item(uint32_t* W, float* colf, int flags, int lr,
                                           const GroupCounter<ROWS>& acc) {
    const int pos = lr >> 16;
    if (pos < 0) return;
#pragma unroll
    for (int h = 0; h < ROWS / 32; h++) {
        uint32_t w[8];
#pragma unroll
        for (int k = 0; k < 8; k++) w[k] = acc.c[h].plane[k];
        transpose_planes8(w);
        if (flags & kItemSplit) {
#pragma unroll
            for (int k = 0; k < 8; k++) atomicAdd(W + (8 * h + k) * WIN + pos, w[k]);
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) W[(8 * h + k) * WIN + pos] = w[k];
        }
    }
    if (flags & kItemFirst) {
        const uint32_t mag = (uint32_t)lr & 0xFFFFu;
        colf[pos] = mag ? small_int_to_float(mag) : -1.0f;
    }
}

__device__ __forceinline__ void group_barrier(int group, int threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "r"(threads) : "memory");
}

template <bool RARE, int G, int ROWS>
__global__ void __launch_bounds__(kSThreads, 1) k_rows_sched(const GroupParams p, const SchedArgs a) {
    constexpr int P = kSWarpsAll / G;          // warps of a group
    constexpr int TG = P * 32;                 // threads of a group
    constexpr int WIN = kSColsAll<ROWS> / G;   // columns of a window
    constexpr int Q = WIN / 4;                 // 4-column quads of a window
    constexpr int NW = ROWS / 4;               // staging words per column
    constexpr int KS = TG / Q;                 // phase 2: threads per quad (word stride)
    static_assert(TG % Q == 0 && NW % KS == 0 && NW / KS == 4,
                  "phase 2 maps each thread to one quad and four of its count words");
    static_assert(((KS * 1) & 7) + KS <= 8 && ((KS * 2) & 7) + KS <= 8 && ((KS * 3) & 7) + KS <= 8,
                  "phase 2's row offsets from row kk are compile-time constants");
    using RS = typename std::conditional<ROWS == 32, RowSmem, RowSmem64>::type;
    extern __shared__ __align__(16) uint32_t T[];
    __shared__ RS rs;
    // amq[4 w + j]: magnitude of row 32 (w / 8) + w % 8 + 8 j (staging word w, byte j)
    __shared__ __align__(16) float amq[ROWS];
    int nr;
    if constexpr (ROWS == 32) nr = build_table(T, rs, p);   // synchronizes the block
    else nr = build_table64(T, rs, p);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int group = warp / P, wg = warp - group * P, tg = threadIdx.x - group * TG;
    uint32_t* W = T + p.tab_words + (size_t)group * (NW + 1) * WIN;   // [NW][WIN] staged counts of this group
    float* colf = reinterpret_cast<float*>(W + NW * WIN);              // [WIN] column magnitude, -1: IEEE path
    if (threadIdx.x < ROWS) {
        const int r = threadIdx.x;
        amq[4 * (8 * (r >> 5) + (r & 7)) + ((r & 31) >> 3)] = rs.amagf[r];
    }
    for (int i = tg * 4; i < NW * WIN; i += TG * 4) *reinterpret_cast<uint4*>(W + i) = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    const int64_t w0 = a.nwin * blockIdx.y / gridDim.y, w1 = a.nwin * (blockIdx.y + 1) / gridDim.y;
    float* outg = a.out + (int64_t)blockIdx.x * ROWS * a.ldo;
    const uint4* E = reinterpret_cast<const uint4*>(p.entries) + lane;
    const char* Eb = reinterpret_cast<const char*>(p.entries);
    const uint64_t k2p23 = f2(8388608.0f, 8388608.0f);
    const int q4 = (tg % Q) * 4;   // phase 2: columns q4 .. q4 + 3
    const int kk = tg / Q;         // phase 2: staging words kk + KS m, m = 0..3
    // phase 2's straight-line path: a full group whose magnitudes all admit
    // div_small, and rows within 32-bit byte offsets of each other
    const bool full_fast = rs.allfast && nr == ROWS && a.ldo < kFullGroupLdo<ROWS>;
    // A warp streams the runs of its windows (w0 + group, then every G-th)
    // as one sequence: the layout stores them back to back, so the two-step
    // register prefetch and the next item's record run straight across the
    // window boundaries.
    const int64_t wfirst = w0 + group;
    const uint4* ptr = E;
    uint4 qa = make_uint4(0u, 0u, 0u, 0u), qb = qa;
    // item records loaded RA items ahead (two, or one when the rare-pair
    // hash's registers leave no room): rec/lr the current item's, rec_n/lr_n
    // the next's, rec_n2/lr_n2 the one after (RA == 2).  rec is the item's
    // steps and flags (the .y of its record; the kernel needs no chunk).
    constexpr int RA = RARE ? 1 : 2;
    // the two steps of a loop iteration share one carry-save addition of
    // their weight-8 carries (64-row groups of the hash kernel lack the
    // registers)
    constexpr bool PAIRED = !RARE || ROWS == 32;
    int it = 0, left = 0;
    const int* iflags = reinterpret_cast<const int*>(a.items) + 1;   // item i's steps and flags: iflags[2 i]
    int rec = 0, rec_n = 0, rec_n2 = 0;
    int lr = -1, lr_n = -1, lr_n2 = -1;   // this lane's records
    int2 rr = make_int2(0, 0), rr_n = rr;     // its rare entries (split vocabulary)
    uint32_t rv0 = 0u, rv1 = 0u;              // the current item's first two rare entries
    bool phase_b = false;   // the next step is held in qb
    if (wfirst < w1) {
        const int64_t sl = wfirst * P + wg;
        const int64_t g0 = __ldg(a.grun + 2 * sl);
        ptr = E + g0;
        qa = __ldg(ptr);
        qb = __ldg(ptr + 32);
        it = __ldg(a.wrun + sl).x;
        rec = __ldg(iflags + 2 * (int64_t)it);
        lr = __ldg(a.lanes + (int64_t)it * 32 + lane);
        rec_n = __ldg(iflags + 2 * (int64_t)(it + 1));
        lr_n = __ldg(a.lanes + (int64_t)(it + 1) * 32 + lane);
        if constexpr (RA == 2) {
            rec_n2 = __ldg(iflags + 2 * (int64_t)(it + 2));
            lr_n2 = __ldg(a.lanes + (int64_t)(it + 2) * 32 + lane);
        }
        if constexpr (RARE) {
            rr = __ldg(a.rare + (int64_t)it * 32 + lane);
            rr_n = __ldg(a.rare + (int64_t)(it + 1) * 32 + lane);
            rare_prefetch(p, rr, rv0, rv1);
        }
        left = rec & kItemStepsMask;
        if (lane == 0) {   // this window's run and the next one's into L2
            for (int64_t w2 = wfirst; w2 < w1 && w2 <= wfirst + G; w2 += G) {
                const int64_t s2 = w2 * P + wg;
                const int64_t b = __ldg(a.grun + 2 * s2), e = __ldg(a.grun + 2 * s2 + 1);
                prefetch_l2(Eb + b * 16, (uint32_t)((e - b) * 16));
            }
        }
    }
    GroupCounter<ROWS> acc;
    acc.clear();
    for (int64_t wnd = wfirst; wnd < w1; wnd += G) {
        const int64_t wbase = wnd * WIN;
        // ---------------------------------------------------------- phase 1
        if (lane == 0) {   // the stream about two windows ahead into L2 (no record to wait for)
            const int64_t g = ptr - E;   // this step's first group
            const int64_t b = g + (int64_t)kPrefetchFrom * 32, e = min(g + (int64_t)kPrefetchTo * 32, a.ngroups);
            if (e > b) prefetch_l2(Eb + b * 16, (uint32_t)((e - b) * 16));
        }
        // ends the items that are complete; false when the window's items are
        // done (rec and lr then hold the next window's first item)
        auto advance = [&]() -> bool {
            while (left == 0) {
                if constexpr (RARE) acc.add_rare(T, p, rr, rv0, rv1);
                flush_item<WIN, ROWS>(W, colf, rec, lr, acc);
                acc.clear();
                const bool last = (rec & kItemLast) != 0;
                ++it;
                rec = rec_n;
                lr = lr_n;
                left = rec & kItemStepsMask;
                if constexpr (RA == 2) {
                    rec_n = rec_n2;
                    lr_n = lr_n2;
                    rec_n2 = __ldg(iflags + 2 * (int64_t)(it + 2));
                    lr_n2 = __ldg(a.lanes + (int64_t)(it + 2) * 32 + lane);
                } else {
                    rec_n = __ldg(iflags + 2 * (int64_t)(it + 1));
                    lr_n = __ldg(a.lanes + (int64_t)(it + 1) * 32 + lane);
                }
                if constexpr (RARE) {
                    rr = rr_n;
                    rr_n = __ldg(a.rare + (int64_t)(it + 1) * 32 + lane);
                    rare_prefetch(p, rr, rv0, rv1);
                }
                if (last) return false;
            }
            return true;
        };
        if (advance()) {
            for (;;) {
                if constexpr (PAIRED) {
                    // ea: the qa step's weight-8 carries while they wait for
                    // the qb step's (zero when qa ended an item or was not run)
                    uint32_t ea[ROWS / 32];
#pragma unroll
                    for (int h = 0; h < ROWS / 32; h++) ea[h] = 0u;
                    if (!phase_b) {   // step held in qa; its register takes the step two ahead
                        uint32_t ix[8];
                        step_vids(qa, ix);
                        qa = __ldg(ptr + 64);
                        acc.step_open(T, ix, ea);
                        --left;
                        if (left == 0) {   // the item ends: its counts complete before the flush
                            acc.close1(ea);
#pragma unroll
                            for (int h = 0; h < ROWS / 32; h++) ea[h] = 0u;
                            if (!advance()) {
                                phase_b = true;
                                break;
                            }
                        }
                    }
                    {   // step held in qb
                        uint32_t ix[8], eb[ROWS / 32];
                        step_vids(qb, ix);
                        qb = __ldg(ptr + 96);
                        acc.step_open(T, ix, eb);
                        acc.close2(ea, eb);
                    }
                } else {
                    if (!phase_b) {   // step held in qa; its register takes the step two ahead
                        uint32_t ix[8], e[ROWS / 32];
                        step_vids(qa, ix);
                        qa = __ldg(ptr + 64);
                        acc.step_open(T, ix, e);
                        acc.close1(e);
                        --left;
                        if (!advance()) {
                            phase_b = true;
                            break;
                        }
                    }
                    {   // step held in qb
                        uint32_t ix[8], e[ROWS / 32];
                        step_vids(qb, ix);
                        qb = __ldg(ptr + 96);
                        acc.step_open(T, ix, e);
                        acc.close1(e);
                    }
                }
                ptr += 64;
                phase_b = false;
                --left;
                if (!advance()) break;
            }
        }
        // every item of the window has been flushed, so the counter is zero
        // here; saying so frees its registers for phase 2
        acc.clear();
        group_barrier(group, TG);
        // ---------------------------------------------------------- phase 2
        const int64_t left_cols = a.nq - wbase;
        const int ncols = left_cols < WIN ? (int)left_cols : WIN;
        const float4 cf = q4 < ncols ? *reinterpret_cast<const float4*>(colf + q4)
                                     : make_float4(-1.0f, -1.0f, -1.0f, -1.0f);
        if (full_fast && q4 + 4 <= ncols && cf.x >= 0.0f && cf.y >= 0.0f && cf.z >= 0.0f && cf.w >= 0.0f) {
            // a full group, a whole quad of columns, every pair exact with
            // div_small: straight-line code, rows addressed by 32-bit byte
            // offsets from row kk
            char* ob = reinterpret_cast<char*>(outg + wbase + q4 + (int64_t)kk * a.ldo);
            const uint32_t row_bytes = (uint32_t)a.ldo * 4u;
            const float bcol[4] = {cf.x, cf.y, cf.z, cf.w};
#pragma unroll
            for (int kq = 0; kq < 4; kq++) {
                const int k = kk + KS * kq;   // staging word: rows 32 (k / 8) + k % 8 + 8 j
                uint32_t* wp = W + k * WIN + q4;
                const uint4 c = *reinterpret_cast<const uint4*>(wp);
                *reinterpret_cast<uint4*>(wp) = make_uint4(0u, 0u, 0u, 0u);
                const float4 a4 = *reinterpret_cast<const float4*>(amq + 4 * k);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
                const uint32_t cw[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const uint32_t sel = 0x7440u | (uint32_t)j;   // 0x4B0000cc: the float 2^23 + count
                    float t[4];
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) {
                        const float isf = __fsub_rn(__uint_as_float(__byte_perm(cw[cc], 0x4B000000u, sel)), 8388608.0f);
                        const float u = __fsub_rn(__fadd_rn(av[j], bcol[cc]), isf);
                        t[cc] = div_small(isf, u);
                    }
                    // row 32 (k / 8) + k % 8 + 8 j, relative to row kk: kk < KS and
                    // (KS kq) % 8 + KS <= 8, so k / 8 = (KS kq) / 8 and k % 8 = kk + (KS kq) % 8
                    const int rel = 32 * ((KS * kq) >> 3) + ((KS * kq) & 7) + 8 * j;
                    *reinterpret_cast<float4*>(ob + (uint32_t)rel * row_bytes) = make_float4(t[0], t[1], t[2], t[3]);
                }
            }
        } else if (q4 < ncols) {
            const bool fast = rs.allfast && q4 + 4 <= ncols && cf.x >= 0.0f && cf.y >= 0.0f && cf.z >= 0.0f &&
                              cf.w >= 0.0f;
            const uint64_t B01 = f2(cf.x, cf.y), B23 = f2(cf.z, cf.w);
            float* ob = outg + wbase + q4;
#pragma unroll
            for (int kq = 0; kq < 4; kq++) {
                const int k = kk + KS * kq;
                uint32_t* wp = W + k * WIN + q4;
                const uint4 c = *reinterpret_cast<const uint4*>(wp);
                *reinterpret_cast<uint4*>(wp) = make_uint4(0u, 0u, 0u, 0u);
                const float4 a4 = *reinterpret_cast<const float4*>(amq + 4 * k);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = 32 * (k >> 3) + (k & 7) + 8 * j;
                    if (r >= nr) break;
                    float* orow = ob + (int64_t)r * a.ldo;
                    const uint32_t sel = 0x7440u | (uint32_t)j;
                    if (fast) {
                        const uint64_t I01 = sub2(f2(__uint_as_float(__byte_perm(c.x, 0x4B000000u, sel)),
                                                     __uint_as_float(__byte_perm(c.y, 0x4B000000u, sel))), k2p23);
                        const uint64_t I23 = sub2(f2(__uint_as_float(__byte_perm(c.z, 0x4B000000u, sel)),
                                                     __uint_as_float(__byte_perm(c.w, 0x4B000000u, sel))), k2p23);
                        const uint64_t A = f2(av[j], av[j]);
                        const uint64_t Q01 = tanimoto2(I01, add2(A, B01));
                        const uint64_t Q23 = tanimoto2(I23, add2(A, B23));
                        float t0, t1, t2, t3;
                        unf2(Q01, t0, t1);
                        unf2(Q23, t2, t3);
                        *reinterpret_cast<float4*>(orow) = make_float4(t0, t1, t2, t3);
                    } else {
                        const uint32_t cw[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
                        for (int cc = 0; cc < 4; cc++) {
                            if (q4 + cc < ncols) {
                                const int is = (int)((cw[cc] >> (8 * j)) & 0xFFu);
                                orow[cc] = tanimoto_rows(is, rs.amag[r], __ldg(a.qmag + wbase + q4 + cc));
                            }
                        }
                    }
                }
            }
        }
        group_barrier(group, TG);
    }
}

// Permutes 16-byte entry groups into schedule order: new step t (32 groups,
// one per lane) is old step map[t].
__global__ void k_sched_gather(const uint4* __restrict__ src, const int64_t* __restrict__ map, int64_t nsteps,
                               uint4* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsteps * 32) return;
    dst[i] = src[__ldg(map + (i >> 5)) * 32 + (i & 31)];
}

// Per item and lane the record phase 1 needs, in one word: the molecule's
// position in its window << 16 | the column magnitude phase 2 divides by
// (fast magnitudes are 1..32768; 0 when the pair takes the IEEE division),
// or -1 for a padding slot.
static_assert(kMaxWindow <= 32768, "a window position takes the upper 16 bits of a lane record");
__global__ void k_sched_lanes(const int2* __restrict__ items, int64_t nitems, const int4* __restrict__ meta,
                              int64_t per_win, int window, int* __restrict__ lanes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (nitems + 2) * 32) return;
    const int64_t item = i >> 5;
    if (item >= nitems || (items[item].y & kItemEmpty)) {   // padding records and placeholders: no lanes
        lanes[i] = -1;
        return;
    }
    const int64_t chunk = items[item].x;
    const int4 m = meta[chunk * 32 + (i & 31)];
    const int64_t wbase = chunk / per_win * window;
    const uint32_t mag = fast_mag(m.y, m.z) ? (uint32_t)m.y : 0u;
    lanes[i] = m.x >= 0 ? (int)(((uint32_t)(m.x - wbase) << 16) | mag) : -1;
}

// Per item and lane the molecule's rare entries {first, count} in the
// layout's rare list, given to the item that holds the chunk's first step
// (the others count none, so each molecule's rare entries are added once).
__global__ void k_sched_rare(const int2* __restrict__ items, int64_t nitems, const int4* __restrict__ meta,
                             const int64_t* __restrict__ rare_off, int2* __restrict__ rare) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (nitems + 2) * 32) return;
    const int64_t item = i >> 5;
    if (item >= nitems) {   // the padding records' lanes
        rare[i] = make_int2(0, 0);
        return;
    }
    const int2 it = items[item];
    const int64_t slot = (int64_t)it.x * 32 + (i & 31);
    const bool first = (it.y & kItemFirst) && !(it.y & kItemEmpty) && meta[slot].x >= 0;
    const int64_t b = rare_off[slot], e = rare_off[slot + 1];
    rare[i] = first ? make_int2((int)b, (int)(e - b)) : make_int2(0, 0);
}

// Inverted lists of the rare vids (split vocabulary): pass 0 counts each
// vid's molecules, pass 1 places them (cursor starts at the list offsets).
__global__ void k_post_build(const int4* __restrict__ meta, int64_t slots, const int64_t* __restrict__ rare_off,
                             const uint32_t* __restrict__ rare_vid, int64_t ncommon, int pass,
                             unsigned long long* __restrict__ cnt, int32_t* __restrict__ post_mol) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= slots) return;
    const int32_t m = meta[s].x;
    if (m < 0) return;
    for (int64_t i = rare_off[s]; i < rare_off[s + 1]; i++) {
        const int64_t k = (int64_t)rare_vid[i] - ncommon - 1;
        if (pass == 0) atomicAdd(cnt + k, 1ull);
        else post_mol[atomicAdd(cnt + k, 1ull)] = m;
    }
}

// Sorted-list merge intersection of two compiled molecules
// (pysiml/_CPULingo.c:53-71).
__device__ __forceinline__ int merge_count(const int32_t* a, const int32_t* as, int32_t alen, const int32_t* b,
                                           const int32_t* bs, int32_t blen) {
    int32_t i = 0, j = 0, isct = 0;
    while (i < alen && j < blen) {
        const int32_t x = a[i], y = b[j];
        if (x == y) { isct += min(as[i], bs[j]); i++; j++; }
        else if (x < y) i++;
        else j++;
    }
    return isct;
}

struct FixArgs {
    const uint32_t* row_vid;
    int64_t row_stride;
    int64_t ncommon;
    const int64_t* post_off;
    const int32_t* post_mol;
    const int32_t *rl, *rc, *rlen, *rmag;   // ref set
    int64_t rw;
    const int32_t *ql, *qc, *qlen, *qmag;   // query set
    int64_t qw;
    int64_t rowbase;
    float* out;
    int64_t ldo;
    int* err;   // asynchronous error word (a row whose pairs overfill the hash: not possible within the
                // launch's bound, reported rather than dropped)
    int slots_log2;   // the per-row hash: 2^slots_log2 slots of dynamic shared memory (key, count)
};

// Fix-up pass limits: a row's rare vids and the (row, molecule) pairs they
// touch, counted in a per-row shared-memory hash at most 3/4 full, sized per
// launch (a power of two up to kFixMaxSlots).
constexpr int kFixMaxSlotsLog2 = 13;
constexpr int kFixMaxSlots = 1 << kFixMaxSlotsLog2;
constexpr int kFixMaxVids = 256;

// The common-entry intersection of a pair from the fp32 Tanimoto the table
// pass wrote (t = isct / (amag + bmag - isct), increasing in isct): the
// estimate t S / (1 + t) and its neighbours, each checked by recomputing the
// reference's quotient bit for bit; -1 when none matches or when magnitudes
// this large could make two counts round to the same quotient.
__device__ __forceinline__ int recover_isct(float t, int amag, int bmag) {
    if (amag == 0 || bmag == 0) return 0;   // t is 0 whatever the count
    const float S = (float)amag + (float)bmag;
    if (!(S <= 1048576.0f)) return -1;
    const int c = __float2int_rn(t * S / (1.0f + t));
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int cand = c + (d == 0 ? 0 : (d == 1 ? -1 : 1));
        if (cand >= 0 && __float_as_uint(tanimoto_rows(cand, amag, bmag)) == __float_as_uint(t)) return cand;
    }
    return -1;
}

// The pairs of a full-matrix block that share a rare vid (one CTA per row).
// The table pass counted their common entries only.  Each molecule's shared
// rare vids are counted in shared memory from the rare vids' molecule lists;
// its common count comes back from the quotient already written, and the
// quotient is written again for the full count (the reference's merge when
// the count cannot be recovered).
__global__ void __launch_bounds__(256) k_rare_fix(const FixArgs f) {
    extern __shared__ int32_t fix_hash[];
    const int nslots = 1 << f.slots_log2;
    int32_t* key = fix_hash;            // molecule + 1, 0: empty
    int32_t* add = fix_hash + nslots;   // shared rare vids
    __shared__ uint32_t rv_s[kFixMaxVids];
    __shared__ int nrv;
    const int tid = threadIdx.x;
    const int64_t r = f.rowbase + blockIdx.x;
    for (int i = tid; i < nslots; i += blockDim.x) {
        key[i] = 0;
        add[i] = 0;
    }
    if (tid == 0) nrv = 0;
    __syncthreads();
    const uint32_t* rv = f.row_vid + r * f.row_stride;
    for (int64_t e = tid; e < f.row_stride; e += blockDim.x) {
        const uint32_t v = rv[e];
        if ((int64_t)v > f.ncommon) {
            const int k = atomicAdd(&nrv, 1);
            if (k < kFixMaxVids) rv_s[k] = v;
        }
    }
    __syncthreads();
    // the launch admits rows of at most kFixMaxVids rare vids; more is
    // reported, not dropped unseen
    if (nrv > kFixMaxVids && tid == 0 && f.err) atomicOr(f.err, kErrBadRowVid);
    const int n = min(nrv, kFixMaxVids);
    for (int j = 0; j < n; j++) {
        const int64_t k = (int64_t)rv_s[j] - f.ncommon - 1;
        const int64_t b = f.post_off[k], en = f.post_off[k + 1];
        for (int64_t i = b + tid; i < en; i += blockDim.x) {
            const int32_t m = f.post_mol[i];
            uint32_t h = ((uint32_t)m * 0x9E3779B1u) >> (32 - f.slots_log2);
            int probe = 0;
            for (; probe < nslots; probe++) {   // at most 3/4 full: ends
                const int32_t prev = atomicCAS(&key[h], 0, m + 1);
                if (prev == 0 || prev == m + 1) {
                    atomicAdd(&add[h], 1);
                    break;
                }
                h = (h + 1) & (nslots - 1);
            }
            if (probe == nslots && f.err) atomicOr(f.err, kErrBadRowVid);
        }
    }
    __syncthreads();
    const int32_t alen = f.rlen[r], amag = f.rmag[r];
    float* orow = f.out + (int64_t)blockIdx.x * f.ldo;
    for (int s = tid; s < nslots; s += blockDim.x) {
        const int32_t km = key[s];
        if (km == 0) continue;
        const int32_t m = km - 1, bmag = f.qmag[m];
        const int i0 = recover_isct(orow[m], amag, bmag);
        const int is = i0 >= 0 ? i0 + add[s]
                               : merge_count(f.rl + r * f.rw, f.rc + r * f.rw, alen, f.ql + (int64_t)m * f.qw,
                                             f.qc + (int64_t)m * f.qw, f.qlen[m]);
        orow[m] = tanimoto_rows(is, amag, bmag);
    }
}

struct SchedItem {
    int64_t chunk;
    int s0, ns;
    bool split;
};

}  // namespace

namespace {

// Shared memory beside the table: the staging and column magnitudes, the
// rare-pair hash (when a split needs it), the row data and amq, with a margin
// for static shared memory.
int64_t sched_extra_smem(int rows, bool hash) {
    if (rows == 64)
        return (int64_t)kSchedExtraSmem<64> + (hash ? (int64_t)kRare64Slots * 12 : 0) + (int64_t)sizeof(RowSmem64) +
               64 * 4 + 2048;
    return (int64_t)kSchedExtraSmem<32> + (hash ? (int64_t)kRareSlots * 8 : 0) + (int64_t)sizeof(RowSmem) + 32 * 4 +
           2048;
}

// Table words of ncommon common vids: one per vid (32 rows) or two (64 rows),
// vids 0..ncommon, rounded up to 16 bytes.
int64_t sched_table_words(int rows, int64_t ncommon) {
    return rows == 64 ? (ncommon + 1 + 1) / 2 * 4 : (ncommon + 1 + 3) / 4 * 4;
}

}  // namespace

int64_t sched_capacity(siml_engine* h) {
    if (sched_whole_fits(h, h->vocab.nvid)) return h->vocab.nvid;
    // a vocabulary in slot order makes no useful split: the kernel takes it
    // whole or not at all; one numbered by frequency lends any prefix
    if (!h->vocab.freq_ordered) return 0;
    const int rows = h->sched_rows;
    const int64_t words = ((int64_t)h->smem_optin - sched_extra_smem(rows, true)) / 4;
    int64_t cap = rows == 64 ? words / 4 * 2 - 2 : words / 4 * 4 - 4;   // sched_table_words(cap) <= words
    return std::max<int64_t>(0, std::min<int64_t>(cap, h->vocab.nvid));
}

bool sched_whole_fits(siml_engine* h, int64_t nvid) {
    const int rows = h->sched_rows;
    return sched_table_words(rows, nvid) * 4 + sched_extra_smem(rows, false) <= (int64_t)h->smem_optin;
}

bool rows_sched_fits(siml_engine* h) {
    const int np = planes_needed(std::min(h->ref.max_entries, h->qry.max_entries));
    if (np > 8) return false;   // staged counts are bytes
    const int64_t nc = std::min<int64_t>(h->vocab.ncommon, sched_capacity(h));
    if (nc <= 0) return false;
    if (nc < h->vocab.nvid && nc < 1024) return false;   // a split that leaves too little in the table
    return true;
}

void free_sched(DbLayout& d) {
    if (d.sched_items) cudaFree(d.sched_items);
    if (d.sched_wrun) cudaFree(d.sched_wrun);
    if (d.sched_grun) cudaFree(d.sched_grun);
    if (d.sched_lanes) cudaFree(d.sched_lanes);
    if (d.sched_rare) cudaFree(d.sched_rare);
    if (d.post_off) cudaFree(d.post_off);
    if (d.post_mol) cudaFree(d.post_mol);
    d.sched_lanes = nullptr;
    d.sched_rare = nullptr;
    d.post_off = nullptr;
    d.post_mol = nullptr;
    d.post_max = 0;
    d.sched_items = nullptr;
    d.sched_wrun = nullptr;
    d.sched_grun = nullptr;
}

namespace {

// Wrap-around fill of one window's chunks (steps L[0..n), ascending; the
// longest first) into P warps of capacity M, an item costing its steps plus
// icost: a chunk goes whole into the current warp while it fits, else
// the warp is filled to M and the rest continues in the next warp.  Returns
// false when P warps do not suffice.
bool fill_window(const int32_t* L, int n, int P, double M, std::vector<SchedItem>* pw, int64_t c0, double icost) {
    for (int w = 0; w < P; w++) pw[w].clear();
    std::vector<double> load((size_t)P, 0.0);
    int w = 0;
    for (int c = n - 1; c >= 0; c--) {
        int rem = L[c], s0 = 0;
        if (rem == 0) {   // molecules with no streamed entries: counts 0, column data still written
            if (load[(size_t)w] + icost > M && w < P - 1) w++;
            load[(size_t)w] += icost;
            pw[w].push_back({c0 + c, 0, 0, false});
            continue;
        }
        while (rem > 0) {
            const int cap = (int)std::floor(M - load[(size_t)w] - icost);
            if (cap <= 0) {
                if (w == P - 1) return false;
                w++;
                continue;
            }
            const int take = rem <= cap ? rem : cap;
            pw[w].push_back({c0 + c, s0, take, false});
            load[(size_t)w] += take + icost;
            s0 += take;
            rem -= take;
            if (load[(size_t)w] >= M - 0.5 && rem > 0) {
                if (w == P - 1) return false;
                w++;
            }
        }
    }
    return true;
}

}  // namespace

// The molecules of each rare vid of a split layout (d.post_off, d.post_mol,
// d.post_max): counted on the device, offsets on the host, placed on the
// device.
static int build_postings(siml_engine* h, DbLayout& d) {
    cudaStream_t st = h->stream;
    const int64_t nrv = h->vocab.nvid - d.ncommon, slots = d.nchunks * 32;
    std::vector<unsigned long long> hc((size_t)nrv + 1, 0ull);
    std::vector<int64_t> ho((size_t)nrv + 1, 0);
    int rc;
    void* cnt = nullptr;
    if ((rc = dev_alloc_bytes(&cnt, hc.size() * 8))) return rc;
    cudaError_t e = cudaMemsetAsync(cnt, 0, hc.size() * 8, st);
    if (e == cudaSuccess && slots > 0) {
        k_post_build<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(d.meta, slots, d.rare_off, d.rare_vid,
                                                                      d.ncommon, 0, (unsigned long long*)cnt, nullptr);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cnt, hc.size() * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int64_t total = 0, longest = 0;
    for (int64_t i = 0; i < nrv; i++) {
        ho[(size_t)i] = total;
        longest = std::max<int64_t>(longest, (int64_t)hc[(size_t)i]);
        total += (int64_t)hc[(size_t)i];
        hc[(size_t)i] = (unsigned long long)ho[(size_t)i];   // cursor of the placing pass
    }
    ho[(size_t)nrv] = total;
    void* off = nullptr;
    void* mol = nullptr;
    if (e == cudaSuccess) {
        if ((rc = dev_alloc_bytes(&off, ho.size() * 8)) ||
            (rc = dev_alloc_bytes(&mol, (size_t)std::max<int64_t>(total, 1) * 4))) {
            if (off) cudaFree(off);
            cudaFree(cnt);
            return rc;
        }
        e = cudaMemcpyAsync(off, ho.data(), ho.size() * 8, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt, hc.data(), hc.size() * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && slots > 0) {
        k_post_build<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(d.meta, slots, d.rare_off, d.rare_vid,
                                                                      d.ncommon, 1, (unsigned long long*)cnt,
                                                                      (int32_t*)mol);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(cnt);
    if (e != cudaSuccess) {
        if (off) cudaFree(off);
        if (mol) cudaFree(mol);
        return cuda_fail(e, "scheduled layout: rare-vid lists");
    }
    d.post_off = (int64_t*)off;
    d.post_mol = (int32_t*)mol;
    d.post_max = longest;
    return SIML_OK;
}

// Builds the per-(window, warp) schedule of a freshly built window-sorted
// layout (windows of d.window, 2-byte entries, chunk c's step s of lane l at
// group off[c] + 32 s + l) for groups of P warps, and permutes its entries
// into schedule order.
int sched_arrange(siml_engine* h, DbLayout& d) {
    cudaStream_t st = h->stream;
    const int P = d.sched_warps;
    const int cols = d.sched_rows == 64 ? kSColsAll<64> : kSColsAll<32>;
    if (d.entry_bytes != 2 || P < 1 || P > kSWarpsAll || d.window != (cols * P) / kSWarpsAll)
        return fail(SIML_ERR_UNSUPPORTED, "scheduled layout: bad base layout");
    const int64_t nch = d.nchunks;
    std::vector<int32_t> ng((size_t)std::max<int64_t>(nch, 1));
    std::vector<int64_t> off((size_t)nch + 1);
    if (nch > 0) {
        SIML_CUDA(cudaMemcpyAsync(ng.data(), d.ng, (size_t)nch * 4, cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaMemcpyAsync(off.data(), d.off, (size_t)(nch + 1) * 8, cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaStreamSynchronize(st));
    }
    const int64_t per_win = d.window / kChunk;
    const int64_t nwin = (d.n + d.window - 1) / d.window;
    const int G = kSWarpsAll / P;
    const double icost = item_cost(d.sched_rows);
    // each (window, warp) run is scheduled first, then the runs are stored in
    // stream order: a warp of group g takes windows g, g + G, g + 2G, ...,
    // so its runs of consecutive such windows are stored back to back
    std::vector<std::vector<SchedItem>> runs((size_t)nwin * P);
    std::vector<std::vector<SchedItem>> pw((size_t)P);
    int64_t max_steps = 0;
    for (int64_t wnd = 0; wnd < nwin; wnd++) {
        const int64_t c0 = wnd * per_win, c1 = std::min<int64_t>(nch, c0 + per_win);
        int n = 0;   // chunks with molecules (padding slots sort last)
        double cost = 0.0;
        int32_t longest = 0;
        for (int64_t c = c0; c < c1 && c * kChunk < d.n; c++, n++) {
            cost += ng[(size_t)c] + icost;
            longest = std::max(longest, ng[(size_t)c]);
        }
        // the smallest share that the fill fits into P warps (bisection)
        double lo = std::max(1.0, cost / P), hi = 2.0 * cost / P + longest + 4.0 * icost + 1.0;
        while (!fill_window(ng.data() + c0, n, P, hi, pw.data(), c0, icost)) hi *= 2.0;
        for (int iter = 0; iter < 24 && hi - lo > 0.25; iter++) {
            const double mid = 0.5 * (lo + hi);
            if (fill_window(ng.data() + c0, n, P, mid, pw.data(), c0, icost)) hi = mid;
            else lo = mid;
        }
        fill_window(ng.data() + c0, n, P, hi, pw.data(), c0, icost);
        // chunks with more than one item add their counts atomically
        std::vector<int> parts((size_t)per_win, 0);
        for (auto& v : pw)
            for (auto& x : v) parts[(size_t)(x.chunk - c0)]++;
        for (int ww = 0; ww < P; ww++) {
            auto& r = runs[(size_t)(wnd * P + ww)];
            r = pw[(size_t)ww];
            for (auto& x : r) {
                x.split = parts[(size_t)(x.chunk - c0)] > 1;
                max_steps = std::max<int64_t>(max_steps, x.ns);
            }
        }
    }
    std::vector<int2> items;
    items.reserve((size_t)nch * 2 + 64);
    std::vector<int2> wrun((size_t)std::max<int64_t>(nwin * P, 1));
    std::vector<int64_t> grun((size_t)std::max<int64_t>(nwin * P, 1) * 2);
    std::vector<int64_t> map;
    map.reserve((size_t)(d.ngroups_total / 32) + 1);
    int64_t gpos = 0;
    for (int g = 0; g < G; g++)
        for (int ww = 0; ww < P; ww++)
            for (int64_t wnd = g; wnd < nwin; wnd += G) {
                const size_t sl = (size_t)(wnd * P + ww);
                wrun[sl].x = (int)items.size();
                grun[2 * sl] = gpos;
                for (auto& x : runs[sl]) {
                    int flags = x.ns;
                    if (x.split) flags |= kItemSplit;
                    if (x.s0 == 0) flags |= kItemFirst;
                    items.push_back(make_int2((int)x.chunk, flags));
                    for (int s2 = 0; s2 < x.ns; s2++) map.push_back(off[(size_t)x.chunk] / 32 + x.s0 + s2);
                    gpos += (int64_t)x.ns * 32;
                }
                // the kernel ends a window's run at its flagged last item;
                // a run with no items gets a placeholder to carry the flag
                if (runs[sl].empty()) items.push_back(make_int2((int)(wnd * per_win), kItemEmpty));
                items.back().y |= kItemLast;
                wrun[sl].y = (int)items.size();
                grun[2 * sl + 1] = gpos;
            }
    // padding records: the stream reads up to two records ahead
    items.push_back(make_int2(0, 0));
    items.push_back(make_int2(0, 0));
    if (gpos != d.ngroups_total) return fail(SIML_ERR_CUDA, "scheduled layout: %lld groups scheduled of %lld",
                                             (long long)gpos, (long long)d.ngroups_total);
    if (items.size() > 0x7FFFFFFFu) return fail(SIML_ERR_UNSUPPORTED, "scheduled layout: too many items");
    int rc;
    void* p = nullptr;
    if ((rc = dev_alloc_bytes(&p, items.size() * sizeof(int2)))) return rc;
    d.sched_items = (int2*)p;
    if ((rc = dev_alloc_bytes(&p, wrun.size() * sizeof(int2)))) return rc;
    d.sched_wrun = (int2*)p;
    if ((rc = dev_alloc_bytes(&p, grun.size() * sizeof(int64_t)))) return rc;
    d.sched_grun = (int64_t*)p;
    SIML_CUDA(cudaMemcpyAsync(d.sched_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    if ((rc = dev_alloc_bytes(&p, items.size() * 32 * sizeof(int)))) return rc;
    d.sched_lanes = (int*)p;
    {
        const int64_t n = (int64_t)items.size() * 32;
        k_sched_lanes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d.sched_items, (int64_t)items.size() - 2, d.meta,
                                                                   per_win, d.window, d.sched_lanes);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
    }
    if (d.rare_off) {   // split vocabulary: each lane's rare entries, loaded ahead by the kernel
        if (d.nrare > 0x7FFFFFFF) return fail(SIML_ERR_UNSUPPORTED, "scheduled layout: too many rare entries");
        if ((rc = dev_alloc_bytes(&p, items.size() * 32 * sizeof(int2)))) return rc;
        d.sched_rare = (int2*)p;
        const int64_t n = (int64_t)items.size() * 32;
        k_sched_rare<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d.sched_items, (int64_t)items.size() - 2, d.meta,
                                                                  d.rare_off, d.sched_rare);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        if ((rc = build_postings(h, d))) return rc;
    }
    SIML_CUDA(cudaMemcpyAsync(d.sched_wrun, wrun.data(), wrun.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    SIML_CUDA(cudaMemcpyAsync(d.sched_grun, grun.data(), grun.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    d.nitems = (int64_t)items.size() - 2;
    d.nwin = nwin;
    d.max_item_steps = max_steps;
    // entries in schedule order, with kPadSteps steps of zeros after them
    // (the stream loads run two steps ahead without bounds tests)
    const int64_t nsteps = (int64_t)map.size();
    void* dmap = nullptr;
    void* dst = nullptr;
    const size_t dst_bytes = (size_t)(nsteps + kPadSteps) * 32 * 16;
    if ((rc = dev_alloc_bytes(&dst, dst_bytes))) return rc;
    cudaError_t e = cudaMemsetAsync((char*)dst + (size_t)nsteps * 512, 0, (size_t)kPadSteps * 512, st);
    if (e == cudaSuccess && nsteps > 0) {
        if ((rc = dev_alloc_bytes(&dmap, (size_t)nsteps * 8))) {
            cudaFree(dst);
            return rc;
        }
        e = cudaMemcpyAsync(dmap, map.data(), (size_t)nsteps * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            const int64_t n = nsteps * 32;
            k_sched_gather<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const uint4*)d.entries, (const int64_t*)dmap,
                                                                       nsteps, (uint4*)dst);
            h->launches++;
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (dmap) cudaFree(dmap);
    if (e != cudaSuccess) {
        cudaFree(dst);
        return cuda_fail(e, "scheduled layout: entry permutation");
    }
    cudaFree(d.entries);
    d.entries = dst;
    return SIML_OK;
}

int launch_rows_sched(siml_engine* h, const RowsArgs& a, bool* done) {
    *done = false;
    if (a.mode != kModeRows || !rows_use_sched(h)) return SIML_OK;
    if (((uintptr_t)a.out & 15u) || (a.ldo & 3)) return SIML_OK;   // 16-byte row stores
    const DbLayout* d = nullptr;
    int rc = ensure_sched_layout(h, &d);
    if (rc) return rc;
    const int64_t rows = a.rowlimit - a.rowbase;
    GroupParams p;
    size_t smem = 0;
    int np = 0;
    if (!table_params(h, d, a.rowbase, rows, kModeRows, p, smem, np) || np != 8 || d->entry_bytes != 2) return SIML_OK;
    const int R = d->sched_rows;
    const bool split = d->ncommon < h->vocab.nvid;
    // Split vocabulary: when the pairs that share a rare vid are few (at most
    // 3/4 of kFixMaxSlots per row, bounded by the row with the most rare
    // entries and the longest molecule list), the table pass skips rare vids
    // and a second pass adds them to those pairs; otherwise the rare vids go
    // through the group's hash inside the table pass.
    const int64_t fix_pairs = h->rows.max_rare_sched * d->post_max;   // bound on one row's pairs
    const bool fixup = split && h->rare_fixup && d->post_off != nullptr &&
                       h->rows.max_rare_sched <= kFixMaxVids && fix_pairs * 4 <= (int64_t)kFixMaxSlots * 3;
    const bool hash = split && !fixup;
    if (R == 64) {
        // the 64-row table: two words per vid, then the 64-bit-mask hash
        if (hash && h->rows.max_rare_sched > kRare64RowMax) return SIML_OK;
        p.vt_words = (int)sched_table_words(64, d->ncommon);
        p.rare_slots = hash ? kRare64Slots : 0;
        p.tab_words = p.vt_words + (hash ? 3 * kRare64Slots : 0);
        smem = (size_t)p.tab_words * 4;
    } else if (fixup) {
        p.rare_slots = 0;
        p.tab_words = p.vt_words;
        smem = (size_t)p.tab_words * 4;
    }
    p.rare_fixup = fixup ? 1 : 0;
    const size_t sm = smem + (R == 64 ? kSchedExtraSmem<64> : kSchedExtraSmem<32>);
    if ((int64_t)smem + sched_extra_smem(R, false) > (int64_t)h->smem_optin) return SIML_OK;
    void (*kern)(const GroupParams, const SchedArgs) = nullptr;
    switch ((kSWarpsAll / d->sched_warps) * 100 + R) {
        case 232: kern = hash ? k_rows_sched<true, 2, 32> : k_rows_sched<false, 2, 32>; break;
        case 432: kern = hash ? k_rows_sched<true, 4, 32> : k_rows_sched<false, 4, 32>; break;
        case 264: kern = hash ? k_rows_sched<true, 2, 64> : k_rows_sched<false, 2, 64>; break;
        case 464: kern = hash ? k_rows_sched<true, 4, 64> : k_rows_sched<false, 4, 64>; break;
        default: return SIML_OK;
    }
    if ((rc = set_smem(kern, sm))) return rc;
    SchedArgs sa;
    sa.items = d->sched_items;
    sa.lanes = d->sched_lanes;
    sa.rare = d->sched_rare;
    if (hash && !sa.rare) return SIML_OK;
    sa.wrun = d->sched_wrun;
    sa.grun = d->sched_grun;
    sa.qmag = h->qry.mag;
    sa.nq = h->qry.n;
    sa.nwin = d->nwin;
    sa.out = a.out;
    sa.ldo = a.ldo;
    sa.ngroups = d->ngroups_total + (int64_t)kPadSteps * 32;
    const int64_t groups = (rows + R - 1) / R;
    // windows per CTA: groups x splits fills whole waves of one CTA per SM
    int splits = 1;
    double best = 1e300;
    for (int64_t s = 1; s <= std::max<int64_t>(1, std::min<int64_t>(d->nwin, 1024)); s++) {
        const int64_t waves = (groups * s + h->num_sms - 1) / h->num_sms;
        const double cost = (double)waves * (1.0 / (double)s + 0.004);
        if (cost < best * 0.999) {
            best = cost;
            splits = (int)s;
        }
    }
    dim3 grid((unsigned)groups, (unsigned)splits);
    SIML_CUDA(mark(h, h->ev0));
    kern<<<grid, kSThreads, sm, h->stream>>>(p, sa);
    SIML_CUDA(cudaGetLastError());
    if (fixup && rows > 0) {
        const RawSet &rs = h->ref, &qs = h->qry;
        FixArgs f{h->rows.vid, h->rows.stride, d->ncommon, d->post_off, d->post_mol,
                  rs.lingos, rs.counts, rs.len, rs.mag, rs.width,
                  qs.lingos, qs.counts, qs.len, qs.mag, qs.width,
                  a.rowbase, a.out, a.ldo, h->d_async_err, 10};
        while (f.slots_log2 < kFixMaxSlotsLog2 && (int64_t)(1 << f.slots_log2) * 3 < fix_pairs * 4) f.slots_log2++;
        const size_t fsm = (size_t)2 * 4 << f.slots_log2;
        if ((rc = set_smem(k_rare_fix, fsm))) return rc;
        k_rare_fix<<<(unsigned)rows, 256, fsm, h->stream>>>(f);
        SIML_CUDA(cudaGetLastError());
        h->launches++;
    }
    SIML_CUDA(mark(h, h->ev1));
    h->timed = true;
    h->launches++;
    h->rows_rare_path = fixup ? 2 : hash ? 1 : 0;
    h->rows_rare_gen = h->generation;
    *done = true;
    return SIML_OK;
}

}  // namespace siml
