// Engine state shared by the host orchestration (engine.cu) and the kernels
// (kernels.cu).  Everything here is internal; the public surface is
// include/siml_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "siml_internal.h"

namespace siml {

// A SMILES set as uploaded: row-major [n, width] codes and counts, lengths,
// effective magnitudes (user-given or the count sums) and count sums.
struct RawSet {
    int64_t n = -1;
    int64_t width = 0;
    int32_t* lingos = nullptr;
    int32_t* counts = nullptr;
    int32_t* len = nullptr;
    int32_t* mag = nullptr;
    int32_t* cmag = nullptr;
    int64_t max_entries = 0;   // max over molecules of the count sum
    int64_t total_entries = 0; // sum of count sums
};

// Open-addressing hash of the database's (code, level) pairs.  key =
// (level << 32) | (uint32)code, empty slots hold kEmptyKey; vid[slot] is the
// dense virtual id (1..nvid) of an occupied slot.
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;
//
// When the table of all vids does not fit in shared memory the vocabulary
// is split: vids are renumbered by falling database frequency, vids
// 1..ncommon are "common" and keep the direct shared-memory table, and the
// rest are "rare": a database molecule's rare entries are kept in a separate
// list per molecule and looked up in a small per-row-group hash of the rows'
// rare vids.  Without a split ncommon == nvid.
constexpr int kRareSlotsLog2 = 12;
constexpr int kRareSlots = 1 << kRareSlotsLog2;   // per-group hash of the rows' rare vids
constexpr int kRareRowMax = 96;                    // 32 rows x 96 <= 3/4 of the hash
struct Vocab {
    unsigned long long* keys = nullptr;
    uint32_t* vid = nullptr;
    int64_t cap = 0;      // power of two
    int64_t nvid = 0;     // number of (code, level) pairs; vids are 1..nvid
    int64_t ncommon = 0;  // vids 1..ncommon go to the shared-memory table
    bool split = false;   // ncommon < nvid
    // vids numbered by falling database frequency, so that every prefix
    // 1..k holds the k most frequent pairs (a split vocabulary, or one whose
    // whole table fits some kernels but not the scheduled one's)
    bool freq_ordered = false;
};

// Database (query set) layout.  Molecules are cut into chunks of 32 (one
// warp, one molecule per lane), either in their natural order (full-matrix
// output: a warp's 32 stores per row are one contiguous 128-byte line) or
// sorted by entry count inside windows of 256 (fused kernels, where lanes of
// a warp then have nearly equal amounts of work).  A chunk's entries are stored as ng groups of 16
// bytes per lane, interleaved [group][lane] so a warp's load of one group is
// 512 contiguous bytes; an entry is a vid (uint16 when nvid < 65536, else
// uint32), 0 padding a molecule's list to the chunk's length.
constexpr int kMaxWindow = 8192;   // largest sort window (one CTA sorts it in shared memory)
constexpr int kChunk = 32;
struct DbLayout {
    int64_t n = 0;
    int64_t nchunks = 0;
    int entry_bytes = 2;          // 2 or 4
    int32_t* perm = nullptr;      // [nchunks*32] original index or -1
    int4* meta = nullptr;         // [nchunks*32] {original index or -1, magnitude, count sum, length}
    int32_t* ng = nullptr;        // [nchunks] 16-byte groups per lane
    int64_t* off = nullptr;       // [nchunks + 1] first group (16-byte units); chunks are contiguous
    void* entries = nullptr;      // 16-byte groups
    int64_t ngroups_total = 0;
    int64_t max_ng = 0;
    bool sorted = false;
    int window = kChunk;          // molecules are sorted by entry count inside windows of this size
    bool offsets = false;         // 4-byte entries hold byte offsets (vid * 4) into the table
    int2* crange = nullptr;       // [nchunks] {smallest, largest} magnitude of the chunk's molecules
    bool balanced = false;        // a chunk's entries spread evenly over its lanes (full-matrix layout)
    // split vocabulary: the streamed entries are the common ones; slot s's
    // rare vids are rare_vid[rare_off[s] .. rare_off[s + 1])
    int64_t* rare_off = nullptr;  // [nchunks*32 + 1]
    uint32_t* rare_vid = nullptr;
    int64_t nrare = 0;
    int64_t ncommon = 0;          // vids the layout streams (<= the vocabulary's ncommon)
    // scheduled full-matrix layout (window-sorted): the entries of each
    // (window, warp of a group) are one contiguous run of work items, each
    // item a chunk or a range of a chunk's steps (rows_sched.cu)
    bool scheduled = false;
    int2* sched_items = nullptr;  // [nitems + 2] {chunk, steps | kItemSplit | kItemFirst}, two padding records last
    int* sched_lanes = nullptr;   // [nitems + 2][32] window position << 16 | fast magnitude, or -1
    int2* sched_rare = nullptr;   // split vocabulary: [nitems + 2][32] {first rare entry, count}
    // split vocabulary, scheduled layout: the molecules (natural index) that
    // hold each rare vid, vid ncommon + 1 + i at post_mol[post_off[i] ..
    // post_off[i + 1]); post_max is the longest list
    int64_t* post_off = nullptr;
    int32_t* post_mol = nullptr;
    int64_t post_max = 0;
    int2* sched_wrun = nullptr;   // [nwin * warps] {first item, end item} of (window, warp of a group)
    int64_t* sched_grun = nullptr; // [nwin * warps][2] first and end 16-byte group of (window, warp)
    int64_t nitems = 0;
    int64_t nwin = 0;
    int64_t max_item_steps = 0;
    int sched_warps = 0;          // warps of a group (one window per group)
    int sched_rows = 0;           // ref rows per CTA of the kernel the layout was built for (32 or 64)
};

// Ref-set rows as vid lists (levels expanded, codes absent from the database
// dropped), stride `stride` entries, zero padded.
struct RowEntries {
    int64_t n = 0;
    int64_t stride = 0;
    uint32_t* vid = nullptr;
    int64_t max_rare = 0;      // most rare-vid entries in one row (split vocabulary)
    int64_t max_rare_bal = 0;  // the same against the balanced layout's smaller common set
    int64_t max_rare_sched = 0; // the same against the scheduled layout's common set
};

}  // namespace siml

struct siml_engine {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    size_t smem_optin = 0;
    siml::RawSet ref, qry;
    bool layout_valid = false;   // vocabulary of the current query set
    bool rows_valid = false;
    siml::Vocab vocab;
    siml::DbLayout db_nat, db_sorted, db_sched;
    bool nat_valid = false, sorted_valid = false, sched_valid = false;
    siml::RowEntries rows;
    // device scratch reused across calls, one buffer per purpose (siml::kSlot*)
    void* scratch[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t scratch_bytes[4] = {0, 0, 0, 0};
    int* d_err = nullptr;                 // device error word (calls that wait for their kernels)
    // error word of kernels whose callers do not wait (top-k's bounded lock
    // waits): host-mapped, so a waiting caller reads it with no copy; sticky
    // until reported by siml_sync / siml_async_status or a waiting top-k call
    int* h_async_err = nullptr;
    int* d_async_err = nullptr;
    unsigned long long* d_eval = nullptr;  // pairs the threshold kernels evaluated (chunks not skipped)
    unsigned long long* d_counter = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    bool hold_timing = false;             // a multi-kernel call times itself as a whole
    int64_t launches = 0;
    uint64_t generation = 0;              // bumped whenever a set is replaced (plans made before are stale)
    int rows_window = siml::kChunk;       // sort window of the full-matrix layout (kChunk: natural order)
    int rows_entries = 0;                 // entry format of the full-matrix layout (SIML_TUNE_ROWS_ENTRIES)
    int64_t row_stride_hint = 0;          // least entries per ref row list (SIML_TUNE_ROW_STRIDE)
    int sorted_window = 2048;             // sort window of the fused-kernel layout (SIML_TUNE_SORT_WINDOW)
    int rows_layout = SIML_ROWS_SCHEDULED; // full-matrix layout (SIML_TUNE_ROWS_LAYOUT)
    int sched_groups = 4;                  // warp groups of the scheduled kernel (SIML_TUNE_SCHED_GROUPS)
    int sched_rows = 64;                   // ref rows per CTA of the scheduled kernel (SIML_TUNE_SCHED_ROWS)
    int rare_fixup = 1;                    // rare pairs by a second pass when few (SIML_TUNE_RARE_FIXUP)
    int rows_rare_path = -1;               // the last scheduled launch: 0 no rare pairs, 1 hash, 2 second pass
    uint64_t rows_rare_gen = 0;            // generation of that launch
};

namespace siml {

// engine.cu
int ensure_prepared(siml_engine* h);
// Natural-order (sorted == false) or window-sorted database layout.
int ensure_layout(siml_engine* h, bool sorted, const DbLayout** out);
// The scheduled full-matrix layout (window-sorted, entries in per-warp
// schedule order); rows_sched.cu arranges it.  A CTA's 32 warps form
// sched_groups groups, each on its own window of 2048 / sched_groups columns.
constexpr int kSchedColumns32 = 2048;   // database columns in flight per CTA, 32-row groups
constexpr int kSchedColumns64 = 1024;   // the same, 64-row groups (twice the staging per column)
int ensure_sched_layout(siml_engine* h, const DbLayout** out);
// getMultipleRows runs on the scheduled layout (settings and sets allow it;
// the sets must be prepared).
bool rows_use_sched(siml_engine* h);
// rows_sched.cu: common vids the scheduled kernel's table can hold beside its
// staging (with a split vocabulary), whether it fits the current sets, the
// schedule and entry permutation of a freshly built window-sorted layout,
// and the launch (*done = false when the call is not one it serves).
int64_t sched_capacity(siml_engine* h);
bool sched_whole_fits(siml_engine* h, int64_t nvid);
bool rows_sched_fits(siml_engine* h);
int sched_arrange(siml_engine* h, DbLayout& d);
void free_sched(DbLayout& d);
// Scratch slots: host-call staging, per-call row order, top-k partial heaps,
// small counters.
constexpr int kSlotStage = 0;
constexpr int kSlotOrder = 1;
constexpr int kSlotPartial = 2;
constexpr int kSlotSmall = 3;
int scratch_reserve(siml_engine* h, size_t bytes, void** out, int slot = kSlotStage);
// Rows [rowbase, rowlimit) of the ref set ordered by magnitude (absolute row
// indices, device array of rowlimit - rowbase entries, in kSlotOrder).
int row_order_by_magnitude(siml_engine* h, int64_t rowbase, int64_t rowlimit, const int32_t** order);
// The same into caller buffers: order[rowlimit - rowbase], bucket[4096].
constexpr int kOrderBuckets = 4096;
int row_order_into(siml_engine* h, int64_t rowbase, int64_t rowlimit, int32_t* order, int32_t* bucket);
int cuda_fail(cudaError_t e, const char* what);
// cudaMalloc through the engines' allocator (siml_debug_fail_alloc can refuse it).
int dev_alloc_bytes(void** p, size_t bytes);
// Lets `kernel` launch with up to `need` bytes of dynamic shared memory on
// the current device.  The limit is an attribute of the function, shared by
// every engine and host thread, so it is raised once per kernel and device
// to the most the kernel can use (the opt-in limit less its static shared
// memory) and never set per launch: a smaller value set for one engine
// would make another thread's larger launch of the same kernel fail.
int raise_smem_limit(const void* kernel, size_t need);
// Reports (and clears) an expired top-k lock wait recorded by queued kernels;
// call only once their work is known to be complete.
int take_async_error(siml_engine* h);
// topk_noalloc.cu: resolves the no-allocation entry point's static scratch on
// `device` (the current device); called when an engine is created.
void noalloc_prepare(int device);

// kernels.cu — launchers; all queue work on h->stream and return a status.
struct RowsArgs {
    int64_t rowbase, rowlimit;
    float* out;          // device, [rows, ldo]
    int64_t ldo;
    int mode;            // kModeRows or kModeSingle
};
constexpr int kModeRows = 0;    // getMultipleRows: CPU-order fp32 union, zero test on magnitudes
constexpr int kModeSingle = 1;  // getTanimotoRow: count-sum magnitudes, zero test on lengths
int launch_rows(siml_engine* h, const RowsArgs& a);
int launch_rows_sched(siml_engine* h, const RowsArgs& a, bool* done);
// The balanced full-matrix kernel's shared memory (table + per-warp pieces)
// fits for the current sets.
bool rows_balanced_fits(siml_engine* h);
struct NbrCall {
    int64_t rowbase, rowlimit;
    int64_t col_begin, col_end;   // database columns searched
    float lo, hi;
    int64_t pitch;
    int32_t* idx;        // device [rows, pitch]
    float* sims;         // device [rows, pitch] or null
    int32_t* counts;     // device [rows]
};
int launch_neighbors(siml_engine* h, const NbrCall& c);
// Batched neighbour search: items (two int4 each) pulled by a persistent
// kernel over ordered ref rows `order`, then the per-output-row finish;
// rowinfo[rows_out] = {ref row, col_begin, col_end, 0} (ref row -1: unused
// row).  Queued on st only.  Items that fail the kernel's extent checks
// (order_len entries of order, rows_out output rows) are skipped and set
// bit 2 of the asynchronous error word.
int batch_nbr_usable(siml_engine* h, const DbLayout* d);
// Whether a direct table of nvid vids fits in shared memory, and the number
// of common vids a split vocabulary keeps (its table, the rare-vid hash and
// the largest kernel extras then fit).
bool direct_table_fits(siml_engine* h, int64_t nvid);
int64_t split_table_capacity(siml_engine* h);
// Common vids of the balanced full-matrix layout with a split vocabulary
// (its table, the rare-vid hash and the per-warp piece buffers fit).
int64_t split_balanced_capacity(siml_engine* h);
int launch_batch_neighbors(siml_engine* h, const DbLayout* d, const int4* items, int64_t nitems, unsigned int* head,
                           const int32_t* order, int64_t order_len, const int4* rowinfo, int64_t rows_out, float lo,
                           float hi, int64_t pitch, int32_t* idx, float* sims, int32_t* counts, cudaStream_t st);
// Chunks of the window-sorted layout that hold database columns [c0, c1).
void sorted_chunk_range(const DbLayout* d, int64_t c0, int64_t c1, int64_t& chunk_begin, int64_t& chunk_end);
// Per-row 101-bin int32 histograms (out [rows, ldo], zeroed here) or one
// 1000-bin uint64 histogram accumulated into out.
int launch_hist(siml_engine* h, int64_t rowbase, int64_t rowlimit, bool global, void* out, int64_t ldo);
// Per-row top-k into idx / sims [rows, k]; a bounded lock wait that expires
// sets *h->d_err (read back by the caller).
int launch_topk(siml_engine* h, int64_t rowbase, int64_t rowlimit, int k, int32_t* idx, float* sims);
// The same in pieces, for callers that bring their own buffers: the plan
// gives the number of database splits of the table path (0: per-row scan
// without scratch) and the partial-heap entries it needs; the core takes the
// row order (rows ordered by magnitude, ignored by the scan) and partial
// buffers float[partial_entries] / int[partial_entries].
struct TopkPlan {
    int splits = 0;
    size_t partial_entries = 0;
};
int topk_plan(siml_engine* h, const DbLayout* d, int64_t rowbase, int64_t rowlimit, int k, TopkPlan& plan);
int launch_topk_core(siml_engine* h, const DbLayout* d, int64_t rowbase, int64_t rowlimit, int k,
                     const TopkPlan& plan, const int32_t* order, float* part_t, int* part_i, int32_t* idx,
                     float* sims);
// rowHistogram101 of a dense fp32 / fp64 device matrix into uint32 [rows, 101].
int launch_row_hist101(siml_engine* h, const void* data, bool f64, int64_t rows, int64_t cols, int64_t ld,
                       uint32_t* hist);

}  // namespace siml

#define SIML_CUDA(call)                                              \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return siml::cuda_fail(_e, #call);    \
    } while (0)
