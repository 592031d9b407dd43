/*
 * siml_gb300 — C ABI of a GB300-native (sm_103a) LINGO multiset-Tanimoto
 * engine that drops in for pySIML's GPU path (pysiml.GPULingo, pysiml.compiler,
 * pysiml.utilities).
 *
 * Conventions
 *   - Every function returns an int status (SIML_OK == 0) unless noted;
 *     siml_last_error() gives the message of the calling thread's last failure.
 *   - Arrays are plain pointers with explicit sizes and row strides (in
 *     elements).  `where` says whether array arguments are host (SIML_HOST)
 *     or device (SIML_DEVICE) pointers.  Host-pointer calls return when the
 *     result is in host memory; device-pointer calls are queued on the
 *     engine's stream and return at once (siml_sync / siml_query_done).
 *   - A handle is used by one host thread at a time; one handle per GPU
 *     (the reference's "one GPULingo object per device", similarity.txt:121-145).
 *   - "ref set" = the rows of a Tanimoto matrix (pySIML's set_refsmiles),
 *     "query set" = its columns (set_qsmiles), as in
 *     doc/html/_sources/concepts.txt:52-57.
 *
 * Every entry point cites the reference interface it replaces
 * (file:line inside the reference project).
 */
#ifndef SIML_GB300_H
#define SIML_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SIML_OK 0
#define SIML_ERR_INVALID 1     /* bad argument (reference: ValueError / TypeError)      */
#define SIML_ERR_STATE 2       /* set not initialised, no pending result                */
#define SIML_ERR_CUDA 3        /* CUDA runtime failure                                  */
#define SIML_ERR_NOMEM 4       /* device or host allocation failed                      */
#define SIML_ERR_TIMEOUT 5     /* a bounded device wait gave up                         */
#define SIML_ERR_UNSUPPORTED 6 /* input outside what the kernels accept (see message)   */
#define SIML_ERR_RANGE 7       /* row range outside the ref set (reference: bare raise) */

/* pointer location */
#define SIML_HOST 0
#define SIML_DEVICE 1
/* siml_rows and siml_row_single: host memory the device can address (pinned and mapped,
 * e.g. from cudaHostAlloc); the kernels write the block into it directly and
 * the call returns at once, like a device-pointer call (siml_sync /
 * siml_query_done).  Other host memory is refused (SIML_ERR_INVALID). */
#define SIML_HOST_QUEUED 2

/* synthetic length models (siml_synth_*) */
#define SIML_SYNTH_UNIFORM_20_90 0
#define SIML_SYNTH_LOGNORMAL_45 1
#define SIML_SYNTH_BIMODAL_35_110 2
#define SIML_SYNTH_CHEM_45 3         /* lognormal 45 with bracket atoms, charges, %nn rings */

typedef struct siml_engine siml_engine;

/* ---- library ------------------------------------------------------------ */
const char* siml_version(void);
/* Message of the calling thread's last failing call ("" if none). */
const char* siml_last_error(void);

/* ---- engine lifetime ---------------------------------------------------- */
/* GPULingo(deviceID) — pysiml/GPULingo.py:162-173 (context + stream per object). */
int siml_create(int device, siml_engine** out);
int siml_destroy(siml_engine* h);
/* Run subsequent work on a caller-owned cudaStream_t (NULL: the engine's own,
 * a non-blocking stream).  For the legacy default stream pass cudaStreamLegacy
 * ((void*)1), not NULL.  Work on the engine's own stream is not ordered after
 * other streams: device inputs written there must be complete first. */
int siml_set_stream(siml_engine* h, void* cuda_stream);
/* stream.synchronize() inside retrieveAsyncResult — pysiml/GPULingo.py:546. */
int siml_sync(siml_engine* h);
/* asyncOperationsDone — pysiml/GPULingo.py:642-647; *done = 1 when idle. */
int siml_query_done(siml_engine* h, int* done);

/* ---- SMILES sets -------------------------------------------------------- */
/* set_refsmiles(L, C, lengths, mags=None) — pysiml/GPULingo.py:187-242.
 * lingos/counts: [n, width] with row stride ld; lengths/mags: [n].  mags may
 * be NULL: magnitudes are then the sum of each row's first `length` counts
 * (accumulateRefMagnitudes, pysiml/kernels.py:45-61).  Codes of a row must be
 * strictly increasing (signed) and counts non-negative, as the compiler
 * produces them; other input is rejected with SIML_ERR_UNSUPPORTED. */
int siml_set_ref(siml_engine* h, const int32_t* lingos, const int32_t* counts,
                 const int32_t* lengths, const int32_t* mags,
                 int64_t n, int64_t width, int64_t ld, int where);
/* set_qsmiles(L, C, lengths, mags=None) — pysiml/GPULingo.py:246-313.  The query
 * set is the resident database; the engine builds its device layout here. */
int siml_set_query(siml_engine* h, const int32_t* lingos, const int32_t* counts,
                   const int32_t* lengths, const int32_t* mags,
                   int64_t n, int64_t width, int64_t ld, int where);
/* Overwrites ref rows [row0, row0 + n) in place (no reference counterpart;
 * the reference replaces the whole set, pysiml/GPULingo.py:187-242): a
 * request loop keeps a slot buffer of ref rows and writes each batch's query
 * molecules into it.  Host arrays (row stride ld >= width, width <= the ref
 * set's width); codes are validated on the host, the copies and the rows'
 * device preparation are queued on the engine's stream, and the call
 * returns without waiting for earlier work when the arrays are pinned.
 * Rows with more entries than SIML_TUNE_ROW_STRIDE reserves make the next
 * call rebuild every row's entry list. */
int siml_write_ref_rows(siml_engine* h, int64_t row0, const int32_t* lingos, const int32_t* counts,
                        const int32_t* lengths, const int32_t* mags, int64_t n, int64_t width, int64_t ld);
/* Sizes of the current sets (-1 when unset). */
int siml_set_sizes(siml_engine* h, int64_t* nref, int64_t* nquery);

/* ---- similarity calls --------------------------------------------------- */
/* getMultipleRows[_async](rowbase, rowlimit) — pysiml/GPULingo.py:354-404,
 * kernel gpuLingoSim3_multirow pysiml/kernels.py:315-352.  out: fp32
 * [rowlimit-rowbase, nquery] with row stride ldo (>= nquery).  A SIML_HOST
 * block in pinned, mapped host memory is written there by the kernels
 * directly; other host memory receives a copy of a device block. */
int siml_rows(siml_engine* h, int64_t rowbase, int64_t rowlimit,
              float* out, int64_t ldo, int where);
/* getTanimotoRow[_async](row) — pysiml/GPULingo.py:316-351, kernel
 * gpuLingoSim3_srgf_T_tex2ns pysiml/kernels.py:234-270: both magnitudes are
 * recomputed from the counts and a molecule with no LINGOs scores 0. */
int siml_row_single(siml_engine* h, int64_t row, float* out, int where);
/* getNeighbors[_async](rowbase, rowlimit, lo, hi, maxneighbors) —
 * pysiml/GPULingo.py:467-534, kernel gpuGetNeighbors_multirow
 * pysiml/kernels.py:393-475.  pitch = 16*ceil(maxneighbors/16) as the
 * reference computes it (GPULingo.py:491).  idx: int32 [rows, pitch] query
 * indices in ascending order; sims (may be NULL): fp32 [rows, pitch] beside
 * them; counts: int32 [rows], larger than pitch when a row overflowed
 * (counted in whole waves of 128 columns, as the reference does). */
int siml_neighbors(siml_engine* h, int64_t rowbase, int64_t rowlimit,
                   float lo, float hi, int64_t pitch,
                   int32_t* idx, float* sims, int32_t* counts, int where);
/* getMultipleHistogrammedRows[_async](rowbase, rowlimit) —
 * pysiml/GPULingo.py:407-463, kernel gpuHistogrammedLingo_multirow
 * pysiml/kernels.py:606-666.  out: int32 [rows, 101], row stride ldo >= 101. */
int siml_hist101(siml_engine* h, int64_t rowbase, int64_t rowlimit,
                 int32_t* out, int64_t ldo, int where);
/* Per-row top-k (no reference counterpart; extends getNeighbors): the k
 * largest similarities of each row, descending, ties to the lower query
 * index; rows with fewer than k columns are padded with -1 / -1.0f.
 * idx: int32 [rows, k], sims: fp32 [rows, k]. */
int siml_topk(siml_engine* h, int64_t rowbase, int64_t rowlimit, int64_t k,
              int32_t* idx, float* sims, int where);
/* With SIML_DEVICE outputs siml_topk only queues work.  Its kernels' bounded
 * lock waits (k > 256, or rows whose candidates overflow twice) record an
 * expiry in a host-mapped word, which siml_sync reports as SIML_ERR_TIMEOUT.
 * siml_async_status reports it without a stream synchronization, so the
 * caller must know the work is done (an event it waited on); both clear the
 * word. */
int siml_async_status(siml_engine* h);
/* siml_topk without any device allocation (no counterpart in the reference).
 * For callers that cannot allocate device memory on the request path (a
 * caller-owned memory pool, a strict memory budget, a service that must not
 * let a request trigger cudaMalloc): all scratch comes from one 16 MiB static
 * __device__ array of the library, held by every GPU that loads it until the
 * process exits.  idx / sims are device pointers [rows, k].  The engine's
 * window-sorted layout must already exist (siml_topk, siml_neighbors,
 * siml_neighbors_range, siml_hist101, siml_hist_global, siml_vocab_stats or
 * siml_batch_create builds it; siml_rows and siml_db_stats do not), else
 * SIML_ERR_STATE; requests needing more than 16 MiB of scratch are refused
 * with SIML_ERR_INVALID.  All calls share the array and it keeps the last
 * call's contents: calls that overlap on the GPU race, so serialize them.
 * The call waits for its kernels before returning (it synchronizes the
 * engine's stream).  siml_create looks up the array's address on its device;
 * if that failed there, the first call does it, and should come before any
 * stream capture. */
int siml_topk_noalloc(siml_engine* h, int64_t rowbase, int64_t rowlimit, int64_t k,
                      int32_t* idx, float* sims);
/* Global similarity histogram over all pairs of a row block (no reference
 * counterpart; a whole-block form of getMultipleHistogrammedRows):
 * nbins = 1000, bin = min((unsigned)(t*1000.0f), 999).  out: uint64 [1000],
 * accumulated into (not cleared), so successive blocks sum. */
int siml_hist_global(siml_engine* h, int64_t rowbase, int64_t rowlimit,
                     uint64_t* out, int where);

/* getNeighbors restricted to query columns [col_begin, col_end) (no
 * reference counterpart; the reference searches the whole query set,
 * pysiml/kernels.py:420-470).  Same rule, pitch and output as
 * siml_neighbors; indices are absolute query indices and an overflowing row
 * is counted in waves of 128 columns starting at col_begin.  This is the
 * plain one-call-per-job path that siml_batch_* replaces. */
int siml_neighbors_range(siml_engine* h, int64_t rowbase, int64_t rowlimit,
                         int64_t col_begin, int64_t col_end,
                         float lo, float hi, int64_t pitch,
                         int32_t* idx, float* sims, int32_t* counts, int where);

/* ---- batched ragged neighbor jobs --------------------------------------- */
/* Many independent threshold searches of different shapes, planned once and
 * run as one persistent launch (no reference counterpart: the reference
 * issues one getNeighbors call per job, pysiml/GPULingo.py:467-513).
 * jobs: int64 [njobs, 5] = {row_begin, row_end, col_begin, col_end, out_row}:
 * ref rows [row_begin, row_end) against query columns [col_begin, col_end)
 * with getNeighbors' rule, results of ref row r in output row
 * out_row + (r - row_begin).  Output rows of different jobs must not
 * overlap; an output row covered by no job gets count 0.  tile_chunks is
 * the number of 32-molecule chunks per work item; <= 0 lets the plan time
 * candidates on a sample of the jobs and keep the fastest.  A plan is tied
 * to the engine's current sets: siml_batch_run refuses it (SIML_ERR_STATE)
 * once set_ref / set_query replaced them.  Destroy plans before the engine. */
typedef struct siml_batch siml_batch;
int siml_batch_create(siml_engine* h, int64_t njobs, const int64_t* jobs,
                      float lo, float hi, int64_t pitch, int64_t tile_chunks,
                      siml_batch** out);
/* siml_batch_create with the plan's shape given (no reference counterpart):
 * tile_chunks chunks per work item, rows_cap ref rows per item (16 or 32),
 * and jobs of at most merge_rows rows given to the per-pair merge (0: none).
 * tile_chunks <= 0 tunes all three on a sample of the jobs, or reuses the
 * shape tuned earlier in the process for the same kind of plan (database
 * length distribution, job sizes and bound); siml_batch_create tunes the
 * same way when its tile_chunks <= 0 and otherwise uses rows_cap 32, no
 * merge jobs. */
int siml_batch_create_shaped(siml_engine* h, int64_t njobs, const int64_t* jobs,
                             float lo, float hi, int64_t pitch, int64_t tile_chunks,
                             int64_t rows_cap, int64_t merge_rows, siml_batch** out);
/* The plan's shape: out = {tile_chunks, rows_cap, merge_rows, 1 when it was
 * reused from an earlier plan of the same kind rather than timed}. */
int siml_batch_shape(siml_batch* b, int64_t out[4]);
/* rows_out: output rows the plan writes (max out_row + rows over jobs);
 * nitems: work items; tile_chunks: the tile the plan uses; stream_bytes:
 * database bytes (entries and per-molecule metadata) one run streams, every
 * work item's chunks; unique_bytes: every job's database range once.  NULL
 * skips an output. */
int siml_batch_info(siml_batch* b, int64_t* rows_out, int64_t* nitems, int64_t* tile_chunks,
                    int64_t* stream_bytes, int64_t* unique_bytes);
/* Queues the plan on stream (a cudaStream_t; NULL: the engine's stream;
 * cudaStreamLegacy for the legacy default stream):
 * device outputs idx, sims (may be NULL): [rows_out, pitch]; counts:
 * [rows_out], with siml_neighbors' meaning.  No host synchronization and
 * no allocation, so a run may be captured in a CUDA graph and replayed.
 * Runs of one plan must not overlap on the GPU (they share a queue head).
 * The kernel checks every work item against the plan's extents; an item
 * outside them is skipped and the next siml_sync / siml_async_status
 * returns SIML_ERR_STATE. */
int siml_batch_run(siml_batch* b, int32_t* idx, float* sims, int32_t* counts, void* stream);
int siml_batch_destroy(siml_batch* b);

/* ---- SMILES compiler ---------------------------------------------------- */
/* cSMILEStoMatrices / _ccompiler.SMILEStoMatrices — pysiml/compiler.py:53-82,
 * pysiml/_ccompiler.cpp:276-381.  Strings are concatenated in buf, string s
 * at [offsets[s], offsets[s+1]); a NUL, space, '\n' or '\r' ends a string.
 * siml_compile_width returns the number of columns needed (max unique
 * LINGOs over the batch) or a negative status. */
int64_t siml_compile_width(const char* buf, const int64_t* offsets, int64_t n);
/* Writes zero-padded int32 lingos/counts [n, width] and lengths/mags [n]. */
int siml_compile_smiles(const char* buf, const int64_t* offsets, int64_t n,
                        int32_t* lingos, int32_t* counts, int32_t* lengths,
                        int32_t* mags, int64_t width);
/* One-pass form of the two calls above (no reference counterpart; the same
 * output, each string compiled once).  siml_compile_stage writes string s's
 * unique codes and counts, unpadded, to staging arrays of offsets[n] int32
 * each at [offsets[s], offsets[s] + lengths[s]), writes lengths and mags [n],
 * and returns the width or a negative status.  siml_compile_scatter then
 * writes the zero-padded [n, width] rows (width >= the returned width, else
 * SIML_ERR_INVALID). */
int64_t siml_compile_stage(const char* buf, const int64_t* offsets, int64_t n,
                           int32_t* stage_codes, int32_t* stage_counts, int32_t* lengths,
                           int32_t* mags);
int siml_compile_scatter(const int64_t* offsets, int64_t n, const int32_t* stage_codes,
                         const int32_t* stage_counts, const int32_t* lengths,
                         int32_t* lingos, int32_t* counts, int64_t width);
/* The same compiler on the GPU (the reference compiles on the CPU only;
 * same rules and output bytes as siml_compile_smiles).  buf (offsets[n]
 * bytes) and offsets (n+1 int64) are device memory, as are the outputs;
 * work is queued on the engine's stream.  siml_compile_width_gpu returns
 * the width (waits for the stream) or a negative status;
 * siml_compile_smiles_gpu fills [n, width] rows (width >= 1) and returns
 * once they are written.  Strings longer than 1,024 bytes are compiled by a
 * second kernel over device scratch sized for them. */
int64_t siml_compile_width_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n);
int siml_compile_smiles_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n,
                            int32_t* lingos, int32_t* counts, int32_t* lengths,
                            int32_t* mags, int64_t width);
/* One-pass form of the GPU compiler (no reference counterpart; the same
 * output as the two calls above, each string compiled once).
 * siml_compile_stage_gpu compiles every string into device staging arrays of
 * offsets[n] int32 each (string s's unique codes and counts, unpadded, at
 * [offsets[s], offsets[s] + lengths[s])), writes lengths and mags [n], and
 * returns the width (waits for the stream) or a negative status.
 * siml_compile_scatter_gpu then writes the zero-padded [n, width] rows
 * (width >= the returned width, else SIML_ERR_INVALID) and returns once they
 * are written. */
int64_t siml_compile_stage_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n,
                               int32_t* stage_codes, int32_t* stage_counts, int32_t* lengths,
                               int32_t* mags);
int siml_compile_scatter_gpu(siml_engine* h, const int64_t* offsets, int64_t n,
                             const int32_t* stage_codes, const int32_t* stage_counts,
                             const int32_t* lengths, int32_t* lingos, int32_t* counts,
                             int64_t width);

/* ---- utilities ---------------------------------------------------------- */
/* rowHistogram101 — pysiml/utilities.py:44-55, pysiml/_cpuutil.cpp:52-126:
 * per-row 101-bin uint32 histogram of an fp32 matrix [rows, cols] (row
 * stride ld); bin = min((unsigned)(x*100), 100), negatives to bin 0. */
int siml_row_histogram101(siml_engine* h, const float* data, int64_t rows, int64_t cols,
                          int64_t ld, uint32_t* hist, int where);
/* The same for an fp64 matrix (the reference accepts float64 too,
 * pysiml/_cpuutil.cpp:89-101); the product x*100 is formed in fp64. */
int siml_row_histogram101_f64(siml_engine* h, const double* data, int64_t rows, int64_t cols,
                              int64_t ld, uint32_t* hist, int where);

/* ---- synthetic workload sets (benchmarks and tests) --------------------- */
int siml_synth_lengths(uint64_t seed, int dist, int64_t first, int64_t n, int32_t* lens);
int siml_synth_smiles(uint64_t seed, int dist, int64_t first, int64_t n,
                      char* buf, int64_t bufcap, int64_t* offsets);

/* ---- introspection ------------------------------------------------------ */
/* Device-layout statistics (no reference counterpart), prepared on demand:
 * out[0] = (code, level) pairs in the database vocabulary, out[1] = bytes per
 * stored entry, out[2] = 16-byte entry groups stored, out[3] = chunks of 32
 * molecules, out[4] = largest chunk in groups per lane, out[5] = database
 * molecules, out[6] / out[7] = largest count sum in the ref / query set. */
int siml_db_stats(siml_engine* h, int64_t out[8]);
/* Vocabulary split (no counterpart in the reference).  When the table of
 * all (code, level) pairs does not fit in shared memory, the pairs are
 * renumbered by database frequency: the first out[1] ("common") keep the
 * shared-memory table, the rest are "rare" and are looked up per row group
 * in a small hash of the ref rows' rare pairs.  out[0] = pairs, out[1] =
 * common pairs (== out[0] without a split), out[2] = rare entries of the
 * database (window-sorted layout), out[3] = most rare entries in one ref row
 * (table kernels run while it is at most 96; otherwise the per-pair merge). */
int siml_vocab_stats(siml_engine* h, int64_t out[4]);
/* Layout tuning (no reference counterpart).  SIML_TUNE_ROWS_WINDOW: the
 * full-matrix layout (siml_rows, siml_row_single) sorts database molecules by
 * entry count inside windows of 32 (natural order), 64, 128 or 256 molecules;
 * wider windows pad less but scatter each warp's stores over more of a row.
 * Changing it drops the current full-matrix layout (rebuilt on next use). */
#define SIML_TUNE_ROWS_WINDOW 1
/* SIML_TUNE_ROWS_ENTRIES: how the full-matrix layout stores entries:
 * SIML_ENTRIES_AUTO (2-byte vids when the vocabulary allows, else 4-byte),
 * SIML_ENTRIES_U32 (4-byte vids), SIML_ENTRIES_OFFSETS (4-byte table byte
 * offsets: no index arithmetic in the inner loop, twice the bytes of 2-byte
 * vids).  Changing it drops the current full-matrix layout. */
#define SIML_TUNE_ROWS_ENTRIES 2
#define SIML_ENTRIES_AUTO 0
#define SIML_ENTRIES_U16 1     /* as AUTO: 2-byte when the vocabulary allows */
#define SIML_ENTRIES_U32 2
#define SIML_ENTRIES_OFFSETS 3
/* SIML_TUNE_ROW_STRIDE: least number of entries (sum of counts) reserved per
 * ref row's entry list, so rows written later by siml_write_ref_rows up to
 * that size need no rebuild. */
#define SIML_TUNE_ROW_STRIDE 3
/* SIML_TUNE_SORT_WINDOW: the layout of the fused kernels (neighbours,
 * histograms, top-k, batched jobs) sorts database molecules by entry count
 * inside windows of this many molecules (a power of two, 64..8192; default
 * 2048).  Wider windows pad less and give chunks narrower magnitude ranges
 * (more chunks skipped by threshold searches); column-range jobs are rounded
 * out to whole windows.  Changing it drops the layout and invalidates
 * batch plans. */
#define SIML_TUNE_SORT_WINDOW 4
/* SIML_TUNE_ROWS_LAYOUT: the layout of the full-matrix path.
 * SIML_ROWS_SCHEDULED (the default): molecules sorted by entry count inside
 * windows (2048 / SIML_TUNE_SCHED_GROUPS molecules), each window's chunks
 * split into equal per-warp work schedules, counts staged in shared memory
 * and written out in natural order.  The natural-order layouts, which the other settings (and calls
 * the scheduled kernel does not serve) use: SIML_ROWS_PADDED (lane i holds
 * molecule i, padded to the chunk's longest) or SIML_ROWS_BALANCED (the
 * chunk's entries dealt evenly to the lanes, partial counts merged before
 * the row epilogue).  Changing it drops the full-matrix layouts. */
#define SIML_TUNE_ROWS_LAYOUT 5
#define SIML_ROWS_PADDED 0
#define SIML_ROWS_BALANCED 1
#define SIML_ROWS_SCHEDULED 2
/* SIML_TUNE_SCHED_GROUPS: the scheduled full-matrix kernel splits a CTA's
 * 32 warps into this many groups (2 or 4; default 4), each working on its
 * own window of 2048 / groups database columns, so the groups' stream and
 * store phases overlap.  Changing it drops the scheduled layout. */
#define SIML_TUNE_SCHED_GROUPS 6
/* SIML_TUNE_SCHED_ROWS: ref rows per CTA of the scheduled full-matrix kernel,
 * 64 (the default: one 8-byte table word per database pair serves 64 rows;
 * windows of 1024 / SIML_TUNE_SCHED_GROUPS molecules) or 32 (one 4-byte word;
 * windows of 2048 / SIML_TUNE_SCHED_GROUPS).  The 64-row table holds fewer
 * pairs, so larger vocabularies are numbered by frequency and their rarest
 * pairs go through a hash.  Changing it rebuilds the vocabulary and layouts
 * on next use and invalidates batch plans. */
#define SIML_TUNE_SCHED_ROWS 7
/* SIML_TUNE_RARE_FIXUP: with a split vocabulary, 1 (the default) lets the
 * scheduled full-matrix kernel skip the rare pairs when few pairs share one
 * (at most 1/64 of a row's columns) and recompute those pairs afterwards with
 * the reference's merge (k_rare_fix); 0 always counts rare pairs through the
 * kernel's hash. */
#define SIML_TUNE_RARE_FIXUP 8
int siml_set_tuning(siml_engine* h, int key, int64_t value);
int siml_get_tuning(siml_engine* h, int key, int64_t* value);
/* The full-matrix path the current sets and settings use (no reference
 * counterpart): out[0] = 1 when getMultipleRows runs on the scheduled layout
 * (SIML_ROWS_SCHEDULED), out[1..3] = its work items, windows and the most
 * 8-entry steps of one item; out[0] = 0 (and zeros) otherwise.  Builds the
 * layout if needed. */
int siml_rows_info(siml_engine* h, int64_t out[4]);
/* The scheduled layout's vocabulary split (no reference counterpart):
 * out[0] = pairs its shared-memory table holds (the most frequent ones),
 * out[1] = database entries of the other ("rare") pairs, out[2] = most rare
 * entries in one ref row, out[3] = how the last getMultipleRows launch on
 * that layout counted the rare pairs: 0 none to count, 1 a per-group hash
 * inside the table pass, 2 a second pass over the pairs that share one,
 * -1 before such a launch.  Zeros (and -1) when getMultipleRows does not run
 * on the scheduled layout.  Builds the layout if needed. */
int siml_rows_vocab(siml_engine* h, int64_t out[4]);
/* Pairs the threshold kernels (neighbours, batched jobs, top-k collection,
 * histograms) actually evaluated: 32 x group rows per streamed chunk, i.e.
 * without the chunks skipped by the magnitude bound.  Waits for the engine's
 * stream; reset != 0 zeroes the counter afterwards. */
int siml_eval_pairs(siml_engine* h, uint64_t* out, int reset);
/* Free and total device memory of the engine's GPU in bytes
 * (cudaMemGetInfo; no counterpart in the reference, which allocates per
 * call).  The request loop admits batches against it. */
int siml_mem_info(siml_engine* h, int64_t* free_bytes, int64_t* total_bytes);
/* Number of kernel launches this engine has issued since creation. */
int64_t siml_launch_count(siml_engine* h);
/* Test support (no counterpart in the reference): overwrites entry `pos` of
 * ref row `row`'s device vid list, the list the table kernels set their
 * shared table from, to exercise the kernels' and the plans' checks without
 * a GPU fault.  The kernels skip an entry they cannot hold and report it
 * (SIML_ERR_STATE from the call, or from siml_sync for queued calls); batch
 * plans refuse rows whose lists hold such entries.  The next siml_set_ref
 * rebuilds the lists. */
int siml_debug_set_row_vid(siml_engine* h, int64_t row, int64_t pos, uint32_t vid);
/* Test support (no counterpart in the reference; needs no GPU): the status
 * and siml_last_error() message that siml_sync / siml_async_status give for
 * an asynchronous error word the kernels wrote.  Value 1: a top-k lock wait
 * ran out (SIML_ERR_TIMEOUT); 2: a batch work item outside its plan
 * (SIML_ERR_STATE); 4: a ref-row vid the table cannot hold (SIML_ERR_STATE).
 * The lowest set bit decides. */
int siml_debug_async_status(int word);
/* Fault injection for tests (no counterpart in the reference): the nth
 * device allocation from now through the engines' array allocator, in any
 * engine of the process, returns SIML_ERR_NOMEM without calling cudaMalloc,
 * as an out-of-memory GPU would; 0 disarms.  Nothing is faulted on the GPU:
 * the refusal is made on the host.  The engine stays usable, and the next
 * call rebuilds whatever the failed one left unbuilt. */
int siml_debug_fail_alloc(int64_t nth);
/* Average device time (ms) of the dominant kernel of the last call on this
 * engine, measured with CUDA events on the engine's stream (0 if none). */
double siml_last_kernel_ms(siml_engine* h);

#ifdef __cplusplus
}
#endif

#endif /* SIML_GB300_H */
