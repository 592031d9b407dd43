/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the reference's CPU algorithms for the LINGO
 * similarity path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load this library; the product path (siml_gb300) never
 * does.  Every function cites the reference file:line it restates.
 *
 * Parity pin: tests/test_oracle_pin.py checks every function here against
 * (a) the reference's own compiled C code (oracle/_ref, built by
 *     oracle/Makefile from the reference sources, in the build container), and
 * (b) the golden fixtures in tests/golden/, which were produced by running
 *     that compiled reference code (tests/golden/make_golden.py).
 *
 * Functions without a reference CPU implementation (getNeighbors, the fused
 * per-row histogram, top-k and the 1000-bin global histogram are GPU-only or
 * new in the reference's API) restate the reference's CUDA kernel semantics
 * on the CPU, citing the kernel lines.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* Multiset Tanimoto — pysiml/_CPULingo.c:53-71 (multisetTanimoto3_mags).
 * Sorted merge over the two code lists with a signed int32 compare; equal
 * codes add min(countA, countB).  The result expression keeps the reference's
 * operation order: ((float)amag + bmag) - isct, each step in fp32.           */
static inline int32_t o_min(int32_t a, int32_t b) { return a < b ? a : b; }

static float oracle_pair(const int32_t* a, const int32_t* b,
                         const int32_t* asize, const int32_t* bsize,
                         int32_t alen, int32_t blen, int32_t amag, int32_t bmag,
                         int32_t* isct_out) {
    int32_t i = 0, j = 0, isct = 0;
    if (isct_out) *isct_out = 0;
    if (amag == 0 || bmag == 0) return 0.0f;
    while (i < alen && j < blen) {
        if (a[i] == b[j]) {
            isct += o_min(asize[i], bsize[j]);
            i++;
            j++;
        } else if (a[i] < b[j]) {
            i++;
        } else {
            j++;
        }
    }
    if (isct_out) *isct_out = isct;
    return isct / ((float)amag + bmag - isct);
}

ORACLE_API float oracle_tanimoto_pair(const int32_t* a, const int32_t* b,
                                      const int32_t* asize, const int32_t* bsize,
                                      int32_t alen, int32_t blen,
                                      int32_t amag, int32_t bmag) {
    return oracle_pair(a, b, asize, bsize, alen, blen, amag, bmag, NULL);
}

/* Block of Tanimoto rows — pysiml/_CPULingo.c:83-274 (serial) and :277-465
 * (OpenMP `parallel for` over reference rows, static schedule, thread count
 * set by omp_set_num_threads(nprocs)).  Rows come from the ref set, columns
 * from the query set; strides are in int32 elements.                        */
ORACLE_API int oracle_tanimoto_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride,
        float* out, int64_t ldo, int nthreads) {
    int64_t row;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads != 1)
#endif
    for (row = 0; row < nref; row++) {
        const int32_t* a = rl + row * rstride;
        const int32_t* as = rc + row * rstride;
        float* orow = out + row * ldo;
        for (int64_t col = 0; col < nq; col++) {
            orow[col] = oracle_pair(a, ql + col * qstride, as, qc + col * qstride,
                                    rlen[row], qlen[col], rmag[row], qmag[col], NULL);
        }
    }
    return 0;
}

/* Intersection counts only (same merge), used by tests that check the
 * integer part of the path separately from the fp32 epilogue.               */
ORACLE_API int oracle_isct_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, int64_t nq, int64_t qstride,
        int32_t* out, int64_t ldo, int nthreads) {
    int64_t row;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads != 1)
#endif
    for (row = 0; row < nref; row++) {
        for (int64_t col = 0; col < nq; col++) {
            int32_t isct = 0;
            oracle_pair(rl + row * rstride, ql + col * qstride, rc + row * rstride,
                        qc + col * qstride, rlen[row], qlen[col], 1, 1, &isct);
            out[row * ldo + col] = isct;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* getNeighbors semantics — pysiml/kernels.py:393-475 (gpuGetNeighbors_multirow)
 * and pysiml/GPULingo.py:467-513.  Per ref row, query columns are scanned in
 * waves of 128 (kernels.py:433).  A column is a neighbour when the fp32
 * magnitude bound min(ma,mb)/(float)max(ma,mb) >= lo (kernels.py:440-441) and
 * the exact Tanimoto t satisfies lo <= t < hi (kernels.py:447).  Neighbours
 * are written in ascending column order while they fit in `pitch`
 * (kernels.py:462-463); the running count grows by whole waves and the scan
 * stops after the first wave that takes it above `pitch` (kernels.py:466-469),
 * so an overflowing row reports a count larger than `pitch`.  `sims` (may be
 * NULL) receives the fp32 similarity beside each written index (an addition
 * of this project; the reference returns indices only).                      */
ORACLE_API int oracle_neighbors_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride,
        float lo, float hi, int64_t pitch,
        int32_t* idx, float* sims, int32_t* counts, int nthreads) {
    int64_t row;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4) if (nthreads != 1)
#endif
    for (row = 0; row < nref; row++) {
        const int32_t ma = rmag[row];
        int64_t count = 0;
        for (int64_t base = 0; base < nq; base += 128) {
            int64_t wave_valid = 0;
            int64_t wend = base + 128 < nq ? base + 128 : nq;
            for (int64_t col = base; col < wend; col++) {
                const int32_t mb = qmag[col];
                const int32_t mn = ma < mb ? ma : mb;
                const int32_t mx = ma > mb ? ma : mb;
                float bound = mn / ((float)mx);
                if (!(bound >= lo)) continue;
                float t = oracle_pair(rl + row * rstride, ql + col * qstride,
                                      rc + row * rstride, qc + col * qstride,
                                      rlen[row], qlen[col], ma, mb, NULL);
                if (t >= lo && t < hi) {
                    int64_t pos = count + wave_valid;
                    if (pos < pitch) {
                        idx[row * pitch + pos] = (int32_t)col;
                        if (sims) sims[row * pitch + pos] = t;
                    }
                    wave_valid++;
                }
            }
            count += wave_valid;
            if (count > pitch) break;
        }
        counts[row] = (int32_t)count;
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Histogram bin rules.
 * 101 bins: pysiml/_cpuutil.cpp:64-66 (rowHistogram101: (unsigned)(x*100)
 * clamped to 100) and the fused kernel pysiml/kernels.py:660-661
 * ((unsigned)(t*100) into 101 bins).  Values below zero (and NaN) go to bin 0.
 * 1000 bins: defined by this project (the reference has no 1000-bin form):
 * min((unsigned)(t*1000.0f), 999), below zero / NaN to bin 0.               */
static inline uint32_t bin101(float x) {
    float s = x * 100.0f;
    if (!(s >= 0.0f)) return 0u;
    if (s >= 4294967040.0f) return 100u;
    uint32_t b = (uint32_t)s;
    return b < 100u ? b : 100u;
}
static inline uint32_t bin1000(float x) {
    float s = x * 1000.0f;
    if (!(s >= 0.0f)) return 0u;
    if (s >= 4294967040.0f) return 999u;
    uint32_t b = (uint32_t)s;
    return b < 999u ? b : 999u;
}

/* rowHistogram101 — pysiml/_cpuutil.cpp:52-72 (float32 input). */
ORACLE_API int oracle_row_histogram101(const float* data, int64_t rows, int64_t cols,
                                       int64_t ld, uint32_t* hist /* rows x 101 */) {
    memset(hist, 0, (size_t)rows * 101 * sizeof(uint32_t));
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = 0; c < cols; c++) hist[r * 101 + bin101(data[r * ld + c])]++;
    return 0;
}

/* Fused Tanimoto + per-row 101-bin histogram — pysiml/kernels.py:606-666
 * (gpuHistogrammedLingo_multirow), GPULingo.py:420-463.  Output int32 [rows,101]. */
ORACLE_API int oracle_hist101_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride, int32_t* hist, int nthreads) {
    int64_t row;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads != 1)
#endif
    for (row = 0; row < nref; row++) {
        int32_t* h = hist + row * 101;
        memset(h, 0, 101 * sizeof(int32_t));
        for (int64_t col = 0; col < nq; col++) {
            float t = oracle_pair(rl + row * rstride, ql + col * qstride,
                                  rc + row * rstride, qc + col * qstride,
                                  rlen[row], qlen[col], rmag[row], qmag[col], NULL);
            h[bin101(t)]++;
        }
    }
    return 0;
}

/* Global 1000-bin uint64 histogram over all pairs of a row block (new in this
 * project's API; bin rule above).  Accumulates into `hist` (not cleared).    */
ORACLE_API int oracle_hist1000_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride, uint64_t* hist, int nthreads) {
    int nt = 1;
#ifdef _OPENMP
    nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
    uint64_t* part = (uint64_t*)calloc((size_t)nt * 1000, sizeof(uint64_t));
    if (!part) return -1;
    int64_t row;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nt) if (nt != 1)
#endif
    for (row = 0; row < nref; row++) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        uint64_t* h = part + (size_t)tid * 1000;
        for (int64_t col = 0; col < nq; col++) {
            float t = oracle_pair(rl + row * rstride, ql + col * qstride,
                                  rc + row * rstride, qc + col * qstride,
                                  rlen[row], qlen[col], rmag[row], qmag[col], NULL);
            h[bin1000(t)]++;
        }
    }
    for (int t = 0; t < nt; t++)
        for (int b = 0; b < 1000; b++) hist[b] += part[(size_t)t * 1000 + b];
    free(part);
    return 0;
}

/* Per-row top-k (new in this project's API): the k largest similarities of
 * each ref row, descending, ties broken by the lower query index.  Rows with
 * fewer than k columns are padded with index -1 and similarity -1.0f.        */
typedef struct { float t; int32_t i; } o_cand;
/* "worse" = lower similarity, or equal similarity and higher index */
static inline int o_worse(o_cand a, o_cand b) { return a.t < b.t || (a.t == b.t && a.i > b.i); }
static void o_sift_down(o_cand* h, int64_t n, int64_t p) {
    for (;;) {
        int64_t l = 2 * p + 1, r = l + 1, w = p;
        if (l < n && o_worse(h[l], h[w])) w = l;
        if (r < n && o_worse(h[r], h[w])) w = r;
        if (w == p) return;
        o_cand tmp = h[p]; h[p] = h[w]; h[w] = tmp; p = w;
    }
}
static void o_sift_up(o_cand* h, int64_t p) {
    while (p > 0) {
        int64_t par = (p - 1) / 2;
        if (!o_worse(h[p], h[par])) return;
        o_cand tmp = h[p]; h[p] = h[par]; h[par] = tmp; p = par;
    }
}
static int o_cmp_best_first(const void* x, const void* y) {
    const o_cand* a = (const o_cand*)x; const o_cand* b = (const o_cand*)y;
    if (a->t != b->t) return a->t > b->t ? -1 : 1;
    return a->i < b->i ? -1 : (a->i > b->i);
}
ORACLE_API int oracle_topk_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride, int64_t k,
        int32_t* idx, float* sims, int nthreads) {
    int64_t row;
    int fail = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4) if (nthreads != 1)
#endif
    for (row = 0; row < nref; row++) {
        o_cand* h = (o_cand*)malloc((size_t)(k > 0 ? k : 1) * sizeof(o_cand));
        if (!h) { fail = 1; continue; }
        int64_t n = 0;
        for (int64_t col = 0; col < nq; col++) {
            o_cand c;
            c.t = oracle_pair(rl + row * rstride, ql + col * qstride,
                              rc + row * rstride, qc + col * qstride,
                              rlen[row], qlen[col], rmag[row], qmag[col], NULL);
            c.i = (int32_t)col;
            if (n < k) { h[n] = c; o_sift_up(h, n); n++; }
            else if (k > 0 && o_worse(h[0], c)) { h[0] = c; o_sift_down(h, n, 0); }
        }
        qsort(h, (size_t)n, sizeof(o_cand), o_cmp_best_first);
        for (int64_t j = 0; j < k; j++) {
            idx[row * k + j] = j < n ? h[j].i : -1;
            sims[row * k + j] = j < n ? h[j].t : -1.0f;
        }
        free(h);
    }
    return fail ? -1 : 0;
}

/* ------------------------------------------------------------------------- */
/* Every product of a row block from one merge per pair, for parity checks at
 * database sizes where separate passes would take minutes.  Each output
 * follows the rule of its single-purpose function above and may be NULL:
 *   out      fp32 [nref, ldo]     oracle_tanimoto_block (_CPULingo.c:53-71)
 *   nb_*     [nref, pitch], [nref] oracle_neighbors_block (kernels.py:393-475:
 *                                  magnitude bound, [lo, hi), 128-wide waves)
 *   tk_*     [nref, k]            oracle_topk_block (ties to the lower index)
 *   h101     int32 [nref, 101]    oracle_hist101_block (kernels.py:606-666)
 *   h1000    uint64 [1000]        oracle_hist1000_block, accumulated into.    */
ORACLE_API int oracle_scan_block(
        const int32_t* rl, const int32_t* rc, const int32_t* rlen, const int32_t* rmag,
        int64_t nref, int64_t rstride,
        const int32_t* ql, const int32_t* qc, const int32_t* qlen, const int32_t* qmag,
        int64_t nq, int64_t qstride,
        float* out, int64_t ldo,
        float lo, float hi, int64_t pitch, int32_t* nb_idx, float* nb_sims, int32_t* nb_counts,
        int64_t k, int32_t* tk_idx, float* tk_sims,
        int32_t* h101, uint64_t* h1000, int nthreads) {
    int nt = 1;
#ifdef _OPENMP
    nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
    uint64_t* part = (uint64_t*)calloc((size_t)nt * 1000, sizeof(uint64_t));
    float* rowbuf = (float*)malloc((size_t)nt * (size_t)(nq > 0 ? nq : 1) * sizeof(float));
    o_cand* heaps = (o_cand*)malloc((size_t)nt * (size_t)(k > 0 ? k : 1) * sizeof(o_cand));
    if (!part || !rowbuf || !heaps) { free(part); free(rowbuf); free(heaps); return -1; }
    int64_t row;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) if (nt != 1)
#endif
    for (row = 0; row < nref; row++) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        float* t = out ? out + row * ldo : rowbuf + (size_t)tid * (size_t)(nq > 0 ? nq : 1);
        for (int64_t col = 0; col < nq; col++)
            t[col] = oracle_pair(rl + row * rstride, ql + col * qstride, rc + row * rstride, qc + col * qstride,
                                 rlen[row], qlen[col], rmag[row], qmag[col], NULL);
        if (h1000) {
            uint64_t* h = part + (size_t)tid * 1000;
            for (int64_t col = 0; col < nq; col++) h[bin1000(t[col])]++;
        }
        if (h101) {
            int32_t* h = h101 + row * 101;
            memset(h, 0, 101 * sizeof(int32_t));
            for (int64_t col = 0; col < nq; col++) h[bin101(t[col])]++;
        }
        if (nb_counts) {
            const int32_t ma = rmag[row];
            int64_t count = 0;
            for (int64_t base = 0; base < nq; base += 128) {
                int64_t wave_valid = 0;
                const int64_t wend = base + 128 < nq ? base + 128 : nq;
                for (int64_t col = base; col < wend; col++) {
                    const int32_t mb = qmag[col];
                    const int32_t mn = ma < mb ? ma : mb, mx = ma > mb ? ma : mb;
                    const float bound = mn / ((float)mx);
                    if (!(bound >= lo)) continue;
                    if (t[col] >= lo && t[col] < hi) {
                        const int64_t pos = count + wave_valid;
                        if (pos < pitch) {
                            nb_idx[row * pitch + pos] = (int32_t)col;
                            if (nb_sims) nb_sims[row * pitch + pos] = t[col];
                        }
                        wave_valid++;
                    }
                }
                count += wave_valid;
                if (count > pitch) break;
            }
            nb_counts[row] = (int32_t)count;
        }
        if (tk_idx && k > 0) {
            o_cand* h = heaps + (size_t)tid * (size_t)k;
            int64_t n = 0;
            for (int64_t col = 0; col < nq; col++) {
                o_cand c;
                c.t = t[col];
                c.i = (int32_t)col;
                if (n < k) { h[n] = c; o_sift_up(h, n); n++; }
                else if (o_worse(h[0], c)) { h[0] = c; o_sift_down(h, n, 0); }
            }
            qsort(h, (size_t)n, sizeof(o_cand), o_cmp_best_first);
            for (int64_t j = 0; j < k; j++) {
                tk_idx[row * k + j] = j < n ? h[j].i : -1;
                tk_sims[row * k + j] = j < n ? h[j].t : -1.0f;
            }
        }
    }
    if (h1000)
        for (int t = 0; t < nt; t++)
            for (int b = 0; b < 1000; b++) h1000[b] += part[(size_t)t * 1000 + b];
    free(part);
    free(rowbuf);
    free(heaps);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* SMILES -> LINGO multiset compiler.
 * Preprocessing state machine — pysiml/_ccompiler.cpp:178-264
 * (processSMILESdigits): digits become '0' except while copying the digits
 * that follow '+', '-', 'H' or '['; "%nn" becomes "%0"; a space, '\n' or '\r'
 * ends the string (dropping the name).  Returns the processed length.        */
static int o_isdigit(unsigned char c) { return c >= '0' && c <= '9'; }

static int32_t oracle_preprocess(const unsigned char* in, int64_t inlen, unsigned char* out) {
    enum { NORMAL, CHOMP, REPLACE, SPECIALNUMS, DONE };
    int state = NORMAL;
    int32_t length = 0;
    int64_t ip = 0, op = 0;
    while (ip < inlen && in[ip] && state != DONE) {
        const unsigned char ch = in[ip];
        switch (state) {
            case CHOMP:
                ip++;
                state = REPLACE;
                break;
            case REPLACE:
                if (o_isdigit(ch)) { out[op] = '0'; length++; }
                else if (ch == ' ' || ch == '\n' || ch == '\r') { out[op] = 0; state = DONE; }
                else if (ch == '%') { out[op] = ch; state = CHOMP; length++; }
                else { out[op] = ch; state = NORMAL; length++; }
                ip++; op++;
                break;
            case SPECIALNUMS:
                out[op] = ch;
                if (!o_isdigit(ch)) state = NORMAL;
                length++; ip++; op++;
                break;
            default: /* NORMAL */
                if (o_isdigit(ch)) { out[op] = '0'; state = REPLACE; length++; }
                else if (ch == '%') { out[op] = ch; state = CHOMP; length++; }
                else if (ch == '+' || ch == '-' || ch == 'H' || ch == '[') {
                    out[op] = ch; state = SPECIALNUMS; length++;
                }
                else if (ch == ' ' || ch == '\n' || ch == '\r') { out[op] = 0; state = DONE; }
                else { out[op] = ch; length++; }
                ip++; op++;
                break;
        }
    }
    out[op] = 0;
    return length;
}

static int o_cmp_i32(const void* x, const void* y) {
    int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
    return (a > b) - (a < b);
}

/* LingoBag — pysiml/_ccompiler.cpp:83-165.  The processed string is viewed as
 * little-endian int32 words; for each of 4 shifts every word whose top byte
 * is non-zero is a LINGO (the scan of a shift stops at the first word with a
 * zero top byte), then all words move down one byte, the next word's low byte
 * entering at the top (:141).  The reference shifts signed int32 values, so a
 * byte >= 0x80 in the top position fills the top with 0xFF instead (:141,
 * :147); that is kept here.  Codes are sorted (signed) and counted; the
 * magnitude is smilen-3 (:90), and strings shorter than 4 give an empty bag
 * (:91-97).  `codes`/`counts` need room for smilen entries.                  */
static inline uint32_t o_asr8(uint32_t w) { return (w >> 8) | ((w & 0x80000000u) ? 0xFF000000u : 0u); }

static int32_t oracle_lingobag(const unsigned char* proc, int32_t smilen,
                               int32_t* codes, int32_t* counts, int32_t* mag) {
    *mag = 0;
    if (smilen - 3 < 1) return 0;
    const int32_t nblocks = smilen / 4 + 1;
    uint32_t* w = (uint32_t*)calloc((size_t)nblocks + 1, sizeof(uint32_t));
    int32_t* all = (int32_t*)malloc(((size_t)smilen + 8) * sizeof(int32_t));
    int32_t nall = 0;
    for (int32_t i = 0; i < nblocks; i++) {
        uint32_t v = 0;
        for (int b = 0; b < 4; b++) {
            int64_t p = (int64_t)4 * i + b;
            uint32_t byte = p < smilen ? proc[p] : 0u;
            v |= byte << (8 * b);
        }
        w[i] = v;
    }
    for (int shift = 0; shift < 4; shift++) {
        for (int32_t i = 0; i < nblocks; i++) {
            if (((w[i] >> 24) & 0xFFu) == 0u) break;
            all[nall++] = (int32_t)w[i];
        }
        for (int32_t i = 0; i < nblocks; i++) {
            if (i < nblocks - 1) w[i] = o_asr8(w[i]) | ((w[i + 1] & 0xFFu) << 24);
            else w[i] = o_asr8(w[i]);
        }
    }
    qsort(all, (size_t)nall, sizeof(int32_t), o_cmp_i32);
    int32_t n = 0;
    for (int32_t k = 0; k < nall; k++) {
        if (n > 0 && codes[n - 1] == all[k]) counts[n - 1]++;
        else { codes[n] = all[k]; counts[n] = 1; n++; }
    }
    free(all);
    free(w);
    *mag = smilen - 3;
    return n;
}

/* One string: preprocess + bag.  Returns the number of unique codes; `codes`
 * and `counts` need room for (inlen + 8) entries.                            */
ORACLE_API int32_t oracle_compile_one(const char* smiles, int64_t inlen,
                                      int32_t* codes, int32_t* counts, int32_t* mag) {
    unsigned char* proc = (unsigned char*)calloc((size_t)inlen + 8, 1);
    int32_t smilen = oracle_preprocess((const unsigned char*)smiles, inlen, proc);
    int32_t n = oracle_lingobag(proc, smilen, codes, counts, mag);
    free(proc);
    return n;
}

/* SMILEStoMatrices — pysiml/_ccompiler.cpp:276-381: all strings of a batch
 * (concatenated in `buf`, string s at [offsets[s], offsets[s+1])) into
 * zero-padded [n, width] code and count matrices plus lengths and mags.
 * With width <= 0 only the required width (max unique codes) is returned.   */
ORACLE_API int64_t oracle_compile_batch(const char* buf, const int64_t* offsets, int64_t n,
                                        int32_t* lingos, int32_t* counts,
                                        int32_t* lengths, int32_t* mags, int64_t width) {
    int64_t maxw = 0;
    int too_wide = 0;
    int64_t s;
    /* strings are independent: OpenMP over them (the reference loops serially) */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) reduction(max : maxw) reduction(| : too_wide)
#endif
    for (s = 0; s < n; s++) {
        int64_t len = offsets[s + 1] - offsets[s];
        int32_t* c = (int32_t*)malloc(((size_t)len + 8) * sizeof(int32_t));
        int32_t* k = (int32_t*)malloc(((size_t)len + 8) * sizeof(int32_t));
        int32_t mag = 0;
        int32_t u = oracle_compile_one(buf + offsets[s], len, c, k, &mag);
        if (u > maxw) maxw = u;
        if (width > 0) {
            if (u > width) {
                too_wide = 1;
            } else {
                memset(lingos + s * width, 0, (size_t)width * sizeof(int32_t));
                memset(counts + s * width, 0, (size_t)width * sizeof(int32_t));
                memcpy(lingos + s * width, c, (size_t)u * sizeof(int32_t));
                memcpy(counts + s * width, k, (size_t)u * sizeof(int32_t));
                lengths[s] = u;
                mags[s] = mag;
            }
        }
        free(c);
        free(k);
    }
    return too_wide ? -1 : maxw;
}
