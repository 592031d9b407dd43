// Similarity kernels (sm_103a).
//
// k_rows — block of Tanimoto rows (getMultipleRows, pysiml/kernels.py:315-352;
// getTanimotoRow, :234-270).  One CTA per (32-row group, database slice):
//   1. the CTA clears a shared-memory table T[vid] (one 32-bit word per
//      database (code, level) pair) and sets bit r of T[vid] for every entry
//      of its row r — rows are the reference's SIML-ref rows;
//   2. each warp walks database chunks of 32 molecules (one per lane); a lane
//      loads its molecule's entries 8 at a time (one 16-byte coalesced load,
//      512 bytes per warp) and adds the eight T words into a bit-sliced
//      counter, so 32 row intersections advance per table read;
//   3. the counter is transposed into 32 row counts and each pair's Tanimoto
//      is formed in the reference's fp32 operation order and stored.
// k_rows_merge — the reference's per-pair sorted merge, used only when the
// table would not fit in shared memory or counts exceed 16 bits.
#include <algorithm>

#include "engine.h"
#include "lingo_core.cuh"

namespace siml {

namespace {

constexpr int kRowsThreads = 512;

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

struct RowsParams {
    // ref rows
    const uint32_t* row_vid;
    int64_t row_stride;
    const int32_t* row_mag;
    const int32_t* row_cmag;
    const int32_t* row_len;
    int64_t rowbase;
    int rows;
    // database layout
    const void* entries;
    const int64_t* off;
    const int32_t* ng;
    const int32_t* perm;
    const int32_t* dmag;
    const int32_t* dcmag;
    const int32_t* dlen;
    int64_t nchunks;
    int vt_words;
    // output
    float* out;
    int64_t ldo;
    int mode;
};

template <int NP, typename ET>
__global__ void __launch_bounds__(kRowsThreads, 1) k_rows(const RowsParams p) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* T = smem;
    int32_t* s_amag = (int32_t*)(smem + p.vt_words);
    int32_t* s_alen = s_amag + 32;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int64_t row0 = (int64_t)blockIdx.x * 32;  // relative to rowbase
    const int nr = min(32, p.rows - (int)row0);

    for (int i = threadIdx.x * 4; i < p.vt_words; i += blockDim.x * 4)
        *reinterpret_cast<uint4*>(T + i) = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x < 32) {
        const int r = threadIdx.x;
        const int64_t gr = p.rowbase + row0 + r;
        s_amag[r] = r < nr ? (p.mode == kModeSingle ? p.row_cmag[gr] : p.row_mag[gr]) : 0;
        s_alen[r] = r < nr ? p.row_len[gr] : 0;
    }
    __syncthreads();
    for (int r = warp; r < nr; r += nwarps) {
        const uint32_t* rv = p.row_vid + (p.rowbase + row0 + r) * p.row_stride;
        for (int64_t e = lane; e < p.row_stride; e += 32) {
            const uint32_t v = rv[e];
            if (v) atomicOr(&T[v], 1u << r);
        }
    }
    __syncthreads();

    const int64_t cb = p.nchunks * blockIdx.y / gridDim.y;
    const int64_t ce = p.nchunks * (blockIdx.y + 1) / gridDim.y;
    for (int64_t c = cb + warp; c < ce; c += nwarps) {
        const int ng = p.ng[c];
        const uint4* ep = reinterpret_cast<const uint4*>(p.entries) + p.off[c] + lane;
        SlicedCounter<NP> acc;
        acc.clear();
        if (sizeof(ET) == 2) {
            for (int s = 0; s < ng; s++) {
                const uint4 q = __ldg(ep + (int64_t)s * 32);
                acc.add8(T[q.x & 0xFFFFu], T[q.x >> 16], T[q.y & 0xFFFFu], T[q.y >> 16],
                         T[q.z & 0xFFFFu], T[q.z >> 16], T[q.w & 0xFFFFu], T[q.w >> 16]);
            }
        } else {
            for (int s = 0; s < ng; s += 2) {
                const uint4 q0 = __ldg(ep + (int64_t)s * 32);
                const uint4 q1 = __ldg(ep + (int64_t)(s + 1) * 32);
                acc.add8(T[q0.x], T[q0.y], T[q0.z], T[q0.w], T[q1.x], T[q1.y], T[q1.z], T[q1.w]);
            }
        }
        RowCounts<NP> rc;
        counts_from_planes<NP>(acc, rc);
        const int64_t slot = c * 32 + lane;
        const int32_t m = p.perm[slot];
        if (m < 0) continue;
        const int32_t bmag = p.mode == kModeSingle ? p.dcmag[slot] : p.dmag[slot];
        const int32_t blen = p.dlen[slot];
        float* o = p.out + row0 * p.ldo + m;
#pragma unroll
        for (int r = 0; r < 32; r++) {
            if (r < nr) {
                const int is = (int)row_count<NP>(rc, r);
                const float t = p.mode == kModeSingle ? tanimoto_single(is, s_amag[r], bmag, s_alen[r], blen)
                                                      : tanimoto_rows(is, s_amag[r], bmag);
                o[(int64_t)r * p.ldo] = t;
            }
        }
    }
}

struct MergeParams {
    const int32_t *rl, *rc, *rlen, *rmag, *rcmag;
    int64_t rw;
    const int32_t *ql, *qc, *qlen, *qmag, *qcmag;
    int64_t qw, nq;
    int64_t rowbase;
    float* out;
    int64_t ldo;
    int mode;
};

// Sorted merge per pair (pysiml/_CPULingo.c:53-71, pysiml/kernels.py:162-199).
__global__ void k_rows_merge(const MergeParams p) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t r = p.rowbase + blockIdx.y;
    if (col >= p.nq) return;
    const int32_t* a = p.rl + r * p.rw;
    const int32_t* as = p.rc + r * p.rw;
    const int32_t* b = p.ql + col * p.qw;
    const int32_t* bs = p.qc + col * p.qw;
    const int32_t alen = p.rlen[r], blen = p.qlen[col];
    int32_t i = 0, j = 0, isct = 0;
    while (i < alen && j < blen) {
        const int32_t x = a[i], y = b[j];
        if (x == y) { isct += min(as[i], bs[j]); i++; j++; }
        else if (x < y) i++;
        else j++;
    }
    const float t = p.mode == kModeSingle ? tanimoto_single(isct, p.rcmag[r], p.qcmag[col], alen, blen)
                                          : tanimoto_rows(isct, p.rmag[r], p.qmag[col]);
    p.out[(int64_t)blockIdx.y * p.ldo + col] = t;
}

int planes_needed(int64_t max_count) {
    int b = 0;
    while (b < 62 && (1ll << b) <= max_count) b++;
    return b;
}

// Splits of the database per row group so that groups x splits fills whole
// waves of one CTA per SM and every CTA still has plenty of chunks.
int choose_splits(int64_t groups, int64_t nchunks, int num_sms, int nwarps) {
    int best = 1;
    double best_cost = 1e300;
    const int64_t max_s = std::max<int64_t>(1, std::min<int64_t>(1024, nchunks / (4 * nwarps)));
    for (int64_t s = 1; s <= max_s; s++) {
        const int64_t ctas = groups * s;
        const int64_t waves = (ctas + num_sms - 1) / num_sms;
        // time ~ waves * (work per CTA + fixed set-up), work per CTA ~ 1/s
        const double cost = (double)waves * (1.0 / (double)s + 0.004);
        if (cost < best_cost * 0.999) { best_cost = cost; best = (int)s; }
    }
    return best;
}

template <int NP, typename ET>
int launch_rows_t(siml_engine* h, const RowsParams& p, int64_t groups, size_t smem) {
    static bool attr_set = false;
    static size_t attr_bytes = 0;
    if (!attr_set || attr_bytes < smem) {
        SIML_CUDA(cudaFuncSetAttribute(k_rows<NP, ET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
        attr_bytes = smem;
    }
    const int nwarps = kRowsThreads / 32;
    const int s = choose_splits(groups, p.nchunks, h->num_sms, nwarps);
    dim3 grid((unsigned)groups, (unsigned)s);
    SIML_CUDA(cudaEventRecord(h->ev0, h->stream));
    k_rows<NP, ET><<<grid, kRowsThreads, smem, h->stream>>>(p);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(cudaEventRecord(h->ev1, h->stream));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

}  // namespace

int launch_rows(siml_engine* h, const RowsArgs& a) {
    const int64_t rows = a.rowlimit - a.rowbase;
    const int64_t groups = (rows + 31) / 32;
    const int vt_words = (int)((h->vocab.nvid + 1 + 3) / 4 * 4);
    const size_t smem = (size_t)vt_words * 4 + 64 * 4;
    const int np = planes_needed(std::min(h->ref.max_entries, h->qry.max_entries));
    const bool table_ok = smem <= h->smem_optin && np <= 16 && groups <= 0x7FFFFFFF;
    if (table_ok) {
        RowsParams p;
        p.row_vid = h->rows.vid;
        p.row_stride = h->rows.stride;
        p.row_mag = h->ref.mag;
        p.row_cmag = h->ref.cmag;
        p.row_len = h->ref.len;
        p.rowbase = a.rowbase;
        p.rows = (int)rows;
        p.entries = h->db.entries;
        p.off = h->db.off;
        p.ng = h->db.ng;
        p.perm = h->db.perm;
        p.dmag = h->db.mag;
        p.dcmag = h->db.cmag;
        p.dlen = h->db.len;
        p.nchunks = h->db.nchunks;
        p.vt_words = vt_words;
        p.out = a.out;
        p.ldo = a.ldo;
        p.mode = a.mode;
        if (np <= 8)
            return h->db.entry_bytes == 2 ? launch_rows_t<8, uint16_t>(h, p, groups, smem)
                                          : launch_rows_t<8, uint32_t>(h, p, groups, smem);
        return h->db.entry_bytes == 2 ? launch_rows_t<16, uint16_t>(h, p, groups, smem)
                                      : launch_rows_t<16, uint32_t>(h, p, groups, smem);
    }
    MergeParams m;
    m.rl = h->ref.lingos; m.rc = h->ref.counts; m.rlen = h->ref.len; m.rmag = h->ref.mag; m.rcmag = h->ref.cmag;
    m.rw = h->ref.width;
    m.ql = h->qry.lingos; m.qc = h->qry.counts; m.qlen = h->qry.len; m.qmag = h->qry.mag; m.qcmag = h->qry.cmag;
    m.qw = h->qry.width; m.nq = h->qry.n;
    m.rowbase = a.rowbase;
    m.out = a.out;
    m.ldo = a.ldo;
    m.mode = a.mode;
    if (rows > 65535) return fail(SIML_ERR_UNSUPPORTED, "merge path: more than 65535 rows per call");
    dim3 grid((unsigned)((h->qry.n + 255) / 256), (unsigned)rows);
    SIML_CUDA(cudaEventRecord(h->ev0, h->stream));
    k_rows_merge<<<grid, 256, 0, h->stream>>>(m);
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(cudaEventRecord(h->ev1, h->stream));
    h->timed = true;
    h->launches++;
    return SIML_OK;
}

}  // namespace siml
