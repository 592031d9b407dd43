// Engine lifetime, SMILES-set upload and the device layout the similarity
// kernels read.  The public C ABI is declared in include/siml_gb300.h.
//
// Set-up pipeline (all on the GPU except tiny scans):
//   set_ref / set_query   upload [n, width] codes and counts, lengths, mags;
//                         validate (codes strictly increasing, counts >= 0,
//                         0 <= length <= width) and form count sums.
//   vocabulary            hash every database (code, level) pair, level =
//                         1..count, and number the pairs 1..nvid.
//   database layout       windows of 256 molecules sorted by entry count,
//                         chunks of 32, vids interleaved per lane.
//   ref-row entries       each ref row as its list of vids (pairs absent from
//                         the database are dropped; they cannot match).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "engine.h"
#include "lingo_core.cuh"

namespace siml {

int cuda_fail(cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? SIML_ERR_NOMEM : SIML_ERR_CUDA;
    return fail(code, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

namespace {
std::mutex g_smem_mu;
std::map<std::pair<const void*, int>, size_t> g_smem_limit;   // (kernel, device) -> dynamic limit set
}  // namespace

int raise_smem_limit(const void* kernel, size_t need) {
    int dev = 0;
    SIML_CUDA(cudaGetDevice(&dev));
    const std::pair<const void*, int> key(kernel, dev);
    size_t limit = 0;
    {
        std::lock_guard<std::mutex> lk(g_smem_mu);
        auto it = g_smem_limit.find(key);
        if (it != g_smem_limit.end()) limit = it->second;
    }
    if (limit == 0) {
        cudaFuncAttributes a;
        SIML_CUDA(cudaFuncGetAttributes(&a, kernel));
        int optin = 0;
        SIML_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        limit = (size_t)std::max(0, optin - (int)a.sharedSizeBytes);
        SIML_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
        std::lock_guard<std::mutex> lk(g_smem_mu);
        g_smem_limit[key] = limit;
    }
    if (need > limit)
        return fail(SIML_ERR_UNSUPPORTED, "a kernel launch needs %zu bytes of dynamic shared memory, more than the "
                    "%zu this GPU allows it", need, limit);
    return SIML_OK;
}

int scratch_reserve(siml_engine* h, size_t bytes, void** out, int slot) {
    if (bytes > h->scratch_bytes[slot]) {
        if (h->scratch[slot]) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            SIML_CUDA(cudaFree(h->scratch[slot]));
            h->scratch[slot] = nullptr;
            h->scratch_bytes[slot] = 0;
        }
        size_t want = std::max(bytes, (size_t)1 << 16);
        SIML_CUDA(cudaMalloc(&h->scratch[slot], want));
        h->scratch_bytes[slot] = want;
    }
    *out = h->scratch[slot];
    return SIML_OK;
}

namespace {

// Counting sort of rows by min(magnitude, 4095): bucket sizes ...
__global__ void k_order_count(const int32_t* __restrict__ mag, int64_t rowbase, int64_t rows, int32_t* bucket) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) atomicAdd(bucket + min(max(mag[rowbase + i], 0), kOrderBuckets - 1), 1);
}
// ... exclusive prefix over the buckets (one block) ...
__global__ void k_order_scan(int32_t* bucket) {
    __shared__ int32_t part[1024];
    const int t = threadIdx.x;
    int32_t v[4], s = 0;
    for (int j = 0; j < 4; j++) { v[j] = bucket[4 * t + j]; s += v[j]; }
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int32_t x = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    int32_t run = part[t] - s;
    for (int j = 0; j < 4; j++) { bucket[4 * t + j] = run; run += v[j]; }
}
// ... and placement (order inside a bucket is arbitrary; every row's result
// is independent of the grouping).
__global__ void k_order_scatter(const int32_t* __restrict__ mag, int64_t rowbase, int64_t rows, int32_t* bucket,
                                int32_t* order) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows) {
        const int pos = atomicAdd(bucket + min(max(mag[rowbase + i], 0), kOrderBuckets - 1), 1);
        order[pos] = (int32_t)(rowbase + i);
    }
}
}  // namespace

int row_order_into(siml_engine* h, int64_t rowbase, int64_t rowlimit, int32_t* order, int32_t* bucket) {
    const int64_t rows = rowlimit - rowbase;
    SIML_CUDA(cudaMemsetAsync(bucket, 0, kOrderBuckets * 4, h->stream));
    if (rows > 0) {
        const unsigned g = (unsigned)((rows + 255) / 256);
        k_order_count<<<g, 256, 0, h->stream>>>(h->ref.mag, rowbase, rows, bucket);
        k_order_scan<<<1, 1024, 0, h->stream>>>(bucket);
        k_order_scatter<<<g, 256, 0, h->stream>>>(h->ref.mag, rowbase, rows, bucket, order);
        h->launches += 3;
        SIML_CUDA(cudaGetLastError());
    }
    return SIML_OK;
}

int row_order_by_magnitude(siml_engine* h, int64_t rowbase, int64_t rowlimit, const int32_t** order) {
    const int64_t rows = rowlimit - rowbase;
    void* ob = nullptr;
    void* bb = nullptr;
    int rc;
    if ((rc = scratch_reserve(h, (size_t)std::max<int64_t>(rows, 1) * 4, &ob, kSlotOrder))) return rc;
    if ((rc = scratch_reserve(h, kOrderBuckets * 4, &bb, kSlotSmall))) return rc;
    if ((rc = row_order_into(h, rowbase, rowlimit, (int32_t*)ob, (int32_t*)bb))) return rc;
    *order = (const int32_t*)ob;
    return SIML_OK;
}

namespace {
// siml_debug_fail_alloc: allocations left before one is refused (0: none).
std::atomic<int64_t> g_fail_alloc{0};
}  // namespace

int dev_alloc_bytes(void** p, size_t bytes) {
    *p = nullptr;
    int64_t left = g_fail_alloc.load();
    while (left > 0 && !g_fail_alloc.compare_exchange_weak(left, left - 1)) {
    }
    if (left == 1)
        return fail(SIML_ERR_NOMEM, "device allocation of %zu bytes refused (siml_debug_fail_alloc)", bytes);
    SIML_CUDA(cudaMalloc(p, bytes));
    return SIML_OK;
}

namespace {

template <class T>
int dev_alloc(T** p, size_t count) {
    return dev_alloc_bytes(reinterpret_cast<void**>(p), (count == 0 ? 1 : count) * sizeof(T));
}
template <class T>
void dev_free(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

void free_set(RawSet& s) {
    dev_free(s.lingos); dev_free(s.counts); dev_free(s.len); dev_free(s.mag); dev_free(s.cmag);
    s = RawSet();
}
void free_vocab(Vocab& v) { dev_free(v.keys); dev_free(v.vid); v = Vocab(); }
void free_layout(DbLayout& d) {
    dev_free(d.perm); dev_free(d.meta);
    dev_free(d.ng); dev_free(d.off);
    dev_free(d.rare_off); dev_free(d.rare_vid);
    if (d.crange) cudaFree(d.crange);
    if (d.entries) cudaFree(d.entries);
    free_sched(d);
    d = DbLayout();
}
void free_rows(RowEntries& r) { dev_free(r.vid); r = RowEntries(); }

constexpr int kErrUnsorted = 1;
constexpr int kErrNegCount = 2;
constexpr int kErrLength = 4;
constexpr int kErrHashFull = 8;

// ---------------------------------------------------------------- kernels --

// Per molecule: validate, count sum (the magnitude accumulateRefMagnitudes /
// accumulateQueryMagnitudes form, pysiml/kernels.py:45-79), statistics.
__global__ void k_set_stats(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                            const int32_t* __restrict__ len, int64_t n, int64_t width,
                            int32_t* __restrict__ cmag, int* err,
                            unsigned long long* total, unsigned long long* maxe) {
    int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mine = 0;
    if (m < n) {
        int32_t L = len[m];
        int e = 0;
        if (L < 0 || L > width) {
            e |= kErrLength;
            L = 0;
        }
        const int32_t* lr = lingos + m * width;
        const int32_t* cr = counts + m * width;
        long long s = 0;
        for (int32_t j = 0; j < L; j++) {
            const int32_t c = cr[j];
            if (c < 0) e |= kErrNegCount;
            else s += c;
            if (j > 0 && !(lr[j - 1] < lr[j])) e |= kErrUnsorted;
        }
        if (s > 0x7FFFFFFFll) { e |= kErrNegCount; s = 0x7FFFFFFF; }
        cmag[m] = (int32_t)s;
        if (e) atomicOr(err, e);
        mine = (unsigned long long)s;
    }
    // warp-level reduce then one atomic per warp
    unsigned long long sum = mine, mx = mine;
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
        unsigned long long t = __shfl_down_sync(0xFFFFFFFFu, mx, o);
        mx = t > mx ? t : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(total, sum);
        atomicMax(maxe, mx);
    }
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}
__device__ __forceinline__ unsigned long long vkey(int32_t code, int32_t level) {
    return ((unsigned long long)(uint32_t)level << 32) | (unsigned long long)(uint32_t)code;
}

// Inserts every (code, level) pair of the database into the hash.
__global__ void k_vocab_insert(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                               const int32_t* __restrict__ len, int64_t n, int64_t width,
                               unsigned long long* keys, int64_t cap,
                               unsigned long long* inserted, int* err) {
    const int64_t total = n * width;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i / width;
        const int32_t j = (int32_t)(i - m * width);
        if (j >= len[m]) continue;
        const int32_t code = lingos[i];
        const int32_t c = counts[i];
        for (int32_t lvl = 1; lvl <= c; lvl++) {
            const unsigned long long k = vkey(code, lvl);
            unsigned long long slot = mix64(k) & (unsigned long long)(cap - 1);
            int64_t probes = 0;
            for (;;) {
                unsigned long long cur = keys[slot];
                if (cur == k) break;
                if (cur == kEmptyKey) {
                    unsigned long long prev = atomicCAS(&keys[slot], kEmptyKey, k);
                    if (prev == kEmptyKey) { atomicAdd(inserted, 1ull); break; }
                    if (prev == k) break;
                }
                slot = (slot + 1) & (unsigned long long)(cap - 1);
                if (++probes >= cap) { atomicOr(err, kErrHashFull); return; }
            }
        }
    }
}

// Occupied slots per 1024-slot block.
__global__ void k_vocab_count(const unsigned long long* __restrict__ keys, int64_t cap, int32_t* blockcount) {
    __shared__ int warp_n[32];
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    const bool occ = i < cap && keys[i] != kEmptyKey;
    const unsigned b = __ballot_sync(0xFFFFFFFFu, occ);
    if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = warp_n[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
        if (threadIdx.x == 0) blockcount[blockIdx.x] = v;
    }
}

// vid = 1 + (occupied slots before this one), slot order.
__global__ void k_vocab_assign(const unsigned long long* __restrict__ keys, int64_t cap,
                               const int32_t* __restrict__ blockbase, uint32_t* vid) {
    __shared__ int warp_n[32];
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    const bool occ = i < cap && keys[i] != kEmptyKey;
    const unsigned b = __ballot_sync(0xFFFFFFFFu, occ);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_n[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = warp_n[threadIdx.x];
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += t;
        }
        warp_n[threadIdx.x] = incl - v;
    }
    __syncthreads();
    if (i < cap) {
        const int rank = warp_n[w] + __popc(b & ((1u << lane) - 1u));
        vid[i] = occ ? (uint32_t)(1 + blockbase[blockIdx.x] + rank) : 0u;
    }
}

__device__ __forceinline__ uint32_t vocab_lookup(const unsigned long long* __restrict__ keys,
                                                 const uint32_t* __restrict__ vid, int64_t cap,
                                                 int32_t code, int32_t lvl) {
    const unsigned long long k = vkey(code, lvl);
    unsigned long long slot = mix64(k) & (unsigned long long)(cap - 1);
    for (int64_t probes = 0; probes < cap; probes++) {
        const unsigned long long cur = keys[slot];
        if (cur == k) return vid[slot];
        if (cur == kEmptyKey) return 0u;
        slot = (slot + 1) & (unsigned long long)(cap - 1);
    }
    return 0u;
}

// Database frequency of every (code, level) pair: the number of molecules
// holding the code with count >= level, i.e. how often its vid appears in
// the entry stream.  Used to renumber a vocabulary that has to be split.
__global__ void k_vocab_freq(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                             const int32_t* __restrict__ len, int64_t n, int64_t width,
                             const unsigned long long* __restrict__ keys, int64_t cap, uint32_t* freq) {
    const int64_t total = n * width;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i / width;
        const int32_t j = (int32_t)(i - m * width);
        if (j >= len[m]) continue;
        const int32_t code = lingos[i], c = counts[i];
        for (int32_t lvl = 1; lvl <= c; lvl++) {
            const unsigned long long k = vkey(code, lvl);
            unsigned long long slot = mix64(k) & (unsigned long long)(cap - 1);
            for (int64_t probes = 0; probes < cap; probes++) {
                const unsigned long long cur = keys[slot];
                if (cur == k) { atomicAdd(&freq[slot], 1u); break; }
                if (cur == kEmptyKey) break;
                slot = (slot + 1) & (unsigned long long)(cap - 1);
            }
        }
    }
}

// Split vocabulary: per molecule the entries that stay in the stream
// (vid <= ncommon) and the rare ones.
__global__ void k_split_count(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                              const int32_t* __restrict__ len, int64_t n, int64_t width,
                              const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ vid,
                              int64_t cap, int64_t ncommon, int32_t* ccount, int32_t* rcount) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int32_t L = len[m];
    int32_t nc = 0, nrare = 0;
    for (int32_t j = 0; j < L; j++) {
        const int32_t code = lingos[m * width + j], cnt = counts[m * width + j];
        for (int32_t lvl = 1; lvl <= cnt; lvl++) {
            const uint32_t v = vocab_lookup(keys, vid, cap, code, lvl);
            if ((int64_t)v <= ncommon) nc++;
            else nrare++;
        }
    }
    ccount[m] = nc;
    rcount[m] = nrare;
}

// Rare entries per chunk of the layout (slot order).
__global__ void k_rare_chunk(const int32_t* __restrict__ perm, const int32_t* __restrict__ rcount, int64_t nchunks,
                             int64_t* chunk_sum) {
    const int64_t c = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (c >= nchunks) return;
    const int32_t m = perm[c * 32 + (threadIdx.x & 31)];
    int64_t v = m >= 0 ? rcount[m] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0) chunk_sum[c] = v;
}

// rare_off[slot] = chunk base + rare entries of the chunk's earlier lanes.
__global__ void k_rare_off(const int32_t* __restrict__ perm, const int32_t* __restrict__ rcount, int64_t nchunks,
                           const int64_t* __restrict__ chunk_base, int64_t* rare_off) {
    const int64_t c = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const int32_t m = perm[c * 32 + lane];
    const int64_t v = m >= 0 ? rcount[m] : 0;
    int64_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += u;
    }
    rare_off[c * 32 + lane] = chunk_base[c] + incl - v;
    if (c == nchunks - 1 && lane == 31) rare_off[nchunks * 32] = chunk_base[c] + incl;
}

// One CTA of 256 threads per window: rank molecules by (entries, index).
// Sorts each window of w molecules (a power of two, 64..kMaxWindow) by entry
// count: bitonic sort of (count << 32 | position) keys in shared memory;
// positions past the end sort last.
__global__ void k_window_sort(const int32_t* __restrict__ cmag, int64_t n, int w, int32_t* perm) {
    extern __shared__ long long key[];
    const int64_t base = (int64_t)blockIdx.x * w;
    for (int i = threadIdx.x; i < w; i += blockDim.x) {
        const int64_t m = base + i;
        key[i] = m < n ? ((long long)cmag[m] << 32) | i : (0x7FFFFFFFll << 32) | i;
    }
    __syncthreads();
    for (int k = 2; k <= w; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < w; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool asc = (i & k) == 0;
                    const long long a = key[i], b = key[ixj];
                    if ((a > b) == asc) {
                        key[i] = b;
                        key[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < w; i += blockDim.x) {
        const int64_t m = base + (int)(key[i] & 0xFFFFFFFFll);
        perm[base + i] = m < n ? (int32_t)m : -1;
    }
}

// Natural order: slot i holds molecule i.
__global__ void k_identity_perm(int64_t n, int64_t slots, int32_t* perm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < slots) perm[i] = i < n ? (int32_t)i : -1;
}

// Per chunk: 16-byte groups per lane = ceil(max entries / entries-per-group),
// rounded up to an even number of 8-entry steps; plus per-lane metadata.
__global__ void k_chunk_meta(const int32_t* __restrict__ perm, const int32_t* __restrict__ cmag,
                             const int32_t* __restrict__ scount, const int32_t* __restrict__ mag,
                             const int32_t* __restrict__ len, int64_t nchunks, int entries_per_group,
                             int balanced, int32_t* __restrict__ ng, int4* __restrict__ meta,
                             int2* __restrict__ crange) {
    const int64_t c = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const int32_t m = perm[c * 32 + lane];
    meta[c * 32 + lane] = make_int4(m, m >= 0 ? mag[m] : 0, m >= 0 ? cmag[m] : 0, m >= 0 ? len[m] : 0);
    const int32_t e = m >= 0 ? scount[m] : 0;               // streamed entries (all, or the common ones)
    int32_t mx = e;
    int32_t sum = (e + 7) / 8;                              // 8-entry steps of this molecule
    int32_t mlo = m >= 0 ? mag[m] : 0x7FFFFFFF, mhi = m >= 0 ? mag[m] : -1;
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
        sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        mlo = min(mlo, __shfl_xor_sync(0xFFFFFFFFu, mlo, o));
        mhi = max(mhi, __shfl_xor_sync(0xFFFFFFFFu, mhi, o));
    }
    if (lane == 0) {
        // padded: every lane as long as the longest molecule; balanced: the
        // chunk's steps spread evenly over the 32 lanes
        const int32_t steps = balanced ? (sum + 31) / 32 : (mx + 7) / 8;
        ng[c] = steps * (8 / entries_per_group);
        crange[c] = make_int2(mlo, mhi);                    // empty chunk: lo > hi
    }
}

// Padded layout: entry e of lane l's molecule sits in 16-byte group e / EPG
// of that lane.  Balanced layout: the chunk's 8-entry steps, molecule after
// molecule, are dealt to the lanes in runs of L = ng / SPG steps, so entry e
// of molecule l is step P_l + e / 8 of the chunk (P_l = steps of molecules
// before l), i.e. step (P_l + e / 8) % L of lane (P_l + e / 8) / L.
template <typename ET>
__global__ void k_fill_entries(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                               const int32_t* __restrict__ len, const int32_t* __restrict__ cmag, int64_t width,
                               const int32_t* __restrict__ perm, const int64_t* __restrict__ off,
                               const int32_t* __restrict__ ng, int64_t nchunks, int balanced,
                               const unsigned long long* __restrict__ keys,
                               const uint32_t* __restrict__ vid, int64_t cap, int shift,
                               ET* __restrict__ entries, int64_t ncommon, const int64_t* __restrict__ rare_off,
                               uint32_t* __restrict__ rare_vid) {
    constexpr int EPG = 16 / sizeof(ET);
    constexpr int SPG = 8 / EPG;   // 16-byte groups per 8-entry step
    const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nchunks * 32) return;   // whole warps (nchunks * 32 is a multiple of 32)
    const int32_t m = perm[slot];
    const int64_t c = slot >> 5;
    const int lane = (int)(slot & 31);
    int32_t P = 0, Ls = 1;
    if (balanced) {   // cmag: the streamed entries of each molecule
        const int32_t g = m >= 0 ? (cmag[m] + 7) / 8 : 0;
        int32_t incl = g;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        P = incl - g;
        Ls = max(1, ng[c] / SPG);
    }
    if (m < 0) return;
    const int32_t L = len[m];
    const int32_t* lr = lingos + (int64_t)m * width;
    const int32_t* cr = counts + (int64_t)m * width;
    int64_t e = 0, er = 0;   // streamed and rare entries so far
    for (int32_t j = 0; j < L; j++) {
        const int32_t code = lr[j], cnt = cr[j];
        for (int32_t lvl = 1; lvl <= cnt; lvl++) {
            const uint32_t v = vocab_lookup(keys, vid, cap, code, lvl);
            if (rare_off && (int64_t)v > ncommon) {
                rare_vid[rare_off[slot] + er++] = v;
                continue;
            }
            int64_t g;
            if (balanced) {
                const int64_t gs = P + e / 8;
                g = off[c] + ((gs % Ls) * SPG + (e % 8) / EPG) * 32 + gs / Ls;
            } else {
                g = off[c] + (e / EPG) * 32 + lane;
            }
            entries[g * EPG + (e % EPG)] = (ET)(v << shift);
            e++;
        }
    }
}

// Each ref row as its vid list (stride entries, zero padded).
__global__ void k_row_entries(const int32_t* __restrict__ lingos, const int32_t* __restrict__ counts,
                              const int32_t* __restrict__ len, int64_t n, int64_t width,
                              const unsigned long long* __restrict__ keys,
                              const uint32_t* __restrict__ vid, int64_t cap,
                              uint32_t* __restrict__ out, int64_t stride, int64_t ncommon, int64_t ncommon_bal,
                              int64_t ncommon_sched, int* max_rare) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int nrare = 0, nrare_bal = 0, nrare_sched = 0;
    const int32_t L = len[r];
    const int32_t* lr = lingos + r * width;
    const int32_t* cr = counts + r * width;
    uint32_t* o = out + r * stride;
    int64_t e = 0;
    for (int32_t j = 0; j < L; j++) {
        const int32_t code = lr[j], cnt = cr[j];
        for (int32_t lvl = 1; lvl <= cnt; lvl++) {
            const uint32_t v = vocab_lookup(keys, vid, cap, code, lvl);
            if (v == 0u) break;   // higher levels of an absent pair are absent too
            o[e++] = v;
            nrare += (int64_t)v > ncommon;
            nrare_bal += (int64_t)v > ncommon_bal;
            nrare_sched += (int64_t)v > ncommon_sched;
        }
    }
    for (; e < stride; e++) o[e] = 0u;
    if (nrare) atomicMax(max_rare, nrare);
    if (nrare_bal) atomicMax(max_rare + 1, nrare_bal);
    if (nrare_sched) atomicMax(max_rare + 2, nrare_sched);
}

// ------------------------------------------------------------ host helpers --

int upload_set(siml_engine* h, RawSet& s, const int32_t* lingos, const int32_t* counts,
               const int32_t* lengths, const int32_t* mags, int64_t n, int64_t width,
               int64_t ld, const char* what) {
    if (n < 0 || width < 0 || ld < width)
        return fail(SIML_ERR_INVALID, "%s: bad shape (n=%lld, width=%lld, ld=%lld)", what,
                    (long long)n, (long long)width, (long long)ld);
    if (n > 0 && (!lengths || (width > 0 && (!lingos || !counts))))
        return fail(SIML_ERR_INVALID, "%s: NULL array", what);
    if (n > 0x7FFFFFFFll) return fail(SIML_ERR_UNSUPPORTED, "%s: more than 2^31-1 molecules", what);
    free_set(s);
    const int64_t w = std::max<int64_t>(width, 1);
    int rc;
    if ((rc = dev_alloc(&s.lingos, (size_t)(n * w)))) return rc;
    if ((rc = dev_alloc(&s.counts, (size_t)(n * w)))) return rc;
    if ((rc = dev_alloc(&s.len, (size_t)n))) return rc;
    if ((rc = dev_alloc(&s.mag, (size_t)n))) return rc;
    if ((rc = dev_alloc(&s.cmag, (size_t)n))) return rc;
    cudaStream_t st = h->stream;
    if (n > 0) {
        if (width > 0) {
            SIML_CUDA(cudaMemcpy2DAsync(s.lingos, w * 4, lingos, ld * 4, width * 4, n, cudaMemcpyDefault, st));
            SIML_CUDA(cudaMemcpy2DAsync(s.counts, w * 4, counts, ld * 4, width * 4, n, cudaMemcpyDefault, st));
        } else {
            SIML_CUDA(cudaMemsetAsync(s.lingos, 0, n * 4, st));
            SIML_CUDA(cudaMemsetAsync(s.counts, 0, n * 4, st));
        }
        SIML_CUDA(cudaMemcpyAsync(s.len, lengths, n * 4, cudaMemcpyDefault, st));
    }
    SIML_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), st));
    SIML_CUDA(cudaMemsetAsync(h->d_counter, 0, 2 * sizeof(unsigned long long), st));
    if (n > 0) {
        k_set_stats<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s.lingos, s.counts, s.len, n, w, s.cmag,
                                                                h->d_err, h->d_counter, h->d_counter + 1);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        if (mags) SIML_CUDA(cudaMemcpyAsync(s.mag, mags, n * 4, cudaMemcpyDefault, st));
        else SIML_CUDA(cudaMemcpyAsync(s.mag, s.cmag, n * 4, cudaMemcpyDeviceToDevice, st));
    }
    int err = 0;
    unsigned long long stats[2] = {0, 0};
    SIML_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SIML_CUDA(cudaMemcpyAsync(stats, h->d_counter, sizeof(stats), cudaMemcpyDeviceToHost, st));
    SIML_CUDA(cudaStreamSynchronize(st));
    s.n = n;
    s.width = w;
    s.total_entries = (int64_t)stats[0];
    s.max_entries = (int64_t)stats[1];
    if (err & kErrLength) { free_set(s); return fail(SIML_ERR_INVALID, "%s: a length is negative or exceeds the matrix width", what); }
    if (err & kErrUnsorted) { free_set(s); return fail(SIML_ERR_UNSUPPORTED, "%s: LINGO codes of a molecule are not strictly increasing (sorted unique codes are required, as the SMILES compiler produces)", what); }
    if (err & kErrNegCount) { free_set(s); return fail(SIML_ERR_UNSUPPORTED, "%s: negative or overflowing LINGO counts", what); }
    return SIML_OK;
}

int split_vocab(siml_engine* h, int64_t ncommon);

// Common vids of the balanced full-matrix layout: the vocabulary's, or
// fewer with a split vocabulary (room for the piece buffers).
int64_t balanced_ncommon(siml_engine* h) {
    return h->vocab.split ? std::min<int64_t>(h->vocab.ncommon, split_balanced_capacity(h)) : h->vocab.ncommon;
}

// Common vids of the scheduled full-matrix layout: the vocabulary's when
// its whole table fits beside the staging, else those of a split vocabulary
// up to the kernel's capacity.
int64_t sched_ncommon(siml_engine* h) {
    return std::min<int64_t>(h->vocab.ncommon, sched_capacity(h));
}

int build_vocab(siml_engine* h) {
    free_vocab(h->vocab);
    const RawSet& q = h->qry;
    cudaStream_t st = h->stream;
    int64_t cap = 1 << 16;
    while (cap < 4 * std::min<int64_t>(q.total_entries, 1 << 22)) cap <<= 1;
    for (int attempt = 0; attempt < 8; attempt++) {
        Vocab& v = h->vocab;
        int rc;
        if ((rc = dev_alloc(&v.keys, (size_t)cap))) return rc;
        v.cap = cap;
        SIML_CUDA(cudaMemsetAsync(v.keys, 0xFF, cap * sizeof(unsigned long long), st));
        SIML_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), st));
        SIML_CUDA(cudaMemsetAsync(h->d_counter, 0, sizeof(unsigned long long), st));
        if (q.n > 0) {
            const int64_t total = q.n * q.width;
            const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 65535LL * 8);
            k_vocab_insert<<<grid, 256, 0, st>>>(q.lingos, q.counts, q.len, q.n, q.width, v.keys, cap,
                                                 h->d_counter, h->d_err);
            h->launches++;
            SIML_CUDA(cudaGetLastError());
        }
        int err = 0;
        unsigned long long ins = 0;
        SIML_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaMemcpyAsync(&ins, h->d_counter, sizeof(ins), cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaStreamSynchronize(st));
        if ((err & kErrHashFull) || (int64_t)ins * 2 > cap) {
            free_vocab(v);
            cap <<= 2;
            continue;
        }
        // number the occupied slots
        const int64_t nblk = (cap + 1023) / 1024;
        int32_t* bcount = nullptr;
        if ((rc = dev_alloc(&bcount, (size_t)nblk))) return rc;
        if ((rc = dev_alloc(&v.vid, (size_t)cap))) { dev_free(bcount); return rc; }
        k_vocab_count<<<(unsigned)nblk, 1024, 0, st>>>(v.keys, cap, bcount);
        h->launches++;
        std::vector<int32_t> hb((size_t)nblk);
        SIML_CUDA(cudaMemcpyAsync(hb.data(), bcount, nblk * 4, cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaStreamSynchronize(st));
        int64_t acc = 0;
        for (auto& x : hb) { int32_t t = x; x = (int32_t)acc; acc += t; }
        SIML_CUDA(cudaMemcpyAsync(bcount, hb.data(), nblk * 4, cudaMemcpyHostToDevice, st));
        k_vocab_assign<<<(unsigned)nblk, 1024, 0, st>>>(v.keys, cap, bcount, v.vid);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        SIML_CUDA(cudaStreamSynchronize(st));
        dev_free(bcount);
        v.nvid = acc;
        v.ncommon = acc;
        v.split = false;
        if (!direct_table_fits(h, acc)) return split_vocab(h, split_table_capacity(h));
        // the whole table fits the kernels with nothing beside it, but not
        // the scheduled full-matrix kernel with its staging: number the
        // vids by frequency (nothing is split), so that kernel can take the
        // most frequent ones as its common set
        if (!sched_whole_fits(h, acc)) return split_vocab(h, acc);
        return SIML_OK;
    }
    return fail(SIML_ERR_NOMEM, "vocabulary hash could not be sized");
}

// Renumbers the vocabulary by falling database frequency (ties: slot order)
// so that vids 1..ncommon are the most frequent pairs, and marks it split
// when ncommon < nvid.
int split_vocab(siml_engine* h, int64_t ncommon) {
    Vocab& v = h->vocab;
    const RawSet& q = h->qry;
    cudaStream_t st = h->stream;
    ncommon = std::max<int64_t>(0, std::min<int64_t>(ncommon, v.nvid));
    uint32_t* freq = nullptr;
    int rc;
    if ((rc = dev_alloc(&freq, (size_t)v.cap))) return rc;
    std::vector<uint32_t> hf((size_t)v.cap);
    cudaError_t e = cudaMemsetAsync(freq, 0, (size_t)v.cap * 4, st);
    if (e == cudaSuccess && q.n > 0) {
        const int64_t total = q.n * q.width;
        const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 65535LL * 8);
        k_vocab_freq<<<grid, 256, 0, st>>>(q.lingos, q.counts, q.len, q.n, q.width, v.keys, v.cap, freq);
        h->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hf.data(), freq, (size_t)v.cap * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(freq);
    if (e != cudaSuccess) return cuda_fail(e, "vocabulary frequencies");
    std::vector<int64_t> occ;
    occ.reserve((size_t)v.nvid);
    for (int64_t s = 0; s < v.cap; s++)
        if (hf[(size_t)s]) occ.push_back(s);
    if ((int64_t)occ.size() != v.nvid) return fail(SIML_ERR_CUDA, "vocabulary frequencies do not cover the vocabulary");
    auto more = [&](int64_t a, int64_t b) {
        return hf[(size_t)a] != hf[(size_t)b] ? hf[(size_t)a] > hf[(size_t)b] : a < b;
    };
    std::nth_element(occ.begin(), occ.begin() + ncommon, occ.end(), more);
    std::sort(occ.begin(), occ.begin() + ncommon, more);
    std::vector<uint32_t> hv((size_t)v.cap, 0u);
    for (int64_t i = 0; i < ncommon; i++) hv[(size_t)occ[(size_t)i]] = (uint32_t)(i + 1);
    uint32_t next = (uint32_t)ncommon + 1u;
    for (int64_t s = 0; s < v.cap; s++)
        if (hf[(size_t)s] && !hv[(size_t)s]) hv[(size_t)s] = next++;
    SIML_CUDA(cudaMemcpyAsync(v.vid, hv.data(), (size_t)v.cap * 4, cudaMemcpyHostToDevice, st));
    SIML_CUDA(cudaStreamSynchronize(st));
    v.ncommon = ncommon;
    v.split = ncommon < v.nvid;
    v.freq_ordered = true;
    return SIML_OK;
}

// Device scratch freed when the scope ends (layout builds only).
struct DevTemp {
    void* p = nullptr;
    ~DevTemp() { if (p) cudaFree(p); }
};

int build_layout(siml_engine* h, DbLayout& d, bool sorted, bool scheduled = false) {
    free_layout(d);
    const RawSet& q = h->qry;
    cudaStream_t st = h->stream;
    const bool vsplit = h->vocab.split;
    if (scheduled) sorted = true;
    d.n = q.n;
    d.sorted = sorted;
    d.scheduled = scheduled;
    d.window = scheduled ? (h->sched_rows == 64 ? kSchedColumns64 : kSchedColumns32) / h->sched_groups
                         : (sorted ? h->sorted_window : h->rows_window);
    d.sched_warps = scheduled ? 32 / h->sched_groups : 0;
    d.sched_rows = scheduled ? h->sched_rows : 0;
    // k_window_sort is a bitonic sort: a window that is not a power of two
    // would index past its shared keys
    if (d.window < kChunk || (d.window & (d.window - 1)) || d.window > kMaxWindow)
        return fail(SIML_ERR_UNSUPPORTED, "layout window %d is not a power of two in [%d, %d]", d.window, kChunk,
                    kMaxWindow);
    d.offsets = !vsplit && !sorted && h->rows_entries == SIML_ENTRIES_OFFSETS;
    // the balanced kernel reads vids, not byte offsets; with a split
    // vocabulary its piece buffers leave room for fewer common vids
    d.balanced = !sorted && h->rows_window == kChunk &&
                 (h->rows_layout == SIML_ROWS_BALANCED || h->rows_layout == SIML_ROWS_SCHEDULED) && !d.offsets &&
                 rows_balanced_fits(h);
    d.ncommon = scheduled ? sched_ncommon(h) : (vsplit && d.balanced ? balanced_ncommon(h) : h->vocab.ncommon);
    const bool split = d.ncommon < h->vocab.nvid;
    d.entry_bytes = d.ncommon < 65535 ? 2 : 4;
    if (!vsplit && !sorted && (h->rows_entries == SIML_ENTRIES_U32 || d.offsets)) d.entry_bytes = 4;
    const int64_t nwin = (q.n + d.window - 1) / d.window;
    d.nchunks = (q.n + kChunk - 1) / kChunk;
    const int64_t slots = std::max<int64_t>(nwin, 1) * d.window;
    int rc;
    if ((rc = dev_alloc(&d.perm, (size_t)slots))) return rc;
    if ((rc = dev_alloc(&d.meta, (size_t)slots))) return rc;
    if ((rc = dev_alloc(&d.ng, (size_t)d.nchunks))) return rc;
    if ((rc = dev_alloc(&d.off, (size_t)d.nchunks + 1))) return rc;
    if (q.n == 0) return SIML_OK;
    SIML_CUDA(cudaMalloc((void**)&d.crange, (size_t)std::max<int64_t>(d.nchunks, 1) * sizeof(int2)));
    // streamed entries per molecule: all of them, or the common ones of a
    // split vocabulary (the rare ones go to per-slot lists)
    DevTemp t_cc, t_rc;
    const int32_t* scount = q.cmag;
    int32_t* rcount = nullptr;
    if (split) {
        SIML_CUDA(cudaMalloc(&t_cc.p, (size_t)q.n * 4));
        SIML_CUDA(cudaMalloc(&t_rc.p, (size_t)q.n * 4));
        k_split_count<<<(unsigned)((q.n + 255) / 256), 256, 0, st>>>(
            q.lingos, q.counts, q.len, q.n, q.width, h->vocab.keys, h->vocab.vid, h->vocab.cap, d.ncommon,
            (int32_t*)t_cc.p, (int32_t*)t_rc.p);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        scount = (const int32_t*)t_cc.p;
        rcount = (int32_t*)t_rc.p;
    }
    if (d.window > kChunk) {
        const size_t wsm = (size_t)d.window * 8;
        rc = raise_smem_limit(reinterpret_cast<const void*>(k_window_sort), wsm);
        if (rc) return rc;
        k_window_sort<<<(unsigned)nwin, std::min(d.window, 1024), wsm, st>>>(scount, q.n, d.window, d.perm);
    } else {
        k_identity_perm<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(q.n, slots, d.perm);
    }
    h->launches++;
    const int epg = 16 / d.entry_bytes;
    k_chunk_meta<<<(unsigned)((d.nchunks + 7) / 8), 256, 0, st>>>(d.perm, q.cmag, scount, q.mag, q.len, d.nchunks,
                                                                  epg, d.balanced ? 1 : 0, d.ng, d.meta, d.crange);
    h->launches++;
    SIML_CUDA(cudaGetLastError());
    std::vector<int32_t> hng((size_t)d.nchunks);
    std::vector<int64_t> hoff((size_t)d.nchunks + 1);
    SIML_CUDA(cudaMemcpyAsync(hng.data(), d.ng, d.nchunks * 4, cudaMemcpyDeviceToHost, st));
    SIML_CUDA(cudaStreamSynchronize(st));
    int64_t acc = 0, mx = 0;
    for (int64_t c = 0; c < d.nchunks; c++) {
        hoff[(size_t)c] = acc;
        acc += (int64_t)hng[(size_t)c] * 32;
        mx = std::max<int64_t>(mx, hng[(size_t)c]);
    }
    hoff[(size_t)d.nchunks] = acc;
    d.ngroups_total = acc;
    d.max_ng = mx;
    SIML_CUDA(cudaMemcpyAsync(d.off, hoff.data(), (d.nchunks + 1) * 8, cudaMemcpyHostToDevice, st));
    if (split) {
        // slot s's rare vids at rare_off[s]: chunk sums, a host scan over
        // chunks, lane offsets inside each chunk
        DevTemp t_sum, t_base;
        SIML_CUDA(cudaMalloc(&t_sum.p, (size_t)d.nchunks * 8));
        SIML_CUDA(cudaMalloc(&t_base.p, (size_t)d.nchunks * 8));
        k_rare_chunk<<<(unsigned)((d.nchunks + 7) / 8), 256, 0, st>>>(d.perm, rcount, d.nchunks,
                                                                      (int64_t*)t_sum.p);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        std::vector<int64_t> hs((size_t)d.nchunks);
        SIML_CUDA(cudaMemcpyAsync(hs.data(), t_sum.p, (size_t)d.nchunks * 8, cudaMemcpyDeviceToHost, st));
        SIML_CUDA(cudaStreamSynchronize(st));
        int64_t tot = 0;
        for (auto& x : hs) { const int64_t t = x; x = tot; tot += t; }
        SIML_CUDA(cudaMemcpyAsync(t_base.p, hs.data(), (size_t)d.nchunks * 8, cudaMemcpyHostToDevice, st));
        if ((rc = dev_alloc(&d.rare_off, (size_t)d.nchunks * 32 + 1))) return rc;
        if ((rc = dev_alloc(&d.rare_vid, (size_t)std::max<int64_t>(tot, 1)))) return rc;
        d.nrare = tot;
        k_rare_off<<<(unsigned)((d.nchunks + 7) / 8), 256, 0, st>>>(d.perm, rcount, d.nchunks,
                                                                    (const int64_t*)t_base.p, d.rare_off);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        SIML_CUDA(cudaStreamSynchronize(st));   // t_base is freed at scope end
    }
    SIML_CUDA(cudaMalloc(&d.entries, (size_t)std::max<int64_t>(acc, 1) * 16));
    SIML_CUDA(cudaMemsetAsync(d.entries, 0, (size_t)std::max<int64_t>(acc, 1) * 16, st));
    const unsigned grid = (unsigned)((d.nchunks * 32 + 255) / 256);
    const int bal = d.balanced ? 1 : 0;
    const int64_t ncommon = d.ncommon;
    if (d.entry_bytes == 2)
        k_fill_entries<uint16_t><<<grid, 256, 0, st>>>(q.lingos, q.counts, q.len, scount, q.width, d.perm, d.off,
                                                       d.ng, d.nchunks, bal, h->vocab.keys, h->vocab.vid,
                                                       h->vocab.cap, 0, (uint16_t*)d.entries, ncommon,
                                                       d.rare_off, d.rare_vid);
    else
        k_fill_entries<uint32_t><<<grid, 256, 0, st>>>(q.lingos, q.counts, q.len, scount, q.width, d.perm, d.off,
                                                       d.ng, d.nchunks, bal, h->vocab.keys, h->vocab.vid,
                                                       h->vocab.cap, d.offsets ? 2 : 0, (uint32_t*)d.entries,
                                                       ncommon, d.rare_off, d.rare_vid);
    h->launches++;
    SIML_CUDA(cudaGetLastError());
    SIML_CUDA(cudaStreamSynchronize(st));
    if (scheduled) return sched_arrange(h, d);
    return SIML_OK;
}

int build_rows(siml_engine* h) {
    free_rows(h->rows);
    const RawSet& r = h->ref;
    RowEntries& re = h->rows;
    re.n = r.n;
    re.stride = std::max<int64_t>(std::max<int64_t>(1, r.max_entries), h->row_stride_hint);
    int rc;
    if ((rc = dev_alloc(&re.vid, (size_t)(std::max<int64_t>(r.n, 1) * re.stride)))) return rc;
    // rare entries per row against the vocabulary's common set, the balanced
    // layout's and the scheduled layout's
    int max_rare[3] = {0, 0, 0};
    int* d_max = reinterpret_cast<int*>(h->d_counter);
    if (r.n > 0) {
        SIML_CUDA(cudaMemsetAsync(d_max, 0, 3 * sizeof(int), h->stream));
        k_row_entries<<<(unsigned)((r.n + 127) / 128), 128, 0, h->stream>>>(
            r.lingos, r.counts, r.len, r.n, r.width, h->vocab.keys, h->vocab.vid, h->vocab.cap, re.vid, re.stride,
            h->vocab.ncommon, balanced_ncommon(h), sched_ncommon(h), d_max);
        h->launches++;
        SIML_CUDA(cudaGetLastError());
        SIML_CUDA(cudaMemcpyAsync(max_rare, d_max, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    }
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    re.max_rare = max_rare[0];
    re.max_rare_bal = max_rare[1];
    re.max_rare_sched = max_rare[2];
    return SIML_OK;
}

}  // namespace

int ensure_prepared(siml_engine* h) {
    if (h->ref.n < 0 || h->qry.n < 0) return fail(SIML_ERR_STATE, "both the ref set (set_refsmiles) and the query set (set_qsmiles) must be set");
    int rc;
    if (!h->layout_valid) {
        h->rows_valid = false;
        h->nat_valid = h->sorted_valid = h->sched_valid = false;
        free_layout(h->db_nat);
        free_layout(h->db_sorted);
        free_layout(h->db_sched);
        if ((rc = build_vocab(h))) return rc;
        h->layout_valid = true;
    }
    if (!h->rows_valid) {
        if ((rc = build_rows(h))) return rc;
        h->rows_valid = true;
    }
    return SIML_OK;
}

int ensure_layout(siml_engine* h, bool sorted, const DbLayout** out) {
    int rc = ensure_prepared(h);
    if (rc) return rc;
    bool& valid = sorted ? h->sorted_valid : h->nat_valid;
    DbLayout& d = sorted ? h->db_sorted : h->db_nat;
    // a balanced full-matrix layout needs the per-warp pieces next to the
    // table; a ref set with longer rows (16 planes) may no longer fit
    if (valid && !sorted && d.balanced && !rows_balanced_fits(h)) valid = false;
    if (!valid) {
        if ((rc = build_layout(h, d, sorted))) return rc;
        valid = true;
    }
    *out = &d;
    return SIML_OK;
}

bool rows_use_sched(siml_engine* h) {
    return h->rows_layout == SIML_ROWS_SCHEDULED && h->rows_window == kChunk &&
           (h->rows_entries == SIML_ENTRIES_AUTO || h->rows_entries == SIML_ENTRIES_U16) && rows_sched_fits(h);
}

int ensure_sched_layout(siml_engine* h, const DbLayout** out) {
    int rc = ensure_prepared(h);
    if (rc) return rc;
    if (!h->sched_valid) {
        if ((rc = build_layout(h, h->db_sched, true, true))) {
            free_layout(h->db_sched);
            return rc;
        }
        h->sched_valid = true;
    }
    *out = &h->db_sched;
    return SIML_OK;
}

}  // namespace siml

namespace siml {

// Status (and message) of an asynchronous error word; the lowest set bit
// decides when several are set.
int async_error_status(int v) {
    if (!v) return SIML_OK;
    if (v & 1)
        return fail(SIML_ERR_TIMEOUT, "a top-k heap lock wait exceeded its bound in a queued call; that call's "
                    "result is invalid");
    if (v & 2)
        return fail(SIML_ERR_STATE, "a batched neighbour run met a work item outside its plan's extents and "
                    "skipped it; that run's result is invalid");
    return fail(SIML_ERR_STATE, "a ref row's entry list held a vid that fits neither the shared table nor the "
                "rare-vid hash; the entry was not used and the call's result is invalid");
}

int take_async_error(siml_engine* h) {
    volatile int* w = h->h_async_err;
    const int v = w ? *w : 0;
    if (!v) return SIML_OK;
    *w = 0;
    return async_error_status(v);
}

}  // namespace siml

using namespace siml;

#define SIML_GUARD(h)                                                   \
    do {                                                                \
        clear_error();                                                  \
        if (!(h)) return fail(SIML_ERR_INVALID, "NULL engine handle");  \
        cudaError_t _se = cudaSetDevice((h)->device);                   \
        if (_se != cudaSuccess) return cuda_fail(_se, "cudaSetDevice"); \
    } while (0)

extern "C" {

const char* siml_version(void) { return "siml_gb300 0.1 (sm_103a)"; }

int siml_create(int device, siml_engine** out) {
    clear_error();
    if (!out) return fail(SIML_ERR_INVALID, "siml_create: NULL output");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return fail(SIML_ERR_INVALID, "siml_create: no CUDA device %d (%d present)", device, ndev);
    SIML_CUDA(cudaSetDevice(device));
    siml_engine* h = new siml_engine();
    h->device = device;
    cudaDeviceProp prop;
    SIML_CUDA(cudaGetDeviceProperties(&prop, device));
    h->num_sms = prop.multiProcessorCount;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    SIML_CUDA(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;
    SIML_CUDA(cudaMalloc(&h->d_err, sizeof(int)));
    SIML_CUDA(cudaMalloc(&h->d_counter, 4 * sizeof(unsigned long long)));
    SIML_CUDA(cudaMalloc(&h->d_eval, sizeof(unsigned long long)));
    SIML_CUDA(cudaMemset(h->d_eval, 0, sizeof(unsigned long long)));
    SIML_CUDA(cudaHostAlloc((void**)&h->h_async_err, sizeof(int), cudaHostAllocMapped));
    *h->h_async_err = 0;
    SIML_CUDA(cudaHostGetDevicePointer((void**)&h->d_async_err, h->h_async_err, 0));
    SIML_CUDA(cudaEventCreate(&h->ev0));
    SIML_CUDA(cudaEventCreate(&h->ev1));
    noalloc_prepare(device);
    *out = h;
    return SIML_OK;
}

int siml_destroy(siml_engine* h) {
    clear_error();
    if (!h) return SIML_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_set(h->ref);
    free_set(h->qry);
    free_vocab(h->vocab);
    free_layout(h->db_nat);
    free_layout(h->db_sorted);
    free_layout(h->db_sched);
    free_rows(h->rows);
    for (int i = 0; i < 4; i++)
        if (h->scratch[i]) cudaFree(h->scratch[i]);
    if (h->d_err) cudaFree(h->d_err);
    if (h->h_async_err) cudaFreeHost(h->h_async_err);
    if (h->d_eval) cudaFree(h->d_eval);
    if (h->d_counter) cudaFree(h->d_counter);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return SIML_OK;
}

int siml_set_stream(siml_engine* h, void* stream) {
    SIML_GUARD(h);
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return SIML_OK;
}

int siml_sync(siml_engine* h) {
    SIML_GUARD(h);
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);
}

int siml_async_status(siml_engine* h) {
    SIML_GUARD(h);
    return take_async_error(h);
}

int siml_eval_pairs(siml_engine* h, uint64_t* out, int reset) {
    SIML_GUARD(h);
    if (!out) return fail(SIML_ERR_INVALID, "siml_eval_pairs: NULL output");
    unsigned long long v = 0;
    SIML_CUDA(cudaMemcpyAsync(&v, h->d_eval, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    if (reset) SIML_CUDA(cudaMemsetAsync(h->d_eval, 0, sizeof(v), h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    *out = (uint64_t)v;
    return SIML_OK;
}

int siml_query_done(siml_engine* h, int* done) {
    SIML_GUARD(h);
    if (!done) return fail(SIML_ERR_INVALID, "siml_query_done: NULL output");
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) { *done = 1; return SIML_OK; }
    if (e == cudaErrorNotReady) { *done = 0; return SIML_OK; }
    return cuda_fail(e, "cudaStreamQuery");
}

int siml_set_ref(siml_engine* h, const int32_t* lingos, const int32_t* counts, const int32_t* lengths,
                 const int32_t* mags, int64_t n, int64_t width, int64_t ld, int where) {
    SIML_GUARD(h);
    (void)where;
    h->rows_valid = false;
    h->generation++;
    return upload_set(h, h->ref, lingos, counts, lengths, mags, n, width, ld, "set_refsmiles");
}

int siml_write_ref_rows(siml_engine* h, int64_t row0, const int32_t* lingos, const int32_t* counts,
                        const int32_t* lengths, const int32_t* mags, int64_t n, int64_t width, int64_t ld) {
    SIML_GUARD(h);
    RawSet& s = h->ref;
    if (s.n < 0) return fail(SIML_ERR_STATE, "siml_write_ref_rows: no ref set (set_refsmiles first)");
    if (row0 < 0 || n < 0 || row0 + n > s.n)
        return fail(SIML_ERR_RANGE, "siml_write_ref_rows: rows [%lld, %lld) outside the ref set of %lld rows",
                    (long long)row0, (long long)(row0 + n), (long long)s.n);
    if (width < 0 || ld < width || width > s.width)
        return fail(SIML_ERR_INVALID, "siml_write_ref_rows: width %lld (ld %lld) does not fit the ref set's %lld",
                    (long long)width, (long long)ld, (long long)s.width);
    if (n == 0) return SIML_OK;
    if (!lengths || (width > 0 && (!lingos || !counts))) return fail(SIML_ERR_INVALID, "siml_write_ref_rows: NULL array");
    // validate on the host, so the write needs no read-back and stays queued
    int64_t mx = 0;
    for (int64_t r = 0; r < n; r++) {
        const int32_t L = lengths[r];
        if (L < 0 || L > width)
            return fail(SIML_ERR_INVALID, "siml_write_ref_rows: length %d of row %lld outside [0, %lld]", L,
                        (long long)r, (long long)width);
        long long sum = 0;
        for (int32_t j = 0; j < L; j++) {
            const int32_t c = counts[r * ld + j];
            if (c < 0) return fail(SIML_ERR_UNSUPPORTED, "siml_write_ref_rows: negative LINGO count");
            if (j > 0 && !(lingos[r * ld + j - 1] < lingos[r * ld + j]))
                return fail(SIML_ERR_UNSUPPORTED, "siml_write_ref_rows: LINGO codes of a molecule are not strictly "
                            "increasing (sorted unique codes are required, as the SMILES compiler produces)");
            sum += c;
        }
        if (sum > 0x7FFFFFFFll) return fail(SIML_ERR_UNSUPPORTED, "siml_write_ref_rows: overflowing LINGO counts");
        mx = std::max<int64_t>(mx, sum);
    }
    cudaStream_t st = h->stream;
    int32_t* dl = s.lingos + row0 * s.width;
    int32_t* dc = s.counts + row0 * s.width;
    if (width < s.width) {
        SIML_CUDA(cudaMemset2DAsync(dl, s.width * 4, 0, s.width * 4, n, st));
        SIML_CUDA(cudaMemset2DAsync(dc, s.width * 4, 0, s.width * 4, n, st));
    }
    if (width > 0) {
        SIML_CUDA(cudaMemcpy2DAsync(dl, s.width * 4, lingos, ld * 4, width * 4, n, cudaMemcpyHostToDevice, st));
        SIML_CUDA(cudaMemcpy2DAsync(dc, s.width * 4, counts, ld * 4, width * 4, n, cudaMemcpyHostToDevice, st));
    }
    SIML_CUDA(cudaMemcpyAsync(s.len + row0, lengths, n * 4, cudaMemcpyHostToDevice, st));
    // count sums on the device (the host copy above only validated them)
    k_set_stats<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dl, dc, s.len + row0, n, s.width, s.cmag + row0,
                                                            h->d_err, h->d_counter, h->d_counter + 1);
    h->launches++;
    SIML_CUDA(cudaGetLastError());
    if (mags) SIML_CUDA(cudaMemcpyAsync(s.mag + row0, mags, n * 4, cudaMemcpyHostToDevice, st));
    else SIML_CUDA(cudaMemcpyAsync(s.mag + row0, s.cmag + row0, n * 4, cudaMemcpyDeviceToDevice, st));
    s.max_entries = std::max(s.max_entries, mx);
    if (h->rows_valid) {
        if (mx > h->rows.stride) {
            h->rows_valid = false;   // rebuilt, wider, on next use
        } else {
            // with a split vocabulary the rows' rare-entry maximum decides
            // whether the table kernels may run, so it is read back (a
            // stream synchronization only for split vocabularies)
            int* d_max = reinterpret_cast<int*>(h->d_counter);
            if (h->vocab.split) SIML_CUDA(cudaMemsetAsync(d_max, 0, 3 * sizeof(int), st));
            k_row_entries<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(dl, dc, s.len + row0, n, s.width,
                                                                       h->vocab.keys, h->vocab.vid, h->vocab.cap,
                                                                       h->rows.vid + row0 * h->rows.stride,
                                                                       h->rows.stride, h->vocab.ncommon,
                                                                       balanced_ncommon(h), sched_ncommon(h), d_max);
            h->launches++;
            SIML_CUDA(cudaGetLastError());
            if (h->vocab.split) {
                int mr[3] = {0, 0, 0};
                SIML_CUDA(cudaMemcpyAsync(mr, d_max, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
                SIML_CUDA(cudaStreamSynchronize(st));
                h->rows.max_rare = std::max<int64_t>(h->rows.max_rare, mr[0]);
                h->rows.max_rare_bal = std::max<int64_t>(h->rows.max_rare_bal, mr[1]);
                h->rows.max_rare_sched = std::max<int64_t>(h->rows.max_rare_sched, mr[2]);
            }
        }
    }
    return SIML_OK;
}

int siml_set_query(siml_engine* h, const int32_t* lingos, const int32_t* counts, const int32_t* lengths,
                   const int32_t* mags, int64_t n, int64_t width, int64_t ld, int where) {
    SIML_GUARD(h);
    (void)where;
    h->layout_valid = false;
    h->rows_valid = false;
    h->generation++;
    return upload_set(h, h->qry, lingos, counts, lengths, mags, n, width, ld, "set_qsmiles");
}

int siml_set_sizes(siml_engine* h, int64_t* nref, int64_t* nquery) {
    SIML_GUARD(h);
    if (nref) *nref = h->ref.n;
    if (nquery) *nquery = h->qry.n;
    return SIML_OK;
}

int siml_db_stats(siml_engine* h, int64_t out[8]) {
    SIML_GUARD(h);
    if (!out) return fail(SIML_ERR_INVALID, "siml_db_stats: NULL output");
    const DbLayout* d = nullptr;
    int rc = ensure_prepared(h);
    if (rc) return rc;
    // the layout getMultipleRows streams
    rc = rows_use_sched(h) ? ensure_sched_layout(h, &d) : ensure_layout(h, false, &d);
    if (rc) return rc;
    out[0] = h->vocab.nvid;
    out[1] = d->entry_bytes;
    out[2] = d->ngroups_total;
    out[3] = d->nchunks;
    out[4] = d->max_ng;
    out[5] = d->n;
    out[6] = h->ref.max_entries;
    out[7] = h->qry.max_entries;
    return SIML_OK;
}

int siml_rows_info(siml_engine* h, int64_t out[4]) {
    SIML_GUARD(h);
    if (!out) return fail(SIML_ERR_INVALID, "siml_rows_info: NULL output");
    int rc = ensure_prepared(h);
    if (rc) return rc;
    out[0] = out[1] = out[2] = out[3] = 0;
    if (!rows_use_sched(h)) return SIML_OK;
    const DbLayout* d = nullptr;
    if ((rc = ensure_sched_layout(h, &d))) return rc;
    out[0] = 1;
    out[1] = d->nitems;
    out[2] = d->nwin;
    out[3] = d->max_item_steps;
    return SIML_OK;
}

int siml_rows_vocab(siml_engine* h, int64_t out[4]) {
    SIML_GUARD(h);
    if (!out) return fail(SIML_ERR_INVALID, "siml_rows_vocab: NULL output");
    int rc = ensure_prepared(h);
    if (rc) return rc;
    out[0] = out[1] = out[2] = 0;
    out[3] = -1;
    if (!rows_use_sched(h)) return SIML_OK;
    const DbLayout* d = nullptr;
    if ((rc = ensure_sched_layout(h, &d))) return rc;
    out[0] = d->ncommon;
    out[1] = d->nrare;
    out[2] = h->rows.max_rare_sched;
    out[3] = h->rows_rare_gen == h->generation ? h->rows_rare_path : -1;
    return SIML_OK;
}

int siml_vocab_stats(siml_engine* h, int64_t out[4]) {
    SIML_GUARD(h);
    if (!out) return fail(SIML_ERR_INVALID, "siml_vocab_stats: NULL output");
    const DbLayout* d = nullptr;
    int rc = ensure_layout(h, true, &d);
    if (rc) return rc;
    out[0] = h->vocab.nvid;
    out[1] = h->vocab.ncommon;
    out[2] = d->nrare;
    out[3] = h->rows.max_rare;
    return SIML_OK;
}

int siml_set_tuning(siml_engine* h, int key, int64_t value) {
    SIML_GUARD(h);
    switch (key) {
    case SIML_TUNE_ROWS_WINDOW:
        if (value != 32 && value != 64 && value != 128 && value != 256)
            return fail(SIML_ERR_INVALID, "rows window must be 32, 64, 128 or 256 (got %lld)", (long long)value);
        if (value != h->rows_window) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            free_layout(h->db_nat);
            h->nat_valid = false;
            h->rows_window = (int)value;
        }
        return SIML_OK;
    case SIML_TUNE_ROWS_LAYOUT:
        if (value != SIML_ROWS_PADDED && value != SIML_ROWS_BALANCED && value != SIML_ROWS_SCHEDULED)
            return fail(SIML_ERR_INVALID, "rows layout must be SIML_ROWS_PADDED, SIML_ROWS_BALANCED or "
                        "SIML_ROWS_SCHEDULED (got %lld)", (long long)value);
        if (value != h->rows_layout) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            free_layout(h->db_nat);
            free_layout(h->db_sched);
            h->nat_valid = h->sched_valid = false;
            h->rows_layout = (int)value;
        }
        return SIML_OK;
    case SIML_TUNE_SORT_WINDOW:
        if (value < 64 || value > kMaxWindow || (value & (value - 1)))
            return fail(SIML_ERR_INVALID, "sort window must be a power of two in [64, %d] (got %lld)", kMaxWindow,
                        (long long)value);
        if (value != h->sorted_window) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            free_layout(h->db_sorted);
            h->sorted_valid = false;
            h->sorted_window = (int)value;
            h->generation++;   // plans hold chunk ranges of the old layout
        }
        return SIML_OK;
    case SIML_TUNE_ROW_STRIDE:
        if (value < 0 || value > (1 << 20))
            return fail(SIML_ERR_INVALID, "row stride hint must be in [0, 2^20] (got %lld)", (long long)value);
        if (value > h->row_stride_hint && h->rows_valid && value > h->rows.stride) h->rows_valid = false;
        h->row_stride_hint = value;
        return SIML_OK;
    case SIML_TUNE_SCHED_GROUPS:
        if (value != 2 && value != 4)
            return fail(SIML_ERR_INVALID, "scheduled kernel warp groups must be 2 or 4 (got %lld)", (long long)value);
        if (value != h->sched_groups) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            free_layout(h->db_sched);
            h->sched_valid = false;
            h->sched_groups = (int)value;
        }
        return SIML_OK;
    case SIML_TUNE_RARE_FIXUP:
        if (value != 0 && value != 1)
            return fail(SIML_ERR_INVALID, "rare fix-up must be 0 or 1 (got %lld)", (long long)value);
        h->rare_fixup = (int)value;
        return SIML_OK;
    case SIML_TUNE_SCHED_ROWS:
        if (value != 32 && value != 64)
            return fail(SIML_ERR_INVALID, "scheduled kernel rows per group must be 32 or 64 (got %lld)",
                        (long long)value);
        if (value != h->sched_rows) {
            // the vocabulary's numbering depends on the table the kernel holds:
            // everything derived from the query set is rebuilt on next use
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            h->layout_valid = false;
            h->sched_rows = (int)value;
            h->generation++;   // plans hold vids of the old numbering
        }
        return SIML_OK;
    case SIML_TUNE_ROWS_ENTRIES:
        if (value < SIML_ENTRIES_AUTO || value > SIML_ENTRIES_OFFSETS)
            return fail(SIML_ERR_INVALID, "rows entry format must be 0..3 (got %lld)", (long long)value);
        if (value != h->rows_entries) {
            SIML_CUDA(cudaStreamSynchronize(h->stream));
            free_layout(h->db_nat);
            h->nat_valid = false;
            h->rows_entries = (int)value;
        }
        return SIML_OK;
    default:
        return fail(SIML_ERR_INVALID, "unknown tuning key %d", key);
    }
}

int siml_get_tuning(siml_engine* h, int key, int64_t* value) {
    SIML_GUARD(h);
    if (!value) return fail(SIML_ERR_INVALID, "siml_get_tuning: NULL output");
    switch (key) {
    case SIML_TUNE_ROWS_WINDOW: *value = h->rows_window; return SIML_OK;
    case SIML_TUNE_ROWS_ENTRIES: *value = h->rows_entries; return SIML_OK;
    case SIML_TUNE_ROW_STRIDE: *value = h->row_stride_hint; return SIML_OK;
    case SIML_TUNE_SORT_WINDOW: *value = h->sorted_window; return SIML_OK;
    case SIML_TUNE_ROWS_LAYOUT: *value = h->rows_layout; return SIML_OK;
    case SIML_TUNE_SCHED_GROUPS: *value = h->sched_groups; return SIML_OK;
    case SIML_TUNE_SCHED_ROWS: *value = h->sched_rows; return SIML_OK;
    case SIML_TUNE_RARE_FIXUP: *value = h->rare_fixup; return SIML_OK;
    default: return fail(SIML_ERR_INVALID, "unknown tuning key %d", key);
    }
}

int64_t siml_launch_count(siml_engine* h) { return h ? h->launches : -1; }

int siml_mem_info(siml_engine* h, int64_t* free_bytes, int64_t* total_bytes) {
    SIML_GUARD(h);
    size_t f = 0, t = 0;
    SIML_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (int64_t)f;
    if (total_bytes) *total_bytes = (int64_t)t;
    return SIML_OK;
}

int siml_debug_fail_alloc(int64_t nth) {
    clear_error();
    if (nth < 0) return fail(SIML_ERR_INVALID, "siml_debug_fail_alloc: nth must be >= 0");
    siml::g_fail_alloc.store(nth);
    return SIML_OK;
}

int siml_debug_async_status(int word) {
    clear_error();
    return async_error_status(word);
}

int siml_debug_set_row_vid(siml_engine* h, int64_t row, int64_t pos, uint32_t vid) {
    SIML_GUARD(h);
    int rc = ensure_prepared(h);
    if (rc) return rc;
    if (row < 0 || row >= h->rows.n || pos < 0 || pos >= h->rows.stride)
        return fail(SIML_ERR_RANGE, "siml_debug_set_row_vid: entry (%lld, %lld) outside the row lists",
                    (long long)row, (long long)pos);
    SIML_CUDA(cudaMemcpyAsync(h->rows.vid + row * h->rows.stride + pos, &vid, sizeof(uint32_t),
                              cudaMemcpyHostToDevice, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return SIML_OK;
}

double siml_last_kernel_ms(siml_engine* h) {
    if (!h || !h->timed) return 0.0;
    float ms = 0.f;
    if (cudaEventSynchronize(h->ev1) != cudaSuccess) return 0.0;
    if (cudaEventElapsedTime(&ms, h->ev0, h->ev1) != cudaSuccess) return 0.0;
    return (double)ms;
}

static int rows_common(siml_engine* h, int64_t rowbase, int64_t rowlimit, float* out, int64_t ldo,
                       int where, int mode) {
    int rc;
    if ((rc = ensure_prepared(h))) return rc;
    if (rowbase < 0 || rowlimit > h->ref.n || rowlimit < rowbase)
        return fail(SIML_ERR_RANGE, "row range [%lld, %lld) outside the ref set of %lld rows",
                    (long long)rowbase, (long long)rowlimit, (long long)h->ref.n);
    const int64_t rows = rowlimit - rowbase, nq = h->qry.n;
    if (ldo < nq) return fail(SIML_ERR_INVALID, "output row stride %lld < query set size %lld", (long long)ldo, (long long)nq);
    if (rows == 0 || nq == 0) return SIML_OK;
    if (!out) return fail(SIML_ERR_INVALID, "NULL output");
    RowsArgs a{rowbase, rowlimit, out, ldo, mode};
    if (where == SIML_DEVICE) return launch_rows(h, a);
    if (where != SIML_HOST && where != SIML_HOST_QUEUED)
        return fail(SIML_ERR_INVALID, "unknown output location %d", where);
    // Pinned host memory mapped for the device: the kernels write the block
    // there directly, over the host link, instead of into a device buffer
    // that a copy then moves (the link bounds both; the direct write saves
    // the device buffer and the copy's start-up).
    float* mapped = nullptr;
    {
        cudaPointerAttributes attr;
        if (cudaPointerGetAttributes(&attr, out) == cudaSuccess) {
            if (attr.type == cudaMemoryTypeHost && attr.devicePointer) mapped = (float*)attr.devicePointer;
        } else {
            cudaGetLastError();   // not a pointer the runtime knows: plain host memory
        }
    }
    if (where == SIML_HOST_QUEUED && !mapped)
        return fail(SIML_ERR_INVALID, "SIML_HOST_QUEUED output must be pinned host memory mapped for the device");
    if (mapped) {
        a.out = mapped;
        if ((rc = launch_rows(h, a))) return rc;
        if (where == SIML_HOST_QUEUED) return SIML_OK;
        SIML_CUDA(cudaStreamSynchronize(h->stream));
        return take_async_error(h);
    }
    void* dbuf = nullptr;
    if ((rc = scratch_reserve(h, (size_t)(rows * nq) * sizeof(float), &dbuf))) return rc;
    a.out = (float*)dbuf;
    a.ldo = nq;
    if ((rc = launch_rows(h, a))) return rc;
    SIML_CUDA(cudaMemcpy2DAsync(out, ldo * 4, dbuf, nq * 4, nq * 4, rows, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);   // a table build that met an unusable row entry
}

int siml_rows(siml_engine* h, int64_t rowbase, int64_t rowlimit, float* out, int64_t ldo, int where) {
    SIML_GUARD(h);
    return rows_common(h, rowbase, rowlimit, out, ldo, where, kModeRows);
}

int siml_neighbors_range(siml_engine* h, int64_t rowbase, int64_t rowlimit, int64_t col_begin, int64_t col_end,
                         float lo, float hi, int64_t pitch, int32_t* idx, float* sims, int32_t* counts, int where) {
    SIML_GUARD(h);
    int rc;
    if ((rc = ensure_prepared(h))) return rc;
    if (rowbase < 0 || rowlimit > h->ref.n || rowlimit < rowbase)
        return fail(SIML_ERR_RANGE, "row range [%lld, %lld) outside the ref set of %lld rows",
                    (long long)rowbase, (long long)rowlimit, (long long)h->ref.n);
    if (col_begin < 0 || col_end > h->qry.n || col_end < col_begin)
        return fail(SIML_ERR_RANGE, "column range [%lld, %lld) outside the query set of %lld molecules",
                    (long long)col_begin, (long long)col_end, (long long)h->qry.n);
    if (pitch < 0 || pitch > 0x7FFFFFFFll) return fail(SIML_ERR_INVALID, "siml_neighbors: bad pitch %lld", (long long)pitch);
    const int64_t rows = rowlimit - rowbase;
    if (rows == 0) return SIML_OK;
    if (!counts || (pitch > 0 && !idx)) return fail(SIML_ERR_INVALID, "siml_neighbors: NULL output");
    NbrCall c{rowbase, rowlimit, col_begin, col_end, lo, hi, pitch, idx, sims, counts};
    if (where == SIML_DEVICE) return launch_neighbors(h, c);
    const size_t ib = (size_t)(rows * pitch) * 4, cb = (size_t)rows * 4;
    const size_t need = ((ib + 255) / 256 * 256) * (sims ? 2 : 1) + cb;
    void* buf = nullptr;
    if ((rc = scratch_reserve(h, need, &buf))) return rc;
    char* b = (char*)buf;
    c.idx = (int32_t*)b;
    c.sims = sims ? (float*)(b + (ib + 255) / 256 * 256) : nullptr;
    c.counts = (int32_t*)(b + ((ib + 255) / 256 * 256) * (sims ? 2 : 1));
    if ((rc = launch_neighbors(h, c))) return rc;
    if (ib) SIML_CUDA(cudaMemcpyAsync(idx, c.idx, ib, cudaMemcpyDefault, h->stream));
    if (ib && sims) SIML_CUDA(cudaMemcpyAsync(sims, c.sims, ib, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaMemcpyAsync(counts, c.counts, cb, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);   // a table build that met an unusable row entry
}

int siml_neighbors(siml_engine* h, int64_t rowbase, int64_t rowlimit, float lo, float hi, int64_t pitch,
                   int32_t* idx, float* sims, int32_t* counts, int where) {
    SIML_GUARD(h);
    return siml_neighbors_range(h, rowbase, rowlimit, 0, h->qry.n < 0 ? 0 : h->qry.n, lo, hi, pitch, idx, sims,
                                counts, where);
}

static int check_range(siml_engine* h, int64_t rowbase, int64_t rowlimit) {
    if (rowbase < 0 || rowlimit > h->ref.n || rowlimit < rowbase)
        return fail(SIML_ERR_RANGE, "row range [%lld, %lld) outside the ref set of %lld rows",
                    (long long)rowbase, (long long)rowlimit, (long long)h->ref.n);
    return SIML_OK;
}

int siml_hist101(siml_engine* h, int64_t rowbase, int64_t rowlimit, int32_t* out, int64_t ldo, int where) {
    SIML_GUARD(h);
    int rc;
    if ((rc = ensure_prepared(h))) return rc;
    if ((rc = check_range(h, rowbase, rowlimit))) return rc;
    if (ldo < 101) return fail(SIML_ERR_INVALID, "siml_hist101: row stride %lld < 101", (long long)ldo);
    const int64_t rows = rowlimit - rowbase;
    if (rows == 0) return SIML_OK;
    if (!out) return fail(SIML_ERR_INVALID, "siml_hist101: NULL output");
    if (where == SIML_DEVICE) return launch_hist(h, rowbase, rowlimit, false, out, ldo);
    void* buf = nullptr;
    if ((rc = scratch_reserve(h, (size_t)rows * 101 * 4, &buf))) return rc;
    if ((rc = launch_hist(h, rowbase, rowlimit, false, buf, 101))) return rc;
    SIML_CUDA(cudaMemcpy2DAsync(out, ldo * 4, buf, 101 * 4, 101 * 4, rows, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);   // a table build that met an unusable row entry
}

int siml_hist_global(siml_engine* h, int64_t rowbase, int64_t rowlimit, uint64_t* out, int where) {
    SIML_GUARD(h);
    int rc;
    if ((rc = ensure_prepared(h))) return rc;
    if ((rc = check_range(h, rowbase, rowlimit))) return rc;
    if (!out) return fail(SIML_ERR_INVALID, "siml_hist_global: NULL output");
    if (rowlimit == rowbase) return SIML_OK;
    if (where == SIML_DEVICE) return launch_hist(h, rowbase, rowlimit, true, out, 0);
    void* buf = nullptr;
    if ((rc = scratch_reserve(h, 1000 * 8, &buf))) return rc;
    SIML_CUDA(cudaMemcpyAsync(buf, out, 1000 * 8, cudaMemcpyDefault, h->stream));
    if ((rc = launch_hist(h, rowbase, rowlimit, true, buf, 0))) return rc;
    SIML_CUDA(cudaMemcpyAsync(out, buf, 1000 * 8, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);   // a table build that met an unusable row entry
}

static int row_hist_common(siml_engine* h, const void* data, bool f64, int64_t rows, int64_t cols, int64_t ld,
                           uint32_t* hist, int where) {
    SIML_GUARD(h);
    if (rows < 0 || cols < 0 || ld < cols) return fail(SIML_ERR_INVALID, "rowHistogram101: bad shape");
    if (rows == 0) return SIML_OK;
    if (!data || !hist) return fail(SIML_ERR_INVALID, "rowHistogram101: NULL array");
    if (where == SIML_DEVICE) return launch_row_hist101(h, data, f64, rows, cols, ld, hist);
    const size_t es = f64 ? 8 : 4;
    const size_t in_bytes = (size_t)rows * cols * es, out_bytes = (size_t)rows * 101 * 4;
    void* buf = nullptr;
    int rc;
    if ((rc = scratch_reserve(h, (in_bytes + 255) / 256 * 256 + out_bytes, &buf))) return rc;
    char* b = (char*)buf;
    uint32_t* dh = (uint32_t*)(b + (in_bytes + 255) / 256 * 256);
    if (cols) SIML_CUDA(cudaMemcpy2DAsync(b, cols * es, data, ld * es, cols * es, rows, cudaMemcpyDefault, h->stream));
    if ((rc = launch_row_hist101(h, b, f64, rows, cols, cols, dh))) return rc;
    SIML_CUDA(cudaMemcpyAsync(hist, dh, out_bytes, cudaMemcpyDefault, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return SIML_OK;
}

int siml_row_histogram101(siml_engine* h, const float* data, int64_t rows, int64_t cols, int64_t ld,
                          uint32_t* hist, int where) {
    return row_hist_common(h, data, false, rows, cols, ld, hist, where);
}

int siml_row_histogram101_f64(siml_engine* h, const double* data, int64_t rows, int64_t cols, int64_t ld,
                              uint32_t* hist, int where) {
    return row_hist_common(h, data, true, rows, cols, ld, hist, where);
}

int siml_topk(siml_engine* h, int64_t rowbase, int64_t rowlimit, int64_t k, int32_t* idx, float* sims, int where) {
    SIML_GUARD(h);
    int rc;
    if ((rc = ensure_prepared(h))) return rc;
    if ((rc = check_range(h, rowbase, rowlimit))) return rc;
    if (k < 1 || k > (1 << 20)) return fail(SIML_ERR_INVALID, "siml_topk: k = %lld out of range", (long long)k);
    const int64_t rows = rowlimit - rowbase;
    if (rows == 0) return SIML_OK;
    if (!idx || !sims) return fail(SIML_ERR_INVALID, "siml_topk: NULL output");
    int32_t* di = idx;
    float* ds = sims;
    const size_t ob = (size_t)rows * k * 4;
    void* own = nullptr;
    if (where != SIML_DEVICE) {
        SIML_CUDA(cudaMallocAsync(&own, 2 * ob, h->stream));
        di = (int32_t*)own;
        ds = (float*)((char*)own + ob);
    }
    rc = launch_topk(h, rowbase, rowlimit, (int)k, di, ds);
    if (!rc && where != SIML_DEVICE) {
        SIML_CUDA(cudaMemcpyAsync(idx, di, ob, cudaMemcpyDefault, h->stream));
        SIML_CUDA(cudaMemcpyAsync(sims, ds, ob, cudaMemcpyDefault, h->stream));
        SIML_CUDA(cudaStreamSynchronize(h->stream));
    }
    if (own) cudaFreeAsync(own, h->stream);
    if (rc) return rc;
    // device outputs: queued only; a bounded lock wait that expired is
    // reported by the next siml_sync / siml_async_status
    return where == SIML_DEVICE ? SIML_OK : take_async_error(h);
}

int siml_row_single(siml_engine* h, int64_t row, float* out, int where) {
    SIML_GUARD(h);
    return rows_common(h, row, row + 1, out, h->qry.n, where, kModeSingle);
}

}  // extern "C"
