// Batched ragged neighbour jobs: plan once, run many times.
//
// A job is a range of ref rows searched against a range of database columns
// with getNeighbors' rule (pysiml/kernels.py:393-475).  The reference issues
// one getNeighbors call per job (pysiml/GPULingo.py:467-513); here a plan
// turns all jobs into work items of at most 32 rows (each job's rows ordered
// by magnitude) x a chunk range of the window-sorted layout, largest first,
// and a persistent kernel pulls them from a device queue.  siml_batch_run only enqueues work on the
// caller's stream (no host synchronization, no allocation), so it can be
// captured in a CUDA graph and replayed.
//
// The plan's shape has three parts: the chunk range of one work item
// (tile_chunks), the most ref rows one item takes (rows_cap, 16 or 32: fewer
// rows per table, more items in flight) and the jobs given to the per-pair
// merge instead of the table kernel (merge_rows: jobs of at most that many
// rows, recomputed by the ordered finish kernel).  With tile_chunks <= 0 the
// plan times candidate shapes on a sample of the jobs (tiles first, then the
// row cap, then the merge cut-off) and keeps the fastest; the choice is kept
// per database length distribution and job shape (a signature of both), so
// later plans of the same kind reuse it without timing.  siml_batch_shape
// reports the choice.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.h"

struct siml_batch {
    siml_engine* h = nullptr;
    const siml::DbLayout* d = nullptr;
    uint64_t generation = 0;
    int4* items = nullptr;        // 2 per item
    int32_t* order = nullptr;     // each job's ref rows, ordered by magnitude
    int64_t order_len = 0;
    int64_t nitems = 0;
    int4* rowinfo = nullptr;      // per output row
    int64_t rows_out = 0;
    unsigned int* head = nullptr;
    float lo = 0.f, hi = 0.f;
    int64_t pitch = 0;
    int64_t tile_chunks = 0;
    int64_t rows_cap = 32;
    int64_t merge_rows = 0;
    int from_cache = 0;
    int64_t stream_bytes = 0;
    int64_t unique_bytes = 0;
};

namespace siml {
namespace {

struct HostJob {
    int64_t rb, re, cb, ce, out;
};

// Orders each job's rows by magnitude into `order` (ref rows, stably) and
// cuts each job into items of at most 32 consecutive ordered rows x `tile`
// chunks, largest items first.  Rows of one item then have close
// magnitudes, so whole chunks out of the bound's reach are skipped.
struct Shape {
    int64_t tile = 128;
    int64_t rows_cap = 32;
    int64_t merge_rows = 0;
};

void make_items(const DbLayout* d, const std::vector<HostJob>& jobs, const std::vector<int32_t>& mag,
                const Shape& sh, std::vector<int4>& items, std::vector<int32_t>& order) {
    const int64_t tile = sh.tile;
    struct It {
        int4 a, b;
        int64_t cost;
    };
    std::vector<It> v;
    order.clear();
    for (const HostJob& j : jobs) {
        if (j.re <= j.rb || j.ce <= j.cb) continue;
        if (j.re - j.rb <= sh.merge_rows) continue;   // the ordered finish kernel computes it
        const int64_t pos0 = (int64_t)order.size();
        for (int64_t r = j.rb; r < j.re; r++) order.push_back((int32_t)r);
        std::stable_sort(order.begin() + pos0, order.end(),
                         [&](int32_t x, int32_t y) { return mag[(size_t)x] < mag[(size_t)y]; });
        int64_t c0, c1;
        sorted_chunk_range(d, j.cb, j.ce, c0, c1);
        const int64_t nrows = j.re - j.rb;
        for (int64_t r = 0; r < nrows; r += sh.rows_cap) {
            const int nr = (int)std::min<int64_t>(sh.rows_cap, nrows - r);
            for (int64_t c = c0; c < c1; c += tile) {
                const int64_t ce = std::min(c1, c + tile);
                It it;
                it.a = make_int4((int)(pos0 + r), nr, (int)(j.out - j.rb), (int)j.cb);
                it.b = make_int4((int)j.ce, (int)c, (int)ce, 0);
                it.cost = (int64_t)(ce - c) * (16 + nr);
                v.push_back(it);
            }
        }
    }
    std::stable_sort(v.begin(), v.end(), [](const It& x, const It& y) { return x.cost > y.cost; });
    items.resize(v.size() * 2);
    for (size_t i = 0; i < v.size(); i++) {
        items[2 * i] = v[i].a;
        items[2 * i + 1] = v[i].b;
    }
}

// Copies on the engine's stream and waits, so kernels queued there later see
// the data (the engine's stream need not synchronize with the legacy one).
template <typename T>
int upload_items(siml_engine* h, const std::vector<T>& items, T** out) {
    *out = nullptr;
    SIML_CUDA(cudaMalloc((void**)out, std::max<size_t>(items.size(), 2) * sizeof(T)));
    if (!items.empty()) {
        SIML_CUDA(cudaMemcpyAsync(*out, items.data(), items.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
        SIML_CUDA(cudaStreamSynchronize(h->stream));
    }
    return SIML_OK;
}

// The ref set's magnitudes on the host (plans order each job's rows by them).
int host_mags(siml_engine* h, std::vector<int32_t>& mag) {
    mag.resize((size_t)std::max<int64_t>(h->ref.n, 0));
    if (!mag.empty()) {
        SIML_CUDA(cudaMemcpyAsync(mag.data(), h->ref.mag, mag.size() * 4, cudaMemcpyDeviceToHost, h->stream));
        SIML_CUDA(cudaStreamSynchronize(h->stream));
    }
    return SIML_OK;
}

// Rows of the jobs given to the per-pair merge carry w = 1 in their row
// info (the finish kernel recomputes them in order).
void mark_merge_rows(const std::vector<HostJob>& jobs, int64_t merge_rows, std::vector<int4>& rowinfo) {
    for (const HostJob& j : jobs)
        if (j.re > j.rb && j.re - j.rb <= merge_rows)
            for (int64_t r = j.rb; r < j.re; r++) rowinfo[(size_t)(j.out + r - j.rb)].w = 1;
}

// Times the plan on a sample of the jobs for a sequence of candidate shapes
// and returns the fastest: tiles first (row cap 32, no merge jobs), then the
// row cap 16 at the best tile, then merge cut-offs.  The sample takes jobs
// at an even stride until it holds about kTuneBudget pairs, so tuning costs a
// fraction of a second whatever the batch size.
constexpr double kTuneBudget = 1.0e10;

int autotune_shape(siml_engine* h, const DbLayout* d, const std::vector<HostJob>& jobs,
                   const std::vector<int32_t>& mag, float lo, float hi, int64_t pitch, Shape* best_shape) {
    static const int64_t tiles[] = {64, 128, 256, 512, 1024, 2048, 4096, 8192};
    static const int64_t merges[] = {1, 2, 4, 8};
    std::vector<HostJob> sample;
    int64_t rows = 0;
    double pairs = 0.0;
    const size_t n = jobs.size();
    const size_t stride = n > 64 ? 61 : 1;   // coprime to typical sizes, visits every job once
    for (size_t k = 0, i = 0; k < n && pairs < kTuneBudget; k++, i = (i + stride) % n) {
        HostJob j = jobs[i];
        const double jp = (double)(j.re - j.rb) * (double)(j.ce - j.cb);
        if (jp <= 0.0 || (pairs > 0.0 && pairs + jp > 2.0 * kTuneBudget)) continue;
        j.out = rows;
        rows += j.re - j.rb;
        pairs += jp;
        sample.push_back(j);
    }
    *best_shape = Shape();
    if (rows == 0) return SIML_OK;
    std::vector<int4> rowinfo0((size_t)rows, make_int4(-1, 0, 0, 0));
    for (const HostJob& j : sample)
        for (int64_t r = j.rb; r < j.re; r++)
            rowinfo0[(size_t)(j.out + r - j.rb)] = make_int4((int)r, (int)j.cb, (int)j.ce, 0);
    int4* d_rowinfo = nullptr;
    int32_t *d_idx = nullptr, *d_cnt = nullptr;
    unsigned int* d_head = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = SIML_OK;
    auto cleanup = [&]() {
        if (d_rowinfo) cudaFree(d_rowinfo);
        if (d_idx) cudaFree(d_idx);
        if (d_cnt) cudaFree(d_cnt);
        if (d_head) cudaFree(d_head);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc((void**)&d_rowinfo, rowinfo0.size() * sizeof(int4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_idx, (size_t)rows * (size_t)std::max<int64_t>(pitch, 1) * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_cnt, (size_t)rows * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_head, sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "batch autotune set-up");
    }
    bool warmed = false;
    // time of one run of the sample with shape sh (ms), or a negative status
    auto time_shape = [&](const Shape& sh, double* ms_out) -> int {
        std::vector<int4> items, rowinfo = rowinfo0;
        std::vector<int32_t> order;
        make_items(d, sample, mag, sh, items, order);
        mark_merge_rows(sample, sh.merge_rows, rowinfo);
        int4* d_items = nullptr;
        int32_t* d_order = nullptr;
        int r2 = upload_items(h, items, &d_items);
        if (!r2) r2 = upload_items(h, order, &d_order);
        if (!r2 && cudaMemcpyAsync(d_rowinfo, rowinfo.data(), rowinfo.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                   h->stream) != cudaSuccess)
            r2 = fail(SIML_ERR_CUDA, "batch autotune upload");
        const int64_t ni = (int64_t)items.size() / 2;
        if (!r2 && !warmed) {   // the first launch pays one-time costs; keep it out of the comparison
            r2 = launch_batch_neighbors(h, d, d_items, ni, d_head, d_order, (int64_t)order.size(), d_rowinfo, rows,
                                        lo, hi, pitch, d_idx, nullptr, d_cnt, h->stream);
            warmed = true;
        }
        if (!r2) {
            cudaEventRecord(e0, h->stream);
            r2 = launch_batch_neighbors(h, d, d_items, ni, d_head, d_order, (int64_t)order.size(), d_rowinfo, rows,
                                        lo, hi, pitch, d_idx, nullptr, d_cnt, h->stream);
            cudaEventRecord(e1, h->stream);
        }
        cudaError_t e2 = cudaEventSynchronize(e1);
        if (d_items) cudaFree(d_items);
        if (d_order) cudaFree(d_order);
        if (r2) return r2;
        if (e2 != cudaSuccess) return cuda_fail(e2, "batch autotune");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *ms_out = ms;
        return SIML_OK;
    };
    double best = 1e300;
    Shape cur;
    for (int64_t t : tiles) {
        cur.tile = t;
        double ms = 0.0;
        if ((rc = time_shape(cur, &ms))) break;
        if (ms < best * 0.98) { best = ms; *best_shape = cur; }
    }
    if (!rc) {
        cur = *best_shape;
        cur.rows_cap = 16;
        double ms = 0.0;
        rc = time_shape(cur, &ms);
        if (!rc && ms < best * 0.98) { best = ms; *best_shape = cur; }
    }
    for (int64_t m : merges) {
        if (rc) break;
        cur = *best_shape;
        cur.merge_rows = m;
        double ms = 0.0;
        if ((rc = time_shape(cur, &ms))) break;
        if (ms < best * 0.98) { best = ms; *best_shape = cur; }
    }
    cleanup();
    return rc;
}

// Shapes chosen by the timing, per (database length distribution, job
// shape, bound) signature, for the whole process.
std::mutex g_shape_mu;
std::map<std::tuple<int64_t, int64_t, int64_t, int64_t, int64_t, int64_t>, Shape> g_shapes;

// Signature of a plan's kind: the database's mean 8-entry steps per chunk
// (quarter steps) and their spread (tenths of the mean), its size (log2),
// the jobs' median rows and columns (log2) and the bound (hundredths).
int plan_signature(siml_engine* h, const DbLayout* d, const std::vector<HostJob>& jobs, float lo,
                   std::tuple<int64_t, int64_t, int64_t, int64_t, int64_t, int64_t>* sig) {
    std::vector<int32_t> ng((size_t)std::max<int64_t>(d->nchunks, 1), 0);
    if (d->nchunks > 0) {
        SIML_CUDA(cudaMemcpyAsync(ng.data(), d->ng, (size_t)d->nchunks * 4, cudaMemcpyDeviceToHost, h->stream));
        SIML_CUDA(cudaStreamSynchronize(h->stream));
    }
    double sum = 0.0, sq = 0.0;
    for (int64_t c = 0; c < d->nchunks; c++) {
        sum += ng[(size_t)c];
        sq += (double)ng[(size_t)c] * ng[(size_t)c];
    }
    const double nc = (double)std::max<int64_t>(d->nchunks, 1);
    const double mean = sum / nc, sd = std::sqrt(std::max(0.0, sq / nc - mean * mean));
    std::vector<int64_t> r, c;
    for (const HostJob& j : jobs) {
        r.push_back(j.re - j.rb);
        c.push_back(j.ce - j.cb);
    }
    auto median_log2 = [](std::vector<int64_t>& v) -> int64_t {
        if (v.empty()) return -1;
        std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
        int64_t x = std::max<int64_t>(v[v.size() / 2], 1), b = 0;
        while ((1ll << (b + 1)) <= x) b++;
        return b;
    };
    int64_t nlog = 0;
    while ((1ll << (nlog + 1)) <= std::max<int64_t>(d->n, 1)) nlog++;
    *sig = std::make_tuple((int64_t)std::llround(mean * 4.0), (int64_t)std::llround(mean > 0 ? 10.0 * sd / mean : 0),
                           nlog, median_log2(r), median_log2(c), (int64_t)std::llround((double)lo * 100.0));
    return SIML_OK;
}

// Sets *bad when a ref row named by the plan holds a vid outside the
// database vocabulary (1..limit) in its entry list: such a list was damaged
// after it was built, and the plan refuses it rather than let the table
// builds skip entries.  One warp per ordered row.
__global__ void k_check_row_vids(const int32_t* __restrict__ order, int64_t n, const uint32_t* __restrict__ row_vid,
                                 int64_t stride, int64_t nref, uint32_t limit, int* bad) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const int32_t r = order[w];
    if (r < 0 || r >= nref) {
        if (lane == 0) atomicOr(bad, 1);
        return;
    }
    bool b = false;
    for (int64_t e = lane; e < stride; e += 32) b |= row_vid[(int64_t)r * stride + e] > limit;
    if (__any_sync(0xFFFFFFFFu, b) && lane == 0) atomicOr(bad, 1);
}

int check_plan_rows(siml_engine* h, const int32_t* d_order, int64_t n) {
    if (n == 0) return SIML_OK;
    int* d_bad = reinterpret_cast<int*>(h->d_counter);
    int bad = 0;
    SIML_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream));
    k_check_row_vids<<<(unsigned)((n * 32 + 255) / 256), 256, 0, h->stream>>>(
        d_order, n, h->rows.vid, h->rows.stride, h->ref.n, (uint32_t)h->vocab.nvid, d_bad);
    SIML_CUDA(cudaGetLastError());
    h->launches++;
    SIML_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) return fail(SIML_ERR_STATE, "siml_batch_create: a ref row's entry list holds a vid outside the "
                                         "database vocabulary (damaged after it was built)");
    return SIML_OK;
}

// Bytes one run reads: *streamed = every item's chunks (entry groups and
// per-lane metadata), as the kernel reads them, mostly from L2; *unique =
// every job's chunk range once, the least any schedule must bring from DRAM.
int plan_bytes(siml_engine* h, const DbLayout* d, const std::vector<HostJob>& jobs, const std::vector<int4>& items,
               int64_t* streamed, int64_t* unique) {
    std::vector<int64_t> off((size_t)d->nchunks + 1);
    SIML_CUDA(cudaMemcpyAsync(off.data(), d->off, off.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    auto range_bytes = [&](int64_t c0, int64_t c1) {
        return (off[(size_t)c1] - off[(size_t)c0]) * 16 + (c1 - c0) * 32 * (int64_t)sizeof(int4);
    };
    int64_t b = 0, u = 0;
    for (size_t i = 1; i < items.size(); i += 2) b += range_bytes(items[i].y, items[i].z);
    for (const HostJob& j : jobs) {
        if (j.re <= j.rb || j.ce <= j.cb) continue;
        int64_t c0, c1;
        sorted_chunk_range(d, j.cb, j.ce, c0, c1);
        u += range_bytes(c0, c1);
    }
    *streamed = b;
    *unique = u;
    return SIML_OK;
}

}  // namespace
}  // namespace siml

using namespace siml;

extern "C" {

int siml_batch_create(siml_engine* h, int64_t njobs, const int64_t* jobs, float lo, float hi, int64_t pitch,
                      int64_t tile_chunks, siml_batch** out) {
    return siml_batch_create_shaped(h, njobs, jobs, lo, hi, pitch, tile_chunks, 32, 0, out);
}

int siml_batch_create_shaped(siml_engine* h, int64_t njobs, const int64_t* jobs, float lo, float hi, int64_t pitch,
                             int64_t tile_chunks, int64_t rows_cap, int64_t merge_rows, siml_batch** out) {
    clear_error();
    if (!h || !out) return fail(SIML_ERR_INVALID, "siml_batch_create: NULL argument");
    *out = nullptr;
    SIML_CUDA(cudaSetDevice(h->device));
    if (njobs < 0 || (njobs > 0 && !jobs)) return fail(SIML_ERR_INVALID, "siml_batch_create: bad job list");
    if (pitch < 0 || pitch > 0x7FFFFFFFll) return fail(SIML_ERR_INVALID, "siml_batch_create: bad pitch");
    const DbLayout* d = nullptr;
    int rc = ensure_layout(h, true, &d);
    if (rc) return rc;
    std::vector<HostJob> hj((size_t)njobs);
    int64_t rows_out = 0;
    for (int64_t j = 0; j < njobs; j++) {
        HostJob x{jobs[5 * j], jobs[5 * j + 1], jobs[5 * j + 2], jobs[5 * j + 3], jobs[5 * j + 4]};
        if (x.rb < 0 || x.re < x.rb || x.re > h->ref.n || x.cb < 0 || x.ce < x.cb || x.ce > h->qry.n || x.out < 0)
            return fail(SIML_ERR_RANGE, "siml_batch_create: job %lld out of range (rows [%lld, %lld) of %lld, "
                        "columns [%lld, %lld) of %lld)", (long long)j, (long long)x.rb, (long long)x.re,
                        (long long)h->ref.n, (long long)x.cb, (long long)x.ce, (long long)h->qry.n);
        rows_out = std::max(rows_out, x.out + (x.re - x.rb));
        hj[(size_t)j] = x;
    }
    if (rows_out > 0x7FFFFFFF) return fail(SIML_ERR_UNSUPPORTED, "siml_batch_create: too many output rows");
    std::vector<int4> rowinfo((size_t)rows_out, make_int4(-1, 0, 0, 0));
    for (const HostJob& x : hj)
        for (int64_t r = x.rb; r < x.re; r++) {
            int4& ri = rowinfo[(size_t)(x.out + r - x.rb)];
            if (ri.x >= 0) return fail(SIML_ERR_INVALID, "siml_batch_create: jobs share output row %lld",
                                       (long long)(x.out + r - x.rb));
            ri = make_int4((int)r, (int)x.cb, (int)x.ce, 0);
        }
    // every job row's entry list must hold vocabulary vids only (checked
    // before the tile timing launches the kernel on them)
    {
        std::vector<int32_t> jrows;
        for (const HostJob& x : hj)
            for (int64_t r = x.rb; r < x.re; r++) jrows.push_back((int32_t)r);
        int32_t* d_rows = nullptr;
        if ((rc = upload_items(h, jrows, &d_rows))) return rc;
        rc = check_plan_rows(h, d_rows, (int64_t)jrows.size());
        cudaFree(d_rows);
        if (rc) return rc;
    }
    std::vector<int32_t> mag;
    if ((rc = host_mags(h, mag))) return rc;
    Shape sh;
    int from_cache = 0;
    if (tile_chunks > 0) {
        sh.tile = tile_chunks;
        sh.rows_cap = rows_cap == 16 ? 16 : 32;
        sh.merge_rows = std::max<int64_t>(0, merge_rows);
    } else if (batch_nbr_usable(h, d)) {
        std::tuple<int64_t, int64_t, int64_t, int64_t, int64_t, int64_t> sig;
        if ((rc = plan_signature(h, d, hj, lo, &sig))) return rc;
        bool hit = false;
        {
            std::lock_guard<std::mutex> lk(g_shape_mu);
            auto it = g_shapes.find(sig);
            if (it != g_shapes.end()) { sh = it->second; hit = true; }
        }
        if (hit) {
            from_cache = 1;
        } else {
            if ((rc = autotune_shape(h, d, hj, mag, lo, hi, pitch, &sh))) return rc;
            std::lock_guard<std::mutex> lk(g_shape_mu);
            g_shapes[sig] = sh;
        }
    }
    mark_merge_rows(hj, sh.merge_rows, rowinfo);
    siml_batch* b = new siml_batch();
    b->h = h;
    b->d = d;
    b->generation = h->generation;
    b->lo = lo;
    b->hi = hi;
    b->pitch = pitch;
    b->tile_chunks = sh.tile;
    b->rows_cap = sh.rows_cap;
    b->merge_rows = sh.merge_rows;
    b->from_cache = from_cache;
    b->rows_out = rows_out;
    std::vector<int4> items;
    std::vector<int32_t> order;
    make_items(d, hj, mag, sh, items, order);
    b->nitems = (int64_t)items.size() / 2;
    b->order_len = (int64_t)order.size();
    if ((rc = plan_bytes(h, d, hj, items, &b->stream_bytes, &b->unique_bytes)) ||
        (rc = upload_items(h, items, &b->items)) || (rc = upload_items(h, order, &b->order)) ||
        (rc = upload_items(h, rowinfo, &b->rowinfo))) {
        siml_batch_destroy(b);
        return rc;
    }
    cudaError_t e = cudaMalloc((void**)&b->head, sizeof(unsigned int));
    if (e != cudaSuccess) {
        siml_batch_destroy(b);
        return cuda_fail(e, "cudaMalloc");
    }
    *out = b;
    return SIML_OK;
}

int siml_batch_info(siml_batch* b, int64_t* rows_out, int64_t* nitems, int64_t* tile_chunks,
                    int64_t* stream_bytes, int64_t* unique_bytes) {
    clear_error();
    if (!b) return fail(SIML_ERR_INVALID, "siml_batch_info: NULL batch");
    if (rows_out) *rows_out = b->rows_out;
    if (nitems) *nitems = b->nitems;
    if (tile_chunks) *tile_chunks = b->tile_chunks;
    if (stream_bytes) *stream_bytes = b->stream_bytes;
    if (unique_bytes) *unique_bytes = b->unique_bytes;
    return SIML_OK;
}

int siml_batch_shape(siml_batch* b, int64_t out[4]) {
    clear_error();
    if (!b || !out) return fail(SIML_ERR_INVALID, "siml_batch_shape: NULL argument");
    out[0] = b->tile_chunks;
    out[1] = b->rows_cap;
    out[2] = b->merge_rows;
    out[3] = b->from_cache;
    return SIML_OK;
}

int siml_batch_run(siml_batch* b, int32_t* idx, float* sims, int32_t* counts, void* stream) {
    clear_error();
    if (!b) return fail(SIML_ERR_INVALID, "siml_batch_run: NULL batch");
    siml_engine* h = b->h;
    SIML_CUDA(cudaSetDevice(h->device));
    if (b->generation != h->generation)
        return fail(SIML_ERR_STATE, "siml_batch_run: the engine's sets changed since the plan was made");
    if (b->rows_out == 0) return SIML_OK;
    if (!counts || (b->pitch > 0 && !idx)) return fail(SIML_ERR_INVALID, "siml_batch_run: NULL output");
    cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
    return launch_batch_neighbors(h, b->d, b->items, b->nitems, b->head, b->order, b->order_len, b->rowinfo,
                                  b->rows_out, b->lo, b->hi, b->pitch, idx, sims, counts, st);
}

int siml_batch_destroy(siml_batch* b) {
    clear_error();
    if (!b) return SIML_OK;
    cudaSetDevice(b->h->device);
    if (b->items) cudaFree(b->items);
    if (b->order) cudaFree(b->order);
    if (b->rowinfo) cudaFree(b->rowinfo);
    if (b->head) cudaFree(b->head);
    delete b;
    return SIML_OK;
}

}  // extern "C"
