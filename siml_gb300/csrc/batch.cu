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
// The chunk range of one work item (tile_chunks) is the tile shape.  With
// tile_chunks <= 0 the plan times the candidate shapes on a sample of the
// jobs and keeps the fastest; siml_batch_info reports the choice, so later
// plans of similar jobs can pass it and skip the timing.
#include <algorithm>
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
void make_items(const DbLayout* d, const std::vector<HostJob>& jobs, const std::vector<int32_t>& mag, int64_t tile,
                std::vector<int4>& items, std::vector<int32_t>& order) {
    struct It {
        int4 a, b;
        int64_t cost;
    };
    std::vector<It> v;
    order.clear();
    for (const HostJob& j : jobs) {
        if (j.re <= j.rb || j.ce <= j.cb) continue;
        const int64_t pos0 = (int64_t)order.size();
        for (int64_t r = j.rb; r < j.re; r++) order.push_back((int32_t)r);
        std::stable_sort(order.begin() + pos0, order.end(),
                         [&](int32_t x, int32_t y) { return mag[(size_t)x] < mag[(size_t)y]; });
        int64_t c0, c1;
        sorted_chunk_range(d, j.cb, j.ce, c0, c1);
        const int64_t nrows = j.re - j.rb;
        for (int64_t r = 0; r < nrows; r += 32) {
            const int nr = (int)std::min<int64_t>(32, nrows - r);
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

// Times the persistent kernel for each candidate tile on a sample of the
// jobs and returns the fastest tile.  The sample takes jobs at an even
// stride until it holds about kTuneBudget pairs, so tuning costs a fraction
// of a second whatever the batch size.
constexpr double kTuneBudget = 1.0e10;

int autotune_tile(siml_engine* h, const DbLayout* d, const std::vector<HostJob>& jobs,
                  const std::vector<int32_t>& mag, float lo, float hi, int64_t pitch, int64_t* best_tile) {
    static const int64_t cand[] = {32, 64, 128, 256, 512, 1024, 2048};
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
    *best_tile = 128;
    if (rows == 0) return SIML_OK;
    std::vector<int4> rowinfo((size_t)rows, make_int4(-1, 0, 0, 0));
    for (const HostJob& j : sample)
        for (int64_t r = j.rb; r < j.re; r++)
            rowinfo[(size_t)(j.out + r - j.rb)] = make_int4((int)r, (int)j.cb, (int)j.ce, 0);
    int4* d_rowinfo = nullptr;
    int32_t *d_idx = nullptr, *d_cnt = nullptr, *d_order = nullptr;
    unsigned int* d_head = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = SIML_OK;
    auto cleanup = [&]() {
        if (d_order) cudaFree(d_order);
        if (d_rowinfo) cudaFree(d_rowinfo);
        if (d_idx) cudaFree(d_idx);
        if (d_cnt) cudaFree(d_cnt);
        if (d_head) cudaFree(d_head);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc((void**)&d_rowinfo, rowinfo.size() * sizeof(int4))) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_rowinfo, rowinfo.data(), rowinfo.size() * sizeof(int4), cudaMemcpyHostToDevice,
                             h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_idx, (size_t)rows * (size_t)std::max<int64_t>(pitch, 1) * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_cnt, (size_t)rows * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_head, sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "batch autotune set-up");
    }
    double best = 1e300;
    bool warmed = false;
    for (int64_t t : cand) {
        std::vector<int4> items;
        std::vector<int32_t> order;
        make_items(d, sample, mag, t, items, order);
        int4* d_items = nullptr;
        if (!d_order && (rc = upload_items(h, order, &d_order))) break;   // the same for every tile
        if ((rc = upload_items(h, items, &d_items))) break;
        const int64_t ni = (int64_t)items.size() / 2;
        if (!warmed) {   // first launch pays one-time costs; keep it out of the comparison
            rc = launch_batch_neighbors(h, d, d_items, ni, d_head, d_order, (int64_t)order.size(), d_rowinfo, rows,
                                        lo, hi, pitch, d_idx, nullptr, d_cnt, h->stream);
            warmed = true;
        }
        if (!rc) {
            cudaEventRecord(e0, h->stream);
            rc = launch_batch_neighbors(h, d, d_items, ni, d_head, d_order, (int64_t)order.size(), d_rowinfo, rows,
                                        lo, hi, pitch, d_idx, nullptr, d_cnt, h->stream);
            cudaEventRecord(e1, h->stream);
        }
        e = cudaEventSynchronize(e1);
        cudaFree(d_items);
        if (rc) break;
        if (e != cudaSuccess) { rc = cuda_fail(e, "batch autotune"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best * 0.98) { best = ms; *best_tile = t; }
    }
    cleanup();
    return rc;
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
    std::vector<int32_t> mag;
    if ((rc = host_mags(h, mag))) return rc;
    int64_t tile = tile_chunks;
    if (tile <= 0) {
        if (batch_nbr_usable(h, d)) {
            if ((rc = autotune_tile(h, d, hj, mag, lo, hi, pitch, &tile))) return rc;
        } else {
            tile = 128;
        }
    }
    siml_batch* b = new siml_batch();
    b->h = h;
    b->d = d;
    b->generation = h->generation;
    b->lo = lo;
    b->hi = hi;
    b->pitch = pitch;
    b->tile_chunks = tile;
    b->rows_out = rows_out;
    std::vector<int4> items;
    std::vector<int32_t> order;
    make_items(d, hj, mag, tile, items, order);
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
