// siml_topk_noalloc: per-row top-k that allocates no device memory.
//
// Some callers cannot allocate device memory on the request path: code that
// runs under a caller-owned memory pool or a strict memory budget, services
// that must not let a request trigger cudaMalloc (which can synchronize the
// device and fail under pressure), and embedders whose allocator forbids
// foreign allocations.  This entry point does the same work as siml_topk's
// per-CTA heap path and takes every scratch byte it needs (the
// magnitude-sort buckets, the row order and the per-CTA partial heaps) from
// one file-scope __device__ array of kNoallocScratchBytes (16 MiB).  Every
// GPU that loads the library holds that array until the process exits.
//
// Rules for callers:
//   - idx and sims are device pointers (int32 / fp32 [rows, k]).
//   - The engine's window-sorted device layout must already exist: siml_topk,
//     siml_neighbors, siml_neighbors_range, siml_hist101, siml_hist_global,
//     siml_vocab_stats and siml_batch_create build it (siml_rows and
//     siml_db_stats build only the full-matrix layout).  Otherwise the call
//     fails with SIML_ERR_STATE instead of building it.
//   - A request whose scratch would exceed 16 MiB is refused with
//     SIML_ERR_INVALID.  The heap path needs rows x splits x k x 8 bytes of
//     partial heaps plus 4 bytes per row plus 16 KiB (splits is at most 64;
//     the top-k path picks it from the row count and the database size); the
//     per-row scan (k > 256, or databases too small to split) needs none.
//   - All calls in the process share the one array and it keeps the last
//     call's contents, so calls whose work overlaps on the GPU (another
//     stream, another host thread, another engine on the same device) race
//     on it.  Serialize them.
//   - The call waits for its kernels (it synchronizes the engine's stream)
//     and returns with the results in idx / sims, or with the error of an
//     expired bounded wait.
//   - siml_create looks up the array's device address (cudaGetSymbolAddress,
//     with that device current), which loads this part of the library on the
//     device and maps the array there, so the request path does not.  If
//     that look-up failed at creation, the first call on the device repeats
//     it; make that call before any stream capture.
#include <mutex>

#include "engine.h"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)16 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_topk_scratch[kNoallocScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_topk_scratch on `device` (the current device).  In host
// code the array's name is only a host-side stand-in, never a device address.
int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return siml::fail(SIML_ERR_UNSUPPORTED, "siml_topk_noalloc: device %d", device);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_topk_scratch);
        if (e != cudaSuccess) return siml::cuda_fail(e, "cudaGetSymbolAddress(g_topk_scratch)");
        g_scratch_addr[device] = p;
    }
    *out = (unsigned char*)g_scratch_addr[device];
    return SIML_OK;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

namespace siml {

// Called by siml_create with `device` current: resolves the static scratch's
// address there, so the no-allocation entry point does not map it on the
// request path.  A failure is not an engine failure; the entry point retries.
void noalloc_prepare(int device) {
    unsigned char* p = nullptr;
    if (scratch_address(device, &p) != SIML_OK) {
        cudaGetLastError();   // not sticky: leave no error for the next call
        clear_error();
    }
}

}  // namespace siml

extern "C" int siml_topk_noalloc(siml_engine* h, int64_t rowbase, int64_t rowlimit, int64_t k,
                                 int32_t* idx, float* sims) {
    using namespace siml;
    clear_error();
    if (!h) return fail(SIML_ERR_INVALID, "NULL engine handle");
    cudaError_t se = cudaSetDevice(h->device);
    if (se != cudaSuccess) return cuda_fail(se, "cudaSetDevice");
    // the top-k kernels read the window-sorted layout only
    if (!h->layout_valid || !h->rows_valid || !h->sorted_valid)
        return fail(SIML_ERR_STATE, "siml_topk_noalloc: the window-sorted device layout of the current sets is not "
                                    "built yet (siml_topk, siml_neighbors, siml_hist101, siml_hist_global, "
                                    "siml_vocab_stats or siml_batch_create build it; this entry point allocates "
                                    "nothing)");
    if (rowbase < 0 || rowlimit > h->ref.n || rowlimit < rowbase)
        return fail(SIML_ERR_RANGE, "row range [%lld, %lld) outside the ref set of %lld rows",
                    (long long)rowbase, (long long)rowlimit, (long long)h->ref.n);
    if (k < 1 || k > (1 << 20)) return fail(SIML_ERR_INVALID, "siml_topk_noalloc: k = %lld out of range", (long long)k);
    const int64_t rows = rowlimit - rowbase;
    if (rows == 0) return SIML_OK;
    if (!idx || !sims) return fail(SIML_ERR_INVALID, "siml_topk_noalloc: NULL output");
    const DbLayout* d = &h->db_sorted;
    TopkPlan plan;
    int rc = topk_plan(h, d, rowbase, rowlimit, (int)k, plan);
    if (rc) return rc;
    unsigned char* base = nullptr;
    if ((rc = scratch_address(h->device, &base))) return rc;
    // buckets and row order serve the heap path only; the per-row scan takes
    // no scratch
    int32_t* bucket = reinterpret_cast<int32_t*>(base);
    int32_t* order = reinterpret_cast<int32_t*>(base + align256((size_t)kOrderBuckets * 4));
    unsigned char* part = base + align256((size_t)kOrderBuckets * 4) + align256((size_t)rows * 4);
    const size_t need = plan.splits > 0 ? (size_t)(part - base) + plan.partial_entries * 8 : 0;
    if (need > kNoallocScratchBytes)
        return fail(SIML_ERR_INVALID, "siml_topk_noalloc: %lld rows x %d splits x k %lld needs %zu bytes of scratch, "
                    "more than the %zu-byte static scratch; use fewer rows per call",
                    (long long)rows, plan.splits, (long long)k, need, kNoallocScratchBytes);
    float* pt = nullptr;
    int* pi = nullptr;
    if (plan.splits > 0) {
        pt = reinterpret_cast<float*>(part);
        pi = reinterpret_cast<int*>(pt + plan.partial_entries);
        if ((rc = row_order_into(h, rowbase, rowlimit, order, bucket))) return rc;
    }
    if ((rc = launch_topk_core(h, d, rowbase, rowlimit, (int)k, plan, order, pt, pi, idx, sims))) return rc;
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    return take_async_error(h);
}
