// SMILES -> LINGO compiler on the GPU: the same output as the host compiler
// (lingo_compiler.cpp) and the reference's C compiler
// (pysiml/_ccompiler.cpp:276-381), for strings already in device memory, so
// a database can be compiled and made resident without a host round trip.
//
// One warp per string.  A string free of the bytes that carry state (see
// lingo::stateful_byte) is preprocessed by all lanes at once, each mapping
// its own bytes; otherwise the warp runs the preprocessing state machine in
// parallel over segments of the string (preprocess_warp), in place.  The lanes then form the windows in parallel, sort them with a
// bitonic network, and mark run starts with ballots: the unique codes and
// their counts go straight to the string's output row.  Strings of up to
// kCompileCap bytes work in shared memory; longer ones are listed and
// compiled by the same code over global scratch.
#include <algorithm>
#include <vector>

#include "engine.h"
#include "lingo_compile_core.h"

namespace siml {
namespace {

constexpr int kCompileCap = 1024;       // bytes of a string held in shared memory
constexpr int kCompileWarps = 8;        // warps (strings in flight) per CTA

// ---- warp-parallel preprocessing.  lingo::preprocess is a transducer over
// four states plus a terminal one (a terminator or NUL ends the string);
// each input byte yields at most one output byte.  A warp takes the string
// in rounds of 32 segments of kSeg bytes: each lane maps every start state
// to the state its segment ends in, a warp scan composes the maps to give
// each lane its true start state, each lane replays its segment from it, and
// a prefix sum of the bytes they keep places their output.
constexpr int kSeg = 2;
constexpr int kDone = 4;   // terminal state

// One step of lingo::preprocess: the next state, and the byte kept (-1: none).
__device__ __forceinline__ int pp_step(int st, unsigned char ch, int& emit) {
    emit = -1;
    if (st == kDone || ch == 0) return kDone;
    if (st == 1) return 2;   // kSwallow: the byte after '%' is dropped
    if (st == 3) {           // kVerbatimDigits: copied until a non-digit
        emit = ch;
        return lingo::is_digit(ch) ? 3 : 0;
    }
    if (ch == ' ' || ch == '\n' || ch == '\r') return kDone;
    if (lingo::is_digit(ch)) {
        emit = '0';
        return 2;
    }
    emit = ch;
    if (ch == '%') return 1;
    if (st == 0 && (ch == '+' || ch == '-' || ch == 'H' || ch == '[')) return 3;
    return 0;
}

// Map of 5 start states to end states, 3 bits each: (g after f)[s] = g[f[s]].
__device__ __forceinline__ uint32_t pp_compose(uint32_t f, uint32_t g) {
    uint32_t r = 0;
#pragma unroll
    for (int s = 0; s < 5; s++) r |= ((g >> (3 * ((f >> (3 * s)) & 7u))) & 7u) << (3 * s);
    return r;
}

// lingo::preprocess of buf[0, inlen) in place, by the calling warp; returns
// the processed length.
__device__ int32_t preprocess_warp(unsigned char* buf, int64_t inlen) {
    const int lane = threadIdx.x & 31;
    int state = 0;
    int32_t n = 0;
    for (int64_t base = 0; base < inlen && state != kDone; base += 32 * kSeg) {
        const int64_t b = base + (int64_t)lane * kSeg;
        const int64_t left = inlen - b;
        const int cnt = left <= 0 ? 0 : (left < kSeg ? (int)left : kSeg);
        unsigned char in[kSeg];
#pragma unroll
        for (int i = 0; i < kSeg; i++) in[i] = i < cnt ? buf[b + i] : 0;
        // this segment's map of start states to end states
        uint32_t map = 0;
#pragma unroll
        for (int s = 0; s < 5; s++) {
            int st = s, e;
#pragma unroll
            for (int i = 0; i < kSeg; i++)
                if (i < cnt) st = pp_step(st, in[i], e);
            map |= (uint32_t)st << (3 * s);
        }
        // inclusive scan of the maps: lane l gets segments 0..l composed
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, map, o);
            if (lane >= o) map = pp_compose(prev, map);
        }
        const int end = (int)((map >> (3 * state)) & 7u);
        int st = __shfl_up_sync(0xFFFFFFFFu, end, 1);
        if (lane == 0) st = state;
        // replay from the true start state
        uint32_t kept[(kSeg + 3) / 4] = {};
        int k = 0;
#pragma unroll
        for (int i = 0; i < kSeg; i++) {
            if (i < cnt) {
                int e;
                st = pp_step(st, in[i], e);
                if (e >= 0) {
                    kept[k >> 2] |= (uint32_t)e << (8 * (k & 3));
                    k++;
                }
            }
        }
        int pre = k;   // exclusive prefix of the kept counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xFFFFFFFFu, pre, o);
            if (lane >= o) pre += t;
        }
        const int total = __shfl_sync(0xFFFFFFFFu, pre, 31);
        pre -= k;
        __syncwarp();   // every lane has read its input before any output lands
        for (int i = 0; i < k; i++) buf[n + pre + i] = (unsigned char)(kept[i >> 2] >> (8 * (i & 3)));
        __syncwarp();
        n += total;
        state = __shfl_sync(0xFFFFFFFFu, end, 31);
    }
    return n;
}

// Compiles one string with the calling warp.  buf holds >= inlen + 8 bytes
// and codes >= max(next power of two >= inlen, 32) words of scratch.
// Always raises *maxw to the number of unique codes.  width > 0: also
// writes the row (zero padded to width when pad), length and magnitude,
// unless the string has more unique codes than width (the caller then
// reports it).  No write leaves the row.
__device__ void compile_one(const unsigned char* __restrict__ raw, int64_t inlen, unsigned char* buf, int32_t* codes,
                            int64_t width, int32_t* lrow, int32_t* crow, int32_t* length, int32_t* mag, int* maxw,
                            bool pad = true) {
    const int lane = threadIdx.x & 31;
    bool stateful = false;
    for (int64_t i = lane; i < inlen; i += 32) {
        const unsigned char c = raw[i];
        buf[i] = c;
        stateful |= lingo::stateful_byte(c);
    }
    int32_t len = (int32_t)inlen;
    if (__ballot_sync(0xFFFFFFFFu, stateful) == 0u) {
        // digits become '0', every other byte stays: each lane maps its own bytes
        for (int64_t i = lane; i < inlen; i += 32)
            if (lingo::is_digit(buf[i])) buf[i] = '0';
    } else {
        __syncwarp();
        len = preprocess_warp(buf, inlen);
    }
    __syncwarp();
    int32_t m = 0;
    if (len >= 4) {
        bool high = false;
        for (int32_t q = lane; q < len; q += 32) high |= buf[q] >= 0x80u;
        const bool ascii = __ballot_sync(0xFFFFFFFFu, high) == 0u;
        m = len - 3;
        for (int32_t p = lane; p < m; p += 32)
            codes[p] = ascii ? lingo::ascii_window(buf, p) : lingo::window_code(buf, len, p / 4, p % 4);
        if (!ascii) {
            int32_t extra = 0;
            if (lane == 0) {
                for (int k = 1; k <= 3; k++) {
                    int32_t c;
                    if (lingo::tail_window(buf, len, k, &c)) codes[m + extra++] = c;
                }
            }
            m += __shfl_sync(0xFFFFFFFFu, extra, 0);
        }
        __syncwarp();
        // bitonic sort of codes[0, N) ascending (signed), padded with INT32_MAX
        int32_t N = 32;
        while (N < m) N <<= 1;
        for (int32_t i = m + lane; i < N; i += 32) codes[i] = 0x7FFFFFFF;
        __syncwarp();
        for (int32_t k = 2; k <= N; k <<= 1) {
            for (int32_t j = k >> 1; j > 0; j >>= 1) {
                for (int32_t i = lane; i < N; i += 32) {
                    const int32_t o = i ^ j;
                    if (o > i) {
                        const int32_t a = codes[i], b = codes[o];
                        if ((a > b) == ((i & k) == 0)) {
                            codes[i] = b;
                            codes[o] = a;
                        }
                    }
                }
                __syncwarp();
            }
        }
    }
    // run starts: rank r of start i is the number of starts before it; with
    // an output row the start positions go to crow[r] first and become
    // counts in a second sweep
    int32_t nu = 0;
    for (int32_t base = 0; base < m; base += 32) {
        const int32_t i = base + lane;
        const bool start = i < m && (i == 0 || codes[i] != codes[i - 1]);
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, start);
        if (start && width > 0) {
            const int32_t r = nu + __popc(bal & ((1u << lane) - 1u));
            if (r < width) {
                lrow[r] = codes[i];
                crow[r] = i;
            }
        }
        nu += __popc(bal);
    }
    if (lane == 0) atomicMax(maxw, nu);
    if (width == 0 || nu > width) return;
    __syncwarp();
    for (int32_t base = 0; base < nu; base += 32) {
        const int32_t r = base + lane;
        int32_t a = 0, b = 0;
        if (r < nu) {
            a = crow[r];
            b = r + 1 < nu ? crow[r + 1] : m;
        }
        __syncwarp();
        if (r < nu) crow[r] = b - a;
        __syncwarp();
    }
    if (pad) {
        for (int64_t j = nu + lane; j < width; j += 32) {
            lrow[j] = 0;
            crow[j] = 0;
        }
    }
    if (lane == 0) {
        *length = nu;
        *mag = len >= 4 ? len - 3 : 0;
    }
}

// Output row of string s: row s of [n, width] (zero padded), or with STAGED
// its stretch [off[s], off[s+1]) of the staging arrays, which holds its
// unique codes unpadded (a string has at most as many unique windows as
// bytes).
struct RowOut {
    int64_t row;
    int64_t width;
};
template <bool STAGED>
__device__ __forceinline__ RowOut row_out(int64_t s, int64_t b, int64_t inlen, int64_t width) {
    if (STAGED) return {b, inlen > 0 ? inlen : 1};
    return {s * width, width};
}

// Strings of at most kCompileCap bytes; longer ones are appended to `longs`.
template <bool STAGED>
__global__ void __launch_bounds__(kCompileWarps * 32) k_compile(const unsigned char* __restrict__ text,
                                                                const int64_t* __restrict__ off, int64_t n,
                                                                int64_t width, int32_t* lingos, int32_t* counts,
                                                                int32_t* lengths, int32_t* mags, int* maxw,
                                                                int64_t* longs, int* nlong) {
    __shared__ __align__(16) unsigned char sbuf[kCompileWarps][kCompileCap + 16];
    __shared__ __align__(16) int32_t scodes[kCompileWarps][kCompileCap];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * kCompileWarps;
    for (int64_t s = (int64_t)blockIdx.x * kCompileWarps + warp; s < n; s += nwarps) {
        const int64_t b = off[s], inlen = off[s + 1] - b;
        if (inlen > kCompileCap) {
            if (lane == 0) longs[atomicAdd(nlong, 1)] = s;
            continue;
        }
        const RowOut o = row_out<STAGED>(s, b, inlen, width);
        compile_one(text + b, inlen, sbuf[warp], scodes[warp], o.width, lingos + o.row, counts + o.row, lengths + s,
                    mags + s, maxw, !STAGED);
        __syncwarp();
    }
}

// The listed long strings, one warp each, over global scratch at
// scratch_off[i] bytes (bytes first, then the code words, 16-byte aligned).
template <bool STAGED>
__global__ void __launch_bounds__(32) k_compile_long(const unsigned char* __restrict__ text,
                                                     const int64_t* __restrict__ off, const int64_t* __restrict__ longs,
                                                     const int64_t* __restrict__ scratch_off, char* scratch,
                                                     int64_t width, int32_t* lingos, int32_t* counts,
                                                     int32_t* lengths, int32_t* mags, int* maxw) {
    const int64_t s = longs[blockIdx.x];
    const int64_t b = off[s], inlen = off[s + 1] - b;
    char* base = scratch + scratch_off[blockIdx.x];
    unsigned char* buf = reinterpret_cast<unsigned char*>(base);
    int32_t* codes = reinterpret_cast<int32_t*>(base + ((inlen + 16 + 15) / 16) * 16);
    const RowOut o = row_out<STAGED>(s, b, inlen, width);
    compile_one(text + b, inlen, buf, codes, o.width, lingos + o.row, counts + o.row, lengths + s, mags + s, maxw,
                !STAGED);
}

// Staged rows into [n, width]: warp per string, zero padded past its unique
// codes.  A string's count is bounded by its staging stretch, so no read
// leaves it; *bad is set when a string has more codes than width.
__global__ void k_compile_scatter(const int64_t* __restrict__ off, int64_t n, const int32_t* __restrict__ sc,
                                  const int32_t* __restrict__ sn, const int32_t* __restrict__ lengths, int64_t width,
                                  int32_t* __restrict__ lingos, int32_t* __restrict__ counts, int* bad) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < n; s += nwarps) {
        const int64_t b = off[s];
        const int64_t nu = min((int64_t)max(lengths[s], 0), off[s + 1] - b);
        if (lane == 0 && nu > width) atomicOr(bad, 1);
        int32_t* lr = lingos + s * width;
        int32_t* cr = counts + s * width;
        for (int64_t j = lane; j < width; j += 32) {
            const bool in = j < nu;
            lr[j] = in ? sc[b + j] : 0;
            cr[j] = in ? sn[b + j] : 0;
        }
    }
}

int64_t pow2_at_least(int64_t v) {
    int64_t p = 32;
    while (p < v) p <<= 1;
    return p;
}

// Runs both kernels; width == 0 computes the width into *maxw_out.  staged:
// lingos/counts are staging arrays of off[n] words (width is ignored) and
// every string's row, length and magnitude are written.
int compile_gpu(siml_engine* h, const char* text, const int64_t* off, int64_t n, int64_t width, int32_t* lingos,
                int32_t* counts, int32_t* lengths, int32_t* mags, int64_t* maxw_out, bool staged = false) {
    cudaStream_t st = h->stream;
    if (n == 0) {
        if (maxw_out) *maxw_out = 0;
        return SIML_OK;
    }
    int* d_small = nullptr;     // {maxw, nlong}
    int64_t* d_longs = nullptr;
    SIML_CUDA(cudaMallocAsync((void**)&d_small, 2 * sizeof(int), st));
    cudaError_t e = cudaMallocAsync((void**)&d_longs, (size_t)n * sizeof(int64_t), st);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_small, st);
        return cuda_fail(e, "compile scratch");
    }
    auto done = [&](int rc) {
        cudaFreeAsync(d_longs, st);
        cudaFreeAsync(d_small, st);
        return rc;
    };
    if ((e = cudaMemsetAsync(d_small, 0, 2 * sizeof(int), st)) != cudaSuccess) return done(cuda_fail(e, "memset"));
    const int64_t per_cta = kCompileWarps;
    const int64_t grid = std::min<int64_t>((n + per_cta - 1) / per_cta, (int64_t)h->num_sms * 16);
    auto kc = staged ? k_compile<true> : k_compile<false>;
    kc<<<(unsigned)grid, kCompileWarps * 32, 0, st>>>((const unsigned char*)text, off, n, width, lingos, counts,
                                                      lengths, mags, d_small, d_longs, d_small + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return done(cuda_fail(e, "k_compile"));
    h->launches++;
    int hs[2] = {0, 0};
    if ((e = cudaMemcpyAsync(hs, d_small, sizeof(hs), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return done(cuda_fail(e, "k_compile"));
    const int nlong = hs[1];
    if (nlong > 0) {
        // scratch per long string: its bytes, then next-power-of-two code words
        std::vector<int64_t> ids((size_t)nlong), lo((size_t)nlong), hi((size_t)nlong), soff((size_t)nlong);
        if ((e = cudaMemcpy(ids.data(), d_longs, (size_t)nlong * 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return done(cuda_fail(e, "long strings"));
        int64_t total = 0;
        for (int i = 0; i < nlong; i++) {
            if ((e = cudaMemcpy(&lo[(size_t)i], off + ids[(size_t)i], 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
                (e = cudaMemcpy(&hi[(size_t)i], off + ids[(size_t)i] + 1, 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
                return done(cuda_fail(e, "long strings"));
            const int64_t inlen = hi[(size_t)i] - lo[(size_t)i];
            soff[(size_t)i] = total;
            total += ((inlen + 16 + 15) / 16) * 16 + pow2_at_least(inlen) * 4;
        }
        char* scratch = nullptr;
        int64_t* d_soff = nullptr;
        if ((e = cudaMallocAsync((void**)&scratch, (size_t)total, st)) != cudaSuccess)
            return done(cuda_fail(e, "long-string scratch"));
        if ((e = cudaMallocAsync((void**)&d_soff, (size_t)nlong * 8, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_soff, soff.data(), (size_t)nlong * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
            cudaFreeAsync(scratch, st);
            return done(cuda_fail(e, "long-string scratch"));
        }
        auto kl = staged ? k_compile_long<true> : k_compile_long<false>;
        kl<<<(unsigned)nlong, 32, 0, st>>>((const unsigned char*)text, off, d_longs, d_soff, scratch, width, lingos,
                                           counts, lengths, mags, d_small);
        e = cudaGetLastError();
        h->launches++;
        if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d_small, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // soff is a host vector
        cudaFreeAsync(d_soff, st);
        cudaFreeAsync(scratch, st);
        if (e != cudaSuccess) return done(cuda_fail(e, "k_compile_long"));
    }
    if (maxw_out) *maxw_out = hs[0];
    return done(SIML_OK);
}

// Offsets must be non-decreasing and start at 0 or more; checked on the
// device copy's endpoints and by one pass on the device.
__global__ void k_check_offsets(const int64_t* off, int64_t n, int* bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (off[i + 1] < off[i] || off[i] < 0) atomicOr(bad, 1);
}

int check_offsets_gpu(siml_engine* h, const int64_t* off, int64_t n) {
    if (n <= 0) return SIML_OK;
    int* d_bad = nullptr;
    SIML_CUDA(cudaMallocAsync((void**)&d_bad, sizeof(int), h->stream));
    int bad = 0;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int), h->stream);
    if (e == cudaSuccess) {
        const int64_t grid = std::min<int64_t>((n + 255) / 256, (int64_t)h->num_sms * 8);
        k_check_offsets<<<(unsigned)grid, 256, 0, h->stream>>>(off, n, d_bad);
        e = cudaGetLastError();
        h->launches++;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFreeAsync(d_bad, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "offset check");
    return bad ? fail(SIML_ERR_INVALID, "GPU compiler: offsets must be non-negative and non-decreasing") : SIML_OK;
}

}  // namespace
}  // namespace siml

using namespace siml;

extern "C" {

int64_t siml_compile_width_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n) {
    clear_error();
    if (!h) return -fail(SIML_ERR_INVALID, "siml_compile_width_gpu: NULL engine");
    if (n < 0 || (n > 0 && (!buf || !offsets))) return -fail(SIML_ERR_INVALID, "siml_compile_width_gpu: bad arguments");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaSetDevice");
    int rc = check_offsets_gpu(h, offsets, n);
    if (rc) return -rc;
    int64_t w = 0;
    rc = compile_gpu(h, buf, offsets, n, 0, nullptr, nullptr, nullptr, nullptr, &w);
    return rc ? -rc : w;
}

int siml_compile_smiles_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n, int32_t* lingos,
                            int32_t* counts, int32_t* lengths, int32_t* mags, int64_t width) {
    clear_error();
    if (!h) return fail(SIML_ERR_INVALID, "siml_compile_smiles_gpu: NULL engine");
    if (n < 0 || width < 1 || (n > 0 && (!buf || !offsets || !lingos || !counts || !lengths || !mags)))
        return fail(SIML_ERR_INVALID, "siml_compile_smiles_gpu: bad arguments");
    SIML_CUDA(cudaSetDevice(h->device));
    int rc = check_offsets_gpu(h, offsets, n);
    if (rc) return rc;
    int64_t w = 0;
    if ((rc = compile_gpu(h, buf, offsets, n, width, lingos, counts, lengths, mags, &w))) return rc;
    if (w > width)
        return fail(SIML_ERR_INVALID, "siml_compile_smiles_gpu: width smaller than a string's unique LINGO count");
    return SIML_OK;
}

int64_t siml_compile_stage_gpu(siml_engine* h, const char* buf, const int64_t* offsets, int64_t n,
                               int32_t* stage_codes, int32_t* stage_counts, int32_t* lengths, int32_t* mags) {
    clear_error();
    if (!h) return -fail(SIML_ERR_INVALID, "siml_compile_stage_gpu: NULL engine");
    if (n < 0 || (n > 0 && (!buf || !offsets || !stage_codes || !stage_counts || !lengths || !mags)))
        return -fail(SIML_ERR_INVALID, "siml_compile_stage_gpu: bad arguments");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaSetDevice");
    int rc = check_offsets_gpu(h, offsets, n);
    if (rc) return -rc;
    int64_t w = 0;
    rc = compile_gpu(h, buf, offsets, n, 0, stage_codes, stage_counts, lengths, mags, &w, true);
    return rc ? -rc : w;
}

int siml_compile_scatter_gpu(siml_engine* h, const int64_t* offsets, int64_t n, const int32_t* stage_codes,
                             const int32_t* stage_counts, const int32_t* lengths, int32_t* lingos, int32_t* counts,
                             int64_t width) {
    clear_error();
    if (!h) return fail(SIML_ERR_INVALID, "siml_compile_scatter_gpu: NULL engine");
    if (n < 0 || width < 1 || (n > 0 && (!offsets || !stage_codes || !stage_counts || !lengths || !lingos || !counts)))
        return fail(SIML_ERR_INVALID, "siml_compile_scatter_gpu: bad arguments");
    if (n == 0) return SIML_OK;
    SIML_CUDA(cudaSetDevice(h->device));
    SIML_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    const int64_t grid = std::min<int64_t>((n + 7) / 8, (int64_t)h->num_sms * 16);
    k_compile_scatter<<<(unsigned)grid, 256, 0, h->stream>>>(offsets, n, stage_codes, stage_counts, lengths, width,
                                                            lingos, counts, h->d_err);
    SIML_CUDA(cudaGetLastError());
    h->launches++;
    int bad = 0;
    SIML_CUDA(cudaMemcpyAsync(&bad, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SIML_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) return fail(SIML_ERR_INVALID, "siml_compile_scatter_gpu: width smaller than a string's unique LINGO count");
    return SIML_OK;
}

}  // extern "C"
