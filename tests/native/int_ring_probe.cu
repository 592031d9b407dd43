// Integer issue probe (measurement support, not part of the library): the
// rate of 32-bit integer instructions on the current GPU, printed as
// instructions per second and as integer lanes per SM per clock.  Its result
// is recorded in profiles/int_issue_probe.md, which bench.py reads for the
// work-reduction figure of the reference's merge (pysiml/_CPULingo.c:53-71:
// per merge step one compare, one select/advance and one min-accumulate).
//
// Each thread runs eight chains in a ring: every stage computes eight new
// words, each from three (or two) words of the previous stage, so a stage
// holds eight independent instructions and no two stages fold into one
// instruction.  Three rings are timed: three-input XOR (a LOP3), a
// three-input add (an IADD3) and alternating min / max (IMNMX).  Eight
// 256-thread CTAs per SM, best of three launches of about a millisecond each.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 int_ring_probe.cu -o probe && ./probe
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

constexpr int kRing = 8;

template <int KIND>
__global__ void __launch_bounds__(256) k_int_ring(const uint32_t* __restrict__ seed, int stages,
                                                  uint32_t* __restrict__ sink) {
    uint32_t a[kRing];
#pragma unroll
    for (int i = 0; i < kRing; i++) a[i] = seed[(threadIdx.x + i) & 31] + (uint32_t)(blockIdx.x * 977 + i);
    for (int s = 0; s < stages; s++) {
        uint32_t n[kRing];
#pragma unroll
        for (int i = 0; i < kRing; i++) {
            const uint32_t x = a[i], y = a[(i + 1) % kRing], z = a[(i + 3) % kRing];
            if (KIND == 0) n[i] = x ^ y ^ z;
            else if (KIND == 1) n[i] = x + y + z;
            else n[i] = (s & 1) ? max(x, y) : min(x, y);
        }
#pragma unroll
        for (int i = 0; i < kRing; i++) a[i] = n[i];
    }
    uint32_t v = 0u;
#pragma unroll
    for (int i = 0; i < kRing; i++) v ^= a[i];
    if (v == 0x9E3779B9u) sink[blockIdx.x] = v;   // keeps the chains live
}

#define CK(x)                                                                              \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            std::printf("CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return 1;                                                                      \
        }                                                                                  \
    } while (0)

template <int KIND>
int time_ring(int sms, const uint32_t* seed, uint32_t* sink, cudaEvent_t e0, cudaEvent_t e1, double* ops) {
    const int blocks = sms * 8, threads = 256, stages = 1 << 14;
    k_int_ring<KIND><<<blocks, threads>>>(seed, 256, sink);   // warm-up
    CK(cudaGetLastError());
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        CK(cudaEventRecord(e0));
        k_int_ring<KIND><<<blocks, threads>>>(seed, stages, sink);
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        best = ms < best ? ms : best;
    }
    *ops = (double)blocks * threads * (double)stages * kRing / (best * 1e-3);
    return 0;
}

int main() {
    int dev = 0, sms = 0, khz = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    uint32_t* buf = nullptr;
    CK(cudaMalloc(&buf, 64 * sizeof(uint32_t) + (size_t)sms * 8 * sizeof(uint32_t)));
    CK(cudaMemset(buf, 0x5A, 64 * sizeof(uint32_t)));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double r[3] = {0, 0, 0};
    if (time_ring<0>(sms, buf, buf + 64, e0, e1, &r[0]) || time_ring<1>(sms, buf, buf + 64, e0, e1, &r[1]) ||
        time_ring<2>(sms, buf, buf + 64, e0, e1, &r[2]))
        return 1;
    const char* name[3] = {"lop3", "iadd3", "imnmx"};
    for (int i = 0; i < 3; i++)
        std::printf("%s: %.4g instructions/s = %.1f lanes/SM/clock at the %d MHz maximum clock\n", name[i], r[i],
                    r[i] / ((double)sms * khz * 1e3), khz / 1000);
    cudaFree(buf);
    return 0;
}
