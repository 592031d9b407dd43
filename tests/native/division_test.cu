// Exhaustive check of div_small_int (siml_gb300/csrc/lingo_core.cuh) against
// the IEEE division __fdiv_rn: every 0 <= a <= b <= 65536, plus a sample of
// a up to 2^24 for each b.  Prints the mismatch count; exit status 0 when
// there is none.  One block per divisor b; no thread waits on another.
#include <cstdio>
#include <cuda_runtime.h>
#include "lingo_core.cuh"

__global__ void check(int bmax, unsigned long long* bad, int* first_a, int* first_b) {
    const int b = blockIdx.x + 1;
    if (b > bmax) return;
    unsigned long long nbad = 0;
    for (int a = threadIdx.x; a <= b; a += blockDim.x) {
        const float want = __fdiv_rn((float)a, (float)b);
        const float got = siml::div_small_int(a, b);
        if (__float_as_uint(want) != __float_as_uint(got)) {
            if (nbad == 0) { *first_a = a; *first_b = b; }
            nbad++;
        }
    }
    // larger numerators: a = k * 4099 + b, up to 2^24
    for (int k = threadIdx.x; k < 4096; k += blockDim.x) {
        const long long a64 = (long long)k * 4099 + b;
        if (a64 > (1 << 24)) break;
        const int a = (int)a64;
        const float want = __fdiv_rn((float)a, (float)b);
        const float got = siml::div_small_int(a, b);
        if (__float_as_uint(want) != __float_as_uint(got)) nbad++;
    }
    if (nbad) atomicAdd(bad, nbad);
}

int main() {
    const int bmax = 65536;
    unsigned long long* d_bad = nullptr;
    int* d_ab = nullptr;
    if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess) return 2;
    if (cudaMalloc(&d_ab, 2 * sizeof(int)) != cudaSuccess) return 2;
    cudaMemset(d_bad, 0, sizeof(unsigned long long));
    cudaMemset(d_ab, 0xFF, 2 * sizeof(int));
    check<<<bmax, 256>>>(bmax, d_bad, d_ab, d_ab + 1);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { std::printf("cuda error %s\n", cudaGetErrorString(e)); return 2; }
    unsigned long long bad = 0;
    int ab[2];
    cudaMemcpy(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost);
    cudaMemcpy(ab, d_ab, sizeof(ab), cudaMemcpyDeviceToHost);
    std::printf("div_small_int mismatches: %llu (first a=%d b=%d)\n", bad, ab[0], ab[1]);
    return bad == 0 ? 0 : 1;
}
