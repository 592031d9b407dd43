// Host-side unit test of the bit-sliced intersection counter and the plane
// transpose used by the CUDA kernels (siml_gb300/csrc/lingo_core.cuh): random
// 32-row masks are accumulated and every row's count is compared with a
// scalar popcount sum.  Exit status 0 on success.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include "lingo_core.cuh"

static uint64_t state = 88172645463325252ull;
static uint32_t rnd() { state ^= state << 13; state ^= state >> 7; state ^= state << 17; return (uint32_t)state; }

template <int NP>
static int run(int trials, int max_masks) {
    for (int t = 0; t < trials; t++) {
        siml::SlicedCounter<NP> c;
        c.clear();
        uint32_t ref[32] = {0};
        int nmask = (int)(rnd() % (uint32_t)(max_masks + 1));
        int n8 = (nmask + 7) / 8;
        for (int b = 0; b < n8; b++) {
            uint32_t m[8];
            for (int i = 0; i < 8; i++) {
                int idx = b * 8 + i;
                uint32_t density = rnd() % 4;
                uint32_t v = rnd();
                if (density == 0) v &= rnd();
                if (density == 1) v |= rnd();
                if (density == 2) v = (rnd() & 1) ? 0xFFFFFFFFu : 0u;
                m[i] = idx < nmask ? v : 0u;
                for (int r = 0; r < 32; r++) ref[r] += (m[i] >> r) & 1u;
            }
            c.add8(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7]);
        }
        siml::RowCounts<NP> rc;
        siml::counts_from_planes<NP>(c, rc);
        for (int r = 0; r < 32; r++) {
            uint32_t got = siml::row_count<NP>(rc, r);
            if (siml::row_count_dyn<NP>(rc, r) != got) {
                std::printf("NP=%d row_count_dyn differs at row %d\n", NP, r);
                return 1;
            }
            if (got != ref[r]) {
                std::printf("NP=%d trial %d row %d: got %u want %u (nmask %d)\n", NP, t, r, got, ref[r], nmask);
                return 1;
            }
        }
    }
    return 0;
}

int main() {
    if (run<8>(20000, 255)) return 1;
    if (run<16>(5000, 4000)) return 1;
    std::printf("sliced counter ok\n");
    return 0;
}
