// Seeded synthetic SMILES-like strings for the benchmark workloads.
//
// Molecule i of a set depends only on (seed, i): a counter-based generator
// (splitmix64 seeding a xoshiro256** stream) and integer/IEEE-double
// arithmetic only, compiled without FMA contraction, so x86 hosts and Arm GPU
// hosts produce byte-identical sets.
//
// Token model: atoms {C,c,N,n,O,o,S,F,Cl,Br} with C and c together drawing 50%
// of all tokens; '(' ')' and ring digits 1-6 are emitted in balanced pairs;
// '=' and '#' bonds.  Length models (characters):
//   SIML_SYNTH_UNIFORM_20_90   uniform integer in [20, 90]
//   SIML_SYNTH_LOGNORMAL_45    lognormal, median 45, sigma 0.5, clipped [10, 200]
//   SIML_SYNTH_BIMODAL_35_110  70% lognormal median 35 (sigma 0.35),
//                              30% lognormal median 110 (sigma 0.3), clipped [10, 250]
//   SIML_SYNTH_CHEM_45         lengths as SIML_SYNTH_LOGNORMAL_45, and real-chemistry
//                              tokens: 12% of atoms are bracket atoms (charges,
//                              explicit hydrogens, stereo centres, isotopes, metals),
//                              '/' and '\\' bonds, and a fifth of ring closures written as
//                              two-digit %nn labels.  These are the bytes that carry
//                              state through the reference's preprocessor (digits after
//                              '+', '-', 'H', '[' are kept; "%nn" becomes "%0").
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "siml_internal.h"

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    Rng(uint64_t seed, uint64_t idx) {
        uint64_t x = seed * 0xD1B54A32D192ED03ull + idx * 0x8CB92BA72F3D8DD7ull + 0x1234567ull;
        for (auto& v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform integer in [0, n)
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
    // uniform double in [0, 1) with 53 random bits
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// exp(x) for |x| <= 8 from the Taylor series of exp(x / 1024) followed by ten
// squarings; plain IEEE double operations only, so the value is the same on
// every host that does not fuse multiply-adds.
double det_exp(double x) {
    double y = x / 1024.0;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 12; k++) {
        term = term * y / (double)k;
        sum = sum + term;
    }
    for (int k = 0; k < 10; k++) sum = sum * sum;
    return sum;
}

// approximately standard normal: Irwin-Hall sum of 12 uniforms minus 6
double approx_normal(Rng& r) {
    double acc = 0.0;
    for (int k = 0; k < 12; k++) acc = acc + r.unit();
    return acc - 6.0;
}

int32_t clampi(int64_t v, int32_t lo, int32_t hi) { return (int32_t)(v < lo ? lo : (v > hi ? hi : v)); }

int32_t lognormal_len(Rng& r, double median, double sigma, int32_t lo, int32_t hi) {
    double v = median * det_exp(sigma * approx_normal(r));
    return clampi((int64_t)(v + 0.5), lo, hi);
}

int32_t draw_length(Rng& r, int dist) {
    switch (dist) {
        case SIML_SYNTH_UNIFORM_20_90: return 20 + (int32_t)r.below(71);
        case SIML_SYNTH_LOGNORMAL_45:
        case SIML_SYNTH_CHEM_45: return lognormal_len(r, 45.0, 0.5, 10, 200);
        case SIML_SYNTH_BIMODAL_35_110:
            if (r.below(100) < 70) return lognormal_len(r, 35.0, 0.35, 10, 250);
            return lognormal_len(r, 110.0, 0.3, 10, 250);
        default: return 40;
    }
}

// token table: cumulative weights in 1/1000
struct Tok { const char* s; int w; int kind; };  // kind: 0 atom, 1 bond, 2 branch-open, 3 ring-open
const Tok kTokens[] = {
    {"C", 250, 0}, {"c", 250, 0}, {"N", 50, 0}, {"n", 50, 0}, {"O", 50, 0},
    {"o", 40, 0}, {"S", 30, 0}, {"F", 20, 0}, {"Cl", 20, 0}, {"Br", 20, 0},
    {"(", 70, 2}, {"=", 40, 1}, {"#", 10, 1}, {"1", 100, 3},
};
constexpr int kNumTokens = sizeof(kTokens) / sizeof(kTokens[0]);

// bracket atoms of the chemistry-like model
const char* const kBracket[] = {"[NH+]", "[NH2+]", "[NH3+]", "[O-]", "[N+]", "[nH]", "[C@@H]", "[C@H]",
                                "[S@@]", "[Na+]", "[Cl-]", "[N-]", "[13CH3]", "[2H]", "[Fe+2]", "[Si]",
                                "[Se]", "[B-]", "[P+]", "[Co+3]"};
constexpr int kNumBracket = sizeof(kBracket) / sizeof(kBracket[0]);

// Writes one molecule into out (capacity >= target + 24); returns its length.
int32_t gen_one(Rng& r, int32_t target, char* out, bool chem) {
    int32_t len = 0;
    int depth = 0;             // open branches
    int open_rings[6] = {0};   // ring i open: 1 written as digit i+1, 2 as "%1" + digit i
    int nopen_rings = 0;
    bool last_atom = false;
    auto put = [&](const char* s) { while (*s) out[len++] = *s++; };
    auto atom = [&]() {
        if (chem && r.below(100) < 12) {
            put(kBracket[r.below(kNumBracket)]);
        } else {
            // atoms only, same relative weights
            uint32_t u = r.below(780);  // sum of the atom weights
            int acc = 0;
            for (int t = 0; t < 10; t++) {
                acc += kTokens[t].w;
                if ((int)u < acc) { put(kTokens[t].s); break; }
            }
        }
        last_atom = true;
    };
    auto ring_label = [&](int k, int kind) {
        if (kind == 2) {
            out[len++] = '%';
            out[len++] = '1';
        }
        out[len++] = (char)((kind == 2 ? '0' : '1') + k);
    };
    atom();
    while (len + depth + nopen_rings < target) {
        // close a branch or a ring with some probability once an atom is down
        if (last_atom && depth > 0 && r.below(100) < 30) { put(")"); depth--; last_atom = false; atom(); continue; }
        if (last_atom && nopen_rings > 0 && r.below(100) < 25) {
            int k = (int)r.below(6);
            while (!open_rings[k]) k = (k + 1) % 6;
            ring_label(k, open_rings[k]);
            open_rings[k] = 0;
            nopen_rings--;
            continue;
        }
        uint32_t u = r.below(1000);
        int acc = 0, t = 0;
        for (; t < kNumTokens; t++) {
            acc += kTokens[t].w;
            if ((int)u < acc) break;
        }
        const Tok& tk = kTokens[t];
        switch (tk.kind) {
            case 0: put(tk.s); last_atom = true; break;
            case 1:
                if (last_atom) {
                    if (chem && r.below(100) < 20) put(r.below(2) ? "/" : "\\");
                    else put(tk.s);
                    atom();
                }
                break;
            case 2: if (last_atom && depth < 4) { put("("); depth++; atom(); } break;
            case 3:
                if (last_atom && nopen_rings < 6) {
                    int k = (int)r.below(6);
                    while (open_rings[k]) k = (k + 1) % 6;
                    const int kind = chem && r.below(100) < 20 ? 2 : 1;
                    ring_label(k, kind);
                    open_rings[k] = kind;
                    nopen_rings++;
                }
                break;
        }
    }
    for (int k = 0; k < 6; k++)
        if (open_rings[k]) ring_label(k, open_rings[k]);
    while (depth-- > 0) put(")");
    return len;
}

}  // namespace

extern "C" {

// Byte lengths of molecules [first, first+n) of the set (seed, dist) — call
// this first to size the buffer for siml_synth_smiles.
int siml_synth_lengths(uint64_t seed, int dist, int64_t first, int64_t n, int32_t* lens) {
    if (n < 0 || !lens || first < 0) return siml::fail(SIML_ERR_INVALID, "siml_synth_lengths: bad arguments");
    if (dist < SIML_SYNTH_UNIFORM_20_90 || dist > SIML_SYNTH_CHEM_45)
        return siml::fail(SIML_ERR_INVALID, "siml_synth_lengths: unknown length model");
    siml::parallel_for(n, [&](int64_t i) {
        Rng r(seed, (uint64_t)(first + i));
        char tmp[640];
        int32_t target = draw_length(r, dist);
        lens[i] = gen_one(r, target, tmp, dist == SIML_SYNTH_CHEM_45);
    });
    return SIML_OK;
}

// Molecules [first, first+n) of the set (seed, dist), concatenated into buf;
// offsets[n+1] receives the start of each string (no separators, no NULs).
int siml_synth_smiles(uint64_t seed, int dist, int64_t first, int64_t n,
                      char* buf, int64_t bufcap, int64_t* offsets) {
    if (n < 0 || !buf || !offsets || first < 0) return siml::fail(SIML_ERR_INVALID, "siml_synth_smiles: bad arguments");
    if (dist < SIML_SYNTH_UNIFORM_20_90 || dist > SIML_SYNTH_CHEM_45)
        return siml::fail(SIML_ERR_INVALID, "siml_synth_smiles: unknown length model");
    std::vector<int32_t> lens((size_t)n);
    int rc = siml_synth_lengths(seed, dist, first, n, lens.data());
    if (rc) return rc;
    offsets[0] = 0;
    for (int64_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + lens[(size_t)i];
    if (offsets[n] > bufcap) return siml::fail(SIML_ERR_INVALID, "siml_synth_smiles: buffer too small");
    siml::parallel_for(n, [&](int64_t i) {
        Rng r(seed, (uint64_t)(first + i));
        char tmp[640];
        int32_t target = draw_length(r, dist);
        int32_t L = gen_one(r, target, tmp, dist == SIML_SYNTH_CHEM_45);
        std::memcpy(buf + offsets[i], tmp, (size_t)L);
    });
    return SIML_OK;
}

}  // extern "C"
