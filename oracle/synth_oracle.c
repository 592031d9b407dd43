/*
 * ORACLE — test infrastructure only.
 *
 * The seeded synthetic SMILES generator of the benchmark workloads, in plain
 * C, so that the CPU reference arm of bench.py generates its inputs without
 * loading the product library.  It must produce the same bytes as the
 * product's generator (siml_gb300/csrc/synth.cpp); tests/test_compiler.py
 * compares the two.  Molecule i of a set depends only on (seed, model, i):
 * splitmix64 seeds a xoshiro256** stream per molecule, and only integer and
 * IEEE-double arithmetic is used (no libm; built with -ffp-contract=off), so
 * x86 and Arm hosts agree.
 *
 * Length models (characters): 0 uniform [20, 90]; 1 lognormal median 45,
 * sigma 0.5, clipped [10, 200]; 2 bimodal, 70% lognormal median 35 (sigma
 * 0.35), 30% median 110 (sigma 0.3), clipped [10, 250]; 3 as 1 with the
 * chemistry-like tokens (bracket atoms, '/' '\\' bonds, %nn ring labels).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

typedef struct { uint64_t s[4]; } o_rng;

static uint64_t o_splitmix(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void o_rng_init(o_rng* r, uint64_t seed, uint64_t idx) {
    uint64_t x = seed * 0xD1B54A32D192ED03ull + idx * 0x8CB92BA72F3D8DD7ull + 0x1234567ull;
    for (int i = 0; i < 4; i++) r->s[i] = o_splitmix(&x);
}

static uint64_t o_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t o_next(o_rng* r) {
    uint64_t* s = r->s;
    const uint64_t res = o_rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = o_rotl(s[3], 45);
    return res;
}

static uint32_t o_below(o_rng* r, uint32_t n) { return (uint32_t)(((o_next(r) >> 32) * (uint64_t)n) >> 32); }
static double o_unit(o_rng* r) { return (double)(o_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* exp(x) for |x| <= 8: Taylor series of exp(x / 1024), then ten squarings */
static double o_exp(double x) {
    double y = x / 1024.0, term = 1.0, sum = 1.0;
    for (int k = 1; k <= 12; k++) {
        term = term * y / (double)k;
        sum = sum + term;
    }
    for (int k = 0; k < 10; k++) sum = sum * sum;
    return sum;
}

/* Irwin-Hall sum of 12 uniforms minus 6 */
static double o_normal(o_rng* r) {
    double acc = 0.0;
    for (int k = 0; k < 12; k++) acc = acc + o_unit(r);
    return acc - 6.0;
}

static int32_t o_clamp(int64_t v, int32_t lo, int32_t hi) { return (int32_t)(v < lo ? lo : (v > hi ? hi : v)); }

static int32_t o_lognormal(o_rng* r, double median, double sigma, int32_t lo, int32_t hi) {
    double v = median * o_exp(sigma * o_normal(r));
    return o_clamp((int64_t)(v + 0.5), lo, hi);
}

static int32_t o_length(o_rng* r, int model) {
    switch (model) {
        case 0: return 20 + (int32_t)o_below(r, 71);
        case 1:
        case 3: return o_lognormal(r, 45.0, 0.5, 10, 200);
        case 2:
            if (o_below(r, 100) < 70) return o_lognormal(r, 35.0, 0.35, 10, 250);
            return o_lognormal(r, 110.0, 0.3, 10, 250);
        default: return 40;
    }
}

/* tokens with weights in 1/1000; kind 0 atom, 1 bond, 2 branch, 3 ring digit */
static const char* const o_tok_s[] = {"C", "c", "N", "n", "O", "o", "S", "F", "Cl", "Br", "(", "=", "#", "1"};
static const int o_tok_w[] = {250, 250, 50, 50, 50, 40, 30, 20, 20, 20, 70, 40, 10, 100};
static const int o_tok_k[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 1, 1, 3};
#define O_NTOK 14

static const char* const o_bracket[] = {"[NH+]", "[NH2+]", "[NH3+]", "[O-]", "[N+]", "[nH]", "[C@@H]", "[C@H]",
                                       "[S@@]", "[Na+]", "[Cl-]", "[N-]", "[13CH3]", "[2H]", "[Fe+2]", "[Si]",
                                       "[Se]", "[B-]", "[P+]", "[Co+3]"};
#define O_NBRACKET 20

typedef struct {
    char* out;
    int32_t len;
    int depth, nrings, last_atom, chem;
    int rings[6];   /* 1: written as digit i+1, 2: as "%1" + digit i */
} o_gen;

static void o_put(o_gen* g, const char* s) { while (*s) g->out[g->len++] = *s++; }

static void o_atom(o_gen* g, o_rng* r) {
    if (g->chem && o_below(r, 100) < 12) {
        o_put(g, o_bracket[o_below(r, O_NBRACKET)]);
    } else {
        uint32_t u = o_below(r, 780);   /* sum of the atom weights */
        int acc = 0;
        for (int t = 0; t < 10; t++) {
            acc += o_tok_w[t];
            if ((int)u < acc) { o_put(g, o_tok_s[t]); break; }
        }
    }
    g->last_atom = 1;
}

static void o_ring_label(o_gen* g, int k, int kind) {
    if (kind == 2) {
        g->out[g->len++] = '%';
        g->out[g->len++] = '1';
    }
    g->out[g->len++] = (char)((kind == 2 ? '0' : '1') + k);
}

/* one molecule into out (capacity >= target + 24); returns its length */
static int32_t o_gen_one(o_rng* r, int32_t target, char* out, int chem) {
    o_gen g;
    memset(&g, 0, sizeof(g));
    g.out = out;
    g.chem = chem;
    o_atom(&g, r);
    while (g.len + g.depth + g.nrings < target) {
        if (g.last_atom && g.depth > 0 && o_below(r, 100) < 30) {
            o_put(&g, ")");
            g.depth--;
            g.last_atom = 0;
            o_atom(&g, r);
            continue;
        }
        if (g.last_atom && g.nrings > 0 && o_below(r, 100) < 25) {
            int k = (int)o_below(r, 6);
            while (!g.rings[k]) k = (k + 1) % 6;
            o_ring_label(&g, k, g.rings[k]);
            g.rings[k] = 0;
            g.nrings--;
            continue;
        }
        uint32_t u = o_below(r, 1000);
        int acc = 0, t = 0;
        for (; t < O_NTOK; t++) {
            acc += o_tok_w[t];
            if ((int)u < acc) break;
        }
        switch (o_tok_k[t]) {
            case 0: o_put(&g, o_tok_s[t]); g.last_atom = 1; break;
            case 1:
                if (g.last_atom) {
                    if (g.chem && o_below(r, 100) < 20) o_put(&g, o_below(r, 2) ? "/" : "\\");
                    else o_put(&g, o_tok_s[t]);
                    o_atom(&g, r);
                }
                break;
            case 2: if (g.last_atom && g.depth < 4) { o_put(&g, "("); g.depth++; o_atom(&g, r); } break;
            case 3:
                if (g.last_atom && g.nrings < 6) {
                    int k = (int)o_below(r, 6);
                    while (g.rings[k]) k = (k + 1) % 6;
                    const int kind = g.chem && o_below(r, 100) < 20 ? 2 : 1;
                    o_ring_label(&g, k, kind);
                    g.rings[k] = kind;
                    g.nrings++;
                }
                break;
        }
    }
    for (int k = 0; k < 6; k++)
        if (g.rings[k]) o_ring_label(&g, k, g.rings[k]);
    while (g.depth-- > 0) o_put(&g, ")");
    return g.len;
}

/* Byte lengths of molecules [first, first + n) of the set (seed, model). */
ORACLE_API int oracle_synth_lengths(uint64_t seed, int model, int64_t first, int64_t n, int32_t* lens) {
    if (n < 0 || first < 0 || model < 0 || model > 3) return -1;
    int64_t i;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (i = 0; i < n; i++) {
        o_rng r;
        char tmp[640];
        o_rng_init(&r, seed, (uint64_t)(first + i));
        lens[i] = o_gen_one(&r, o_length(&r, model), tmp, model == 3);
    }
    return 0;
}

/* Molecules [first, first + n), concatenated into buf (offsets[s] is the start
 * of string s, offsets[n] the total; no separators). */
ORACLE_API int oracle_synth_smiles(uint64_t seed, int model, int64_t first, int64_t n, char* buf, int64_t bufcap,
                                   int64_t* offsets) {
    if (n < 0 || first < 0 || model < 0 || model > 3) return -1;
    int32_t* lens = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    if (!lens) return -1;
    oracle_synth_lengths(seed, model, first, n, lens);
    offsets[0] = 0;
    for (int64_t i = 0; i < n; i++) offsets[i + 1] = offsets[i] + lens[i];
    free(lens);
    if (offsets[n] > bufcap) return -1;
    int64_t i;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (i = 0; i < n; i++) {
        o_rng r;
        char tmp[640];
        o_rng_init(&r, seed, (uint64_t)(first + i));
        const int32_t L = o_gen_one(&r, o_length(&r, model), tmp, model == 3);
        memcpy(buf + offsets[i], tmp, (size_t)L);
    }
    return 0;
}
