/*
 * ORACLE -- test infrastructure only.
 *
 * The seeded synthetic inputs of the benchmark workloads, restated for the
 * host side that must not load the shipped library: the reference arm of the
 * benchmark and the CPU baselines generate their instances here, and a CPU
 * test checks that every output equals the library's own generator
 * (gpsat_gen_random_ksat / gpsat_gen_trails) bit for bit.
 *
 * Generator: splitmix64 with one independent stream per clause or per trail,
 * stream state = mix(seed * golden + mix(stream + c)); uniform(n) is the high
 * 64 bits of draw * n (multiply-shift).  Random k-SAT: per clause, k distinct
 * variables by rejection, each with a fair sign from the draw's top bit.
 * Trails: length round(n * (fmin + (fmax - fmin) * u)) clamped to [1, n],
 * distinct variables by Floyd's sampling, a Fisher-Yates shuffle, fair signs.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define GOLDEN 0x9E3779B97F4A7C15ULL

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

typedef struct { uint64_t s; } rng_t;

static inline rng_t rng_make(uint64_t seed, uint64_t stream)
{
    rng_t r;
    r.s = mix64(seed * GOLDEN + mix64(stream + 0x632BE59BD9B4E019ULL));
    return r;
}
static inline uint64_t rng_next(rng_t *r) { return mix64(r->s += GOLDEN); }
/* high 64 bits of x * n for n < 2^32, from 32-bit halves */
static inline uint32_t rng_below(rng_t *r, uint32_t n)
{
    uint64_t x = rng_next(r);
    uint64_t lo = (x & 0xFFFFFFFFULL) * n, hi = (x >> 32) * n;
    return (uint32_t)((hi + (lo >> 32)) >> 32);
}
static inline double rng_unit(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

int orc_gen_random_ksat(uint64_t seed, int32_t n_vars, int64_t n_clauses, int32_t k, int32_t *lits)
{
    if (n_vars <= 0 || n_clauses < 0 || k <= 0 || k > n_vars || k > 64) return -1;
    for (int64_t c = 0; c < n_clauses; c++) {
        rng_t r = rng_make(seed, (uint64_t)c);
        int32_t *out = lits + c * k;
        for (int32_t i = 0; i < k; i++) {
            uint32_t v;
            int dup;
            do {
                v = rng_below(&r, (uint32_t)n_vars);
                dup = 0;
                for (int32_t j = 0; j < i; j++) dup |= (uint32_t)(abs(out[j]) - 1) == v;
            } while (dup);
            out[i] = (rng_next(&r) >> 63) ? (int32_t)v + 1 : -((int32_t)v + 1);
        }
    }
    return 0;
}

static int64_t trail_len(uint64_t seed, int32_t t, int32_t n, double fmin, double fmax)
{
    rng_t r = rng_make(seed, 0x7472616900000000ULL + (uint64_t)t);
    double f = fmin + (fmax - fmin) * rng_unit(&r);
    int64_t u = (int64_t)llround(f * n);
    if (u > n) u = n;
    return u < 1 ? 1 : u;
}

/* offsets[n_trails + 1]; lits may be NULL (offsets only) */
int orc_gen_trails(uint64_t seed, int32_t n_vars, int32_t n_trails, double fmin, double fmax, int64_t *offsets,
                   int32_t *lits)
{
    if (n_vars <= 0 || n_trails < 0 || !offsets || !(fmin >= 0.0) || !(fmax >= fmin) || fmax > 1.0) return -1;
    offsets[0] = 0;
    for (int32_t t = 0; t < n_trails; t++) offsets[t + 1] = offsets[t] + trail_len(seed, t, n_vars, fmin, fmax);
    if (!lits) return 0;
    uint64_t *bits = (uint64_t *)calloc(((size_t)n_vars + 63) / 64, 8);
    if (!bits) return -2;
    for (int32_t t = 0; t < n_trails; t++) {
        int64_t u = offsets[t + 1] - offsets[t], cnt = 0;
        int32_t *out = lits + offsets[t];
        rng_t r = rng_make(seed, 0x5452414900000000ULL + (uint64_t)t);
        for (int64_t j = n_vars - u; j < n_vars; j++) {
            uint32_t x = rng_below(&r, (uint32_t)(j + 1));
            if ((bits[x >> 6] >> (x & 63)) & 1) x = (uint32_t)j;
            bits[x >> 6] |= 1ULL << (x & 63);
            out[cnt++] = (int32_t)x;
        }
        for (int64_t i = u - 1; i > 0; i--) {
            int64_t j = rng_below(&r, (uint32_t)(i + 1));
            int32_t tmp = out[i];
            out[i] = out[j];
            out[j] = tmp;
        }
        for (int64_t i = 0; i < u; i++) {
            int32_t v = out[i];
            bits[(uint32_t)v >> 6] = 0;
            out[i] = (rng_next(&r) >> 63) ? v + 1 : -(v + 1);
        }
    }
    free(bits);
    return 0;
}
