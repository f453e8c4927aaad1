// Seeded synthetic inputs: uniform random k-SAT, planted k-SAT with community
// structure, and random partial trails.
//
// Generator: splitmix64 with one independent stream per clause or per trail
// (stream state = mix(seed, index)), so the output is the same whatever the
// number of host threads.  uniform(n) is the high 64 bits of draw * n
// (Lemire's multiply-shift; the bias is below 2^-32 for n < 2^32).
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "internal.h"

namespace gpsat {

namespace {

inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s;
    Rng(uint64_t seed, uint64_t stream) : s(mix64(seed * 0x9E3779B97F4A7C15ULL + mix64(stream + 0x632BE59BD9B4E019ULL))) {}
    uint64_t next() { return mix64(s += 0x9E3779B97F4A7C15ULL); }
    uint32_t below(uint32_t n) { return (uint32_t)(((unsigned __int128)next() * n) >> 64); }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

template <class F>
void parallel_for(int64_t n, F fn)
{
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int64_t nt = std::min<int64_t>(hw, std::max<int64_t>(1, n / 256));
    if (nt <= 1) {
        fn(0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; t++) {
        int64_t b = n * t / nt, e = n * (t + 1) / nt;
        th.emplace_back([=] { fn(b, e, (int)t); });
    }
    for (auto &x : th) x.join();
}

int64_t trail_len(uint64_t seed, int32_t t, int32_t n, double fmin, double fmax)
{
    Rng r(seed, 0x7472616900000000ULL + (uint64_t)t);
    double f = fmin + (fmax - fmin) * r.unit();
    int64_t u = (int64_t)std::llround(f * n);
    return std::max<int64_t>(1, std::min<int64_t>(u, n));
}

}  // namespace

}  // namespace gpsat

using namespace gpsat;

extern "C" int gpsat_gen_random_ksat(uint64_t seed, int32_t n_vars, int64_t n_clauses, int32_t k, int32_t *lits)
{
    if (n_vars <= 0 || n_clauses < 0 || k <= 0 || k > n_vars || k > 64 || (n_clauses > 0 && !lits))
        return set_error(GPSAT_ERR_ARG, "gpsat_gen_random_ksat: need 0 < k <= min(n_vars, 64)");
    parallel_for(n_clauses, [&](int64_t b, int64_t e, int) {
        for (int64_t c = b; c < e; c++) {
            Rng r(seed, (uint64_t)c);
            int32_t *out = lits + c * k;
            for (int32_t i = 0; i < k; i++) {
                uint32_t v;
                bool dup;
                do {
                    v = r.below((uint32_t)n_vars);
                    dup = false;
                    for (int32_t j = 0; j < i; j++) dup |= (uint32_t)(std::abs(out[j]) - 1) == v;
                } while (dup);
                out[i] = (r.next() >> 63) ? (int32_t)v + 1 : -((int32_t)v + 1);
            }
        }
    });
    return GPSAT_OK;
}

extern "C" int gpsat_gen_trails(uint64_t seed, int32_t n_vars, int32_t n_trails, double fmin, double fmax,
                                int64_t *offsets, int32_t *lits)
{
    if (n_vars <= 0 || n_trails < 0 || !offsets || !(fmin >= 0.0) || !(fmax >= fmin) || fmax > 1.0)
        return set_error(GPSAT_ERR_ARG, "gpsat_gen_trails: need n_vars > 0, 0 <= fmin <= fmax <= 1");
    offsets[0] = 0;
    for (int32_t t = 0; t < n_trails; t++) offsets[t + 1] = offsets[t] + trail_len(seed, t, n_vars, fmin, fmax);
    if (!lits) return GPSAT_OK;
    parallel_for(n_trails, [&](int64_t b, int64_t e, int) {
        // Floyd's sampling of distinct variables with a bitmap, then a
        // Fisher-Yates shuffle for a uniformly random order.
        std::vector<uint64_t> bits(((size_t)n_vars + 63) / 64, 0);
        for (int64_t t = b; t < e; t++) {
            int64_t u = offsets[t + 1] - offsets[t];
            int32_t *out = lits + offsets[t];
            Rng r(seed, 0x5452414900000000ULL + (uint64_t)t);
            int64_t cnt = 0;
            for (int64_t j = n_vars - u; j < n_vars; j++) {
                uint32_t x = r.below((uint32_t)(j + 1));
                if (bits[x >> 6] >> (x & 63) & 1) x = (uint32_t)j;
                bits[x >> 6] |= 1ULL << (x & 63);
                out[cnt++] = (int32_t)x;
            }
            for (int64_t i = u - 1; i > 0; i--) {
                int64_t j = r.below((uint32_t)(i + 1));
                std::swap(out[i], out[j]);
            }
            for (int64_t i = 0; i < u; i++) {
                int32_t v = out[i];
                bits[(uint32_t)v >> 6] = 0;
                out[i] = (r.next() >> 63) ? v + 1 : -(v + 1);
            }
        }
    });
    return GPSAT_OK;
}

extern "C" int gpsat_gen_planted(uint64_t seed, int32_t n_vars, int64_t n_clauses, int32_t k, int32_t n_communities,
                                 double p_in, int32_t *lits, int8_t *planted)
{
    if (n_vars <= 0 || n_clauses < 0 || k <= 0 || k > 64 || n_communities <= 0 || n_communities > n_vars ||
        k > n_vars / n_communities || !(p_in >= 0.0 && p_in <= 1.0) || (n_clauses > 0 && !lits))
        return set_error(GPSAT_ERR_ARG,
                         "gpsat_gen_planted: need 0 < k <= n_vars / n_communities, k <= 64, 0 <= p_in <= 1");
    // the hidden assignment: one bit per variable from its own stream
    auto value = [&](int32_t v) { return (Rng(seed, 0x504C414E00000000ULL + (uint64_t)v).next() >> 63) != 0; };
    if (planted)
        parallel_for(n_vars, [&](int64_t b, int64_t e, int) {
            for (int64_t v = b; v < e; v++) planted[v] = value((int32_t)v) ? 1 : -1;
        });
    // community g holds variables [g*n/G, (g+1)*n/G)
    auto first = [&](int64_t g) { return (int32_t)(g * n_vars / n_communities); };
    parallel_for(n_clauses, [&](int64_t b, int64_t e, int) {
        for (int64_t c = b; c < e; c++) {
            Rng r(seed, (uint64_t)c);
            int32_t *out = lits + c * k;
            const int32_t g = (int32_t)r.below((uint32_t)n_communities);
            const int32_t lo = first(g), size = first(g + 1) - lo;
            for (int32_t i = 0; i < k; i++) {
                const bool inside = r.unit() < p_in;
                uint32_t v;
                bool dup;
                do {
                    v = inside ? (uint32_t)lo + r.below((uint32_t)size) : r.below((uint32_t)n_vars);
                    dup = false;
                    for (int32_t j = 0; j < i; j++) dup |= (uint32_t)(std::abs(out[j]) - 1) == v;
                } while (dup);
                out[i] = (int32_t)v + 1;
            }
            // signs: uniform over the patterns the hidden assignment satisfies
            // (rejection: a pattern is redrawn while every literal is false)
            bool sat = false;
            while (!sat) {
                for (int32_t i = 0; i < k; i++) {
                    const int32_t v = std::abs(out[i]);
                    const bool pos = (r.next() >> 63) != 0;
                    out[i] = pos ? v : -v;
                    sat |= pos == value(v - 1);
                }
            }
        }
    });
    return GPSAT_OK;
}
