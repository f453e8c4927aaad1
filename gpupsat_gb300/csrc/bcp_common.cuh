// Shared by the BCP kernels (bcp_window.cuh, built at several window widths)
// and the host code in bcp.cu: the device view of a BCP launch, the literal
// and assignment helpers, and the reference's process_clause for long
// clauses.  See bcp_window.cuh for the algorithm and the layout.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstddef>
#include <cstdint>

#include "internal.h"

namespace gpsat {
namespace bcp {


constexpr unsigned FULL = 0xffffffffu;
constexpr int KIN = 4;            // clause literals stored inside a watch entry
constexpr uint32_t EPMAX = 255;   // epochs per slot before a wipe
constexpr int MAXLEN = 2048;      // clause length limit (11-bit watch indices)
constexpr int MAXSC = 32;         // window scans (the current one + 31 following)
constexpr int LB = 128;           // look-ahead ring positions
constexpr int CHUNK = 32;         // ring refill granularity (one warp)
constexpr int LEAD = 96;          // ring positions kept ahead of the trail cursor
constexpr int64_t MAX_ITERS = int64_t(1) << 26;  // per-trail loop iterations before GPSAT_BCP_BUDGET

constexpr int MIN_WARPS = 2, MAX_WARPS = 8;    // window widths built: 64, 128 and 256 entries
constexpr int DEFAULT_WARPS = 4;

enum : int { A_NONE = 0, A_SW1 = 1, A_SW2 = 2, A_BLOCK = 3, A_IMPLY = 4, A_CONFLICT = 5 };

struct Dev {
    int32_t n_vars;
    int32_t n_clauses;
    const int32_t *__restrict__ lits;
    const uint32_t *__restrict__ w0off;
    const int4 *__restrict__ w0ent;   // 2 int4 per entry
    uint32_t *asg;
    uint32_t *dh;
    uint32_t *cst;
    int4 *arena;                      // 2 int4 per entry
    int2 *stack;
    int32_t *impl;
    uint32_t *epoch;
    unsigned int *next_trail;
    const int32_t *order;             // trails in processing order (null: index order)
    int64_t n_words, n_pad, m_pad, arena_cap, impl_cap;
    int32_t n_slots;
    const int32_t *__restrict__ trail;
    const int64_t *__restrict__ toff;
    int32_t n_trails;
    int32_t *status, *conflict, *stop;
    int64_t *nimpl;
    int32_t *ilit, *ireason;
    int64_t *counters;
    // trails applied beforehand (apply_kernel): trail t's assignment words at
    // tasg + t * n_words and its bad-trail flag tbad[t]; null: each block
    // assigns its trail into its slot's asg words and clears them after
    uint32_t *tasg;
    const int32_t *tbad;
};

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
template <class T>
__device__ __forceinline__ T warp_sum(T x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    return x;
}
__device__ __forceinline__ int32_t dimacs_of(int32_t l) { return (l & 1) ? (l >> 1) + 1 : -((l >> 1) + 1); }

// assignment bits of variable v inside its word: bit 0 assigned, bit 1 sign (1 = true)
__device__ __forceinline__ uint32_t asg_bits(uint32_t word, int32_t v) { return (word >> ((v & 15) << 1)) & 3u; }
// literal l is consistent (unassigned, or true) given its variable's bits
__device__ __forceinline__ bool cons_of(uint32_t b, int32_t l) { return !(b & 1u) || ((b >> 1) == (uint32_t)(l & 1)); }

struct Eval {
    int act;
    int nw1, nw2;       // new watch indices (switch)
    int32_t t1, t2;     // switch target vars
    int32_t unit;       // unit literal (imply)
    int acnt;           // assignment lookups as the reference counts them
};

// process_clause of the reference for a clause too long for the inline path
// (literals and their assignment words read from memory one by one).
static __device__ __noinline__ void eval_long(const Dev &d, const uint32_t *asg, int off, int len, int w1, int w2, Eval &r)
{
    const int32_t *L = d.lits + off;
    const int32_t l1 = L[w1], l2 = L[w2];
    const bool c1 = cons_of(asg_bits(asg[(l1 >> 1) >> 4], l1 >> 1), l1);
    const bool c2 = cons_of(asg_bits(asg[(l2 >> 1) >> 4], l2 >> 1), l2);
    r.acnt = 2;
    r.act = A_NONE;
    if (c1 && c2) return;
    int pend = (!c1 && !c2) ? 2 : 1, f1 = -1, f2 = -1;
    for (int i = 0; pend > 0 && i < len; i++) {
        if (i == w1 || i == w2) continue;
        const int32_t l = L[i];
        r.acnt++;
        if (cons_of(asg_bits(asg[(l >> 1) >> 4], l >> 1), l)) {
            if (f1 < 0) f1 = i;
            else f2 = i;
            pend--;
        }
    }
    int32_t unit = -1;
    if (c1 || c2) {
        if (f1 < 0) {
            unit = c1 ? l1 : l2;
        } else {
            r.act = A_SW1;
            r.nw1 = c1 ? w1 : f1;
            r.nw2 = c1 ? f1 : w2;
            r.t1 = L[f1] >> 1;
            return;
        }
    } else if (f1 >= 0 && f2 >= 0) {
        r.act = A_SW2;
        r.nw1 = f1;
        r.nw2 = f2;
        r.t1 = L[f1] >> 1;
        r.t2 = L[f2] >> 1;
        return;
    } else if (f1 >= 0) {
        unit = L[f1];
    } else {
        r.act = A_CONFLICT;
        return;
    }
    r.unit = unit;
    r.act = (asg_bits(asg[(unit >> 1) >> 4], unit >> 1) & 1u) ? A_BLOCK : A_IMPLY;
}

// commit-cut keys: (window position << 7) | (window scan << 1) | after
constexpr int NO_CUT = INT_MAX;
__device__ __forceinline__ int key_before(int pos, int scan) { return (pos << 7) | (scan << 1); }
__device__ __forceinline__ int key_after(int pos, int scan) { return ((pos + 1) << 7) | (scan << 1) | 1; }

// The ring chunk that warp 1 carries between rounds: lanes hold trail
// positions [ring_hi + 32, +32) as literals (stage 1) and [ring_hi, +32) as
// variable, initial-list range and list head in flight (stage 2).
struct RingPipe {
    int32_t lit;
    int32_t var;
    uint32_t a, b, h;
};

// One build of the BCP kernel per window width (warps per block): its launch
// and its resident blocks per SM (bcp_w2.cu, bcp_w4.cu, bcp_w8.cu).
struct Variant {
    int warps;
    cudaError_t (*launch)(const Dev &d, int blocks, cudaStream_t st);
    cudaError_t (*occupancy)(int *blocks_per_sm);
};
const Variant *variant(int warps);   // nullptr for a width not built

}  // namespace bcp
}  // namespace gpsat
