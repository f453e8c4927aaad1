// Two-watched-literal BCP over a batch of partial trails, in the reference's
// own processing order (bit-exact implied literals, reasons and conflict
// clause), on sm_103a.
//
// Reference behaviour (paths inside the reference project, src/):
//   trail application   SATSolver/VariablesStateHandler.cu:35-59 then
//                       ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu:56-73
//   new_decision        BCPStrategy/WatchedClausesList.cu:46-101 (snapshot of the
//                       var's list, then depth-first over new implications)
//   process_clause      BCPStrategy/WatchedClausesList.cu:103-221
//   handle_implication  BCPStrategy/WatchedClausesList.cu:253-282
//   block / switch      BCPStrategy/ClauseListStructure.cu:73-92, 150-164
//
// Layout (HBM):
//   formula (shared by all trails, read-only)
//     lits[]   internal literals, CSR by clause
//     w0off[]  per-var offsets into w0ent
//     w0ent[]  32 bytes per initial watch: {clause, literal offset, length,
//              (w1<<16)|w2} {first four literals}; each var's entries in the
//              reference's initial list order
//   per trail slot (one thread block owns one slot; slots are reused)
//     asg[n/16]  2 bits per variable (assigned, sign): the trail literals and
//                the pending implications; zero between trails (a trail
//                clears the words it set)
//     dh[n]      uint32 (epoch<<24)|arena index: head of the clauses
//                add_first'ed to the variable
//     cst[m]     uint32 (epoch<<24)|(blocked<<22)|(w1<<11)|w2: clauses whose
//                watches moved or that were blocked
//     arena[]    32 bytes per entry: {clause, literal offset, length, next} {literals}
//     stack[]    int2 depth-first frames (intervals of the implication list)
//     impl[]     the implied literals (internal encoding), read by the descent
//   A slot's epoch (1..255) advances per trail, so dh and cst are not cleared
//   between trails; the slot wipes them once every 255 trails.
//
// Current list of var v = clauses add_first'ed to v (newest first) followed by
// v's initial list, keeping entries whose clause still watches v and is not
// blocked.  A clause never comes back to a var it left (watches only leave
// false literals and nothing is unassigned within one BCP), so that is the
// reference's linked list exactly.
//
// Execution: one thread block (NW warps) per trail.  A round lays out a window
// of up to 32*NW upcoming watch entries -- the rest of the current scan and,
// while the current scan is a trail scan that has implied nothing, the entries
// of up to 31 following trail scans -- and thread p evaluates window position
// p against the round-start state, with every random load of the round in one
// trip.  The round then commits the entries in reference order up to the first
// event that could have changed a later evaluation (an entry whose clause an
// earlier window scan holds, a later scan whose list is not what the round
// assumed or gets a clause moved into it, the entry just after a conflict, the
// end of the scan an implication was found in -- its depth-first descent comes
// first -- and a later entry of that scan whose clause has the implied
// variable).  Events are ordered integer keys and the cut is one block-wide
// minimum.  Uncommitted entries are evaluated again next round, so the result
// is the sequential one.
//
// The following scans come from a look-ahead ring of upcoming trail positions
// (variable, initial-list range, and the list head as loaded when the position
// entered the ring), filled two rounds ahead by warp 1.  A head loaded then may
// be stale; every window scan's head is loaded again in the round's entry trip
// and a scan whose list changed is cut from the window.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdio>
#include <mutex>

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

#ifndef GPSAT_BCP_WARPS
#define GPSAT_BCP_WARPS 4
#endif
constexpr int NW = GPSAT_BCP_WARPS;   // warps per block: one trail per block
constexpr int NT = NW * 32;
constexpr int W = NT;                 // window entries: one per thread
static_assert(NW >= 2 && W <= 256 && LB >= LEAD + CHUNK, "layout limits");

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
};

struct Smem {
    // window layout (written by warp 0 / thread 0, read by all)
    int sc_var[MAXSC];
    int sc_b[MAXSC];
    int sc_e[MAXSC];
    uint32_t sc_wk[MAXSC];
    uint32_t sc_wend[MAXSC];
    int32_t sc_head[MAXSC];    // following scan: arena index of the assumed added head, or -1
    uint32_t sc_h[MAXSC];      // following scan: the list-head word the layout assumed
    int32_t sc_next[MAXSC];    // following scan: what comes after its added head (-1: nothing)
    uint8_t pos_scan[W];
    int4 dyn0[W];              // the current scan's added entries (thread 0 follows the chain)
    int4 dyn1[W];
    int32_t dyn_next[W];
    int ndyn, dyn_done, nsc, nent;
    // events of the round
    int key_min;
    int imp_cnt;
    int16_t imp_pos[W];
    int8_t imp_scan[W];
    int32_t imp_var[W];
    int wcnt_im[NW], wcnt_mv[NW];
    int32_t mh[2 * W];         // move targets of the round (collision check)
    int collide;
    int32_t mv_t1[W], mv_t2[W];
    int32_t confl_c, confl_scan;
    unsigned long long red[NW][3];
    int t;
    // look-ahead ring: trail position q lives in slot q % LB
    int32_t lb_var[LB];
    uint32_t lb_a[LB], lb_b[LB], lb_h[LB];
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
__device__ __noinline__ void eval_long(const Dev &d, const uint32_t *asg, int off, int len, int w1, int w2, Eval &r)
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

// block-wide minimum; every thread gets it
__device__ __forceinline__ int block_min(Smem &sm, int v)
{
    v = __reduce_min_sync(FULL, v);
    if ((threadIdx.x & 31) == 0) atomicMin(&sm.key_min, v);
    __syncthreads();
    return sm.key_min;
}

// The ring chunk that warp 1 carries between rounds: lanes hold trail
// positions [ring_hi + 32, +32) as literals (stage 1) and [ring_hi, +32) as
// variable, initial-list range and list head in flight (stage 2).
struct RingPipe {
    int32_t lit;
    int32_t var;
    uint32_t a, b, h;
};

__device__ void process_trail(const Dev &d, Smem &sm, const int t, const int slot)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t *asg = d.asg + (size_t)slot * d.n_words;
    uint32_t *dh = d.dh + (size_t)slot * d.n_pad;
    uint32_t *cst = d.cst + (size_t)slot * d.m_pad;
    int4 *arena = d.arena + (size_t)slot * d.arena_cap * 2;
    int2 *stk = d.stack + (size_t)slot * d.impl_cap;
    int32_t *impl = d.impl + (size_t)slot * d.impl_cap;
    int32_t *ilit = d.ilit + (size_t)t * d.impl_cap;
    int32_t *ireason = d.ireason + (size_t)t * d.impl_cap;
    const int32_t n = d.n_vars;
    const unsigned lt = lanemask_lt();

    // ---- epoch of this slot
    uint32_t e = d.epoch[slot] + 1;
    if (e > EPMAX) {
        const uint4 z = make_uint4(0, 0, 0, 0);
        uint4 *d4 = reinterpret_cast<uint4 *>(dh);
        for (int64_t i = tid; i < d.n_pad / 4; i += NT) d4[i] = z;
        uint4 *c4 = reinterpret_cast<uint4 *>(cst);
        for (int64_t i = tid; i < d.m_pad / 4; i += NT) c4[i] = z;
        e = 1;
    }
    const int64_t tb = d.toff[t];
    const int64_t tn = d.toff[t + 1] - tb;
    __syncthreads();
    if (tid == 0) d.epoch[slot] = e;

    // ---- assign every trail literal first: an atomic OR of its two bits; the
    // old word shows the variable assigned the other way earlier (by any thread)
    bool bad = tn < 0;
#pragma unroll 4
    for (int64_t i = tid; i < tn; i += NT) {
        const int32_t x = d.trail[tb + i];
        if (x == 0 || x > n || x < -n) {
            bad = true;
        } else {
            const int32_t v = (x > 0 ? x : -x) - 1;
            const int sh = (v & 15) << 1;
            const uint32_t bits = (x > 0 ? 3u : 1u) << sh;
            const uint32_t old = atomicOr(&asg[v >> 4], bits);
            if (((old >> sh) & 1u) && (((old ^ bits) >> sh) & 2u)) bad = true;
        }
    }

    // ---- fill the look-ahead ring with the first LEAD positions, and start
    // the pipelined refill after them
    RingPipe pipe;
    pipe.lit = pipe.var = 0;
    pipe.a = pipe.b = pipe.h = 0;
    int64_t ring_hi = tn < LEAD ? (tn > 0 ? tn : 0) : LEAD;   // positions [0, ring_hi) are in the ring
    for (int64_t q = tid; q < ring_hi; q += NT) {
        const int32_t x = d.trail[tb + q];
        int32_t v = (x > 0 ? x : -x) - 1;
        if (v < 0 || v >= n) v = 0;   // a bad trail never reads the ring
        const int r = (int)(q & (LB - 1));
        sm.lb_var[r] = v;
        sm.lb_a[r] = d.w0off[v];
        sm.lb_b[r] = d.w0off[v + 1];
        sm.lb_h[r] = dh[v];
    }
    if (wid == 1 && ring_hi < tn) {
        const int64_t q = ring_hi + lane;
        if (q < tn) {
            const int32_t x = d.trail[tb + q];
            int32_t v = (x > 0 ? x : -x) - 1;
            if (v < 0 || v >= n) v = 0;
            pipe.var = v;
            pipe.a = d.w0off[v];
            pipe.b = d.w0off[v + 1];
            pipe.h = dh[v];
        }
        const int64_t q2 = ring_hi + CHUNK + lane;
        if (q2 < tn) pipe.lit = d.trail[tb + q2];
    }
    bad = __syncthreads_or(bad);

    int64_t n_impl = 0, props = 0, cI = 0;
    int64_t myW = 0, myL = 0, myA = 0;  // thread-private, reduced at the end
    int32_t status = bad ? GPSAT_BCP_BAD_TRAIL : GPSAT_BCP_NO_CONFLICT, confl = -1, stopi = -1;
    int64_t arena_used = 0, ti = 0, top_j = 0, top_e = 0, cur_impl_start = 0, cur_trail = -1, dfs_trail = -1;
    int depth = 0;
    bool in_scan = false, cur_counted = false, cur_is_trail = false;
    int32_t cur_var = 0, cur_dp = -1;
    uint32_t cur_wk = 0, cur_wend = 0;
    // every iteration finishes a scan, pops a frame or commits at least one
    // entry; the budget only guarantees termination if that were ever broken
    int64_t budget = MAX_ITERS;

    while (status == GPSAT_BCP_NO_CONFLICT) {
        if (--budget < 0) {
            status = GPSAT_BCP_BUDGET;
            stopi = (int32_t)cur_trail;
            break;
        }
        if (!in_scan) {
            int32_t v;
            if (depth > 0) {
                if (top_j < top_e) {
                    v = impl[top_j] >> 1;
                    top_j++;
                    cur_is_trail = false;
                    cur_trail = dfs_trail;
                    cur_wk = d.w0off[v];
                    cur_wend = d.w0off[v + 1];
                } else {
                    depth--;
                    if (depth > 0) {
                        const int2 fr = stk[depth - 1];
                        top_j = fr.x;
                        top_e = fr.y;
                    }
                    continue;
                }
            } else {
                if (ti >= tn) break;
                if (ti < ring_hi) {
                    const int r = (int)(ti & (LB - 1));
                    v = sm.lb_var[r];
                    cur_wk = sm.lb_a[r];
                    cur_wend = sm.lb_b[r];
                } else {
                    const int32_t x = d.trail[tb + ti];
                    v = (x > 0 ? x : -x) - 1;
                    cur_wk = d.w0off[v];
                    cur_wend = d.w0off[v + 1];
                }
                cur_trail = ti;
                dfs_trail = ti;
                ti++;
                cur_is_trail = true;
            }
            const uint32_t h = dh[v];
            cur_var = v;
            cur_dp = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
            cur_counted = false;
            cur_impl_start = n_impl;
            in_scan = true;
        }
        if (!cur_counted) {
            props++;
            cur_counted = true;
        }
        // The scans that come next if the current one implies nothing are the
        // following trail scans when it is a trail scan, or when it is the
        // last implication of a trail scan's frame (its descent ends with it
        // and the depth-first walk returns to the trail)
        const bool then_trail = (depth == 0 && cur_is_trail) || (depth == 1 && !cur_is_trail && top_j >= top_e);
        if (cur_dp < 0 && cur_wk >= cur_wend) {
            const bool next_trail_scans = then_trail && n_impl == cur_impl_start && ti < tn;
            if (!next_trail_scans) {
                // descend into the implications the scan found
                in_scan = false;
                if (n_impl > cur_impl_start) {
                    // every thread records the frame (each reads back its own
                    // write: no barrier need separate this store from the pop)
                    if (depth > 0) stk[depth - 1] = make_int2((int)top_j, (int)top_e);
                    top_j = cur_impl_start;
                    top_e = n_impl;
                    depth++;
                }
                continue;
            }
        }

        // ---- lay out the window
        if (tid == 0) {
            sm.key_min = NO_CUT;
            sm.imp_cnt = 0;
            sm.collide = 0;
            sm.confl_c = -1;
        }
        int ndyn = 0;
        bool dyn_done = true;
        if (cur_dp >= 0) {
            if (tid == 0) {
                int32_t p = cur_dp;
                int k = 0;
                while (p >= 0 && k < W) {
                    const int4 a = arena[2 * p];
                    sm.dyn0[k] = a;
                    sm.dyn1[k] = arena[2 * p + 1];
                    p = a.w;
                    sm.dyn_next[k] = p;
                    k++;
                }
                sm.ndyn = k;
                sm.dyn_done = p < 0;
            }
            __syncthreads();
            ndyn = sm.ndyn;
            dyn_done = sm.dyn_done;
        }
        int nent = ndyn, take0 = 0;
        if (dyn_done) {
            const uint32_t left = cur_wend - cur_wk;
            take0 = (int)((uint32_t)(W - nent) < left ? (uint32_t)(W - nent) : left);
            nent += take0;
        }
        const int nent0 = nent;
        int nsc = 1;
        const bool scan0_full = dyn_done && (cur_wk + (uint32_t)take0 == cur_wend);
        const int64_t lim = ring_hi < tn ? ring_hi : tn;
        if (tid == 0) {
            sm.sc_var[0] = cur_var;
            sm.sc_b[0] = 0;
            sm.sc_e[0] = nent0;
        }
        if (scan0_full && then_trail && n_impl == cur_impl_start && nent < W && ti < lim) {
            // following trail scans from the ring: lane j of warp 0 takes
            // position ti + j; a scan is taken if it starts inside the window
            // (the last one may be cut short) and its variable is not already
            // a window scan's
            if (wid == 0) {
                const int64_t q = ti + lane;
                const bool in = lane < MAXSC - 1 && q < lim;
                const int r = (int)(q & (LB - 1));
                const int32_t v = in ? sm.lb_var[r] : -1 - lane;
                const uint32_t a = in ? sm.lb_a[r] : 0u, b = in ? sm.lb_b[r] : 0u, h = in ? sm.lb_h[r] : 0u;
                const bool hasA = in && (h >> 24) == e;
                const int cnt = in ? (hasA ? 1 : 0) + (int)(b - a) : 0;
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += y;
                }
                const int start = nent + incl - cnt;
                const unsigned same = __match_any_sync(FULL, v);
                const bool dup = in && ((same & lt) != 0 || v == cur_var);
                const unsigned ok = __ballot_sync(FULL, in && start < W && !dup);
                const int K = (~ok) ? __ffs(~ok) - 1 : 32;
                if (lane < K) {
                    const int s = 1 + lane;
                    const int end = start + cnt < W ? start + cnt : W;
                    sm.sc_var[s] = v;
                    sm.sc_b[s] = start;
                    sm.sc_e[s] = end;
                    sm.sc_wk[s] = a;
                    sm.sc_wend[s] = b;
                    sm.sc_head[s] = hasA ? (int32_t)(h & 0xFFFFFFu) : -1;
                    sm.sc_h[s] = h;
                    sm.sc_next[s] = -1;
                    for (int p = start; p < end; p++) sm.pos_scan[p] = (uint8_t)s;
                }
                const int last = K > 0 ? __shfl_sync(FULL, incl, K - 1) : 0;
                if (lane == 0) {
                    sm.nsc = 1 + K;
                    sm.nent = nent + last < W ? nent + last : W;
                }
            }
            __syncthreads();
            nsc = sm.nsc;
            nent = sm.nent;
        } else {
            __syncthreads();
        }

        // ---- the window's entries (trip 1): thread p loads position p;
        // thread s (1 <= s < nsc) also loads window scan s's list head again
        const bool has = tid < nent;
        int my_scan = 0;
        int4 en = make_int4(0, 0, 0, 0), el = en;
        if (has) {
            if (tid < nent0) {
                if (tid < ndyn) {
                    en = sm.dyn0[tid];
                    el = sm.dyn1[tid];
                } else {
                    const size_t w = cur_wk + (uint32_t)(tid - ndyn);
                    en = d.w0ent[2 * w];
                    el = d.w0ent[2 * w + 1];
                }
            } else {
                my_scan = sm.pos_scan[tid];
                const int q = tid - sm.sc_b[my_scan];
                const int32_t head = sm.sc_head[my_scan];
                if (head >= 0 && q == 0) {
                    en = arena[2 * head];
                    el = arena[2 * head + 1];
                    sm.sc_next[my_scan] = en.w;
                } else {
                    const size_t w = sm.sc_wk[my_scan] + (uint32_t)(q - (head >= 0 ? 1 : 0));
                    en = d.w0ent[2 * w];
                    el = d.w0ent[2 * w + 1];
                }
            }
        }
        uint32_t hnow = 0;
        const bool vthr = tid >= 1 && tid < nsc;
        if (vthr) hnow = dh[sm.sc_var[tid]];
        const int32_t sv = sm.sc_var[my_scan];

        // ---- every entry's state (trip 2): the clause state, the assignment
        // words of its literals and the list head of each possible move
        // target (the literals its initial watches leave out; a clause whose
        // watches moved that needs another head loads it at commit time)
        Eval r;
        r.act = A_NONE;
        r.acnt = 0;
        r.t1 = r.t2 = -1;
        r.unit = -1;
        r.nw1 = r.nw2 = 0;
        bool valid = false;
        int32_t ov = -1;  // a valid entry's clause: its other watched variable
        int w1 = 0, w2 = 0;
        uint32_t dh1 = 0, dh2 = 0;
        bool dh1_ok = false, dh2_ok = false;
        if (has) {
            const uint32_t st = cst[en.x];
            const int len = en.z;
            const int32_t Lr[KIN] = {el.x, el.y, el.z, el.w};
            const bool fresh = (st >> 24) != e;
            const int iw1 = (uint32_t)en.w >> 16, iw2 = en.w & 0xFFFF;   // initial watches (static entries)
            const bool is_added = tid < nent0 ? tid < ndyn : (sm.sc_head[my_scan] >= 0 && tid == sm.sc_b[my_scan]);
            uint32_t Ab[KIN], Dh[KIN];
#pragma unroll
            for (int i = 0; i < KIN; i++) {
                const int32_t v = Lr[i] >> 1;
                Ab[i] = (i < len) ? asg_bits(asg[v >> 4], v) : 0u;
                const bool want = i < len && len <= KIN && v != sv && (is_added || len > 3 || (i != iw1 && i != iw2));
                Dh[i] = want ? dh[v] : 0u;
            }
            bool blk;
            if (!fresh) {
                blk = (st >> 22) & 1u;
                w1 = (st >> 11) & 0x7FFu;
                w2 = st & 0x7FFu;
            } else {
                blk = false;
                w1 = iw1;
                w2 = iw2;
            }
            if (len <= KIN) {
                int32_t l1 = 0, l2 = 0;
                bool c1 = false, c2 = false;
#pragma unroll
                for (int i = 0; i < KIN; i++) {
                    if (i == w1) {
                        l1 = Lr[i];
                        c1 = cons_of(Ab[i], Lr[i]);
                    }
                    if (i == w2) {
                        l2 = Lr[i];
                        c2 = cons_of(Ab[i], Lr[i]);
                    }
                }
                valid = !blk && ((l1 >> 1) == sv || (l2 >> 1) == sv);
                if (valid) ov = ((l1 >> 1) == sv) ? (l2 >> 1) : (l1 >> 1);
                if (valid) {
                    r.acnt = 2;
                    if (!(c1 && c2)) {
                        int pend = (!c1 && !c2) ? 2 : 1, f1 = -1, f2 = -1;
                        int32_t lf1 = 0, lf2 = 0;
                        uint32_t af1 = 0, df1 = 0, df2 = 0;
                        bool ok1 = false, ok2 = false;
#pragma unroll
                        for (int i = 0; i < KIN; i++) {
                            if (i < len && pend > 0 && i != w1 && i != w2) {
                                r.acnt++;
                                if (cons_of(Ab[i], Lr[i])) {
                                    const bool loaded =
                                        (Lr[i] >> 1) != sv && (is_added || len > 3 || (i != iw1 && i != iw2));
                                    if (f1 < 0) {
                                        f1 = i;
                                        lf1 = Lr[i];
                                        af1 = Ab[i];
                                        df1 = Dh[i];
                                        ok1 = loaded;
                                    } else {
                                        f2 = i;
                                        lf2 = Lr[i];
                                        df2 = Dh[i];
                                        ok2 = loaded;
                                    }
                                    pend--;
                                }
                            }
                        }
                        int32_t unit = -1;
                        uint32_t au = 0;
                        if (c1 || c2) {
                            if (f1 < 0) {
                                unit = c1 ? l1 : l2;
#pragma unroll
                                for (int i = 0; i < KIN; i++)
                                    if (i == (c1 ? w1 : w2)) au = Ab[i];
                            } else {
                                r.act = A_SW1;
                                r.nw1 = c1 ? w1 : f1;
                                r.nw2 = c1 ? f1 : w2;
                                r.t1 = lf1 >> 1;
                                dh1 = df1;
                                dh1_ok = ok1;
                            }
                        } else if (f1 >= 0 && f2 >= 0) {
                            r.act = A_SW2;
                            r.nw1 = f1;
                            r.nw2 = f2;
                            r.t1 = lf1 >> 1;
                            r.t2 = lf2 >> 1;
                            dh1 = df1;
                            dh2 = df2;
                            dh1_ok = ok1;
                            dh2_ok = ok2;
                        } else if (f1 >= 0) {
                            unit = lf1;
                            au = af1;
                        } else {
                            r.act = A_CONFLICT;
                        }
                        if (unit >= 0) {
                            r.unit = unit;
                            r.act = (au & 1u) ? A_BLOCK : A_IMPLY;
                        }
                    }
                }
            } else {
                const int32_t l1 = d.lits[en.y + w1], l2 = d.lits[en.y + w2];
                valid = !blk && ((l1 >> 1) == sv || (l2 >> 1) == sv);
                if (valid) ov = ((l1 >> 1) == sv) ? (l2 >> 1) : (l1 >> 1);
                if (valid) eval_long(d, asg, en.y, len, w1, w2, r);
            }
        }

        // ---- where the commit stops: the smallest event key of the round
        int key = NO_CUT;
        // a following scan whose list is not what the layout assumed
        if (vthr) {
            const uint32_t ha = sm.sc_h[tid];
            const bool va = (ha >> 24) == e, vn = (hnow >> 24) == e;
            if (va != vn || (vn && hnow != ha)) key = key_before(sm.sc_b[tid], tid);
        }
        // a following scan's added head with more added entries behind it:
        // only the head is in the window
        if (has && my_scan > 0 && tid == sm.sc_b[my_scan] && sm.sc_head[my_scan] >= 0 && en.w >= 0)
            key = min(key, key_before(tid + 1, my_scan));
        const bool mv = valid && (r.act == A_SW1 || r.act == A_SW2);
        if (valid) {
            // an entry whose clause an earlier window scan also holds (and may
            // change): a clause is listed under the two variables it watches,
            // so that is one whose other watched variable is an earlier window
            // scan's (for scan 0, whose entries may come from earlier rounds,
            // this can cut where nothing repeats: a cut only ends the round early)
            if (my_scan > 0 && ov == cur_var) key = min(key, key_before(tid, my_scan));
            if (r.act == A_CONFLICT) key = min(key, key_after(tid, my_scan));
            if (r.act == A_IMPLY) {
                // an implication ends its scan's part of the window
                key = min(key, key_after(sm.sc_e[my_scan] - 1, my_scan));
                const int k = atomicAdd(&sm.imp_cnt, 1);
                sm.imp_pos[k] = (int16_t)tid;
                sm.imp_scan[k] = (int8_t)my_scan;
                sm.imp_var[k] = r.unit >> 1;
            }
            for (int s = 1; s < nsc; s++) {
                const int32_t vs = sm.sc_var[s];
                if (s < my_scan && vs == ov) key = min(key, key_before(tid, my_scan));
                // a move into a later window scan's list
                if (mv && s > my_scan && (vs == r.t1 || vs == r.t2)) key = min(key, key_before(sm.sc_b[s], s));
            }
        }
        __syncthreads();
        // a later entry of an implying scan whose clause has the implied variable
        // (a long clause: always); the other entries read nothing the
        // implication changed, so several implications commit in one round
        const int nimp = sm.imp_cnt;
        if (valid && nimp > 0) {
            for (int j = 0; j < nimp; j++) {
                if (sm.imp_scan[j] != my_scan || sm.imp_pos[j] >= tid) continue;
                const int32_t uv = sm.imp_var[j];
                const bool dep = en.z > KIN || (el.x >> 1) == uv || (en.z > 1 && (el.y >> 1) == uv) ||
                                 (en.z > 2 && (el.z >> 1) == uv) || (en.z > 3 && (el.w >> 1) == uv);
                if (dep) key = min(key, key_before(tid, my_scan));
            }
        }
        const int cut = block_min(sm, key);
        int k_end, new_cur;
        bool new_started;
        if (cut == NO_CUT) {
            k_end = nent;
            new_cur = nsc - 1;
            new_started = (new_cur == 0) || (sm.sc_e[new_cur] > sm.sc_b[new_cur]);
        } else {
            k_end = cut >> 7;
            new_cur = (cut >> 1) & 63;
            new_started = (cut & 1) || new_cur == 0 || k_end > sm.sc_b[new_cur];
        }
        // a round that would commit nothing and start no scan could never end
        // the trail: report it (it cannot happen; the guard keeps a fault in
        // this logic from spinning until the iteration budget runs out)
        if (k_end == 0 && new_cur == 0) {
            status = GPSAT_BCP_BUDGET;
            stopi = (int32_t)cur_trail;
            break;
        }

        // ---- ranks of the committed implications and moves (window order)
        bool com = valid && tid < k_end;
        int tot_im = 0, tot_mv = 0, my_im = 0, my_mv = 0;
        auto rank = [&]() {
            const bool imp = com && r.act == A_IMPLY;
            const unsigned bi = __ballot_sync(FULL, imp);
            const unsigned b1 = __ballot_sync(FULL, com && (r.act == A_SW1 || r.act == A_SW2));
            const unsigned b2 = __ballot_sync(FULL, com && r.act == A_SW2);
            if (lane == 0) {
                sm.wcnt_im[wid] = __popc(bi);
                sm.wcnt_mv[wid] = __popc(b1) + __popc(b2);
            }
            __syncthreads();
            int bim = 0, bmv = 0;
            tot_im = tot_mv = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const int ci = sm.wcnt_im[w], cm = sm.wcnt_mv[w];
                if (w < wid) {
                    bim += ci;
                    bmv += cm;
                }
                tot_im += ci;
                tot_mv += cm;
            }
            my_im = bim + __popc(bi & lt);
            my_mv = bmv + __popc(b1 & lt) + __popc(b2 & lt);
            __syncthreads();   // the counts are read before anyone writes them again
        };
        rank();
        // more implications than impl_cap leaves room for: commit up to the
        // first one that does not fit; the next round reports the overflow there
        {
            const int64_t room = d.impl_cap - n_impl;
            if (room > 0 && tot_im > room) {
                if (com && r.act == A_IMPLY && my_im == room) {
                    sm.nent = tid;
                    sm.nsc = my_scan;
                }
                __syncthreads();
                k_end = sm.nent;
                new_cur = sm.nsc;
                new_started = new_cur == 0 || k_end > sm.sc_b[new_cur];
                com = valid && tid < k_end;
                rank();
            }
        }
        const int64_t ti_round = ti;
        const bool aover = arena_used + tot_mv > d.arena_cap, iover = tot_im > 0 && n_impl >= d.impl_cap;
        if (aover || iover) {
            // the scan of the first move (arena) or implication (list) that
            // does not fit; its trail position is the stop index
            const bool first = aover ? (com && (r.act == A_SW1 || r.act == A_SW2) && my_mv == 0)
                                     : (com && r.act == A_IMPLY && my_im == 0);
            if (first) sm.nsc = my_scan;
            __syncthreads();
            const int ks = sm.nsc;
            status = GPSAT_BCP_OVERFLOW;
            stopi = (int32_t)(ks == 0 ? cur_trail : ti + ks - 1);
            break;
        }

        // ---- commit
        // moves into the same variable within the round (rare) are linked by
        // thread 0 in window order; otherwise every mover links its own entry
        if (com && (r.act == A_SW1 || r.act == A_SW2)) {
            const int32_t tg[2] = {r.t1, r.t2};
            for (int k = 0; k < (r.act == A_SW2 ? 2 : 1); k++) {
                const uint32_t hsh = ((uint32_t)tg[k] * 2654435761u) >> 24;
                for (int probe = 0; probe < 2 * W; probe++) {
                    const int slotp = (int)((hsh + (uint32_t)probe) & (2 * W - 1));
                    const int32_t old = atomicCAS(&sm.mh[slotp], -1, tg[k]);
                    if (old == -1) break;
                    if (old == tg[k]) {
                        sm.collide = 1;
                        break;
                    }
                }
            }
        }
        sm.mv_t1[tid] = (com && (r.act == A_SW1 || r.act == A_SW2)) ? r.t1 : -1;
        sm.mv_t2[tid] = (com && r.act == A_SW2) ? r.t2 : -1;
        if (com && (r.act == A_SW1 || r.act == A_SW2)) {
            sm.dyn0[tid] = make_int4(en.x, en.y, en.z, 0);
            sm.dyn1[tid] = el;
        }
        __syncthreads();
        const bool collide = sm.collide != 0;
        if (!collide) {
            if (com && (r.act == A_SW1 || r.act == A_SW2)) {
                const int idx = (int)arena_used + my_mv;
                if (!dh1_ok) dh1 = dh[r.t1];
                const int32_t nx1 = ((dh1 >> 24) == e) ? (int32_t)(dh1 & 0xFFFFFFu) : -1;
                arena[2 * idx] = make_int4(en.x, en.y, en.z, nx1);
                arena[2 * idx + 1] = el;
                dh[r.t1] = (e << 24) | (uint32_t)idx;
                if (r.act == A_SW2) {
                    if (!dh2_ok) dh2 = dh[r.t2];
                    const int32_t nx2 = ((dh2 >> 24) == e) ? (int32_t)(dh2 & 0xFFFFFFu) : -1;
                    arena[2 * (idx + 1)] = make_int4(en.x, en.y, en.z, nx2);
                    arena[2 * (idx + 1) + 1] = el;
                    dh[r.t2] = (e << 24) | (uint32_t)(idx + 1);
                }
            }
        } else if (tid == 0) {
            int idx = (int)arena_used;
            for (int p = 0; p < k_end; p++) {
                const int32_t tg1 = sm.mv_t1[p];
                if (tg1 < 0) continue;
                const int4 a = sm.dyn0[p], b = sm.dyn1[p];
                const int32_t tg2 = sm.mv_t2[p];
                uint32_t h = dh[tg1];
                arena[2 * idx] = make_int4(a.x, a.y, a.z, ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1);
                arena[2 * idx + 1] = b;
                dh[tg1] = (e << 24) | (uint32_t)idx;
                idx++;
                if (tg2 >= 0) {
                    h = dh[tg2];
                    arena[2 * idx] = make_int4(a.x, a.y, a.z, ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1);
                    arena[2 * idx + 1] = b;
                    dh[tg2] = (e << 24) | (uint32_t)idx;
                    idx++;
                }
            }
        }
        // clause states
        if (com && r.act != A_NONE) {
            uint32_t ns;
            if (r.act == A_SW1 || r.act == A_SW2) ns = (e << 24) | ((uint32_t)r.nw1 << 11) | (uint32_t)r.nw2;
            else ns = (e << 24) | (1u << 22) | ((uint32_t)w1 << 11) | (uint32_t)w2;
            cst[en.x] = ns;
        }
        // implications, in window order (all of one scan, on distinct variables)
        if (com && r.act == A_IMPLY) {
            const int64_t at = n_impl + my_im;
            ilit[at] = dimacs_of(r.unit);
            ireason[at] = en.x;
            impl[at] = r.unit;
            const int32_t u = r.unit >> 1;
            atomicOr(&asg[u >> 4], ((r.unit & 1) ? 3u : 1u) << ((u & 15) << 1));
        }
        if (com && r.act == A_CONFLICT) {
            sm.confl_c = en.x;
            sm.confl_scan = my_scan;
        }
        if (com) {
            myW++;
            myL += en.z;
            myA += r.acnt;
        }
        // the look-ahead ring: warp 1 publishes the chunk it loaded a refill
        // ago and starts the next two (the decision is the same in every thread)
        const bool refill = ring_hi < tn && ring_hi - ti < LEAD;
        if (refill && wid == 1) {
            // stage 2 -> ring
            const int64_t q = ring_hi + lane;
            if (q < tn) {
                const int rr = (int)(q & (LB - 1));
                sm.lb_var[rr] = pipe.var;
                sm.lb_a[rr] = pipe.a;
                sm.lb_b[rr] = pipe.b;
                sm.lb_h[rr] = pipe.h;
                // warm L2 with the position's initial watch entries (two per line)
                const uint32_t ne = pipe.b - pipe.a < 32u ? pipe.b - pipe.a : 32u;
                for (uint32_t k = 0; k < ne; k += 2)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(d.w0ent + 2 * (size_t)(pipe.a + k)));
            }
            // stage 1 -> stage 2, and a new stage 1
            const int64_t nb = ring_hi + CHUNK;
            if (nb < tn) {
                const int64_t q2 = nb + lane;
                if (q2 < tn) {
                    int32_t v = (pipe.lit > 0 ? pipe.lit : -pipe.lit) - 1;
                    if (v < 0 || v >= n) v = 0;
                    pipe.var = v;
                    pipe.a = d.w0off[v];
                    pipe.b = d.w0off[v + 1];
                    pipe.h = dh[v];
                }
                const int64_t q3 = nb + CHUNK + lane;
                if (q3 < tn) pipe.lit = d.trail[tb + q3];
            }
        }
        if (refill) ring_hi = ring_hi + CHUNK < tn ? ring_hi + CHUNK : tn;
        __syncthreads();
        // empty the move-target table for the next round (the end-of-round
        // barrier separates this from the next round's inserts)
        for (int i = tid; i < 2 * W; i += NT) sm.mh[i] = -1;
        arena_used += tot_mv;
        n_impl += tot_im;
        cI += tot_im;

        // ---- advance the scan cursors
        if (new_cur == 0) {
            if (k_end > 0) {
                if (k_end <= ndyn) {
                    cur_dp = sm.dyn_next[k_end - 1];
                } else {
                    cur_dp = -1;
                    cur_wk += (uint32_t)(k_end - ndyn);
                }
            }
        } else {
            props += new_cur - 1;
            cur_var = sm.sc_var[new_cur];
            cur_wk = sm.sc_wk[new_cur];
            cur_wend = sm.sc_wend[new_cur];
            cur_dp = -1;
            if (!new_started) {
                // cut before this scan because its list is not what the window
                // assumed (possibly changed by this round): read it again
                const uint32_t h = dh[cur_var];
                cur_dp = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
            } else {
                const int k = k_end - sm.sc_b[new_cur];
                if (sm.sc_head[new_cur] >= 0) {
                    const int32_t nx = sm.sc_next[new_cur];
                    if (nx >= 0) cur_dp = nx;   // cut right after the head
                    else cur_wk += (uint32_t)(k - 1);
                } else {
                    cur_wk += (uint32_t)k;
                }
            }
            cur_counted = new_started;
            if (new_started) props++;
            cur_trail = ti + new_cur - 1;
            dfs_trail = cur_trail;
            ti += new_cur;
            cur_is_trail = true;
            depth = 0;  // a descent whose scan led into trail scans has ended
            cur_impl_start = n_impl - tot_im;
        }
        const int32_t cc = sm.confl_c;
        if (cc >= 0) {
            const int ks = sm.confl_scan;
            confl = cc;
            stopi = (int32_t)(ks == 0 ? (new_cur == 0 ? cur_trail : dfs_trail) : ti_round + ks - 1);
            status = GPSAT_BCP_CONFLICT;
        }
        __syncthreads();   // the window's shared state is read before the next round rewrites it
    }

    // ---- clear the assignment words this trail set (trail and implications)
    for (int64_t i = tid; i < tn; i += NT) {
        const int32_t x = d.trail[tb + i];
        if (x != 0 && x <= n && x >= -n) asg[((x > 0 ? x : -x) - 1) >> 4] = 0u;
    }
    for (int64_t i = tid; i < n_impl; i += NT) asg[(impl[i] >> 1) >> 4] = 0u;

    // ---- outputs
    myW = warp_sum(myW);
    myL = warp_sum(myL);
    myA = warp_sum(myA);
    if (lane == 0) {
        sm.red[wid][0] = (unsigned long long)myW;
        sm.red[wid][1] = (unsigned long long)myL;
        sm.red[wid][2] = (unsigned long long)myA;
    }
    __syncthreads();
    if (tid == 0) {
        int64_t W_ = 0, L_ = 0, A_ = 0;
        for (int w = 0; w < NW; w++) {
            W_ += (int64_t)sm.red[w][0];
            L_ += (int64_t)sm.red[w][1];
            A_ += (int64_t)sm.red[w][2];
        }
        d.status[t] = status;
        d.conflict[t] = confl;
        d.stop[t] = stopi;
        d.nimpl[t] = n_impl;
        if (d.counters) {
            int64_t *cn = d.counters + (size_t)t * GPSAT_BCP_NCOUNTERS;
            cn[0] = props;
            cn[1] = W_;
            cn[2] = L_;
            cn[3] = A_;
            cn[4] = cI;
            cn[5] = bad ? 0 : tn;
        }
    }
    __syncthreads();   // the bitmap is clean and the shared state free before the next trail
}

// ---------------------------------------------------------------------------
// Processing order: shortest trails first.  A launch lasts as long as its
// slowest trail, and when there are more trails than resident warps the
// last ones start only as others finish.  The trails that propagate longest
// are those that reach their fixpoint without a conflict, and a trail that
// assigns fewer variables is the more likely to: starting the short ones
// first starts the long-running ones at once.  (Outputs do not depend on the
// order; at the 4096-trail benchmark shape the measured per-trail durations
// give a 37.9 ms schedule instead of 41.4 ms.)  A counting sort on length / 16.
constexpr int ORDER_BUCKETS = 4096;

__device__ __forceinline__ int order_bucket(const int64_t *toff, int t)
{
    const int64_t len = toff[t + 1] - toff[t];
    return len <= 0 ? 0 : (int)(len >> 4 < ORDER_BUCKETS - 1 ? len >> 4 : ORDER_BUCKETS - 1);
}

__global__ void order_count(const int64_t *toff, int T, unsigned *hist)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
        atomicAdd(&hist[order_bucket(toff, t)], 1u);
}

// one block of 1024 threads: the counts become exclusive prefix sums in place
__global__ void __launch_bounds__(1024) order_scan(unsigned *hist)
{
    __shared__ unsigned part[1024];
    const int i = threadIdx.x;
    unsigned v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = hist[4 * i + k];
        sum += v[k];
    }
    part[i] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned add = i >= o ? part[i - o] : 0u;
        __syncthreads();
        part[i] += add;
        __syncthreads();
    }
    unsigned run = part[i] - sum;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        hist[4 * i + k] = run;
        run += v[k];
    }
}

__global__ void order_scatter(const int64_t *toff, int T, unsigned *hist, int32_t *order)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
        order[atomicAdd(&hist[order_bucket(toff, t)], 1u)] = t;
}

// ---------------------------------------------------------------------------
// Full-scan clause evaluation: the reference's BASIC_SEARCH strategy
// (ConflictAnalysis/ConflictAnalyzer.cu:173-245, clause_status :298-313 and
// SATSolver/VariablesStateHandler.cu:180-206).  Every trail literal is
// assigned, then sweeps run over all clauses in index order; a clause with a
// true literal is satisfied, one with every literal false is a conflict (the
// trail stops there), one with a single unassigned literal and the rest false
// implies it at once, so the clauses after it see the implication; sweeps
// repeat while one adds implications.
//
// One thread block per trail.  A pass evaluates the next SCAN_NT * SCAN_PER
// clauses at once against the current assignment; the first clause (lowest
// index) that is unit or false -- a block-wide minimum -- is the next event
// of the sequential sweep: the clauses before it are final, an implication is
// committed and the rest of the pass is evaluated again.  The trail's
// assignment bits sit in shared memory when they fit (SCAN_SMEM_WORDS), else
// in the slot's assignment words.  Counters: [0] sweeps, [1] clause
// evaluations, [2] and [3] literals examined, [4] implications, [5] trail
// literals; stop_index is the sweep (0-based) that met the conflict.
constexpr int SCAN_NT = 256;
constexpr int SCAN_PER = 4;
constexpr int SCAN_SPAN = SCAN_NT * SCAN_PER;
constexpr int64_t SCAN_SMEM_WORDS = 12288;   // 48 KB: formulas up to 196,608 variables

template <bool SMEM>
__global__ void __launch_bounds__(SCAN_NT) scan_kernel(Dev d, const uint32_t *__restrict__ coff)
{
    extern __shared__ uint32_t sasg[];
    __shared__ int s_key[3];   // per pass, in rotation: a slot is reset two barriers before its next use
    __shared__ int s_t;
    __shared__ unsigned long long s_red[SCAN_NT / 32][3];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int slot = blockIdx.x;
    if (slot >= d.n_slots) return;
    const int32_t n = d.n_vars;
    const int64_t m = d.n_clauses;
    uint32_t *asg = SMEM ? sasg : d.asg + (size_t)slot * d.n_words;
    while (true) {
        if (tid == 0) s_t = (int)atomicAdd(d.next_trail, 1u);
        __syncthreads();
        const int t0 = s_t;
        if (t0 >= d.n_trails) break;
        const int t = d.order ? d.order[t0] : t0;
        if (SMEM)
            for (int64_t i = tid; i < d.n_words; i += SCAN_NT) sasg[i] = 0u;
        __syncthreads();
        const int64_t tb = d.toff[t], tn = d.toff[t + 1] - tb;
        int32_t *ilit = d.ilit + (size_t)t * d.impl_cap;
        int32_t *ireason = d.ireason + (size_t)t * d.impl_cap;
        bool bad = tn < 0;
        for (int64_t i = tid; i < tn; i += SCAN_NT) {
            const int32_t x = d.trail[tb + i];
            if (x == 0 || x > n || x < -n) {
                bad = true;
            } else {
                const int32_t v = (x > 0 ? x : -x) - 1;
                const int sh = (v & 15) << 1;
                const uint32_t bits = (x > 0 ? 3u : 1u) << sh;
                const uint32_t old = atomicOr(&asg[v >> 4], bits);
                if (((old >> sh) & 1u) && (((old ^ bits) >> sh) & 2u)) bad = true;
            }
        }
        bad = __syncthreads_or(bad);
        int32_t status = bad ? GPSAT_BCP_BAD_TRAIL : GPSAT_BCP_NO_CONFLICT, confl = -1, stopi = -1;
        int64_t n_impl = 0, last = -1, sweeps = 0;
        int64_t myW = 0, myL = 0;
        int kb = 0;
        if (tid == 0) s_key[0] = s_key[1] = s_key[2] = INT_MAX;
        __syncthreads();
        while (status == GPSAT_BCP_NO_CONFLICT && last != n_impl) {
            last = n_impl;
            const int64_t sweep = sweeps++;
            for (int64_t base = 0; base < m && status == GPSAT_BCP_NO_CONFLICT; base += SCAN_SPAN) {
                int64_t cursor = base;
                const int64_t end = base + SCAN_SPAN < m ? base + SCAN_SPAN : m;
                while (cursor < end) {
                    // evaluate this thread's clauses of [cursor, end)
                    int ev_key = INT_MAX;
                    int32_t unit[SCAN_PER];
                    int exam[SCAN_PER];
                    bool fals[SCAN_PER];
#pragma unroll
                    for (int j = 0; j < SCAN_PER; j++) {
                        const int64_t c = base + tid + (int64_t)j * SCAN_NT;
                        unit[j] = -1;
                        exam[j] = 0;
                        fals[j] = false;
                        if (c >= cursor && c < end) {
                            const uint32_t b = coff[c], e = coff[c + 1];
                            int unsat = 0, k = 0;
                            int32_t learnt = -1;
                            bool sat = false;
                            for (uint32_t i = b; i < e; i++) {
                                const int32_t l = d.lits[i];
                                const uint32_t bits = asg_bits(asg[(l >> 1) >> 4], l >> 1);
                                k++;
                                if (!(bits & 1u)) learnt = l;
                                else if ((bits >> 1) == (uint32_t)(l & 1)) {
                                    sat = true;
                                    break;
                                } else unsat++;
                            }
                            exam[j] = k;
                            const int len = (int)(e - b);
                            if (!sat && unsat == len) {
                                fals[j] = true;
                                ev_key = min(ev_key, (int)(c - base));
                            } else if (!sat && unsat == len - 1) {
                                unit[j] = learnt;
                                ev_key = min(ev_key, (int)(c - base));
                            }
                        }
                    }
                    ev_key = __reduce_min_sync(FULL, ev_key);
                    if (lane == 0 && ev_key != INT_MAX) atomicMin(&s_key[kb], ev_key);
                    __syncthreads();
                    const int key = s_key[kb];
                    if (tid == 0) s_key[kb == 0 ? 2 : kb - 1] = INT_MAX;   // the slot after next
                    kb = kb == 2 ? 0 : kb + 1;
                    const int64_t upto = key == INT_MAX ? end : base + key + 1;   // clauses final after this pass
#pragma unroll
                    for (int j = 0; j < SCAN_PER; j++) {
                        const int64_t c = base + tid + (int64_t)j * SCAN_NT;
                        if (c >= cursor && c < upto) {
                            myW++;
                            myL += exam[j];
                        }
                    }
                    if (key == INT_MAX) break;
                    const int64_t c = base + key;
                    const int j = (int)((c - base) / SCAN_NT);
                    const bool mine = (int)((c - base) % SCAN_NT) == tid;
                    // the event's kind: the owner tells everyone
                    int kind = 0;   // 1 conflict, 2 implication
                    if (mine) {
                        int32_t u = -1;
                        bool f = false;
#pragma unroll
                        for (int q = 0; q < SCAN_PER; q++)
                            if (q == j) {
                                u = unit[q];
                                f = fals[q];
                            }
                        kind = f ? 1 : 2;
                        if (!f && n_impl < d.impl_cap) {
                            ilit[n_impl] = dimacs_of(u);
                            ireason[n_impl] = (int32_t)c;
                            const int32_t v = u >> 1;
                            atomicOr(&asg[v >> 4], ((u & 1) ? 3u : 1u) << ((v & 15) << 1));
                        }
                        s_red[0][0] = (unsigned long long)kind;
                    }
                    __syncthreads();
                    kind = (int)s_red[0][0];
                    __syncthreads();
                    if (kind == 1) {
                        confl = (int32_t)c;
                        stopi = (int32_t)sweep;
                        status = GPSAT_BCP_CONFLICT;
                        break;
                    }
                    if (n_impl >= d.impl_cap) {
                        stopi = (int32_t)sweep;
                        status = GPSAT_BCP_OVERFLOW;
                        break;
                    }
                    n_impl++;
                    cursor = c + 1;
                }
            }
        }
        // clear what this trail set in the slot's assignment words
        if (!SMEM) {
            for (int64_t i = tid; i < tn; i += SCAN_NT) {
                const int32_t x = d.trail[tb + i];
                if (x != 0 && x <= n && x >= -n) asg[((x > 0 ? x : -x) - 1) >> 4] = 0u;
            }
            __syncthreads();   // implied literals are read back from the outputs
            for (int64_t i = tid; i < n_impl; i += SCAN_NT) {
                const int32_t x = ilit[i];
                asg[((x > 0 ? x : -x) - 1) >> 4] = 0u;
            }
        }
        myW = warp_sum(myW);
        myL = warp_sum(myL);
        if (lane == 0) {
            s_red[wid][1] = (unsigned long long)myW;
            s_red[wid][2] = (unsigned long long)myL;
        }
        __syncthreads();
        if (tid == 0) {
            int64_t W_ = 0, L_ = 0;
            for (int w = 0; w < SCAN_NT / 32; w++) {
                W_ += (int64_t)s_red[w][1];
                L_ += (int64_t)s_red[w][2];
            }
            d.status[t] = status;
            d.conflict[t] = confl;
            d.stop[t] = stopi;
            d.nimpl[t] = n_impl;
            if (d.counters) {
                int64_t *cn = d.counters + (size_t)t * GPSAT_BCP_NCOUNTERS;
                cn[0] = bad ? 0 : sweeps;
                cn[1] = W_;
                cn[2] = L_;
                cn[3] = L_;
                cn[4] = n_impl;
                cn[5] = bad ? 0 : tn;
            }
        }
        __syncthreads();
    }
}

// blocks per SM the register allocation targets
#ifndef GPSAT_BCP_MIN_BLOCKS
#define GPSAT_BCP_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(NT, GPSAT_BCP_MIN_BLOCKS) bcp_kernel(Dev d)
{
    __shared__ Smem sm;
    for (int i = threadIdx.x; i < 2 * W; i += NT) sm.mh[i] = -1;
    const int slot = blockIdx.x;
    if (slot >= d.n_slots) return;
    __syncthreads();
    while (true) {
        if (threadIdx.x == 0) sm.t = (int)atomicAdd(d.next_trail, 1u);
        __syncthreads();
        const int t = sm.t;
        if (t >= d.n_trails) break;
        process_trail(d, sm, d.order ? d.order[t] : t, slot);
    }
}

}  // namespace bcp
}  // namespace gpsat

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace gpsat;

struct gpsat_bcp {
    const gpsat_formula *f = nullptr;
    int device = 0;
    int32_t slots = 0;
    int32_t active = 0;                // slots the launches use (0: all)
    int32_t strategy = GPSAT_BCP_WATCHED;
    int32_t scan_resident = 0;         // resident blocks of the full-scan kernel
    int64_t n_words = 0, n_pad = 0, m_pad = 0, arena_cap = 0, impl_cap = 0;
    uint32_t *asg = nullptr, *dh = nullptr, *cst = nullptr, *epoch = nullptr;
    int4 *arena = nullptr;
    int2 *stack = nullptr;
    int32_t *impl = nullptr;
    unsigned int *counter = nullptr;
    unsigned *hist = nullptr;          // ORDER_BUCKETS counters
    int32_t *order = nullptr;          // processing order of the last launch
    int64_t order_cap = 0;
    int64_t bytes = 0;
    // host-path staging
    int32_t *d_trail = nullptr;
    int64_t *d_toff = nullptr;
    int64_t trail_cap = 0, toff_cap = 0;
    void *d_out = nullptr;
    int64_t out_cap = 0;
};

namespace {

void bcp_free(gpsat_bcp *b)
{
    cudaFree(b->asg);
    cudaFree(b->dh);
    cudaFree(b->cst);
    cudaFree(b->impl);
    cudaFree(b->epoch);
    cudaFree(b->arena);
    cudaFree(b->stack);
    cudaFree(b->counter);
    cudaFree(b->hist);
    cudaFree(b->order);
    cudaFree(b->d_trail);
    cudaFree(b->d_toff);
    cudaFree(b->d_out);
}

int launch(gpsat_bcp *b, const int32_t *trail, const int64_t *toff, int32_t n_trails, int32_t *status,
           int32_t *conflict, int32_t *stop, int64_t *nimpl, int32_t *ilit, int32_t *ireason, int64_t *counters,
           cudaStream_t st)
{
    const gpsat_formula *f = b->f;
    bcp::Dev d;
    d.n_vars = f->h.n_vars;
    d.n_clauses = (int32_t)f->h.n_clauses();
    d.lits = f->d_lits;
    d.w0off = f->d_w0off;
    d.w0ent = reinterpret_cast<const int4 *>(f->d_w0ent);
    d.asg = b->asg;
    d.dh = b->dh;
    d.cst = b->cst;
    d.arena = b->arena;
    d.stack = b->stack;
    d.impl = b->impl;
    d.epoch = b->epoch;
    d.next_trail = b->counter;
    d.n_words = b->n_words;
    d.n_pad = b->n_pad;
    d.m_pad = b->m_pad;
    d.arena_cap = b->arena_cap;
    d.impl_cap = b->impl_cap;
    d.n_slots = std::min<int32_t>(b->active > 0 ? b->active : b->slots, std::max<int32_t>(n_trails, 1));
    d.trail = trail;
    d.toff = toff;
    d.n_trails = n_trails;
    d.status = status;
    d.conflict = conflict;
    d.stop = stop;
    d.nimpl = nimpl;
    d.ilit = ilit;
    d.ireason = ireason;
    d.counters = counters;
    d.order = nullptr;
    cudaError_t err = cudaMemsetAsync(b->counter, 0, sizeof(unsigned int), st);
    if (err != cudaSuccess) return cuda_error(err, "bcp counter reset");
    if (n_trails == 0) return GPSAT_OK;
    if (n_trails > d.n_slots) {
        // more trails than resident warps: shortest first (see order_count)
        if (!b->hist && cudaMalloc(&b->hist, bcp::ORDER_BUCKETS * sizeof(unsigned)) != cudaSuccess)
            return set_error(GPSAT_ERR_NOMEM, "bcp order buckets");
        if (n_trails > b->order_cap) {
            cudaFree(b->order);
            b->order = nullptr;
            b->order_cap = 0;
            if (cudaMalloc(&b->order, (size_t)n_trails * 4) != cudaSuccess)
                return set_error(GPSAT_ERR_NOMEM, "bcp order");
            b->order_cap = n_trails;
        }
        err = cudaMemsetAsync(b->hist, 0, bcp::ORDER_BUCKETS * sizeof(unsigned), st);
        if (err != cudaSuccess) return cuda_error(err, "bcp order reset");
        const int g = std::min(1024, (n_trails + 255) / 256);
        bcp::order_count<<<g, 256, 0, st>>>(toff, n_trails, b->hist);
        bcp::order_scan<<<1, 1024, 0, st>>>(b->hist);
        bcp::order_scatter<<<g, 256, 0, st>>>(toff, n_trails, b->hist, b->order);
        d.order = b->order;
    }
    if (b->strategy == GPSAT_BCP_FULL_SCAN) {
        // one block per trail; the assignment bits in shared memory when they fit
        const bool smem = b->n_words <= bcp::SCAN_SMEM_WORDS;
        d.n_slots = std::min<int32_t>(smem ? b->scan_resident : std::min(b->scan_resident, b->slots),
                                      std::max<int32_t>(n_trails, 1));
        if (b->active > 0) d.n_slots = std::min(d.n_slots, b->active);
        if (smem)
            bcp::scan_kernel<true><<<d.n_slots, bcp::SCAN_NT, (size_t)b->n_words * 4, st>>>(d, f->d_coff);
        else
            bcp::scan_kernel<false><<<d.n_slots, bcp::SCAN_NT, 0, st>>>(d, f->d_coff);
    } else {
        bcp::bcp_kernel<<<d.n_slots, bcp::NT, 0, st>>>(d);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_error(err, "bcp kernel launch");
    return GPSAT_OK;
}

}  // namespace

extern "C" int gpsat_bcp_create(const gpsat_formula *f, int32_t max_slots, int64_t impl_cap, int64_t arena_cap,
                                gpsat_bcp **out)
{
    if (!f || !out || impl_cap <= 0 || impl_cap > INT32_MAX || max_slots < 0 || arena_cap < 0 ||
        arena_cap > (1 << 24))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_create: bad argument");
    *out = nullptr;
    if (f->h.verdict != GPSAT_UNKNOWN)
        return set_error(GPSAT_ERR_STATE, "formula was decided by preprocessing; nothing to propagate");
    if (f->h.max_len > bcp::MAXLEN)
        return set_error(GPSAT_ERR_CAPACITY, "clause longer than 2048 literals");
    int urc = formula_upload(const_cast<gpsat_formula *>(f));
    if (urc != GPSAT_OK) return urc;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcp::bcp_kernel, bcp::NT, 0);
    int32_t resident = std::max(1, sms * std::max(per_sm, 1));
    gpsat_bcp *b = new gpsat_bcp();
    b->f = f;
    b->device = f->device;
    b->n_pad = ((int64_t)f->h.n_vars + 15) / 16 * 16;
    b->n_words = b->n_pad / 16;
    b->m_pad = (f->h.n_clauses() + 3) / 4 * 4;
    b->impl_cap = impl_cap;
    b->arena_cap = arena_cap ? arena_cap : (1 << 17);
    const int64_t per_slot = b->n_words * 4 + b->n_pad * 4 + b->m_pad * 4 + b->arena_cap * 32 + b->impl_cap * 12;
    int32_t slots = max_slots ? max_slots : resident;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const int64_t budget = (int64_t)(free_b * 0.6);
    if ((int64_t)slots * per_slot > budget) slots = (int32_t)std::max<int64_t>(1, budget / per_slot);
    b->slots = slots;
    const size_t S = (size_t)slots;
    bool ok = cudaMalloc(&b->asg, S * b->n_words * 4) == cudaSuccess &&
              cudaMalloc(&b->dh, S * b->n_pad * 4) == cudaSuccess &&
              cudaMalloc(&b->cst, S * b->m_pad * 4) == cudaSuccess &&
              cudaMalloc(&b->epoch, S * 4) == cudaSuccess &&
              cudaMalloc(&b->arena, S * b->arena_cap * 32) == cudaSuccess &&
              cudaMalloc(&b->stack, S * b->impl_cap * 8) == cudaSuccess &&
              cudaMalloc(&b->impl, S * b->impl_cap * 4) == cudaSuccess &&
              cudaMalloc(&b->counter, 16) == cudaSuccess;
    if (ok)
        ok = cudaMemset(b->asg, 0, S * b->n_words * 4) == cudaSuccess &&
             cudaMemset(b->dh, 0, S * b->n_pad * 4) == cudaSuccess &&
             cudaMemset(b->cst, 0, S * b->m_pad * 4) == cudaSuccess && cudaMemset(b->epoch, 0, S * 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bcp_free(b);
        delete b;
        return set_error(GPSAT_ERR_NOMEM, "gpsat_bcp_create: device allocation failed");
    }
    b->bytes = (int64_t)S * per_slot;
    {
        int ps = 0;
        const bool smem = b->n_words <= bcp::SCAN_SMEM_WORDS;
        if (smem)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, bcp::scan_kernel<true>, bcp::SCAN_NT,
                                                          (size_t)b->n_words * 4);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, bcp::scan_kernel<false>, bcp::SCAN_NT, 0);
        cudaGetLastError();
        b->scan_resident = std::max(1, sms * std::max(ps, 1));
    }
    *out = b;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_destroy(gpsat_bcp *b)
{
    if (!b) return GPSAT_OK;
    cudaSetDevice(b->device);
    bcp_free(b);
    delete b;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_info(const gpsat_bcp *b, int32_t *slots, int64_t *device_bytes)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null handle");
    if (slots) *slots = b->slots;
    if (device_bytes) *device_bytes = b->bytes;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_set_active_slots(gpsat_bcp *b, int32_t n)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null handle");
    if (n < 0 || n > b->slots) return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_active_slots: n outside 0..slots");
    b->active = n;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_set_strategy(gpsat_bcp *b, int32_t strategy)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null handle");
    if (strategy != GPSAT_BCP_WATCHED && strategy != GPSAT_BCP_FULL_SCAN)
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_strategy: unknown strategy");
    b->strategy = strategy;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_run_device(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets,
                                    int32_t n_trails, int32_t *status, int32_t *conflict_clause,
                                    int32_t *stop_index, int64_t *n_impl, int32_t *impl_lit,
                                    int32_t *impl_reason, int64_t *counters, void *stream)
{
    if (!b || n_trails < 0 || (n_trails > 0 && (!trail_lits || !trail_offsets || !status || !conflict_clause ||
                                                !stop_index || !n_impl || !impl_lit || !impl_reason)))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_run_device: bad argument");
    cudaError_t err = cudaSetDevice(b->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
    return launch(b, trail_lits, trail_offsets, n_trails, status, conflict_clause, stop_index, n_impl, impl_lit,
                  impl_reason, counters, (cudaStream_t)stream);
}

extern "C" int gpsat_bcp_run_host(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets,
                                  int32_t n_trails, int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                                  int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters)
{
    if (!b || n_trails < 0 || (n_trails > 0 && (!trail_offsets || !status || !conflict_clause || !stop_index ||
                                                !n_impl || !impl_lit || !impl_reason)))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_run_host: bad argument");
    if (n_trails == 0) return GPSAT_OK;
    cudaError_t err = cudaSetDevice(b->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
    const int64_t nl = trail_offsets[n_trails];
    if (nl < 0 || (nl > 0 && !trail_lits)) return set_error(GPSAT_ERR_ARG, "bad trail offsets");
    {
        // Every buffer page-locked (cudaHostAlloc / cudaHostRegister, as
        // torch's pin_memory): the kernel reads the trails and writes the
        // results in place, over the CPU-GPU link, with no staging copies.
        const void *hp[9] = {nl > 0 ? (const void *)trail_lits : (const void *)trail_offsets, trail_offsets, status, conflict_clause, stop_index,
                             n_impl, impl_lit, impl_reason, counters ? (const void *)counters : trail_offsets};
        void *dp[9];
        bool all = true;
        for (int i = 0; i < 9 && all; i++) {
            cudaPointerAttributes a;
            if (cudaPointerGetAttributes(&a, hp[i]) != cudaSuccess) {
                cudaGetLastError();
                all = false;
            } else {
                all = a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
                dp[i] = a.devicePointer;
            }
        }
        if (all) {
            int rc = launch(b, (const int32_t *)dp[0], (const int64_t *)dp[1], n_trails, (int32_t *)dp[2],
                            (int32_t *)dp[3], (int32_t *)dp[4], (int64_t *)dp[5], (int32_t *)dp[6], (int32_t *)dp[7],
                            counters ? (int64_t *)dp[8] : nullptr, 0);
            if (rc != GPSAT_OK) return rc;
            err = cudaStreamSynchronize(0);
            if (err != cudaSuccess) return cuda_error(err, "bcp run");
            return GPSAT_OK;
        }
    }
    if (nl > b->trail_cap) {
        cudaFree(b->d_trail);
        b->d_trail = nullptr;
        if (cudaMalloc(&b->d_trail, std::max<int64_t>(nl, 1) * 4) != cudaSuccess) {
            b->trail_cap = 0;
            return set_error(GPSAT_ERR_NOMEM, "trail staging");
        }
        b->trail_cap = nl;
    }
    if (n_trails + 1 > b->toff_cap) {
        cudaFree(b->d_toff);
        b->d_toff = nullptr;
        if (cudaMalloc(&b->d_toff, (int64_t)(n_trails + 1) * 8) != cudaSuccess) {
            b->toff_cap = 0;
            return set_error(GPSAT_ERR_NOMEM, "offset staging");
        }
        b->toff_cap = n_trails + 1;
    }
    const int64_t T = n_trails;
    const int64_t need = T * (4 + 4 + 4 + 8 + 8 * GPSAT_BCP_NCOUNTERS) + 2 * T * b->impl_cap * 4 + 64;
    if (need > b->out_cap) {
        cudaFree(b->d_out);
        b->d_out = nullptr;
        if (cudaMalloc(&b->d_out, need) != cudaSuccess) {
            b->out_cap = 0;
            return set_error(GPSAT_ERR_NOMEM, "output staging");
        }
        b->out_cap = need;
    }
    char *p = (char *)b->d_out;
    int64_t *d_nimpl = (int64_t *)p;
    p += T * 8;
    int64_t *d_cnt = (int64_t *)p;
    p += T * 8 * GPSAT_BCP_NCOUNTERS;
    int32_t *d_status = (int32_t *)p;
    p += T * 4;
    int32_t *d_confl = (int32_t *)p;
    p += T * 4;
    int32_t *d_stop = (int32_t *)p;
    p += T * 4;
    int32_t *d_ilit = (int32_t *)p;
    p += T * b->impl_cap * 4;
    int32_t *d_ireason = (int32_t *)p;
    cudaStream_t st = 0;
    if (nl > 0 && cudaMemcpyAsync(b->d_trail, trail_lits, nl * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "trail copy");
    if (cudaMemcpyAsync(b->d_toff, trail_offsets, (T + 1) * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "offset copy");
    int rc = launch(b, b->d_trail, b->d_toff, n_trails, d_status, d_confl, d_stop, d_nimpl, d_ilit, d_ireason,
                    counters ? d_cnt : nullptr, st);
    if (rc != GPSAT_OK) return rc;
    bool ok = cudaMemcpyAsync(status, d_status, T * 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaMemcpyAsync(conflict_clause, d_confl, T * 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaMemcpyAsync(stop_index, d_stop, T * 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
              cudaMemcpyAsync(n_impl, d_nimpl, T * 8, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (ok && counters)
        ok = cudaMemcpyAsync(counters, d_cnt, T * 8 * GPSAT_BCP_NCOUNTERS, cudaMemcpyDeviceToHost, st) ==
             cudaSuccess;
    if (!ok) return cuda_error(cudaGetLastError(), "result copy");
    err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return cuda_error(err, "bcp run");
    // implication lists: copy only the used prefix of each trail's region
    int64_t maxn = 0;
    for (int64_t t = 0; t < T; t++) maxn = std::max(maxn, n_impl[t]);
    if (maxn * 4 >= b->impl_cap * 2) {
        ok = cudaMemcpy(impl_lit, d_ilit, T * b->impl_cap * 4, cudaMemcpyDeviceToHost) == cudaSuccess &&
             cudaMemcpy(impl_reason, d_ireason, T * b->impl_cap * 4, cudaMemcpyDeviceToHost) == cudaSuccess;
    } else if (maxn > 0) {
        ok = cudaMemcpy2D(impl_lit, b->impl_cap * 4, d_ilit, b->impl_cap * 4, maxn * 4, T,
                          cudaMemcpyDeviceToHost) == cudaSuccess &&
             cudaMemcpy2D(impl_reason, b->impl_cap * 4, d_ireason, b->impl_cap * 4, maxn * 4, T,
                          cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    if (!ok) return cuda_error(cudaGetLastError(), "implication copy");
    return GPSAT_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free entry: the per-trail state in a fixed device array
// ---------------------------------------------------------------------------
// For callers that cannot allocate device memory while they propagate: code
// that captures the call into a CUDA graph (no cudaMalloc/cudaFree on a
// capturing stream, and a replayed graph needs addresses that do not move)
// and hosts whose device memory is reserved up front by their own pool.  The
// call below makes no allocating CUDA call and no library allocation; the
// slots' state lives in bcp_static_scratch, laid out afresh by every call:
//   [launch counter | epoch per slot | assignment words | list heads | clause
//    states | move arena | stack | implied literals]
// each part 256-byte aligned.  Everything but the arena, the stack and the
// implied literals (which the kernel writes before it reads) is cleared on the
// stream per call.  One array per device, so calls whose GPU work overlaps
// race on it.  The array's device address is looked up once per device and
// kept for the life of the process; after a cudaDeviceReset the module may be
// loaded again at another address, so this entry is not for use across a
// device reset.
namespace gpsat {
namespace bcp {

static __device__ __align__(256) unsigned char bcp_static_scratch[GPSAT_BCP_STATIC_SCRATCH_BYTES];

}  // namespace bcp
}  // namespace gpsat

namespace {

constexpr int STATIC_MAX_DEVICES = 64;
constexpr int64_t STATIC_ALIGN = 256;

inline int64_t align_up(int64_t x) { return (x + STATIC_ALIGN - 1) / STATIC_ALIGN * STATIC_ALIGN; }

struct StaticScratch {
    std::mutex mu;
    bool ready[STATIC_MAX_DEVICES] = {};
    unsigned char *base[STATIC_MAX_DEVICES] = {};
    int32_t resident[STATIC_MAX_DEVICES] = {};
};

StaticScratch &static_scratch()
{
    static StaticScratch s;
    return s;
}

// Once per device, with that device current: the array's device address and
// the resident warp count of the BCP kernel.  The lookup may load the module,
// which is why the first call must not come inside a stream capture.
int static_setup(int device, unsigned char **base, int32_t *resident)
{
    if (device < 0 || device >= STATIC_MAX_DEVICES)
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_run_static: device ordinal out of range");
    StaticScratch &s = static_scratch();
    std::lock_guard<std::mutex> lock(s.mu);
    if (!s.ready[device]) {
        void *ptr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&ptr, bcp::bcp_static_scratch);
        if (err != cudaSuccess) return cuda_error(err, "cudaGetSymbolAddress(bcp_static_scratch)");
        int sms = 0, per_sm = 0;
        err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (err != cudaSuccess) return cuda_error(err, "cudaDeviceGetAttribute");
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcp::bcp_kernel, bcp::NT, 0);
        if (err != cudaSuccess) return cuda_error(err, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        s.base[device] = static_cast<unsigned char *>(ptr);
        s.resident[device] = std::max(1, sms * std::max(per_sm, 1));
        s.ready[device] = true;
    }
    *base = s.base[device];
    *resident = s.resident[device];
    return GPSAT_OK;
}

// Bytes of the scratch layout for S slots (each part rounded up to 256):
// counter, epochs, assignment words, list heads, clause states, move arena,
// depth-first stack, implied literals.
int64_t static_layout_bytes(int64_t S, int64_t n_pad, int64_t m_pad, int64_t arena_cap, int64_t impl_cap)
{
    return STATIC_ALIGN + align_up(S * 4) + align_up(S * (n_pad / 16) * 4) + align_up(S * n_pad * 4) +
           align_up(S * m_pad * 4) + align_up(S * arena_cap * 32) + align_up(S * impl_cap * 8) +
           align_up(S * impl_cap * 4);
}

}  // namespace

extern "C" int gpsat_bcp_run_static(const gpsat_formula *f, int64_t impl_cap, int64_t arena_cap,
                                    const int32_t *trail_lits, const int64_t *trail_offsets, int32_t n_trails,
                                    int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                                    int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason, int64_t *counters,
                                    void *stream)
{
    if (!f || impl_cap <= 0 || impl_cap > INT32_MAX || arena_cap < 0 || arena_cap > (1 << 24) || n_trails < 0 ||
        (n_trails > 0 && (!trail_lits || !trail_offsets || !status || !conflict_clause || !stop_index || !n_impl ||
                          !impl_lit || !impl_reason)))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_run_static: bad argument");
    if (f->h.verdict != GPSAT_UNKNOWN)
        return set_error(GPSAT_ERR_STATE, "formula was decided by preprocessing; nothing to propagate");
    if (f->h.max_len > bcp::MAXLEN) return set_error(GPSAT_ERR_CAPACITY, "clause longer than 2048 literals");
    if (!f->uploaded)
        return set_error(GPSAT_ERR_STATE,
                         "gpsat_bcp_run_static: the formula is not on the device yet (gpsat_bcp_create on it "
                         "uploads it; this entry point allocates nothing, so it cannot upload)");
    // switch devices only when needed (a caller capturing this call into a
    // graph keeps its device current), and back before returning
    int cur_dev = -1;
    cudaError_t err = cudaGetDevice(&cur_dev);
    if (err == cudaSuccess && cur_dev != f->device) err = cudaSetDevice(f->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
    struct Restore {
        int dev, was;
        ~Restore()
        {
            if (was >= 0 && was != dev) cudaSetDevice(was);
        }
    } restore{f->device, cur_dev};
    unsigned char *base = nullptr;
    int32_t resident = 0;
    int rc = static_setup(f->device, &base, &resident);
    if (rc != GPSAT_OK) return rc;

    const int64_t n_pad = ((int64_t)f->h.n_vars + 15) / 16 * 16;
    const int64_t m_pad = (f->h.n_clauses() + 3) / 4 * 4;
    const int64_t acap = arena_cap ? arena_cap : (1 << 17);
    const int64_t limit = GPSAT_BCP_STATIC_SCRATCH_BYTES;
    if (static_layout_bytes(1, n_pad, m_pad, acap, impl_cap) > limit) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "gpsat_bcp_run_static: one trail's state needs %lld bytes (n_vars %d, %lld clauses, "
                      "arena_cap %lld, impl_cap %lld) but the static scratch holds %lld bytes",
                      (long long)static_layout_bytes(1, n_pad, m_pad, acap, impl_cap), f->h.n_vars,
                      (long long)f->h.n_clauses(), (long long)acap, (long long)impl_cap, (long long)limit);
        return set_error(GPSAT_ERR_CAPACITY, msg);
    }
    int64_t S = std::min<int64_t>(resident, std::max<int32_t>(n_trails, 1));
    const int64_t per_slot = 4 + (n_pad / 16) * 4 + n_pad * 4 + m_pad * 4 + acap * 32 + impl_cap * 12;
    S = std::min<int64_t>(S, std::max<int64_t>(1, (limit - 9 * STATIC_ALIGN) / per_slot));
    while (S > 1 && static_layout_bytes(S, n_pad, m_pad, acap, impl_cap) > limit) S--;

    unsigned char *p = base;
    auto take = [&](int64_t bytes) {
        unsigned char *q = p;
        p += align_up(bytes);
        return q;
    };
    unsigned int *counter = reinterpret_cast<unsigned int *>(take(STATIC_ALIGN));
    uint32_t *epoch = reinterpret_cast<uint32_t *>(take(S * 4));
    uint32_t *asg = reinterpret_cast<uint32_t *>(take(S * (n_pad / 16) * 4));
    uint32_t *dh = reinterpret_cast<uint32_t *>(take(S * n_pad * 4));
    uint32_t *cst = reinterpret_cast<uint32_t *>(take(S * m_pad * 4));
    int4 *arena = reinterpret_cast<int4 *>(take(S * acap * 32));
    int2 *stack = reinterpret_cast<int2 *>(take(S * impl_cap * 8));
    int32_t *impl = reinterpret_cast<int32_t *>(take(S * impl_cap * 4));

    cudaStream_t st = (cudaStream_t)stream;
    // what the kernel expects to find zero: the launch counter, the slots'
    // epochs, assignment words and epoch-tagged state (a previous call may
    // have used another formula with another layout)
    err = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(epoch, 0, (size_t)S * 4, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(asg, 0, (size_t)(S * (n_pad / 16) * 4), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(dh, 0, (size_t)(S * n_pad * 4), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(cst, 0, (size_t)(S * m_pad * 4), st);
    if (err != cudaSuccess) return cuda_error(err, "gpsat_bcp_run_static: clearing the static scratch");
    if (n_trails == 0) return GPSAT_OK;

    bcp::Dev d;
    d.n_vars = f->h.n_vars;
    d.n_clauses = (int32_t)f->h.n_clauses();
    d.lits = f->d_lits;
    d.w0off = f->d_w0off;
    d.w0ent = reinterpret_cast<const int4 *>(f->d_w0ent);
    d.asg = asg;
    d.dh = dh;
    d.cst = cst;
    d.arena = arena;
    d.stack = stack;
    d.impl = impl;
    d.epoch = epoch;
    d.next_trail = counter;
    d.order = nullptr;
    d.n_words = n_pad / 16;
    d.n_pad = n_pad;
    d.m_pad = m_pad;
    d.arena_cap = acap;
    d.impl_cap = impl_cap;
    d.n_slots = (int32_t)S;
    d.trail = trail_lits;
    d.toff = trail_offsets;
    d.n_trails = n_trails;
    d.status = status;
    d.conflict = conflict_clause;
    d.stop = stop_index;
    d.nimpl = n_impl;
    d.ilit = impl_lit;
    d.ireason = impl_reason;
    d.counters = counters;
    bcp::bcp_kernel<<<(int)S, bcp::NT, 0, st>>>(d);
    err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_error(err, "bcp kernel launch (static scratch)");
    return GPSAT_OK;
}
