// Device CDCL: one warp solves one job (an instance, optionally restricted to
// a cube of assumption literals); a persistent grid pulls jobs from a global
// counter until none are left.
//
// Roles of the reference solver (paths inside the reference project, src/)
// and their counterparts here:
//   BCPStrategy (two watched literals)  WatchedClausesList.cu  -> propagate(): per-literal
//       watch lists with blockers, one list at a time, 32 watches per step
//   ConflictAnalysis                    ConflictAnalyzer.cu, GraphAnalyzer.cu  -> analyze():
//       first-UIP cut over the trail (the reference cuts at the decision),
//       basic clause minimisation
//   ClauseLearning                      LearntClausesManager.cu  -> learn(): clauses are
//       appended to a per-job arena and watched; reduce() keeps the better half by LBD
//       (the reference keeps a ring of 20)
//   DecisionStrategy                    DecisionMaker.cu, VSIDS.cu  -> decide(): VSIDS with
//       float activities, bump/decay, phase saving; or the reference's default
//       "last free variable, positive" rule
//   Restarts                            GeometricRestartsManager.cu  -> Luby or geometric
//   Backtracker                         Backtracker.cu -> backtrack(): non-chronological
//   SATSolver::solve                    SATSolver.cu:67-218 -> solve_job() with a conflict
//       budget instead of the reference's iteration cap
//
// Per-job state lives in a per-warp slot in HBM: variable arrays (value, level,
// reason, trail, activity, phase), per-literal watch lists, a clause arena
// ([len|flags][lbd][literals...]) and the list of live clause references.
// Clause literals 0 and 1 are the watched ones; a reason clause has its implied
// literal at position 0.
//
// A watch list that outgrows its room moves to the free tail of the slot's
// watch area; only when that tail is used up is the whole area rebuilt.
//
// Every loop is bounded: conflicts by the budget, decisions by the variable
// count between conflicts, propagation by the trail length, list moves by the
// tail and full rebuilds by a guard; a job that outgrows its slot ends UNKNOWN
// with FL_RESOURCE and the exhausted limit (ResourceCode) in bits 16..23 of
// its flags.
#include <cuda_runtime.h>

#include <cfloat>

#include "cdcl.cuh"
#include "internal.h"

namespace gpsat {
namespace cdcl {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WARPS = 4;
enum : int { W_KEEP = 0, W_MOVE = 1, W_IMPLY = 2, W_CONFL = 3 };
enum : int { R_RUN = 0, R_SAT = 10, R_UNSAT = 20, R_UNKNOWN = 0 };

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
// position of the n-th set bit of m (n >= 1, m holds at least n set bits)
__device__ __forceinline__ int nth_set_bit(unsigned m, int n)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc(m & ((1u << w) - 1u));
        if (c < n) {
            n -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

template <class T>
__device__ __forceinline__ T wsum(T x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    return x;
}
__device__ __forceinline__ int wmax(int x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(FULL, x, o));
    return x;
}
__device__ __forceinline__ int wscan_incl(int x, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

struct Ctx {
    int lane;
    int n;
    int8_t *val, *phase;
    uint8_t *seen;
    int32_t *level, *reason, *trail, *tlim, *learnt, *lstamp, *tmp;
    float *act;
    float *bmax;     // per block of 32 variables: >= the largest activity of its unassigned
                     // variables (-1: none left); exact for a block pick_branch last tightened
    bool use_bmax;   // large formulas pick through the block bounds, small ones scan
    int32_t *wl_start, *wl_size, *wl_cap;
    int2 *watches;
    int32_t *arena, *crefs;
    int32_t *sm64;   // 64 ints of shared memory for this warp
    int32_t *part;
    int32_t *occ;    // per variable: occurrences in learnt clauses (optional)
    int64_t WCAP, ACAP, CCAP;
    int64_t wtop;    // first watch entry of the free tail (lists outgrown are moved there)
    // warp-uniform state
    int32_t tsize, qhead, dlevel;
    int32_t arena_top, n_crefs, n_orig, orig_top;
    int32_t stamp;
    float var_inc;
    int32_t minimize;
    bool resource;
    int32_t check;   // first failed consistency check (CheckCode), 0 if none
    int32_t why;     // which limit set `resource` (ResourceCode)
    int64_t conflicts, decisions, props, restarts, reduces, rebuilds;
    int32_t *proof;  // this job's proof log (null: none)
    int64_t plen;    // words logged, -1 once the log overflowed
};

__device__ __forceinline__ void fail_check(Ctx &C, int code)
{
    if (C.check == 0) C.check = code;
    C.resource = true;
}
__device__ __forceinline__ void out_of(Ctx &C, int why)
{
    if (C.why == 0) C.why = why;
    C.resource = true;
}

__device__ __forceinline__ int lval(const Ctx &C, int32_t l)
{
    int a = C.val[l >> 1];
    return (l & 1) ? a : -a;
}

// ---------------------------------------------------------------- watches
// Rebuilds every watch list from clause positions 0 and 1 (deterministic
// order: clause reference order), compacting the watch area.  Each list gets
// up to half its length again as room to grow and the rest of the area stays
// a free tail that lists which outgrow their room move to (relocate), so a
// full rebuild is needed only when that tail is used up.  Returns false when
// the watches alone do not fit the slot.
__device__ bool rebuild_watches(Ctx &C)
{
    const int lane = C.lane;
    const int nl = 2 * C.n;
    // the list sizes count each literal's watches first; the layout below
    // reads each count once and then sets the size to zero
    for (int i = lane; i < nl; i += 32) C.wl_size[i] = 0;
    __syncwarp();
    for (int k = lane; k < C.n_crefs; k += 32) {
        const int32_t r = C.crefs[k];
        const uint32_t h = (uint32_t)C.arena[r];
        if (!(h & F_DELETED) && (h & LEN_MASK) >= 2) {
            atomicAdd(&C.wl_size[C.arena[r + HDR]], 1);
            atomicAdd(&C.wl_size[C.arena[r + HDR + 1]], 1);
        }
    }
    __syncwarp();
    // half the spare capacity at most is shared out in proportion to each
    // list's length plus one; the other half is the free tail
    int64_t total = 0;
    for (int i = lane; i < nl; i += 32) total += C.wl_size[i];
    total = wsum(total);
    if (total > C.WCAP) return false;
    const int64_t spare = C.WCAP - total, weight = 2 * (total + nl);
    int64_t running = 0;
    for (int b = 0; b < nl; b += 32) {
        const int i = b + lane;
        const int c = i < nl ? C.wl_size[i] : 0;
        const int room = min((int)(spare * (c + 1) / weight), c / 2 + 8);
        const int cap = i < nl ? c + room : 0;
        const int incl = wscan_incl(cap, lane);
        if (i < nl) {
            C.wl_start[i] = (int32_t)(running + incl - cap);
            C.wl_cap[i] = cap;
            C.wl_size[i] = 0;
        }
        running += __shfl_sync(FULL, incl, 31);
    }
    C.rebuilds++;
    if (running > C.WCAP) return false;
    C.wtop = running;
    __syncwarp();
    for (int b = 0; b < C.n_crefs; b += 32) {
        const int k = b + lane;
        bool ok = false;
        int32_t r = 0, t0 = -1, t1 = -1;
        if (k < C.n_crefs) {
            r = C.crefs[k];
            const uint32_t h = (uint32_t)C.arena[r];
            ok = !(h & F_DELETED) && (h & LEN_MASK) >= 2;
            if (ok) {
                t0 = C.arena[r + HDR];
                t1 = C.arena[r + HDR + 1];
            }
        }
        C.sm64[2 * lane] = ok ? t0 : -1;
        C.sm64[2 * lane + 1] = ok ? t1 : -1;
        __syncwarp();
        int rk0 = 0, rk1 = 0;
        if (ok) {
            for (int q = 0; q < 2 * lane; q++) {
                const int tq = C.sm64[q];
                rk0 += tq == t0;
                rk1 += tq == t1;
            }
            rk1 += (t0 == t1);
        }
        int p0 = 0, p1 = 0;
        if (ok) {
            p0 = C.wl_start[t0] + C.wl_size[t0] + rk0;
            p1 = C.wl_start[t1] + C.wl_size[t1] + rk1;
        }
        __syncwarp();
        if (ok) {
            C.watches[p0] = make_int2(r, t1);
            C.watches[p1] = make_int2(r, t0);
            atomicAdd(&C.wl_size[t0], 1);
            atomicAdd(&C.wl_size[t1], 1);
        }
        __syncwarp();
    }
    return true;
}

// append one watch; false on overflow (caller relocates the list or rebuilds)
__device__ __forceinline__ bool watch_push(Ctx &C, int32_t lit, int32_t ref, int32_t blk)
{
    const int32_t pos = atomicAdd(&C.wl_size[lit], 1);
    if (pos < C.wl_cap[lit]) {
        C.watches[C.wl_start[lit] + pos] = make_int2(ref, blk);
        return true;
    }
    atomicSub(&C.wl_size[lit], 1);
    return false;
}

// Warp-collective: moves the list of `lit` to the free tail with twice its
// length (plus 8) as capacity; its old entries become waste until the next
// rebuild.  False when the tail is used up.  Every lane must have finished
// its pushes (a __syncwarp) before the call.
__device__ bool relocate(Ctx &C, int32_t lit)
{
    const int32_t sz = C.wl_size[lit];
    const int32_t from = C.wl_start[lit];
    const int64_t cap = 2 * (int64_t)sz + 8;
    if (C.wtop + cap > C.WCAP) return false;
    const int32_t to = (int32_t)C.wtop;
    for (int k = C.lane; k < sz; k += 32) C.watches[to + k] = C.watches[from + k];
    __syncwarp();
    if (C.lane == 0) {
        C.wl_start[lit] = to;
        C.wl_cap[lit] = (int32_t)cap;
    }
    C.wtop += cap;
    __syncwarp();
    return true;
}

// Warp-collective append of one watch by lane 0, growing the list into the
// free tail when it is full.  False only when the tail is used up.
__device__ bool attach_watch(Ctx &C, int32_t lit, int32_t ref, int32_t blk)
{
    for (int tries = 0; tries < 4; tries++) {
        bool ok = false;
        if (C.lane == 0) ok = watch_push(C, lit, ref, blk);
        if (__shfl_sync(FULL, ok, 0)) return true;
        __syncwarp();
        if (!relocate(C, lit)) return false;
    }
    return false;
}

// ---------------------------------------------------------------- BCP
// Evaluates one watch of false literal x: keep (blocker or other watch true),
// move (a non-false replacement at position kpos), imply l0, or conflict.
__device__ __forceinline__ void eval_watch(const Ctx &C, int32_t x, int2 w, int &act, int32_t &blk, int32_t &imp,
                                           int32_t &tgt, int32_t &l0, int &kpos, bool &swapped)
{
    int32_t *CL = C.arena + w.x + HDR;
    const int len = (int)((uint32_t)C.arena[w.x] & LEN_MASK);
    l0 = CL[0];
    if (l0 == x) {
        l0 = CL[1];
        swapped = true;
    }
    const int v0 = lval(C, l0);
    if (v0 == 1) {
        blk = l0;
        return;
    }
    // first literal at position >= 2 that is not false, four literals per
    // 16-byte load (chunks aligned in the arena, whose slot base and capacity
    // are multiples of 4 words)
    int k = len;
    int32_t lk = 0;
    const int64_t a0 = (int64_t)w.x + HDR + 2, a1 = (int64_t)w.x + HDR + len;
    for (int64_t c = a0 & ~int64_t(3); c < a1 && k == len; c += 4) {
        const int4 q = *reinterpret_cast<const int4 *>(C.arena + c);
        const int32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
            const int64_t at = c + jj;
            if (k == len && at >= a0 && at < a1 && lval(C, qq[jj]) != -1) {
                k = (int)(at - ((int64_t)w.x + HDR));
                lk = qq[jj];
            }
        }
    }
    blk = l0;
    if (k < len) {
        act = W_MOVE;
        tgt = lk;
        kpos = k;
    } else {
        act = (v0 == -1) ? W_CONFL : W_IMPLY;
        imp = l0;
    }
}

// Several pending literals whose watch lists fit together in one 32-wide
// step are propagated at once: lane k takes entry k of the concatenated lists.
// (A CDCL solver may propagate its queue in any order, and every action below
// is valid against the state before the step, as in the one-list step.)
// Returns the number of literals consumed (0: not applicable, the caller takes
// the one-list path); sets confl / overflow like it.
__device__ int propagate_multi(Ctx &C, int32_t &confl, bool &overflow)
{
    const int lane = C.lane;
    const unsigned lt = lanemask_lt();
    const int npend = min(32, C.tsize - C.qhead);
    if (npend < 2) return 0;
    int32_t xl = 0, sl = 0, nl = 0;
    if (lane < npend) {
        xl = C.trail[C.qhead + lane] ^ 1;
        sl = C.wl_start[xl];
        nl = C.wl_size[xl];
    }
    int incl = nl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    // sizes are >= 0, so the lists that fit form a prefix of the queue
    const unsigned fit = __ballot_sync(FULL, lane < npend && incl <= 32);
    const int K = __popc(fit);
    if (K < 2) return 0;
    const int total = __shfl_sync(FULL, incl, K - 1);
    const int excl = incl - nl;
    // entry position -> list: rank among the lists that start at or before it
    const bool nonempty = lane < K && nl > 0;
    const unsigned nem = __ballot_sync(FULL, nonempty);
    const unsigned starts = __reduce_or_sync(FULL, nonempty ? (1u << excl) : 0u);
    bool has = lane < total;
    int li = 0;
    if (has) li = nth_set_bit(nem, __popc(starts & (lane == 31 ? FULL : ((2u << lane) - 1u))));
    const int32_t x = __shfl_sync(FULL, xl, li), s = __shfl_sync(FULL, sl, li), e0 = __shfl_sync(FULL, excl, li);
    int2 w = has ? C.watches[s + lane - e0] : make_int2(-1, 0);
    if (__any_sync(FULL, has && (w.x < 0 || w.x >= C.arena_top || w.y < 0 || w.y >= 2 * C.n))) {
        fail_check(C, CK_CREF);
        confl = -1;
        return -1;
    }
    // a clause in two of these lists (both its watches false): take only the
    // lists before the later one (the one-list path when that leaves one)
    const unsigned dup = __match_any_sync(FULL, has ? w.x : -1 - lane);
    const int kd = __reduce_min_sync(FULL, (has && (dup & lt)) ? (unsigned)li : 32u);
    int K2 = K;
    if (kd < K2) {
        K2 = kd;
        if (K2 < 2) return 0;
        has = lane < __shfl_sync(FULL, incl, K2 - 1);
        if (!has) w = make_int2(-1, 0);
    }
    C.qhead += K2;
    C.props += K2;
    int act = W_KEEP;
    int32_t blk = w.y, imp = -1, tgt = -1, l0 = 0;
    int kpos = -1;
    bool swapped = false;
    if (has && lval(C, w.y) != 1) eval_watch(C, x, w, act, blk, imp, tgt, l0, kpos, swapped);
    bool moved = false, full = false;
    if (act == W_MOVE) {
        moved = watch_push(C, tgt, w.x, l0);
        full = !moved;
    }
    __syncwarp();
    while (__any_sync(FULL, full)) {
        const int ld = __ffs(__ballot_sync(FULL, full)) - 1;
        const int32_t L = __shfl_sync(FULL, tgt, ld);
        if (!relocate(C, L)) break;
        if (full && tgt == L) {
            moved = watch_push(C, tgt, w.x, l0);
            full = !moved;
        }
        __syncwarp();
    }
    overflow |= __any_sync(FULL, full);
    if (moved) {
        int32_t *CL = C.arena + w.x + HDR;
        CL[0] = l0;
        CL[1] = tgt;
        CL[kpos] = x;
    }
    const bool is_imp = act == W_IMPLY;
    bool winner = false;
    if (__any_sync(FULL, is_imp)) {
        const int32_t key = is_imp ? (imp >> 1) : -1 - lane;
        const unsigned grp = __match_any_sync(FULL, key);
        const int lead = __ffs(grp) - 1;
        const int32_t lead_lit = __shfl_sync(FULL, imp, lead);
        winner = is_imp && lead == lane;
        if (is_imp && !winner) act = (imp == lead_lit) ? W_KEEP : W_CONFL;
    }
    const unsigned wm = __ballot_sync(FULL, winner);
    if (C.tsize + __popc(wm) > C.n) {
        fail_check(C, CK_TRAIL);
        return -1;
    }
    if (winner) {
        int32_t *CL = C.arena + w.x + HDR;
        if (swapped) {
            CL[0] = l0;
            CL[1] = x;
        }
        const int pos = C.tsize + __popc(wm & lt);
        const int32_t v = imp >> 1;
        C.val[v] = (imp & 1) ? 1 : -1;
        C.level[v] = C.dlevel;
        C.reason[v] = w.x;
        C.trail[pos] = imp;
    }
    C.tsize += __popc(wm);
    const unsigned cm = __ballot_sync(FULL, act == W_CONFL);
    if (cm) confl = __shfl_sync(FULL, w.x, __ffs(cm) - 1);
    // each list keeps its entries that did not move, in order, at its start
    const bool kept = has && !moved;
    const unsigned km = __ballot_sync(FULL, kept);
    const unsigned seg = __match_any_sync(FULL, has ? li : -1 - lane);
    if (kept) C.watches[s + __popc(km & lt & seg)] = make_int2(w.x, blk);
    __syncwarp();
    // new list sizes: the first lane of each list writes its count
    if (has && (seg & lt) == 0) C.wl_size[x] = __popc(km & seg);
    __syncwarp();
    return K2;
}

// Returns the conflicting clause reference, or -1.
__device__ int32_t propagate(Ctx &C)
{
    const int lane = C.lane;
    const unsigned lt = lanemask_lt();
    int32_t confl = -1;
    int guard = 0;
    while (C.qhead < C.tsize && confl < 0) {
        bool moverflow = false;
        const int took = propagate_multi(C, confl, moverflow);
        if (took < 0) return -1;
        if (took > 0) {
            if (moverflow) {
                if (!rebuild_watches(C)) {
                    out_of(C, RS_WATCHES);
                    return -1;
                }
                if (confl < 0) C.qhead = (C.dlevel > 0) ? C.tlim[C.dlevel - 1] : 0;
                if (++guard > 64) {
                    out_of(C, RS_REBUILD_LOOP);
                    return -1;
                }
            }
            continue;
        }
        const int32_t p = C.trail[C.qhead];
        C.qhead++;
        C.props++;
        const int32_t x = p ^ 1;  // the literal that became false
        const int32_t s = C.wl_start[x];
        const int32_t nsz = C.wl_size[x];
        int32_t i = 0, j = 0;
        bool overflow = false;
        while (i < nsz) {
            const int cnt = min(32, nsz - i);
            const bool has = lane < cnt;
            int2 w = has ? C.watches[s + i + lane] : make_int2(-1, 0);
            // a watch must name a clause of this job and a literal of its variables
            if (__any_sync(FULL, has && (w.x < 0 || w.x >= C.arena_top || w.y < 0 || w.y >= 2 * C.n))) {
                fail_check(C, CK_CREF);
                return -1;
            }
            // every watch of the batch has a true blocker: it stays as it is
            // (moved down over the entries earlier batches moved away)
            if (__all_sync(FULL, !has || lval(C, w.y) == 1)) {
                if (j != i && has) C.watches[s + j + lane] = w;
                j += cnt;
                i += cnt;
                __syncwarp();
                continue;
            }
            int act = W_KEEP;
            int32_t blk = w.y, imp = -1, tgt = -1, l0 = 0;
            int kpos = -1;
            bool swapped = false;
            if (has && lval(C, w.y) != 1) {
                int32_t *CL = C.arena + w.x + HDR;
                const int len = (int)((uint32_t)C.arena[w.x] & LEN_MASK);
                l0 = CL[0];
                if (l0 == x) {
                    l0 = CL[1];
                    swapped = true;
                }
                const int v0 = lval(C, l0);
                if (v0 == 1) {
                    blk = l0;
                } else {
                    // first literal at position >= 2 that is not false, four
                    // literals per 16-byte load (chunks aligned in the arena,
                    // whose slot base and capacity are multiples of 4 words)
                    int k = len;
                    int32_t lk = 0;
                    const int64_t a0 = (int64_t)w.x + HDR + 2, a1 = (int64_t)w.x + HDR + len;
                    for (int64_t c = a0 & ~int64_t(3); c < a1 && k == len; c += 4) {
                        const int4 q = *reinterpret_cast<const int4 *>(C.arena + c);
                        const int32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int64_t at = c + j;
                            if (k == len && at >= a0 && at < a1 && lval(C, qq[j]) != -1) {
                                k = (int)(at - ((int64_t)w.x + HDR));
                                lk = qq[j];
                            }
                        }
                    }
                    blk = l0;
                    if (k < len) {
                        act = W_MOVE;
                        tgt = lk;
                        kpos = k;
                    } else {
                        act = (v0 == -1) ? W_CONFL : W_IMPLY;
                        imp = l0;
                    }
                }
            }
            bool moved = false, full = false;
            if (act == W_MOVE) {
                moved = watch_push(C, tgt, w.x, l0);
                full = !moved;
            }
            __syncwarp();
            // a full target list grows into the free tail (one list at a time,
            // every lane moving to it retries); when the tail is used up the
            // clause stays here and the whole area is rebuilt below
            while (__any_sync(FULL, full)) {
                const int ld = __ffs(__ballot_sync(FULL, full)) - 1;
                const int32_t L = __shfl_sync(FULL, tgt, ld);
                if (!relocate(C, L)) break;
                if (full && tgt == L) {
                    moved = watch_push(C, tgt, w.x, l0);
                    full = !moved;
                }
                __syncwarp();
            }
            overflow |= full;
            if (moved) {
                int32_t *CL = C.arena + w.x + HDR;
                CL[0] = l0;
                CL[1] = tgt;
                CL[kpos] = x;
            }
            // several lanes may imply the same variable: the lowest lane wins,
            // the same literal again is kept, the opposite one is a conflict
            const bool is_imp = act == W_IMPLY;
            bool winner = false;
            if (__any_sync(FULL, is_imp)) {
                const int32_t key = is_imp ? (imp >> 1) : -1 - lane;
                const unsigned grp = __match_any_sync(FULL, key);
                const int lead = __ffs(grp) - 1;
                const int32_t lead_lit = __shfl_sync(FULL, imp, lead);
                winner = is_imp && lead == lane;
                if (is_imp && !winner) act = (imp == lead_lit) ? W_KEEP : W_CONFL;
            }
            const unsigned wm = __ballot_sync(FULL, winner);
            if (C.tsize + __popc(wm) > C.n) {  // more assignments than variables
                fail_check(C, CK_TRAIL);
                return -1;
            }
            if (winner) {
                int32_t *CL = C.arena + w.x + HDR;
                if (swapped) {
                    CL[0] = l0;
                    CL[1] = x;
                }
                const int pos = C.tsize + __popc(wm & lt);
                const int32_t v = imp >> 1;
                C.val[v] = (imp & 1) ? 1 : -1;
                C.level[v] = C.dlevel;
                C.reason[v] = w.x;
                C.trail[pos] = imp;
            }
            C.tsize += __popc(wm);
            const unsigned cm = __ballot_sync(FULL, act == W_CONFL);
            if (cm) confl = __shfl_sync(FULL, w.x, __ffs(cm) - 1);
            const bool kept = has && !moved;
            const unsigned km = __ballot_sync(FULL, kept);
            if (kept) C.watches[s + j + __popc(km & lt)] = make_int2(w.x, blk);
            j += __popc(km);
            i += cnt;
            __syncwarp();
            if (confl >= 0 && i < nsz) {
                // keep the unscanned tail of the list
                for (int t = 0; t < nsz - i; t += 32) {
                    int2 v = (t + lane < nsz - i) ? C.watches[s + i + t + lane] : make_int2(0, 0);
                    __syncwarp();
                    if (t + lane < nsz - i) C.watches[s + j + t + lane] = v;
                    __syncwarp();
                }
                j += nsz - i;
                i = nsz;
            }
        }
        if (lane == 0) C.wl_size[x] = j;
        __syncwarp();
        // a push fails on one lane, but the rebuild is warp-collective
        if (__any_sync(FULL, overflow)) {
            // a target list was full: share the spare capacity out again and
            // rescan this level
            if (!rebuild_watches(C)) {
                out_of(C, RS_WATCHES);
                return -1;
            }
            // every list a failed move left behind belongs to a literal of the
            // current level, whose scans all start at this level's first entry
            if (confl < 0) C.qhead = (C.dlevel > 0) ? C.tlim[C.dlevel - 1] : 0;
            if (++guard > 64) {
                out_of(C, RS_REBUILD_LOOP);
                return -1;
            }
        }
    }
    return confl;
}

// ---------------------------------------------------------------- analysis
// Activities are >= 0, so their float bits order like ints: atomicMax on the
// bits raises a block bound.
__device__ __forceinline__ void raise_bound(Ctx &C, int32_t v, float a)
{
    if (C.use_bmax) atomicMax(reinterpret_cast<int *>(&C.bmax[v >> 5]), __float_as_int(a));
}

__device__ __forceinline__ void bump(Ctx &C, int32_t v, bool &big)
{
    float a = C.act[v] + C.var_inc;
    C.act[v] = a;
    raise_bound(C, v, a);
    big |= a > 1e30f;
}

__device__ void rescale(Ctx &C)
{
    for (int v = C.lane; v < C.n; v += 32) C.act[v] *= 1e-30f;
    if (C.use_bmax)
        for (int b = C.lane; b < (C.n + 31) / 32; b += 32)
            if (C.bmax[b] >= 0.f) C.bmax[b] *= 1e-30f;
    C.var_inc *= 1e-30f;
    __syncwarp();
}

// First-UIP learning.  Writes the learnt clause to C.learnt[0..len), the
// asserting literal at 0 and a literal of the backjump level at 1.
__device__ void analyze(Ctx &C, int32_t confl, int &out_len, int &bt_level, int &lbd)
{
    const int lane = C.lane;
    const unsigned lt = lanemask_lt();
    int len = 1, pathC = 0, idx = C.tsize - 1;
    int32_t p = -1, c = confl;
    bool big = false;
    for (int guard = 0; guard <= C.tsize + 1; guard++) {
        const int32_t *CL = C.arena + c + HDR;
        const int clen = (int)((uint32_t)C.arena[c] & LEN_MASK);
        const int start = (p == -1) ? 0 : 1;
        for (int b = start; b < clen; b += 32) {
            const int k = b + lane;
            const bool has = k < clen;
            const int32_t q = has ? CL[k] : 0;
            const int32_t v = q >> 1;
            const bool take = has && !C.seen[v] && C.level[v] > 0;
            bool cur = false;
            if (take) {
                C.seen[v] = 1;
                bump(C, v, big);
                if (C.part) atomicAdd(&C.part[v], 1);
                cur = C.level[v] >= C.dlevel;
            }
            pathC += __popc(__ballot_sync(FULL, cur));
            const unsigned lm = __ballot_sync(FULL, take && !cur);
            if (take && !cur) C.learnt[len + __popc(lm & lt)] = q;
            len += __popc(lm);
        }
        __syncwarp();
        if (pathC <= 0) {  // a conflict must involve the current level
            fail_check(C, p == -1 ? CK_NO_CURRENT : CK_UIP);
            break;
        }
        // walk the trail down to the next seen variable
        for (;;) {
            const int k = idx - lane;
            const bool hit = k >= 0 && C.seen[C.trail[k] >> 1];
            const unsigned bm = __ballot_sync(FULL, hit);
            if (bm) {
                idx -= __ffs(bm) - 1;
                break;
            }
            idx -= 32;
            if (idx < 0) break;  // cannot happen while pathC > 0
        }
        if (idx < 0) {
            fail_check(C, CK_UIP);
            break;
        }
        p = C.trail[idx];
        c = C.reason[p >> 1];
        if (lane == 0) C.seen[p >> 1] = 0;
        pathC--;
        idx--;
        __syncwarp();
        if (pathC <= 0) break;
        if (c < 0 || c >= C.arena_top) {  // an implied variable without a usable reason
            fail_check(C, CK_REASON);
            break;
        }
    }
    if (C.check) {
        // leave no seen mark behind for the next job
        for (int v = lane; v < C.n; v += 32) C.seen[v] = 0;
        out_len = 0;
        bt_level = 0;
        lbd = 0;
        __syncwarp();
        return;
    }
    if (lane == 0) C.learnt[0] = p ^ 1;
    if (__any_sync(FULL, big)) rescale(C);
    __syncwarp();
    // basic minimisation: drop a literal whose reason's other literals are all
    // seen or fixed at level 0
    // (decisions first, into tmp; seen marks are cleared only after all of them)
    int keep_n = 1;
    if (C.minimize) {
        for (int k = 1 + lane; k < len; k += 32) {
            const int32_t q = C.learnt[k];
            bool keep = true;
            const int32_t r = C.reason[q >> 1];
            if (r >= 0) {
                const int32_t *RL = C.arena + r + HDR;
                const int rl = (int)((uint32_t)C.arena[r] & LEN_MASK);
                bool red = true;
                for (int t = 1; t < rl && red; t++) {
                    const int32_t v = RL[t] >> 1;
                    red = C.seen[v] || C.level[v] == 0;
                }
                keep = !red;
            }
            C.tmp[k] = keep ? q : -1;
        }
    } else {
        for (int k = 1 + lane; k < len; k += 32) C.tmp[k] = C.learnt[k];
    }
    __syncwarp();
    for (int k = 1 + lane; k < len; k += 32) C.seen[C.learnt[k] >> 1] = 0;
    __syncwarp();
    for (int b = 1; b < len; b += 32) {
        const int k = b + lane;
        const int32_t q = (k < len) ? C.tmp[k] : -1;
        const unsigned km = __ballot_sync(FULL, q >= 0);
        if (q >= 0) C.learnt[keep_n + __popc(km & lt)] = q;
        keep_n += __popc(km);
    }
    __syncwarp();
    len = keep_n;
    // backjump level: highest level among literals 1.., moved to position 1
    int best = -1, bestk = 0;
    for (int k = 1 + lane; k < len; k += 32) {
        const int lv = C.level[C.learnt[k] >> 1];
        if (lv > best) {
            best = lv;
            bestk = k;
        }
    }
    int bl = wmax(best);
    const unsigned bm = __ballot_sync(FULL, best == bl && bl >= 0);
    int kk = __shfl_sync(FULL, bestk, bm ? __ffs(bm) - 1 : 0);
    if (len > 1 && lane == 0 && kk != 1) {
        int32_t t = C.learnt[1];
        C.learnt[1] = C.learnt[kk];
        C.learnt[kk] = t;
    }
    bt_level = len > 1 ? bl : 0;
    __syncwarp();
    // LBD: distinct levels
    C.stamp++;
    int cntl = 0;
    for (int k = lane; k < len; k += 32) {
        const int lv = C.level[C.learnt[k] >> 1];
        if (atomicExch(&C.lstamp[lv], C.stamp) != C.stamp) cntl++;
    }
    lbd = wsum(cntl);
    out_len = len;
    __syncwarp();
}

// ---------------------------------------------------------------- trail
__device__ void backtrack(Ctx &C, int lvl)
{
    if (C.dlevel <= lvl) return;
    const int from = C.tlim[lvl];
    for (int k = from + C.lane; k < C.tsize; k += 32) {
        const int32_t l = C.trail[k];
        C.phase[l >> 1] = (int8_t)(l & 1);
        C.val[l >> 1] = 0;
        raise_bound(C, l >> 1, C.act[l >> 1]);
    }
    C.tsize = from;
    C.qhead = from;
    C.dlevel = lvl;
    __syncwarp();
}

__device__ __forceinline__ void assign_lane0(Ctx &C, int32_t l, int32_t reason, int lvl)
{
    if (C.lane == 0) {
        const int32_t v = l >> 1;
        C.val[v] = (l & 1) ? 1 : -1;
        C.level[v] = lvl;
        C.reason[v] = reason;
        C.trail[C.tsize] = l;
    }
    C.tsize++;
    __syncwarp();
}

// ---------------------------------------------------------------- clause DB
// Moves live clauses down over deleted ones and remaps reasons.
__device__ void collect_garbage(Ctx &C)
{
    const int lane = C.lane;
    int32_t dst = C.orig_top;
    // new reference of every learnt clause (clauses are listed in arena order)
    for (int k = C.n_orig; k < C.n_crefs; k++) {
        const int32_t r = C.crefs[k];
        const int sz = HDR + (int)((uint32_t)C.arena[r] & LEN_MASK);
        for (int t = 0; t < sz; t += 32) {
            const int32_t v = (t + lane < sz) ? C.arena[r + t + lane] : 0;
            __syncwarp();
            if (t + lane < sz) C.arena[dst + t + lane] = v;
            __syncwarp();
        }
        if (lane == 0) C.tmp[k] = dst;
        dst += sz;
    }
    __syncwarp();
    // reasons: binary search of the old reference among crefs
    for (int k = lane; k < C.tsize; k += 32) {
        const int32_t v = C.trail[k] >> 1;
        const int32_t r = C.reason[v];
        if (r >= C.orig_top) {
            int lo = C.n_orig, hi = C.n_crefs - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (C.crefs[mid] < r) lo = mid + 1;
                else hi = mid;
            }
            C.reason[v] = C.tmp[lo];
        }
    }
    __syncwarp();
    for (int k = C.n_orig + lane; k < C.n_crefs; k += 32) C.crefs[k] = C.tmp[k];
    C.arena_top = dst;
    __syncwarp();
}

// Deletes about half of the learnt clauses, highest LBD first, never a
// clause that is the reason of a current assignment or has LBD <= 2.
__device__ void reduce_db(Ctx &C)
{
    const int lane = C.lane;
    const unsigned lt = lanemask_lt();
    int32_t *hist = C.sm64;
    for (int i = lane; i < 64; i += 32) hist[i] = 0;
    __syncwarp();
    const int nlearnt = C.n_crefs - C.n_orig;
    for (int k = C.n_orig + lane; k < C.n_crefs; k += 32) {
        const int32_t r = C.crefs[k];
        const int32_t l0 = C.arena[r + HDR];
        const bool locked = C.reason[l0 >> 1] == r && lval(C, l0) == 1;
        const int lbd = min(C.arena[r + 1], 63);
        C.tmp[k] = locked ? -1 : lbd;
        if (!locked && lbd > 2) atomicAdd(&hist[lbd], 1);
    }
    __syncwarp();
    const int target = nlearnt / 2;
    int thr = 64, above = 0;
    for (int L = 63; L > 2; L--) {
        if (above + hist[L] >= target) {
            thr = L;
            break;
        }
        above += hist[L];
        thr = L;
    }
    int quota = target - above;  // deletions allowed at LBD == thr
    int kept = 0;
    for (int b = C.n_orig; b < C.n_crefs; b += 32) {
        const int k = b + lane;
        int cls = -2;  // -2 none, else lbd or -1 locked
        if (k < C.n_crefs) cls = C.tmp[k];
        const bool over = cls > thr;
        const bool at = cls == thr && cls > 2;
        const unsigned am = __ballot_sync(FULL, at);
        const int rank = __popc(am & lt);
        const bool del = over || (at && rank < quota);
        quota -= min(quota, __popc(am));
        const int32_t r = (k < C.n_crefs) ? C.crefs[k] : 0;
        if (k < C.n_crefs && del) C.arena[r] = (int32_t)((uint32_t)C.arena[r] | F_DELETED);
        const bool keep = k < C.n_crefs && !del;
        const unsigned km = __ballot_sync(FULL, keep);
        __syncwarp();
        if (keep) C.crefs[C.n_orig + kept + __popc(km & lt)] = r;
        kept += __popc(km);
        __syncwarp();
    }
    C.n_crefs = C.n_orig + kept;
    C.reduces++;
    __syncwarp();
}

// Appends the learnt clause; returns its reference or -1 when the slot is full.
__device__ int32_t store_learnt(Ctx &C, int len, int lbd)
{
    if (C.arena_top + HDR + len > C.ACAP || C.n_crefs >= C.CCAP) {
        reduce_db(C);
        collect_garbage(C);
        if (!rebuild_watches(C)) return -1;
        if (C.arena_top + HDR + len > C.ACAP || C.n_crefs >= C.CCAP) return -1;
    }
    const int32_t r = C.arena_top;
    if (C.lane == 0) {
        C.arena[r] = (int32_t)((uint32_t)len | F_LEARNT);
        C.arena[r + 1] = lbd;
        C.crefs[C.n_crefs] = r;
    }
    for (int k = C.lane; k < len; k += 32) C.arena[r + HDR + k] = C.learnt[k];
    C.arena_top += HDR + len;
    C.n_crefs++;
    __syncwarp();
    return r;
}

// ---------------------------------------------------------------- decisions
__device__ int32_t pick_branch(Ctx &C, int mode)
{
    const int lane = C.lane;
    if (mode == DECIDE_LAST_FREE) {
        int best = -1;
        for (int v = lane; v < C.n; v += 32)
            if (C.val[v] == 0) best = v;
        best = wmax(best);
        return best < 0 ? -1 : 2 * best + 1;
    }
    // VSIDS: the unassigned variable of largest activity, lowest index on ties.
    if (!C.use_bmax) {
        // small formulas: one warp scan over every variable
        float ba = -FLT_MAX;
        int bv = -1;
        for (int v = lane; v < C.n; v += 32) {
            if (C.val[v] == 0) {
                const float a = C.act[v];
                if (bv < 0 || a > ba) {
                    ba = a;
                    bv = v;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oa = __shfl_xor_sync(FULL, ba, o);
            const int ov = __shfl_xor_sync(FULL, bv, o);
            if (ov >= 0 && (bv < 0 || oa > ba || (oa == ba && ov < bv))) {
                ba = oa;
                bv = ov;
            }
        }
        return bv < 0 ? -1 : 2 * bv + (C.phase[bv] ? 1 : 0);
    }
    // Large formulas: take the block with the largest bound (lowest block on ties), compute its
    // exact best; if that reaches the bound it beats every other block, else
    // tighten the bound and look again.  Every round either answers or makes one
    // bound exact, so the loop ends; the answer is the full scan's.
    const int nb = (C.n + 31) / 32;
    for (int guard = 0; guard <= 2 * nb + 1; guard++) {
        float bb = -2.f;
        int bi = -1;
        for (int b = lane; b < nb; b += 32) {
            const float x = C.bmax[b];
            if (x > bb) {
                bb = x;
                bi = b;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(FULL, bb, o);
            const int oi = __shfl_xor_sync(FULL, bi, o);
            if (oi >= 0 && (bi < 0 || ob > bb || (ob == bb && oi < bi))) {
                bb = ob;
                bi = oi;
            }
        }
        if (bi < 0 || bb < 0.f) return -1;  // no unassigned variable left
        const int v = 32 * bi + lane;
        const bool free_v = v < C.n && C.val[v] == 0;
        float ba = free_v ? C.act[v] : -1.f;
        int bv = free_v ? v : -1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oa = __shfl_xor_sync(FULL, ba, o);
            const int ov = __shfl_xor_sync(FULL, bv, o);
            if (ov >= 0 && (bv < 0 || oa > ba || (oa == ba && ov < bv))) {
                ba = oa;
                bv = ov;
            }
        }
        __syncwarp();
        if (lane == 0) C.bmax[bi] = bv < 0 ? -1.f : ba;
        __syncwarp();
        if (bv >= 0 && ba >= bb) return 2 * bv + (C.phase[bv] ? 1 : 0);
    }
    return -1;  // not reached: every round tightens a bound
}

__device__ __forceinline__ double luby(double y, int x)
{
    int size = 1, seq = 0;
    while (size < x + 1) {
        seq++;
        size = 2 * size + 1;
    }
    while (size - 1 != x) {
        size = (size - 1) >> 1;
        seq--;
        x = x % size;
    }
    double r = 1.0;
    for (int i = 0; i < seq; i++) r *= y;
    return r;
}

// Whether another job already found a model for the instance.  Another warp
// may set the flag at any time, so lane 0 reads it once for the whole warp:
// the answer guards warp-collective code and must be warp-uniform.
__device__ __forceinline__ bool instance_closed(const Params &P, int inst)
{
    int v = 0;
    if ((threadIdx.x & 31) == 0) v = *(volatile int32_t *)&P.inst_state[inst];
    return __shfl_sync(FULL, v, 0) != 0;
}

// ---------------------------------------------------------------- one job
__device__ int solve_job(const Params &P, Ctx &C, int job, int inst, int64_t *stats)
{
    const int lane = C.lane;
    const Opts &o = P.o;
    const int cb = P.inst_cb[inst], ce = P.inst_ce[inst];
    const int m = ce - cb;
    const int64_t voff = P.var_off[inst];
    C.n = P.inst_nv[inst];
    C.tsize = C.qhead = C.dlevel = 0;
    C.stamp = 0;
    C.var_inc = 1.0f;
    C.resource = false;
    C.minimize = o.minimize;
    C.check = 0;
    C.why = 0;
    C.conflicts = C.decisions = C.props = C.restarts = C.reduces = C.rebuilds = 0;
    C.proof = P.proof ? P.proof + (size_t)job * (size_t)P.proof_cap : nullptr;
    C.plen = 0;
    C.part = (P.part && o.log_participation) ? P.part + voff : nullptr;
    C.occ = (P.part && o.log_participation >= 2) ? P.part + P.var_total + voff : nullptr;
    for (int v = lane; v < C.n; v += 32) {
        C.val[v] = 0;
        C.seen[v] = 0;
        C.act[v] = P.seed_act ? P.seed_act[voff + v] : 0.0f;
        C.phase[v] = P.seed_phase ? P.seed_phase[voff + v] : (int8_t)o.phase_init;
    }
    for (int v = lane; v <= C.n; v += 32) C.lstamp[v] = 0;
    C.use_bmax = C.n > 1024;
    __syncwarp();
    for (int b = lane; C.use_bmax && b < (C.n + 31) / 32; b += 32) {
        float x = 0.f;
        for (int v = 32 * b; v < 32 * b + 32 && v < C.n; v++) x = fmaxf(x, C.act[v]);
        C.bmax[b] = x;
    }
    // copy the clauses into the arena
    const uint32_t base = P.coff[cb];
    const int64_t otop = (int64_t)(P.coff[ce] - base) + (int64_t)HDR * m;
    if (otop > C.ACAP || m > C.CCAP) {
        stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_INIT << 16);
        return R_UNKNOWN;
    }
    for (int c = lane; c < m; c += 32) {
        const uint32_t a = P.coff[cb + c], e = P.coff[cb + c + 1];
        const int32_t pos = (int32_t)(a - base) + HDR * c;
        C.arena[pos] = (int32_t)(e - a);
        C.arena[pos + 1] = 0;
        for (uint32_t t = a; t < e; t++) C.arena[pos + HDR + (int32_t)(t - a)] = P.lits[t];
        C.crefs[c] = pos;
    }
    C.arena_top = C.orig_top = (int32_t)otop;
    C.n_crefs = C.n_orig = m;
    __syncwarp();
    if (o.phase_init == 2 && !P.seed_phase) {
        // first polarity = the sign the variable has in most of its clause
        // occurrences (ties: false); lstamp counts, and is zero again after
        for (uint32_t t = base + lane; t < P.coff[ce]; t += 32) {
            const int32_t l = P.lits[t];
            atomicAdd(&C.lstamp[l >> 1], (l & 1) ? 1 : -1);
        }
        __syncwarp();
        for (int v = lane; v < C.n; v += 32) {
            C.phase[v] = C.lstamp[v] > 0 ? 1 : 0;
            C.lstamp[v] = 0;
        }
        __syncwarp();
    }
    if (!rebuild_watches(C)) {
        stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_INIT << 16);
        return R_UNKNOWN;
    }
    __syncwarp();
    // level-0 facts: unit clauses and the job's cube
    for (int c = 0; c < m; c++) {
        const uint32_t a = P.coff[cb + c], e = P.coff[cb + c + 1];
        if (e - a == 0) return R_UNSAT;
        if (e - a == 1) {
            const int32_t l = P.lits[a];
            // lane 0's reading for everyone: it also orders the reads before lane 0's write
            const int lv = __shfl_sync(FULL, lval(C, l), 0);
            if (lv == -1) return R_UNSAT;
            if (lv == 0) assign_lane0(C, l, -1, 0);
        }
    }
    if (P.job_cube_len) {
        const int32_t *cube = P.cubes + P.job_cube_off[job];
        for (int k = 0; k < P.job_cube_len[job]; k++) {
            const int32_t l = cube[k];
            const int lv = __shfl_sync(FULL, lval(C, l), 0);
            if (lv == -1) return R_UNSAT;
            if (lv == 0) assign_lane0(C, l, -1, 0);
        }
    }
    int64_t max_learnts = max(o.learnt_first, m / 2);
    int64_t restart_limit = o.restart_base;
    int64_t since_restart = 0;
    double geo = o.restart_base;
    int result = R_UNKNOWN;
    const int64_t decide_guard = (int64_t)C.n + 2;
    int64_t dsince = 0;
    while (true) {
        const int32_t confl = propagate(C);
        if (C.resource) {
            stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)C.why << 16);
            result = R_UNKNOWN;
            break;
        }
        if (confl >= 0) {
            C.conflicts++;
            since_restart++;
            dsince = 0;
            if (C.dlevel == 0) {
                result = R_UNSAT;
                break;
            }
            int len, bt, lbd;
            analyze(C, confl, len, bt, lbd);
            if (C.check) {
                stats[ST_FLAGS] |= FL_INTERNAL | ((int64_t)C.check << 8);
                result = R_UNKNOWN;
                break;
            }
            if (C.occ)
                for (int k = lane; k < len; k += 32) atomicAdd(&C.occ[C.learnt[k] >> 1], 1);
            if (C.proof && C.plen >= 0) {
                // the proof log: the learnt clause as derived, before it is stored
                if (C.plen + 1 + len <= P.proof_cap) {
                    if (lane == 0) C.proof[C.plen] = len;
                    for (int k = lane; k < len; k += 32) C.proof[C.plen + 1 + k] = C.learnt[k];
                    C.plen += 1 + len;
                } else {
                    C.plen = -1;
                }
            }
            backtrack(C, bt);
            int32_t r = -1;
            if (len >= 2) {
                r = store_learnt(C, len, lbd);
                if (r < 0) {
                    stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_CLAUSES << 16);
                    result = R_UNKNOWN;
                    break;
                }
                const bool ok = attach_watch(C, C.learnt[0], r, C.learnt[1]) &&
                                attach_watch(C, C.learnt[1], r, C.learnt[0]);
                if (!ok) {
                    // the rebuild also registers the new clause (it is in crefs)
                    if (!rebuild_watches(C)) {
                        stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_WATCHES << 16);
                        result = R_UNKNOWN;
                        break;
                    }
                }
            }
            const bool asserted_free = lval(C, C.learnt[0]) == 0;
            __syncwarp();  // every lane has read the value before lane 0 assigns it
            if (!asserted_free) {  // the asserting literal must be free after the backjump
                fail_check(C, CK_ASSIGNED);
                stats[ST_FLAGS] |= FL_INTERNAL | ((int64_t)C.check << 8);
                result = R_UNKNOWN;
                break;
            }
            assign_lane0(C, C.learnt[0], r, len >= 2 ? bt : 0);
            C.var_inc *= 1.0f / o.var_decay;
            if (C.var_inc > 1e30f) rescale(C);
            if (C.conflicts >= o.conflict_budget) {
                stats[ST_FLAGS] |= FL_BUDGET;
                result = R_UNKNOWN;
                break;
            }
            if (o.check_every > 0 && (C.conflicts % o.check_every) == 0 && instance_closed(P, inst)) {
                stats[ST_FLAGS] |= FL_CANCELLED;
                result = R_UNKNOWN;
                break;
            }
            if (o.restart != RESTART_NONE && since_restart >= restart_limit) {
                backtrack(C, 0);
                C.restarts++;
                since_restart = 0;
                if (o.restart == RESTART_LUBY) {
                    restart_limit = (int64_t)(luby(2.0, (int)C.restarts) * o.restart_base);
                } else {
                    geo *= o.restart_factor;
                    restart_limit = (int64_t)geo;
                }
            }
            if ((C.n_crefs - C.n_orig) - C.tsize >= max_learnts) {
                reduce_db(C);
                max_learnts += o.learnt_inc;
                if (C.arena_top > C.ACAP * 3 / 4) collect_garbage(C);
                if (!rebuild_watches(C)) {
                    stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_WATCHES << 16);
                    result = R_UNKNOWN;
                    break;
                }
            }
        } else {
            if (++dsince > decide_guard) {  // more decisions than variables: impossible
                stats[ST_FLAGS] |= FL_RESOURCE | ((int64_t)RS_DECISIONS << 16);
                result = R_UNKNOWN;
                break;
            }
            const int32_t d = pick_branch(C, o.decide);
            if (d < 0) {
                result = R_SAT;
                break;
            }
            C.decisions++;
            if (lane == 0) C.tlim[C.dlevel] = C.tsize;
            C.dlevel++;
            assign_lane0(C, d, -1, C.dlevel);
        }
    }
    if (C.proof && lane == 0) P.proof_len[job] = C.plen;
    stats[ST_CONFLICTS] = C.conflicts;
    stats[ST_DECISIONS] = C.decisions;
    stats[ST_PROPS] = C.props;
    stats[ST_RESTARTS] = C.restarts;
    stats[ST_LEARNTS] = C.n_crefs - C.n_orig;
    stats[ST_REDUCES] = C.reduces;
    stats[ST_REBUILDS] = C.rebuilds;
    if (C.check) stats[ST_FLAGS] |= FL_INTERNAL | ((int64_t)C.check << 8);
    return result;
}

__device__ __forceinline__ void cdcl_body(const Params &P)
{
    __shared__ int32_t smem[WARPS][64];
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int slot = blockIdx.x * WARPS + wib;
    if (slot >= P.n_slots) return;
    Ctx C;
    C.lane = lane;
    const size_t N = (size_t)P.N, S = (size_t)slot;
    if (P.smem_per_warp > 0) {
        // small formulas: the arrays every propagation, analysis and decision
        // touch at random sit in this warp's part of shared memory
        unsigned char *b = dyn_smem + (size_t)wib * (size_t)P.smem_per_warp;
        auto carve = [&](size_t bytes) {
            unsigned char *q = b;
            b += bytes;
            return q;
        };
        C.level = (int32_t *)carve(4 * N);
        C.reason = (int32_t *)carve(4 * N);
        C.trail = (int32_t *)carve(4 * N);
        C.act = (float *)carve(4 * N);
        C.bmax = nullptr;  // block bounds: formulas above 1024 variables only
        C.tlim = (int32_t *)carve(4 * (N + 4));
        C.learnt = (int32_t *)carve(4 * (N + 4));
        C.lstamp = (int32_t *)carve(4 * (N + 4));
        C.wl_start = (int32_t *)carve(8 * N);
        C.wl_size = (int32_t *)carve(8 * N);
        C.wl_cap = (int32_t *)carve(8 * N);
        C.val = (int8_t *)carve(N);
        C.phase = (int8_t *)carve(N);
        C.seen = (uint8_t *)carve(N);
    } else {
        C.val = P.val + S * N;
        C.phase = P.phase + S * N;
        C.seen = P.seen + S * N;
        C.level = P.level + S * N;
        C.reason = P.reason + S * N;
        C.trail = P.trail + S * N;
        C.tlim = P.tlim + S * (N + 1);
        C.learnt = P.learnt + S * (N + 1);
        C.lstamp = P.lstamp + S * (N + 1);
        C.act = P.act + S * N;
        C.bmax = P.bmax + S * (N / 16);
        C.wl_start = P.wl_start + S * 2 * N;
        C.wl_size = P.wl_size + S * 2 * N;
        C.wl_cap = P.wl_cap + S * 2 * N;
    }
    C.watches = P.watches + S * (size_t)P.WCAP;
    C.arena = P.arena + S * (size_t)P.ACAP;
    C.crefs = P.crefs + S * (size_t)P.CCAP;
    C.tmp = P.tmp + S * (size_t)P.CCAP;
    C.sm64 = smem[wib];
    C.WCAP = P.WCAP;
    C.ACAP = P.ACAP;
    C.CCAP = P.CCAP;
    while (true) {
        int job = 0;
        if (lane == 0) job = (int)atomicAdd(P.next_job, 1u);
        job = __shfl_sync(FULL, job, 0);
        if (job >= P.n_jobs) break;
        job = P.job_order[job];
        const int inst = P.job_inst[job];
        int64_t st[NSTATS];
        for (int i = 0; i < NSTATS; i++) st[i] = 0;
        int res = R_UNKNOWN;
        if (instance_closed(P, inst)) {
            st[ST_FLAGS] |= FL_CANCELLED;
        } else {
            res = solve_job(P, C, job, inst, st);
        }
        if (res == R_SAT) {
            int won = 0;
            if (lane == 0) won = atomicCAS(&P.inst_state[inst], 0, 1) == 0;
            won = __shfl_sync(FULL, won, 0);
            if (won) {
                const int64_t voff = P.var_off[inst];
                for (int v = lane; v < C.n; v += 32) P.model[voff + v] = C.val[v] > 0 ? 1 : -1;
            }
        }
        if (lane == 0) {
            P.job_verdict[job] = res;
            for (int i = 0; i < NSTATS; i++) P.job_stats[(size_t)job * NSTATS + i] = st[i];
        }
        __syncwarp();
    }
}

// Three builds: 4 blocks/SM (128 registers) with the per-variable arrays in
// HBM; in shared memory, 4 blocks/SM when four blocks of them fit (N up to
// about 250) and 3 (about 160 registers) when only three do (N up to about 290).
__global__ void __launch_bounds__(WARPS * 32, 3) cdcl_kernel_smem(Params P) { cdcl_body(P); }
__global__ void __launch_bounds__(WARPS * 32, 4) cdcl_kernel_smem4(Params P) { cdcl_body(P); }
__global__ void __launch_bounds__(WARPS * 32, 4) cdcl_kernel_hbm(Params P) { cdcl_body(P); }

}  // namespace cdcl
}  // namespace gpsat
