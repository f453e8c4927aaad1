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
//   per trail slot (one warp owns one slot; slots are reused across trails)
//     vr[n]     8 bytes per var: dh  uint32 (epoch<<24)|arena index, head of the
//               clauses add_first'ed to the var; asg uint8 (epoch<<1)|sign, trail
//               + pending implications (one load reads both)
//     cst[m]    uint32 (epoch<<24)|(blocked<<22)|(w1<<11)|w2   clauses touched
//     arena[]   32 bytes per entry: {clause, literal offset, length, next} {literals}
//     stack[]   int2 depth-first frames (intervals of the implication list)
//   A slot's epoch (1..127) advances per trail, so nothing is cleared between
//   trails; the slot is wiped once every 127 trails.
//
// Current list of var v = clauses add_first'ed to v (newest first) followed by
// v's initial list, keeping entries whose clause still watches v and is not
// blocked.  A clause never comes back to a var it left (watches only leave
// false literals and nothing is unassigned within one BCP), so that is the
// reference's linked list exactly.
//
// Execution: one warp per trail.  A round gathers up to 32 upcoming watch
// entries -- the rest of the current scan and, while the current scan is a
// trail scan that has implied nothing, the entries of the following trail
// scans -- and evaluates all of them at once against the current state, with
// every random load of the round (clause state, assignments, list heads) in
// one trip.  It then commits them in reference order up to the first event
// that could have changed a later evaluation: an entry whose clause an earlier
// entry of the round already handled, a later scan whose list is not what the
// round assumed (it has clauses add_first'ed to it, possibly by this round),
// the entry just after a conflict, the end of the scan an implication was
// found in (its depth-first descent comes first), or a later entry of that
// scan whose clause has the implied variable.  Events are encoded as ordered
// keys and the cut is one warp min-reduction.  Uncommitted entries are
// evaluated again next round, so the result is the sequential one.
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
constexpr int WARPS = 4;          // warps per block
constexpr int KIN = 4;            // clause literals stored inside a watch entry
constexpr uint32_t EPMAX = 127;   // epochs per slot before a wipe
constexpr int MAXLEN = 2048;      // clause length limit (11-bit watch indices)
constexpr int64_t MAX_ITERS = int64_t(1) << 26;  // per-trail loop iterations before GPSAT_BCP_BUDGET

enum : int { A_NONE = 0, A_SW1 = 1, A_SW2 = 2, A_BLOCK = 3, A_IMPLY = 4, A_CONFLICT = 5 };

// per-variable record of a trail slot
struct VarRec {
    uint32_t dh;       // (epoch<<24)|arena index: head of the clauses add_first'ed to the var
    uint8_t asg;       // (epoch<<1)|sign: trail literal or pending implication
    uint8_t pad[3];
};
static_assert(sizeof(VarRec) == 8 && offsetof(VarRec, asg) == 4, "the assignment byte starts a 4-byte word");

struct Dev {
    int32_t n_vars;
    int32_t n_clauses;
    const int32_t *__restrict__ lits;
    const uint32_t *__restrict__ w0off;
    const int4 *__restrict__ w0ent;   // 2 int4 per entry
    VarRec *vr;
    uint32_t *cst;
    int4 *arena;                      // 2 int4 per entry
    int2 *stack;
    uint32_t *epoch;
    unsigned int *next_trail;
    const int32_t *order;             // trails in processing order (null: index order)
    int64_t n_pad, m_pad, arena_cap, impl_cap;
    int32_t n_slots;
    const int32_t *__restrict__ trail;
    const int64_t *__restrict__ toff;
    int32_t n_trails;
    int32_t *status, *conflict, *stop;
    int64_t *nimpl;
    int32_t *ilit, *ireason;
    int64_t *counters;
};

struct WarpSmem {
    int4 e0[32];
    int4 e1[32];
    int32_t dp_after[32];
    int32_t sc_var[33];
    int32_t sc_begin[33];
    int32_t sc_end[33];
    uint32_t sc_wk[33];
    uint32_t sc_wend[33];
    uint8_t q2j[1024];      // look-ahead buffer: entry stream offset -> buffer position
};

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned lanemask_gt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_gt;" : "=r"(r));
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

// literal l is consistent (unassigned in this epoch, or true) given its var's asg byte
__device__ __forceinline__ bool cons_of(uint8_t a, int32_t l, uint32_t e)
{
    return ((uint32_t)(a >> 1) != e) || ((a & 1) == (l & 1));
}

struct Eval {
    int act;
    int nw1, nw2;       // new watch indices (switch)
    int32_t t1, t2;     // switch target vars
    uint32_t dh1, dh2;  // their list heads as loaded
    int32_t unit;       // unit literal (imply)
    int acnt;           // assignment lookups as the reference counts them
};

// process_clause of the reference for a clause too long for the inline path
// (literals read from the arena).
__device__ __noinline__ void eval_long(const Dev &d, const VarRec *vr, int off, int len,
                                       int w1, int w2, uint32_t e, Eval &r)
{
    const int32_t *L = d.lits + off;
    int32_t l1 = L[w1], l2 = L[w2];
    bool c1 = cons_of(vr[l1 >> 1].asg, l1, e), c2 = cons_of(vr[l2 >> 1].asg, l2, e);
    r.acnt = 2;
    r.act = A_NONE;
    if (c1 && c2) return;
    int pend = (!c1 && !c2) ? 2 : 1, f1 = -1, f2 = -1;
    for (int i = 0; pend > 0 && i < len; i++) {
        if (i == w1 || i == w2) continue;
        int32_t l = L[i];
        r.acnt++;
        if (cons_of(vr[l >> 1].asg, l, e)) {
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
            r.dh1 = vr[r.t1].dh;
            return;
        }
    } else if (f1 >= 0 && f2 >= 0) {
        r.act = A_SW2;
        r.nw1 = f1;
        r.nw2 = f2;
        r.t1 = L[f1] >> 1;
        r.t2 = L[f2] >> 1;
        r.dh1 = vr[r.t1].dh;
        r.dh2 = vr[r.t2].dh;
        return;
    } else if (f1 >= 0) {
        unit = L[f1];
    } else {
        r.act = A_CONFLICT;
        return;
    }
    r.unit = unit;
    r.act = ((uint32_t)(vr[unit >> 1].asg >> 1) != e) ? A_IMPLY : A_BLOCK;
}

// commit-cut keys: (lane position << 7) | (window scan << 1) | after
constexpr int NO_CUT = INT_MAX;
__device__ __forceinline__ int key_before(int pos, int scan) { return (pos << 7) | (scan << 1); }
__device__ __forceinline__ int key_after(int pos, int scan) { return ((pos + 1) << 7) | (scan << 1) | 1; }

__device__ void process_trail(const Dev &d, WarpSmem &sm, int t, int slot, int lane)
{
    VarRec *vr = d.vr + (size_t)slot * d.n_pad;
    uint32_t *cst = d.cst + (size_t)slot * d.m_pad;
    int4 *arena = d.arena + (size_t)slot * d.arena_cap * 2;
    int2 *stk = d.stack + (size_t)slot * d.impl_cap;
    int32_t *ilit = d.ilit + (size_t)t * d.impl_cap;
    int32_t *ireason = d.ireason + (size_t)t * d.impl_cap;
    const int32_t n = d.n_vars;
    const unsigned lt = lanemask_lt();

    // ---- epoch of this slot
    uint32_t e = 0;
    if (lane == 0) e = d.epoch[slot] + 1;
    e = __shfl_sync(FULL, e, 0);
    if (e > EPMAX) {
        uint4 z = make_uint4(0, 0, 0, 0);
        uint4 *v4 = reinterpret_cast<uint4 *>(vr);
        for (int64_t i = lane; i < d.n_pad / 2; i += 32) v4[i] = z;
        uint4 *c4 = reinterpret_cast<uint4 *>(cst);
        for (int64_t i = lane; i < d.m_pad / 4; i += 32) c4[i] = z;
        e = 1;
        __syncwarp();
    }
    if (lane == 0) d.epoch[slot] = e;

    const int64_t tb = d.toff[t];
    const int64_t tn = d.toff[t + 1] - tb;

    // ---- assign every trail literal first, in one pass: an exchange on the
    // word that holds the assignment byte (the rest of the word is padding)
    // returns what was there, and the same variable given the other sign
    // earlier in this trail (by any lane) shows as this epoch's opposite sign
    bool bad = tn < 0;
    // (unrolled so that several iterations' loads are in flight at once)
#pragma unroll 4
    for (int64_t i = lane; i < tn; i += 32) {
        const int32_t x = d.trail[tb + i];
        if (x == 0 || x > n || x < -n) {
            bad = true;
        } else {
            const unsigned a = (e << 1) | (x > 0 ? 1u : 0u);
            const unsigned old = atomicExch(reinterpret_cast<unsigned *>(&vr[(x > 0 ? x : -x) - 1].asg), a) & 0xFFu;
            if ((old >> 1) == e && old != a) bad = true;
        }
    }
    bad = __any_sync(FULL, bad);
    __syncwarp();

    int64_t n_impl = 0, props = 0, cI = 0;
    int64_t myW = 0, myL = 0, myA = 0;  // lane-private, reduced at the end
    int32_t status = bad ? GPSAT_BCP_BAD_TRAIL : GPSAT_BCP_NO_CONFLICT, confl = -1, stopi = -1;
    int64_t arena_used = 0, ti = 0, top_j = 0, top_e = 0, cur_impl_start = 0, cur_trail = -1, dfs_trail = -1;
    int depth = 0;
    bool in_scan = false, cur_counted = false, cur_is_trail = false;
    int32_t cur_var = 0, cur_dp = -1;
    uint32_t cur_wk = 0, cur_wend = 0;
    // look-ahead buffer: lane j holds trail position lb_base + j (its variable
    // and initial watch-list range; positions past the trail: empty).  When
    // fewer than 16 lie ahead it advances by 16 from values loaded one advance
    // earlier: lanes 0-15 of nx_* hold positions lb_base + 32.. (their list
    // ranges in flight) and nnx the trail literals of lb_base + 48.., so an
    // advance waits on no load.
    int64_t lb_base = INT64_MIN / 2;
    int32_t lb_v = 0, nx_v = 0, nnx = 0;
    uint32_t lb_a = 0, lb_b = 0, nx_a = 0, nx_b = 0;
    int lb_p = 0;
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
                    int32_t x = ilit[top_j];
                    top_j++;
                    v = (x > 0 ? x : -x) - 1;
                    cur_is_trail = false;
                    cur_trail = dfs_trail;
                } else {
                    depth--;
                    if (depth > 0) {
                        int2 fr = stk[depth - 1];
                        top_j = fr.x;
                        top_e = fr.y;
                    }
                    continue;
                }
            } else {
                if (ti >= tn) break;
                v = -1;
                const int64_t bo = ti - lb_base;
                if (bo >= 0 && bo < 32) {
                    // the look-ahead buffer holds this position's variable and range
                    v = __shfl_sync(FULL, lb_v, (int)bo);
                    cur_wk = __shfl_sync(FULL, lb_a, (int)bo);
                    cur_wend = __shfl_sync(FULL, lb_b, (int)bo);
                } else {
                    int32_t x = d.trail[tb + ti];
                    v = (x > 0 ? x : -x) - 1;
                }
                cur_trail = ti;
                dfs_trail = ti;
                ti++;
                cur_is_trail = true;
                if (bo < 0 || bo >= 32) {
                    cur_wk = d.w0off[v];
                    cur_wend = d.w0off[v + 1];
                }
            }
            uint32_t h = vr[v].dh;
            cur_var = v;
            cur_dp = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
            if (!cur_is_trail) {
                cur_wk = d.w0off[v];
                cur_wend = d.w0off[v + 1];
            }
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
            // scan finished.  One that implied nothing and is followed by trail
            // scans leads straight to them: this round's window is those alone
            // (as look-ahead scans, set up from the look-ahead buffer with their
            // list heads loaded in the round's own trip), not a separate setup
            const bool next_trail_scans = then_trail && n_impl == cur_impl_start && ti < tn;
            if (!next_trail_scans) {
                // descend into the implications it found
                in_scan = false;
                if (n_impl > cur_impl_start) {
                    if (depth > 0 && lane == 0) stk[depth - 1] = make_int2((int)top_j, (int)top_e);
                    top_j = cur_impl_start;
                    top_e = n_impl;
                    depth++;
                }
                continue;
            }
        }

        // ---- gather the window
        int ndyn = 0;
        bool dyn_done = true;
        if (cur_dp >= 0) {
            if (lane == 0) {
                int32_t p = cur_dp;
                while (p >= 0 && ndyn < 32) {
                    const int4 a = arena[2 * p];
                    sm.e0[ndyn] = a;
                    sm.e1[ndyn] = arena[2 * p + 1];
                    p = a.w;
                    sm.dp_after[ndyn] = p;
                    ndyn++;
                }
                dyn_done = p < 0;
            }
            ndyn = __shfl_sync(FULL, ndyn, 0);
            dyn_done = __shfl_sync(FULL, dyn_done, 0);
        }
        // Window position p is evaluated by lane p.  Entries from the initial
        // lists are loaded straight into that lane's registers (g*: the
        // current scan, h*: the look-ahead scans), so the loads of both kinds
        // are in flight together and nothing waits on them before the
        // evaluation; only the added-list entries go through shared memory.
        int nent = ndyn;
        int take0 = 0;
        int4 g0 = make_int4(0, 0, 0, 0), g1 = g0, h0 = g0, h1 = g0;
        if (dyn_done) {
            take0 = min(32 - nent, (int)(cur_wend - cur_wk));
            if (lane >= nent && lane < nent + take0) {
                const size_t w = cur_wk + (uint32_t)(lane - nent);
                g0 = d.w0ent[2 * w];
                g1 = d.w0ent[2 * w + 1];
            }
            nent += take0;
        }
        const int nent0 = nent;
        if (lane == 0) {
            sm.sc_var[0] = cur_var;
            sm.sc_begin[0] = 0;
            sm.sc_end[0] = nent;
        }
        int nsc = 1;
        int my_scan = 0;
        const bool scan0_full = dyn_done && (cur_wk + (uint32_t)take0 == cur_wend);
        if (scan0_full && then_trail && n_impl == cur_impl_start && nent < 32 && ti < tn) {
            // following trail scans, assumed to start with an empty added list
            // (checked in the evaluation trip)
            const int room = 32 - nent;
            if (ti - lb_base >= 16 && lb_base + 32 < tn) {
                const int64_t old_base = lb_base;
                if (ti - lb_base >= 32) {
                    // (re)fill at ti: the buffer now, the next 16 and the
                    // trail literals of the 16 after them in flight
                    lb_base = ti;
                    lb_v = 0;
                    lb_a = lb_b = 0;
                    if (ti + lane < tn) {
                        const int32_t x = d.trail[tb + ti + lane];
                        lb_v = (x > 0 ? x : -x) - 1;
                        lb_a = d.w0off[lb_v];
                        lb_b = d.w0off[lb_v + 1];
                    }
                    nx_v = 0;
                    nx_a = nx_b = 0;
                    if (lane < 16 && ti + 32 + lane < tn) {
                        const int32_t x = d.trail[tb + ti + 32 + lane];
                        nx_v = (x > 0 ? x : -x) - 1;
                        nx_a = d.w0off[nx_v];
                        nx_b = d.w0off[nx_v + 1];
                    }
                } else {
                    // advance by 16: lanes 0-15 take lanes 16-31, lanes 16-31
                    // the next 16 (loaded one advance ago)
                    lb_base += 16;
                    const int sl = (lane + 16) & 31;
                    const int32_t hv = __shfl_sync(FULL, lb_v, sl), qv = __shfl_sync(FULL, nx_v, sl);
                    const uint32_t ha = __shfl_sync(FULL, lb_a, sl), qa = __shfl_sync(FULL, nx_a, sl);
                    const uint32_t hb = __shfl_sync(FULL, lb_b, sl), qb = __shfl_sync(FULL, nx_b, sl);
                    lb_v = lane < 16 ? hv : qv;
                    lb_a = lane < 16 ? ha : qa;
                    lb_b = lane < 16 ? hb : qb;
                    nx_v = 0;
                    nx_a = nx_b = 0;
                    if (lane < 16 && lb_base + 32 + lane < tn) {
                        nx_v = (nnx > 0 ? nnx : -nnx) - 1;
                        nx_a = d.w0off[nx_v];
                        nx_b = d.w0off[nx_v + 1];
                    }
                }
                nnx = 0;
                if (lane < 16 && lb_base + 48 + lane < tn) nnx = d.trail[tb + lb_base + 48 + lane];
                // warm L2 with the initial watch entries of the positions that
                // entered the buffer (a line holds four): the rounds of the
                // next trail scans gather them
                if (lb_base + lane >= old_base + 32) {
                    const uint32_t ne = lb_b - lb_a < 32u ? lb_b - lb_a : 32u;
                    for (uint32_t q = 0; q < ne; q += 4)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(d.w0ent + 2 * (size_t)(lb_a + q)));
                }
                // the buffer's entry stream, laid out once per refill: position
                // j's (up to 32) entries follow position j-1's; lb_p is the
                // inclusive prefix of the counts and q2j maps a stream offset
                // back to its buffer position
                const int c = (int)(lb_b - lb_a < 32u ? lb_b - lb_a : 32u);
                int pc = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL, pc, o);
                    if (lane >= o) pc += y;
                }
                lb_p = pc;
                for (int q = pc - c; q < pc; q++) sm.q2j[q] = (uint8_t)lane;
                __syncwarp();
            }
            const int lb_off = (int)(ti - lb_base);
            const int64_t ahead = (32 - lb_off < tn - ti) ? (int64_t)(32 - lb_off) : tn - ti;
            const int nlook = (int)(ahead < 31 ? ahead : 31);
            const int src = (lb_off + lane) & 31;
            const int32_t bv = __shfl_sync(FULL, lb_v, src);
            const uint32_t ba = __shfl_sync(FULL, lb_a, src), bb = __shfl_sync(FULL, lb_b, src);
            const int bp = __shfl_sync(FULL, lb_p, src);
            // stream offset of the window's first look-ahead entry
            const int pbase = lb_off > 0 ? __shfl_sync(FULL, lb_p, (lb_off - 1) & 31) : 0;
            int32_t v = -1;
            uint32_t a = 0, b = 0;
            if (lane < nlook) {
                v = bv;
                a = ba;
                b = bb;
            }
            const int cnt = (lane < nlook) ? (int)(b - a < 32u ? b - a : 32u) : 0;
            const int incl = bp - pbase;  // (lanes below nlook)
            const int excl = incl - cnt;
            const unsigned ok = __ballot_sync(FULL, lane < nlook && excl < room);
            const int K = (~ok) ? __ffs(~ok) - 1 : 32;
            if (lane < K) {
                sm.sc_var[1 + lane] = v;
                sm.sc_begin[1 + lane] = nent + excl;
                sm.sc_end[1 + lane] = min(nent + excl + cnt, 32);
                sm.sc_wk[1 + lane] = a;
                sm.sc_wend[1 + lane] = b;
            }
            if (K > 0) {
                const int total = min(nent + __shfl_sync(FULL, incl, K - 1), 32);
                // window position -> look-ahead scan, through the stream map
                if (lane >= nent && lane < total) my_scan = 1 + (int)sm.q2j[pbase + lane - nent] - lb_off;
                const int jj = my_scan - 1;
                const int ej = __shfl_sync(FULL, excl, jj < 0 ? 0 : jj);
                const uint32_t aj = __shfl_sync(FULL, a, jj < 0 ? 0 : jj);
                if (lane >= nent && lane < total) {
                    const size_t w = aj + (uint32_t)(lane - nent - ej);
                    h0 = d.w0ent[2 * w];
                    h1 = d.w0ent[2 * w + 1];
                }
                nent = total;
                nsc = 1 + K;
            }
        }
        __syncwarp();

        // ---- evaluate every entry of the window at once
        const bool has = lane < nent;
        const int4 en = lane < ndyn ? sm.e0[lane] : (lane < nent0 ? g0 : h0);
        const int4 el = lane < ndyn ? sm.e1[lane] : (lane < nent0 ? g1 : h1);
        const int32_t sv = sm.sc_var[my_scan];
        // lane s (1 <= s < nsc) checks whether window scan s starts with added clauses
        const int32_t scan_v = (lane >= 1 && lane < nsc) ? sm.sc_var[lane] : -1;
        const int32_t scan_b = (lane >= 1 && lane < nsc) ? sm.sc_begin[lane] : 0;
        Eval r;
        r.act = A_NONE;
        r.acnt = 0;
        r.t1 = r.t2 = -1;
        r.dh1 = r.dh2 = 0;
        r.unit = -1;
        r.nw1 = r.nw2 = 0;
        bool valid = false;
        int32_t ov = -1;  // a valid entry's clause: its other watched variable
        int w1 = 0, w2 = 0;
        uint32_t scan_h = 0;
        if (has) {
            const uint32_t st = cst[en.x];
            const int len = en.z;
            const int32_t Lr[KIN] = {el.x, el.y, el.z, el.w};
            uint8_t Av[KIN];
            uint32_t Dh[KIN];
            // every random load of the round in one trip: clause state, the
            // literals' assignments and list heads (unused ones are cheap misses)
#pragma unroll
            for (int i = 0; i < KIN; i++) {
                // one 8-byte load per literal: list head and assignment byte
                const uint2 rv = (i < len) ? *reinterpret_cast<const uint2 *>(&vr[Lr[i] >> 1]) : make_uint2(0, 0);
                Av[i] = (uint8_t)(rv.y & 0xFFu);
                Dh[i] = rv.x;
            }
            if (scan_v >= 0) scan_h = vr[scan_v].dh;
            bool blk;
            if ((st >> 24) == e) {
                blk = (st >> 22) & 1u;
                w1 = (st >> 11) & 0x7FFu;
                w2 = st & 0x7FFu;
            } else {
                blk = false;
                w1 = (uint32_t)en.w >> 16;
                w2 = en.w & 0xFFFF;
            }
            if (len <= KIN) {
                int32_t l1 = 0, l2 = 0;
                bool c1 = false, c2 = false;
#pragma unroll
                for (int i = 0; i < KIN; i++) {
                    if (i == w1) {
                        l1 = Lr[i];
                        c1 = cons_of(Av[i], Lr[i], e);
                    }
                    if (i == w2) {
                        l2 = Lr[i];
                        c2 = cons_of(Av[i], Lr[i], e);
                    }
                }
                valid = !blk && ((l1 >> 1) == sv || (l2 >> 1) == sv);
                if (valid) ov = ((l1 >> 1) == sv) ? (l2 >> 1) : (l1 >> 1);
                if (valid) {
                    r.acnt = 2;
                    if (!(c1 && c2)) {
                        int pend = (!c1 && !c2) ? 2 : 1, f1 = -1, f2 = -1;
                        int32_t lf1 = 0, lf2 = 0;
                        uint32_t df1 = 0, df2 = 0;
                        uint8_t af1 = 0;
#pragma unroll
                        for (int i = 0; i < KIN; i++) {
                            if (i < len && pend > 0 && i != w1 && i != w2) {
                                r.acnt++;
                                if (cons_of(Av[i], Lr[i], e)) {
                                    if (f1 < 0) {
                                        f1 = i;
                                        lf1 = Lr[i];
                                        df1 = Dh[i];
                                        af1 = Av[i];
                                    } else {
                                        f2 = i;
                                        lf2 = Lr[i];
                                        df2 = Dh[i];
                                    }
                                    pend--;
                                }
                            }
                        }
                        int32_t unit = -1;
                        uint8_t au = 0;
                        if (c1 || c2) {
                            if (f1 < 0) {
                                unit = c1 ? l1 : l2;
#pragma unroll
                                for (int i = 0; i < KIN; i++)
                                    if (i == (c1 ? w1 : w2)) au = Av[i];
                            } else {
                                r.act = A_SW1;
                                r.nw1 = c1 ? w1 : f1;
                                r.nw2 = c1 ? f1 : w2;
                                r.t1 = lf1 >> 1;
                                r.dh1 = df1;
                            }
                        } else if (f1 >= 0 && f2 >= 0) {
                            r.act = A_SW2;
                            r.nw1 = f1;
                            r.nw2 = f2;
                            r.t1 = lf1 >> 1;
                            r.t2 = lf2 >> 1;
                            r.dh1 = df1;
                            r.dh2 = df2;
                        } else if (f1 >= 0) {
                            unit = lf1;
                            au = af1;
                        } else {
                            r.act = A_CONFLICT;
                        }
                        if (unit >= 0) {
                            r.unit = unit;
                            r.act = ((uint32_t)(au >> 1) != e) ? A_IMPLY : A_BLOCK;
                        }
                    }
                }
            } else {
                const int32_t l1 = d.lits[en.y + w1], l2 = d.lits[en.y + w2];
                valid = !blk && ((l1 >> 1) == sv || (l2 >> 1) == sv);
                if (valid) ov = ((l1 >> 1) == sv) ? (l2 >> 1) : (l1 >> 1);
                if (valid) eval_long(d, vr, en.y, len, w1, w2, e, r);
            }
        } else if (scan_v >= 0) {
            scan_h = vr[scan_v].dh;
        }

        // ---- where the commit stops: the smallest event key of the round
        int key = NO_CUT;
        {
            // an entry whose clause an earlier entry of the round also holds
            // (and may change).  A clause is listed once per variable and only
            // a valid entry acts, so that is a valid entry whose clause's other
            // watched variable is an earlier window scan's (scan 0: checked
            // here; later scans: in the loop below).  Scan 0 may have entries
            // from earlier rounds, so this can cut where nothing repeats: a
            // cut only ends the round early.
            if (valid && my_scan > 0 && ov == cur_var) key = key_before(lane, my_scan);
            if (valid && r.act == A_CONFLICT) key = min(key, key_after(lane, my_scan));
            // an implication ends its scan's part of the window (its depth-first
            // descent comes before any later scan) ...
            const bool imp = valid && r.act == A_IMPLY;
            if (imp) key = min(key, key_after(sm.sc_end[my_scan] - 1, my_scan));
            // ... and a later entry of the same scan is evaluated again if its
            // clause has the implied variable (a long clause: always); the
            // other entries read nothing the implication changed
            unsigned im = __ballot_sync(FULL, imp);
            while (im) {
                const int k = __ffs(im) - 1;
                im &= im - 1;
                const int32_t uv = __shfl_sync(FULL, r.unit >> 1, k);
                const int ks = __shfl_sync(FULL, my_scan, k);
                if (valid && lane > k && my_scan == ks) {
                    const bool dep = en.z > KIN || (el.x >> 1) == uv || (en.z > 1 && (el.y >> 1) == uv) ||
                                     (en.z > 2 && (el.z >> 1) == uv) || (en.z > 3 && (el.w >> 1) == uv);
                    if (dep) key = min(key, key_before(lane, my_scan));
                }
            }
            // a later window scan whose list starts with added clauses
            if (scan_v >= 0 && (scan_h >> 24) == e) key = min(key, key_before(scan_b, lane));
            // a move of this lane that lands in a later window scan's list, and
            // the repeated clauses of scans 1.. (lane s holds window scan s's
            // variable and start; the loop is uniform, so its shuffles are
            // independent and overlap, and the smallest key is the first scan)
            const bool mv = valid && (r.act == A_SW1 || r.act == A_SW2);
            if (nsc > 1) {
                for (int s = 1; s < nsc; s++) {
                    const int32_t vs = __shfl_sync(FULL, scan_v, s);
                    const int bs = __shfl_sync(FULL, scan_b, s);
                    if (mv && s > my_scan && (vs == r.t1 || vs == r.t2)) key = min(key, key_before(bs, s));
                    if (valid && s < my_scan && vs == ov) key = min(key, key_before(lane, my_scan));
                }
            }
        }
        const int cut = __reduce_min_sync(FULL, key);
        int k_end, new_cur;
        bool new_started;
        if (cut == NO_CUT) {
            k_end = nent;
            new_cur = nsc - 1;
            new_started = (new_cur == 0) || (sm.sc_end[new_cur] > sm.sc_begin[new_cur]);
        } else {
            k_end = cut >> 7;
            new_cur = (cut >> 1) & 63;
            new_started = (cut & 1) || new_cur == 0 || k_end > sm.sc_begin[new_cur];
        }

        // more implications than impl_cap leaves room for: commit up to the
        // first one that does not fit; the next round reports the overflow there
        {
            const unsigned im0 = __ballot_sync(FULL, valid && lane < k_end && r.act == A_IMPLY);
            const int64_t room = d.impl_cap - n_impl;
            if (room > 0 && __popc(im0) > room) {
                const int kk = nth_set_bit(im0, (int)room + 1);
                const int ks = __shfl_sync(FULL, my_scan, kk);
                k_end = kk;
                new_cur = ks;
                new_started = ks == 0 || kk > sm.sc_begin[ks];
            }
        }
        const bool com = valid && lane < k_end;
        // watch moves: add_first into the target var's list, in commit order
        const bool ins1 = com && (r.act == A_SW1 || r.act == A_SW2);
        const bool ins2 = com && r.act == A_SW2;
        const unsigned m1 = __ballot_sync(FULL, ins1), m2 = __ballot_sync(FULL, ins2);
        const int total_ins = __popc(m1) + __popc(m2);
        if (arena_used + total_ins > d.arena_cap) {
            const int ks = __shfl_sync(FULL, my_scan, __ffs(m1) - 1);
            status = GPSAT_BCP_OVERFLOW;
            stopi = (int32_t)(ks == 0 ? cur_trail : ti + ks - 1);
            break;
        }
        const unsigned imask = __ballot_sync(FULL, com && r.act == A_IMPLY);
        if (imask && n_impl >= d.impl_cap) {
            // stop index: the trail literal whose propagation overflowed
            const int ks = __shfl_sync(FULL, my_scan, __ffs(imask) - 1);
            status = GPSAT_BCP_OVERFLOW;
            stopi = (int32_t)(ks == 0 ? cur_trail : ti + ks - 1);
            break;
        }
        if (m2 == 0) {
            const int myidx = (int)arena_used + __popc(m1 & lt);
            const unsigned g = __match_any_sync(FULL, ins1 ? r.t1 : -1 - lane);
            if (ins1) {
                const unsigned before = g & lt;
                int32_t next;
                if (before) {
                    const int pl = 31 - __clz(before);
                    next = (int)arena_used + __popc(m1 & ((1u << pl) - 1u));
                } else {
                    next = ((r.dh1 >> 24) == e) ? (int32_t)(r.dh1 & 0xFFFFFFu) : -1;
                }
                arena[2 * myidx] = make_int4(en.x, en.y, en.z, next);
                arena[2 * myidx + 1] = el;
                if ((g & lanemask_gt()) == 0) vr[r.t1].dh = (e << 24) | (uint32_t)myidx;
            }
        } else {
            // rare (a clause moving both watches needs 4+ literals): lane 0
            // inserts every move serially, in commit order
            int idx = (int)arena_used;
            unsigned rem = m1;
            while (rem) {
                const int k = __ffs(rem) - 1;
                rem &= rem - 1;
                const int32_t c = __shfl_sync(FULL, en.x, k), off = __shfl_sync(FULL, en.y, k),
                              len = __shfl_sync(FULL, en.z, k);
                const int4 lk = make_int4(__shfl_sync(FULL, el.x, k), __shfl_sync(FULL, el.y, k),
                                          __shfl_sync(FULL, el.z, k), __shfl_sync(FULL, el.w, k));
                const int32_t tt1 = __shfl_sync(FULL, r.t1, k), tt2 = __shfl_sync(FULL, r.t2, k);
                const bool two = (m2 >> k) & 1u;
                if (lane == 0) {
                    uint32_t h = vr[tt1].dh;
                    int32_t next = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
                    arena[2 * idx] = make_int4(c, off, len, next);
                    arena[2 * idx + 1] = lk;
                    vr[tt1].dh = (e << 24) | (uint32_t)idx;
                    if (two) {
                        h = vr[tt2].dh;
                        next = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
                        arena[2 * (idx + 1)] = make_int4(c, off, len, next);
                        arena[2 * (idx + 1) + 1] = lk;
                        vr[tt2].dh = (e << 24) | (uint32_t)(idx + 1);
                    }
                }
                idx += two ? 2 : 1;
            }
        }
        arena_used += total_ins;

        // clause states
        if (com && r.act != A_NONE) {
            uint32_t ns;
            if (r.act == A_SW1 || r.act == A_SW2) ns = (e << 24) | ((uint32_t)r.nw1 << 11) | (uint32_t)r.nw2;
            else ns = (e << 24) | (1u << 22) | ((uint32_t)w1 << 11) | (uint32_t)w2;
            cst[en.x] = ns;
        }
        // implications, in commit order (all of one scan, on distinct variables)
        if (imask) {
            if ((imask >> lane) & 1u) {
                const int64_t at = n_impl + __popc(imask & lt);
                ilit[at] = dimacs_of(r.unit);
                ireason[at] = en.x;
                vr[r.unit >> 1].asg = (uint8_t)((e << 1) | (uint32_t)(r.unit & 1));
            }
            n_impl += __popc(imask);
            cI += __popc(imask);
        }
        const unsigned cmask = __ballot_sync(FULL, com && r.act == A_CONFLICT);
        if (com) {
            myW++;
            myL += en.z;
            myA += r.acnt;
        }
        const int64_t ti_round = ti;
        __syncwarp();

        // ---- advance the scan cursors
        if (new_cur == 0) {
            if (k_end > 0) {
                if (k_end <= ndyn) {
                    cur_dp = sm.dp_after[k_end - 1];
                } else {
                    cur_dp = -1;
                    cur_wk += (uint32_t)(k_end - ndyn);
                }
            }
        } else {
            props += new_cur - 1;
            cur_var = sm.sc_var[new_cur];
            cur_dp = -1;
            if (!new_started) {
                // cut before this scan because its list starts with added
                // clauses (possibly added by this round): those come first
                const uint32_t h = vr[cur_var].dh;
                cur_dp = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
            }
            cur_wk = sm.sc_wk[new_cur] + (uint32_t)(k_end - sm.sc_begin[new_cur]);
            cur_wend = sm.sc_wend[new_cur];
            cur_counted = new_started;
            if (new_started) props++;
            cur_trail = ti + new_cur - 1;
            dfs_trail = cur_trail;
            ti += new_cur;
            cur_is_trail = true;
            depth = 0;  // a descent whose scan led into trail scans has ended
            cur_impl_start = n_impl - __popc(imask);
        }
        if (cmask) {
            const int k = __ffs(cmask) - 1;
            confl = __shfl_sync(FULL, en.x, k);
            const int ks = __shfl_sync(FULL, my_scan, k);
            stopi = (int32_t)(ks == 0 ? (new_cur == 0 ? cur_trail : dfs_trail) : ti_round + ks - 1);
            status = GPSAT_BCP_CONFLICT;
        }
        __syncwarp();
    }

    myW = warp_sum(myW);
    myL = warp_sum(myL);
    myA = warp_sum(myA);
    if (lane == 0) {
        d.status[t] = status;
        d.conflict[t] = confl;
        d.stop[t] = stopi;
        d.nimpl[t] = n_impl;
        if (d.counters) {
            int64_t *cn = d.counters + (size_t)t * GPSAT_BCP_NCOUNTERS;
            cn[0] = props;
            cn[1] = myW;
            cn[2] = myL;
            cn[3] = myA;
            cn[4] = cI;
            cn[5] = bad ? 0 : tn;
        }
    }
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

// blocks per SM the register allocation targets: 4 (16 resident warps per SM)
// leaves the kernel its ~100 registers without spills, which measured faster
// than 32 resident warps with spills at 64 registers
#ifndef GPSAT_BCP_MIN_BLOCKS
#define GPSAT_BCP_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(WARPS * 32, GPSAT_BCP_MIN_BLOCKS) bcp_kernel(Dev d)
{
    __shared__ WarpSmem smem[WARPS];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int slot = blockIdx.x * WARPS + wib;
    if (slot >= d.n_slots) return;
    while (true) {
        int t = 0;
        if (lane == 0) t = (int)atomicAdd(d.next_trail, 1u);
        t = __shfl_sync(FULL, t, 0);
        if (t >= d.n_trails) break;
        process_trail(d, smem[wib], d.order ? d.order[t] : t, slot, lane);
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
    int64_t n_pad = 0, m_pad = 0, arena_cap = 0, impl_cap = 0;
    bcp::VarRec *vr = nullptr;
    uint32_t *cst = nullptr, *epoch = nullptr;
    int4 *arena = nullptr;
    int2 *stack = nullptr;
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
    cudaFree(b->vr);
    cudaFree(b->cst);
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
    d.vr = b->vr;
    d.cst = b->cst;
    d.arena = b->arena;
    d.stack = b->stack;
    d.epoch = b->epoch;
    d.next_trail = b->counter;
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
    const int blocks = (d.n_slots + bcp::WARPS - 1) / bcp::WARPS;
    bcp::bcp_kernel<<<blocks, bcp::WARPS * 32, 0, st>>>(d);
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcp::bcp_kernel, bcp::WARPS * 32, 0);
    int32_t resident = std::max(1, sms * std::max(per_sm, 1) * bcp::WARPS);
    gpsat_bcp *b = new gpsat_bcp();
    b->f = f;
    b->device = f->device;
    b->n_pad = ((int64_t)f->h.n_vars + 15) / 16 * 16;
    b->m_pad = (f->h.n_clauses() + 3) / 4 * 4;
    b->impl_cap = impl_cap;
    b->arena_cap = arena_cap ? arena_cap : (1 << 17);
    const int64_t per_slot = b->n_pad * 8 + b->m_pad * 4 + b->arena_cap * 32 + b->impl_cap * 8;
    int32_t slots = max_slots ? max_slots : resident;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const int64_t budget = (int64_t)(free_b * 0.6);
    if ((int64_t)slots * per_slot > budget) slots = (int32_t)std::max<int64_t>(1, budget / per_slot);
    b->slots = slots;
    const size_t S = (size_t)slots;
    bool ok = cudaMalloc(&b->vr, S * b->n_pad * 8) == cudaSuccess &&
              cudaMalloc(&b->cst, S * b->m_pad * 4) == cudaSuccess &&
              cudaMalloc(&b->epoch, S * 4) == cudaSuccess &&
              cudaMalloc(&b->arena, S * b->arena_cap * 32) == cudaSuccess &&
              cudaMalloc(&b->stack, S * b->impl_cap * 8) == cudaSuccess &&
              cudaMalloc(&b->counter, 16) == cudaSuccess;
    if (ok)
        ok = cudaMemset(b->vr, 0, S * b->n_pad * 8) == cudaSuccess &&
             cudaMemset(b->cst, 0, S * b->m_pad * 4) == cudaSuccess && cudaMemset(b->epoch, 0, S * 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bcp_free(b);
        delete b;
        return set_error(GPSAT_ERR_NOMEM, "gpsat_bcp_create: device allocation failed");
    }
    b->bytes = (int64_t)S * per_slot;
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
//   [launch counter | epoch per slot | variable records | cst | move arena | stack]
// each part 256-byte aligned.  Everything but the arena and the stack (which
// the kernel writes before it reads) is cleared on the stream per call.  One
// array per device, so calls whose GPU work overlaps race on it.
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
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcp::bcp_kernel, bcp::WARPS * 32, 0);
        if (err != cudaSuccess) return cuda_error(err, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        s.base[device] = static_cast<unsigned char *>(ptr);
        s.resident[device] = std::max(1, sms * std::max(per_sm, 1) * bcp::WARPS);
        s.ready[device] = true;
    }
    *base = s.base[device];
    *resident = s.resident[device];
    return GPSAT_OK;
}

// Bytes of the scratch layout for S slots (each part rounded up to 256).
int64_t static_layout_bytes(int64_t S, int64_t n_pad, int64_t m_pad, int64_t arena_cap, int64_t impl_cap)
{
    return STATIC_ALIGN + align_up(S * 4) + align_up(S * n_pad * 8) + align_up(S * m_pad * 4) +
           align_up(S * arena_cap * 32) + align_up(S * impl_cap * 8);
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
    // switch devices only when needed: a caller capturing this call into a
    // graph keeps its device current
    int cur_dev = -1;
    cudaError_t err = cudaGetDevice(&cur_dev);
    if (err == cudaSuccess && cur_dev != f->device) err = cudaSetDevice(f->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
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
    const int64_t per_slot = 4 + n_pad * 8 + m_pad * 4 + acap * 32 + impl_cap * 8;
    S = std::min<int64_t>(S, std::max<int64_t>(1, (limit - 7 * STATIC_ALIGN) / per_slot));
    while (S > 1 && static_layout_bytes(S, n_pad, m_pad, acap, impl_cap) > limit) S--;

    unsigned char *p = base;
    auto take = [&](int64_t bytes) {
        unsigned char *q = p;
        p += align_up(bytes);
        return q;
    };
    unsigned int *counter = reinterpret_cast<unsigned int *>(take(STATIC_ALIGN));
    uint32_t *epoch = reinterpret_cast<uint32_t *>(take(S * 4));
    bcp::VarRec *vr = reinterpret_cast<bcp::VarRec *>(take(S * n_pad * 8));
    uint32_t *cst = reinterpret_cast<uint32_t *>(take(S * m_pad * 4));
    int4 *arena = reinterpret_cast<int4 *>(take(S * acap * 32));
    int2 *stack = reinterpret_cast<int2 *>(take(S * impl_cap * 8));

    cudaStream_t st = (cudaStream_t)stream;
    // what the kernel expects to find zero: the launch counter, the slots'
    // epochs and their epoch-tagged state (a previous call may have used
    // another formula with another layout)
    err = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(epoch, 0, (size_t)S * 4, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(vr, 0, (size_t)(S * n_pad * 8), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(cst, 0, (size_t)(S * m_pad * 4), st);
    if (err != cudaSuccess) return cuda_error(err, "gpsat_bcp_run_static: clearing the static scratch");
    if (n_trails == 0) return GPSAT_OK;

    bcp::Dev d;
    d.n_vars = f->h.n_vars;
    d.n_clauses = (int32_t)f->h.n_clauses();
    d.lits = f->d_lits;
    d.w0off = f->d_w0off;
    d.w0ent = reinterpret_cast<const int4 *>(f->d_w0ent);
    d.vr = vr;
    d.cst = cst;
    d.arena = arena;
    d.stack = stack;
    d.epoch = epoch;
    d.next_trail = counter;
    d.order = nullptr;
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
    const int blocks = (int)((S + bcp::WARPS - 1) / bcp::WARPS);
    bcp::bcp_kernel<<<blocks, bcp::WARPS * 32, 0, st>>>(d);
    err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_error(err, "bcp kernel launch (static scratch)");
    return GPSAT_OK;
}
