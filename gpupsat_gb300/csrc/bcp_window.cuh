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
//
// This header is compiled once per window width by bcp_w2.cu, bcp_w4.cu and
// bcp_w8.cu, each defining GPSAT_BCP_WARPS, GPSAT_BCP_MIN_BLOCKS and the
// namespace GPSAT_BCP_NS of its build.
#pragma once

#include "bcp_common.cuh"

namespace gpsat {
namespace bcp {
namespace GPSAT_BCP_NS {

// The window width of this build: GPSAT_BCP_WARPS warps per block, one
// window entry per thread.
constexpr int NW = GPSAT_BCP_WARPS;   // warps per block: one trail per block
constexpr int NT = NW * 32;
constexpr int W = NT;                 // window entries: one per thread
static_assert(NW >= 2 && W <= 256 && LB >= LEAD + CHUNK, "layout limits");

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
    int32_t confl_c[2], confl_scan[2];   // by round parity (see the round's end)
    unsigned long long red[NW][3];
    int t;
    // look-ahead ring: trail position q lives in slot q % LB
    int32_t lb_var[LB];
    uint32_t lb_a[LB], lb_b[LB], lb_h[LB];
};

// block-wide minimum; every thread gets it
__device__ __forceinline__ int block_min(Smem &sm, int v)
{
    v = __reduce_min_sync(FULL, v);
    if ((threadIdx.x & 31) == 0) atomicMin(&sm.key_min, v);
    __syncthreads();
    return sm.key_min;
}

// one 32-byte list entry in one 256-bit load (entries are 32-byte aligned:
// the formula's and each slot's arrays start on 256-byte boundaries); the
// formula's entries through the non-coherent path
__device__ __forceinline__ void ld_entry(const int4 *p, int4 &a, int4 &b)
{
    asm volatile("ld.global.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
                 : "l"(p));
}
__device__ __forceinline__ void ld_entry_nc(const int4 *p, int4 &a, int4 &b)
{
    asm volatile("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
                 : "l"(p));
}

__device__ void process_trail(const Dev &d, Smem &sm, const int t, const int slot)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const bool pre = d.tasg != nullptr;   // the trail was assigned by apply_kernel
    uint32_t *asg = pre ? d.tasg + (size_t)t * d.n_words : d.asg + (size_t)slot * d.n_words;
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
    bool bad = tn < 0 || (pre && d.tbad[t] != 0);
#pragma unroll 4
    for (int64_t i = pre ? tn : tid; i < tn; i += NT) {
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
    int par = 0;   // round parity: the slot of this round's conflict record

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
            sm.confl_c[par] = -1;
        }
        int ndyn = 0;
        bool dyn_done = true;
        if (cur_dp >= 0) {
            if (tid == 0) {
                int32_t p = cur_dp;
                int k = 0;
                while (p >= 0 && k < W) {
                    int4 a, a2;
                    ld_entry(arena + 2 * p, a, a2);
                    sm.dyn0[k] = a;
                    sm.dyn1[k] = a2;
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
                    ld_entry_nc(d.w0ent + 2 * w, en, el);
                }
            } else {
                my_scan = sm.pos_scan[tid];
                const int q = tid - sm.sc_b[my_scan];
                const int32_t head = sm.sc_head[my_scan];
                if (head >= 0 && q == 0) {
                    ld_entry(arena + 2 * head, en, el);
                    sm.sc_next[my_scan] = en.w;
                } else {
                    const size_t w = sm.sc_wk[my_scan] + (uint32_t)(q - (head >= 0 ? 1 : 0));
                    ld_entry_nc(d.w0ent + 2 * w, en, el);
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
            // (no barrier here: the counts are written again only after the
            // commit barrier of this round, or after the barrier that
            // precedes the second call below)
        };
        // the round's moves into the move-target table before the ranking
        // barrier, which publishes both.  Moves into the same variable within
        // the round (rare) are linked by thread 0 in window order; otherwise
        // every mover links its own entry.  (If the implication limit below
        // shortens the commit, the entries it drops may leave false
        // collisions: they only send the round to the serial path.)
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
            for (int i = tid; i < 2 * W; i += NT) sm.mh[i] = -1;   // clean for the next trail
            status = GPSAT_BCP_OVERFLOW;
            stopi = (int32_t)(ks == 0 ? cur_trail : ti + ks - 1);
            break;
        }

        // ---- commit
        // (the move-target table and the movers' records were published by
        // the ranking barrier)
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
            sm.confl_c[par] = en.x;
            sm.confl_scan[par] = my_scan;
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
        // empty the move-target table for the next round (every probe of
        // this round came before the collision barrier; the next round's
        // inserts come after this round's last barrier)
        for (int i = tid; i < 2 * W; i += NT) sm.mh[i] = -1;
        arena_used += tot_mv;
        n_impl += tot_im;
        cI += tot_im;

        // ---- advance the scan cursors (from window state that no thread
        // writes before the next round's layout)
        bool reload = false;
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
                // assumed (possibly changed by this round): read it again once
                // this round's list-head writes are in
                reload = true;
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
        // The round's one closing barrier: this round's commits (list heads,
        // clause states, ring, conflict record) are in before anyone reads
        // them, and every read of this round's window state is done before
        // the next layout rewrites it.  The conflict record alternates
        // between two slots, so the next layout's reset of its own slot cannot
        // race with a late read of this one.
        __syncthreads();
        if (reload) {
            const uint32_t h = dh[cur_var];
            cur_dp = ((h >> 24) == e) ? (int32_t)(h & 0xFFFFFFu) : -1;
        }
        const int32_t cc = sm.confl_c[par];
        if (cc >= 0) {
            const int ks = sm.confl_scan[par];
            confl = cc;
            stopi = (int32_t)(ks == 0 ? (new_cur == 0 ? cur_trail : dfs_trail) : ti_round + ks - 1);
            status = GPSAT_BCP_CONFLICT;
        }
        par ^= 1;
    }

    // ---- clear the assignment words this trail set (trail and implications);
    // a trail's own words (apply_kernel) are cleared for the next launch by
    // the host instead
    for (int64_t i = pre ? tn : tid; i < tn; i += NT) {
        const int32_t x = d.trail[tb + i];
        if (x != 0 && x <= n && x >= -n) asg[((x > 0 ? x : -x) - 1) >> 4] = 0u;
    }
    for (int64_t i = pre ? n_impl : tid; i < n_impl; i += NT) asg[(impl[i] >> 1) >> 4] = 0u;

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

// blocks per SM the register allocation targets (set by the build unit)
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

inline cudaError_t launch(const Dev &d, int blocks, cudaStream_t st)
{
    bcp_kernel<<<blocks, NT, 0, st>>>(d);
    return cudaGetLastError();
}

inline cudaError_t occupancy(int *per_sm)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, bcp_kernel, NT, 0);
}

}  // namespace GPSAT_BCP_NS
}  // namespace bcp
}  // namespace gpsat
