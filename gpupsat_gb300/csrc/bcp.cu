// Host side of the two-watched-literal BCP batch (C ABI) and the kernels
// around it: the shortest-first processing order and the full-scan clause
// evaluation strategy.  The reference-order BCP kernel itself is in
// bcp_window.cuh (built at three window widths).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstddef>
#include <cstdio>
#include <mutex>

#include "bcp_common.cuh"

namespace gpsat {
namespace bcp {

extern const Variant variant_w2, variant_w4, variant_w8;

const Variant *variant(int warps)
{
    switch (warps) {
    case 2: return &variant_w2;
    case 4: return &variant_w4;
    case 8: return &variant_w8;
    default: return nullptr;
    }
}

// ---------------------------------------------------------------------------
// Processing order.  A launch lasts as long as its slowest trail, and when
// there are more trails than resident blocks the last ones start only as
// others finish, so the long-running trails should start first.  The trails
// that propagate longest are those that reach their fixpoint without a
// conflict: a trail that assigns fewer variables is the more likely to, but
// it also has fewer literals to propagate, so the longest ones assign a
// middling number.  The order therefore takes the trails whose length is
// nearest a pivot first (pivot 0: shortest first), and the pivot is tuned on
// the caller's trails (BCPBatch.tune).  (Outputs do not depend on the order.
// At the 4096-trail benchmark shape, the measured per-trail durations of one
// launch give an 18.5 ms list schedule shortest first and 15.0-15.4 ms with
// the pivot at the 25th-30th percentile of the lengths.)  A counting sort on
// |length - pivot| / 16.
constexpr int ORDER_BUCKETS = 4096;

__device__ __forceinline__ int order_bucket(const int64_t *toff, int t, int64_t pivot)
{
    int64_t len = toff[t + 1] - toff[t];
    if (len < 0) len = 0;
    const int64_t dist = len >= pivot ? len - pivot : pivot - len;
    return (int)(dist >> 4 < ORDER_BUCKETS - 1 ? dist >> 4 : ORDER_BUCKETS - 1);
}

__global__ void order_count(const int64_t *toff, int T, int64_t pivot, unsigned *hist)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
        atomicAdd(&hist[order_bucket(toff, t, pivot)], 1u);
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

__global__ void order_scatter(const int64_t *toff, int T, int64_t pivot, unsigned *hist, int32_t *order)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
        order[atomicAdd(&hist[order_bucket(toff, t, pivot)], 1u)] = t;
}

// ---------------------------------------------------------------------------
// Trail application ahead of the BCP kernel.  The reference assigns every
// trail literal before it propagates any (SATSolver/VariablesStateHandler.cu
// :35-59), so the assignment words of all the launch's trails can be built
// at once, in parallel over the whole GPU, instead of by each trail's block
// (one dependent global atomic per literal) before its rounds start.  A block
// builds one trail's words at a time in shared memory, a chunk of variables
// per pass over the trail's literals, and writes every word of the chunk out
// (so the words need no clearing between launches: each launch writes them
// all).  A literal out of range, or a variable given both signs, marks the
// trail bad (the BCP kernel then reports GPSAT_BCP_BAD_TRAIL for it).
constexpr int APPLY_NT = 1024;
constexpr int APPLY_CHUNK_WORDS = 32768;   // 128 KB: 524,288 variables per pass
constexpr int64_t APPLY_MAX_BYTES = int64_t(8) << 30;   // above this the blocks assign their own trails

// trails [t_begin, t_end) of the launch
__global__ void __launch_bounds__(APPLY_NT) apply_kernel(const int32_t *__restrict__ trail,
                                                        const int64_t *__restrict__ toff, int32_t t_begin,
                                                        int32_t t_end, int32_t n, int64_t n_words,
                                                        uint32_t *__restrict__ tasg, int32_t *__restrict__ tbad)
{
    extern __shared__ uint32_t chunk[];   // APPLY_CHUNK_WORDS words
    __shared__ int s_bad;
    for (int t = t_begin + blockIdx.x; t < t_end; t += gridDim.x) {
        const int64_t tb = toff[t], tn = toff[t + 1] - tb;
        uint32_t *out = tasg + (size_t)t * n_words;
        if (threadIdx.x == 0) s_bad = tn < 0;
        for (int64_t w0 = 0; w0 < n_words; w0 += APPLY_CHUNK_WORDS) {
            const int cw = (int)(n_words - w0 < APPLY_CHUNK_WORDS ? n_words - w0 : APPLY_CHUNK_WORDS);
            for (int i = threadIdx.x; i < cw; i += APPLY_NT) chunk[i] = 0u;
            __syncthreads();
            const int64_t v_lo = w0 * 16, v_hi = (w0 + cw) * 16;
            bool bad = false;
#pragma unroll 4
            for (int64_t i = threadIdx.x; i < tn; i += APPLY_NT) {
                const int32_t x = trail[tb + i];
                if (x == 0 || x > n || x < -n) {
                    bad = true;
                    continue;
                }
                const int32_t v = (x > 0 ? x : -x) - 1;
                if (v < v_lo || v >= v_hi) continue;
                const int sh = (v & 15) << 1;
                const uint32_t bits = (x > 0 ? 3u : 1u) << sh;
                const uint32_t old = atomicOr(&chunk[(v >> 4) - w0], bits);
                if (((old >> sh) & 1u) && (((old ^ bits) >> sh) & 2u)) bad = true;
            }
            if (bad) s_bad = 1;   // every writer writes 1
            __syncthreads();
            for (int i = threadIdx.x; i < cw; i += APPLY_NT) out[w0 + i] = chunk[i];
            __syncthreads();   // the chunk is read out before the next pass clears it
        }
        if (threadIdx.x == 0) tbad[t] = s_bad;
        __syncthreads();       // s_bad is read before the next trail resets it
    }
}

// the 128 KB of dynamic shared memory needs the opt-in, once per device
cudaError_t apply_allow()
{
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, APPLY_CHUNK_WORDS * 4);
    if (e == cudaSuccess) done.fetch_or(bit);
    return e;
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
    int64_t pivot = 0;                 // processing order: trail lengths nearest this first
    int32_t strategy = GPSAT_BCP_WATCHED;
    int32_t warps = bcp::DEFAULT_WARPS;    // window width of the two-watched-literal kernel / 32
    int32_t resident[bcp::MAX_WARPS + 1] = {};   // per width: blocks the GPU keeps resident
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
    // trails applied ahead of the BCP kernel (apply_kernel)
    uint32_t *tasg = nullptr;
    int32_t *tbad = nullptr;
    int64_t tasg_cap = 0, tbad_cap = 0;   // words, trails
    int32_t apply_blocks = 0;             // resident blocks of apply_kernel (0: not looked up yet)
    // page-locked host trails: copied in parts on copy_stream, each part
    // applied on the launch stream as soon as it has arrived
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t part_done[4] = {};
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
    cudaFree(b->tasg);
    cudaFree(b->tbad);
    for (cudaEvent_t e : b->part_done)
        if (e) cudaEventDestroy(e);
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
}

// Room for n_trails trails' assignment words (tasg) and bad-trail flags
// (tbad), built by apply_kernel ahead of the BCP kernel and grown on demand;
// false when they would take more than APPLY_MAX_BYTES or cannot be
// allocated, and the BCP kernel's blocks then assign their own trails.
bool apply_prepare(gpsat_bcp *b, int32_t n_trails)
{
    const int64_t words = (int64_t)n_trails * b->n_words;
    if (n_trails <= 0 || words * 4 > bcp::APPLY_MAX_BYTES) return false;
    if (words > b->tasg_cap) {
        cudaFree(b->tasg);
        b->tasg = nullptr;
        b->tasg_cap = 0;
        if (cudaMalloc(&b->tasg, (size_t)words * 4) != cudaSuccess) {
            cudaGetLastError();
            b->tasg = nullptr;
            return false;
        }
        b->tasg_cap = words;
    }
    if (n_trails > b->tbad_cap) {
        cudaFree(b->tbad);
        b->tbad = nullptr;
        b->tbad_cap = 0;
        if (cudaMalloc(&b->tbad, (size_t)n_trails * 4) != cudaSuccess) {
            cudaGetLastError();
            b->tbad = nullptr;
            return false;
        }
        b->tbad_cap = n_trails;
    }
    if (bcp::apply_allow() != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (b->apply_blocks == 0) {
        int per_sm = 0, sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bcp::apply_kernel, bcp::APPLY_NT,
                                                          bcp::APPLY_CHUNK_WORDS * 4) != cudaSuccess)
            cudaGetLastError();
        b->apply_blocks = std::max(1, sms * std::max(per_sm, 1));
    }
    return true;
}

// apply_kernel over trails [t0, t1) on stream st (after apply_prepare)
bool apply_range(gpsat_bcp *b, const int32_t *trail, const int64_t *toff, int32_t t0, int32_t t1, cudaStream_t st)
{
    if (t1 <= t0) return true;
    const int grid = std::min<int32_t>(t1 - t0, b->apply_blocks);
    bcp::apply_kernel<<<grid, bcp::APPLY_NT, bcp::APPLY_CHUNK_WORDS * 4, st>>>(trail, toff, t0, t1, b->f->h.n_vars,
                                                                               b->n_words, b->tasg, b->tbad);
    return cudaGetLastError() == cudaSuccess;
}

bool apply_trails(gpsat_bcp *b, const int32_t *trail, const int64_t *toff, int32_t n_trails, cudaStream_t st)
{
    return apply_prepare(b, n_trails) && apply_range(b, trail, toff, 0, n_trails, st);
}

// applied: the caller already ran apply_kernel over every trail into b->tasg
int launch(gpsat_bcp *b, const int32_t *trail, const int64_t *toff, int32_t n_trails, int32_t *status,
           int32_t *conflict, int32_t *stop, int64_t *nimpl, int32_t *ilit, int32_t *ireason, int64_t *counters,
           cudaStream_t st, bool applied = false)
{
    const gpsat_formula *f = b->f;
    bcp::Dev d{};
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
    // trails in flight: the chosen kernel's resident blocks, at most the
    // workspace's slots, the caller's active setting and the trails
    const bool scan = b->strategy == GPSAT_BCP_FULL_SCAN;
    const bool scan_smem = b->n_words <= bcp::SCAN_SMEM_WORDS;
    int32_t cap = scan ? (scan_smem ? b->scan_resident : std::min(b->scan_resident, b->slots))
                       : std::min(b->resident[b->warps], b->slots);
    if (b->active > 0) cap = std::min(cap, b->active);
    d.n_slots = std::min<int32_t>(cap, std::max<int32_t>(n_trails, 1));
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
        // more trails than blocks in flight: shortest first (see order_count)
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
        bcp::order_count<<<g, 256, 0, st>>>(toff, n_trails, b->pivot, b->hist);
        bcp::order_scan<<<1, 1024, 0, st>>>(b->hist);
        bcp::order_scatter<<<g, 256, 0, st>>>(toff, n_trails, b->pivot, b->hist, b->order);
        d.order = b->order;
    }
    if (scan) {
        // one block per trail; the assignment bits in shared memory when they fit
        if (scan_smem)
            bcp::scan_kernel<true><<<d.n_slots, bcp::SCAN_NT, (size_t)b->n_words * 4, st>>>(d, f->d_coff);
        else
            bcp::scan_kernel<false><<<d.n_slots, bcp::SCAN_NT, 0, st>>>(d, f->d_coff);
        err = cudaGetLastError();
    } else {
        if (applied || apply_trails(b, trail, toff, n_trails, st)) {
            d.tasg = b->tasg;
            d.tbad = b->tbad;
        }
        err = bcp::variant(b->warps)->launch(d, d.n_slots, st);
    }
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
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, f->device);
    gpsat_bcp *b = new gpsat_bcp();
    // slots for the widest residency among the window widths built
    int32_t resident = 1;
    for (int w = bcp::MIN_WARPS; w <= bcp::MAX_WARPS; w *= 2) {
        int per_sm = 0;
        if (bcp::variant(w)->occupancy(&per_sm) != cudaSuccess) cudaGetLastError();
        b->resident[w] = std::max(1, sms * std::max(per_sm, 1));
        resident = std::max(resident, b->resident[w]);
    }
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
    // the slots, plus the per-trail assignment words and staging buffers the
    // runs so far have grown
    if (device_bytes)
        *device_bytes = b->bytes + b->tasg_cap * 4 + b->tbad_cap * 4 + b->trail_cap * 4 + b->toff_cap * 8 + b->out_cap;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_set_active_slots(gpsat_bcp *b, int32_t n)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null handle");
    if (n < 0 || n > b->slots) return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_active_slots: n outside 0..slots");
    b->active = n;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_set_order_pivot(gpsat_bcp *b, int64_t pivot)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_order_pivot: null handle");
    if (pivot < 0) return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_order_pivot: negative pivot");
    b->pivot = pivot;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_set_window(gpsat_bcp *b, int32_t entries)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null handle");
    if (entries % 32 || !bcp::variant(entries / 32))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_set_window: window of 64, 128 or 256 entries");
    b->warps = entries / 32;
    return GPSAT_OK;
}

extern "C" int gpsat_bcp_window_slots(const gpsat_bcp *b, int32_t entries, int32_t *slots)
{
    if (!b || !slots) return set_error(GPSAT_ERR_ARG, "null argument");
    if (entries % 32 || !bcp::variant(entries / 32))
        return set_error(GPSAT_ERR_ARG, "gpsat_bcp_window_slots: window of 64, 128 or 256 entries");
    *slots = std::min(b->resident[entries / 32], b->slots);
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

namespace {
// The handle's trail staging buffers, grown to nl literals and n_trails trails.
int stage_alloc(gpsat_bcp *b, int64_t nl, int32_t n_trails)
{
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
    return GPSAT_OK;
}

// The trails copied into the handle's staging buffers (grown on demand) on
// stream st: device memory that apply_kernel can pass over more than once.
int stage_trails(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets, int32_t n_trails,
                 cudaStream_t st)
{
    const int64_t nl = trail_offsets[n_trails];
    const int rc = stage_alloc(b, nl, n_trails);
    if (rc != GPSAT_OK) return rc;
    if (nl > 0 && cudaMemcpyAsync(b->d_trail, trail_lits, nl * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "trail copy");
    if (cudaMemcpyAsync(b->d_toff, trail_offsets, (int64_t)(n_trails + 1) * 8, cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
        return cuda_error(cudaGetLastError(), "offset copy");
    return GPSAT_OK;
}
// Page-locked host trails: copied to the staging buffers in parts on the
// handle's copy stream, each part's trails applied (apply_kernel) on the
// legacy stream as soon as the part has arrived, so the copy of one part
// overlaps the application of the one before.  False (nothing enqueued that
// matters: the caller copies and applies as usual) when a stream, an event or
// the per-trail words cannot be had.
bool copy_and_apply(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets, int32_t n_trails)
{
    constexpr int P = 4;
    if (!apply_prepare(b, n_trails)) return false;
    if (!b->copy_stream) {
        if (cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            b->copy_stream = nullptr;
            return false;
        }
        for (cudaEvent_t &e : b->part_done)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                e = nullptr;
            }
    }
    for (cudaEvent_t e : b->part_done)
        if (!e) return false;
    cudaStream_t cs = b->copy_stream;
    // the legacy stream's earlier work (a previous run's readers of the
    // staging buffers) is done before the copies start: run_host synchronises
    bool ok = cudaMemcpyAsync(b->d_toff, trail_offsets, (int64_t)(n_trails + 1) * 8, cudaMemcpyHostToDevice, cs) ==
              cudaSuccess;
    for (int k = 0; ok && k < P; k++) {
        const int32_t t0 = (int32_t)((int64_t)n_trails * k / P), t1 = (int32_t)((int64_t)n_trails * (k + 1) / P);
        const int64_t a = trail_offsets[t0], e = trail_offsets[t1];
        ok = (e <= a ||
              cudaMemcpyAsync(b->d_trail + a, trail_lits + a, (e - a) * 4, cudaMemcpyHostToDevice, cs) ==
                  cudaSuccess) &&
             cudaEventRecord(b->part_done[k], cs) == cudaSuccess &&
             cudaStreamWaitEvent(0, b->part_done[k], 0) == cudaSuccess &&
             apply_range(b, b->d_trail, b->d_toff, t0, t1, 0);
    }
    if (!ok) {
        // the caller stages the trails again into the same buffers: no copy
        // of this pass may still be in flight
        cudaGetLastError();
        cudaStreamSynchronize(cs);
        cudaGetLastError();
    }
    return ok;
}
}  // namespace

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
    // every trail inside the nl literals that are copied in
    if (trail_offsets[0] < 0) return set_error(GPSAT_ERR_ARG, "trail offsets must be >= 0");
    for (int32_t t = 0; t < n_trails; t++)
        if (trail_offsets[t + 1] < trail_offsets[t])
            return set_error(GPSAT_ERR_ARG, "trail offsets must be non-decreasing");
    {
        // Every buffer page-locked (cudaHostAlloc / cudaHostRegister, as
        // torch's pin_memory): the trails are copied to the device by DMA
        // (the trail-application kernel passes over them more than once) and
        // the kernel writes the results in place, over the CPU-GPU link, with
        // no staging copies.
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
            int rc = stage_alloc(b, nl, n_trails);
            if (rc != GPSAT_OK) return rc;
            const bool applied = b->strategy == GPSAT_BCP_WATCHED && copy_and_apply(b, trail_lits, trail_offsets, n_trails);
            if (!applied) {
                rc = stage_trails(b, trail_lits, trail_offsets, n_trails, 0);
                if (rc != GPSAT_OK) return rc;
            }
            rc = launch(b, b->d_trail, b->d_toff, n_trails, (int32_t *)dp[2], (int32_t *)dp[3], (int32_t *)dp[4],
                        (int64_t *)dp[5], (int32_t *)dp[6], (int32_t *)dp[7], counters ? (int64_t *)dp[8] : nullptr, 0,
                        applied);
            // also waits for the parts copied on the copy stream (the legacy
            // stream waited for each), so no copy from the caller's buffers
            // is left in flight even when the launch failed
            err = cudaStreamSynchronize(0);
            if (rc != GPSAT_OK) return rc;
            if (err != cudaSuccess) return cuda_error(err, "bcp run");
            return GPSAT_OK;
        }
    }
    int rc = stage_trails(b, trail_lits, trail_offsets, n_trails, 0);
    if (rc != GPSAT_OK) return rc;
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
    rc = launch(b, b->d_trail, b->d_toff, n_trails, d_status, d_confl, d_stop, d_nimpl, d_ilit, d_ireason,
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
        err = bcp::variant(bcp::DEFAULT_WARPS)->occupancy(&per_sm);
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

    bcp::Dev d{};
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
    err = bcp::variant(bcp::DEFAULT_WARPS)->launch(d, (int)S, st);
    if (err != cudaSuccess) return cuda_error(err, "bcp kernel launch (static scratch)");
    return GPSAT_OK;
}
