// Host side of the device CDCL solver: formula batches, jobs (whole
// instances or cubes), the persistent solve launch captured in a CUDA graph,
// model assembly and the device model checker; plus the independent host
// model checker.
//
// Reference counterparts (paths inside the reference project, src/):
//   SATSolver/main.cu:217-310 + Parallelizer.cu:133-228  the parallel path: cube jobs in a
//       queue, one solver per thread, relaunch loop -> one persistent launch per batch,
//       one solver per warp, jobs from a global counter
//   SATSolver/JobsQueue.cu:10-32                         JobsQueue::next_job -> atomicAdd in
//       the kernel's job loop
//   SATSolver/Results.cu:106-155                         model assembly; its "verified"
//       check ignores signs, so both checkers here are new code
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "cdcl.cuh"
#include "internal.h"

namespace gpsat {
namespace cdcl {
__global__ void cdcl_kernel_smem(Params P);
__global__ void cdcl_kernel_smem4(Params P);
__global__ void cdcl_kernel_hbm(Params P);
}
// which build of the solver kernel a workspace runs
enum : int { K_HBM = 0, K_SMEM3 = 1, K_SMEM4 = 2 };

namespace {

constexpr unsigned FULL = 0xffffffffu;

// One warp per formula: every original clause must hold a true literal.
__global__ void check_models_kernel(const int32_t *lits, const uint32_t *coff, const int32_t *cb, const int32_t *ce,
                                    const int64_t *var_off, const int8_t *model, const int32_t *verdict,
                                    int32_t n_formulas, int32_t *ok)
{
    const int lane = threadIdx.x & 31;
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (f >= n_formulas) return;
    if (verdict[f] != GPSAT_SAT) {
        if (lane == 0) ok[f] = -1;
        return;
    }
    const int8_t *mdl = model + var_off[f];
    bool bad = false;
    for (int c = cb[f] + lane; c < ce[f]; c += 32) {
        bool sat = false;
        for (uint32_t k = coff[c]; k < coff[c + 1] && !sat; k++) {
            const int32_t l = lits[k];
            const int8_t v = mdl[l >> 1];
            sat = (l & 1) ? v > 0 : v < 0;
        }
        bad |= !sat;
    }
    bad = __any_sync(FULL, bad);
    if (lane == 0) ok[f] = bad ? 0 : 1;
}

void pad_model(int8_t *m, int32_t n)
{
    for (int32_t v = 0; v < n; v++)
        if (m[v] == 0) m[v] = 1;
}

}  // namespace
}  // namespace gpsat

using namespace gpsat;

struct gpsat_batch {
    int device = 0;
    int32_t n_formulas = 0;
    std::vector<HostFormula> prep;        // preprocessed formulas
    std::vector<int32_t> n_vars;
    std::vector<int64_t> var_off;         // n_formulas + 1
    std::vector<int32_t> olits;           // original clauses, internal encoding
    std::vector<uint32_t> ocoff;
    std::vector<int32_t> ocb, oce;
    // device, preprocessed
    int32_t *d_lits = nullptr, *d_cb = nullptr, *d_ce = nullptr, *d_nv = nullptr;
    uint32_t *d_coff = nullptr;
    int64_t *d_var_off = nullptr;
    // device, original (model checking)
    int32_t *d_olits = nullptr, *d_ocb = nullptr, *d_oce = nullptr;
    uint32_t *d_ocoff = nullptr;
    // per-formula device outputs
    int8_t *d_model = nullptr;
    int32_t *d_state = nullptr, *d_verdict = nullptr, *d_ok = nullptr, *d_part = nullptr;
    int64_t part_cap = 0;
    float *d_seed_act = nullptr;
    int8_t *d_seed_phase = nullptr;
    // jobs
    int32_t *d_job_inst = nullptr, *d_job_cube_off = nullptr, *d_job_cube_len = nullptr, *d_cubes = nullptr;
    int32_t *d_job_order = nullptr;
    int32_t *d_job_verdict = nullptr;
    int64_t *d_job_stats = nullptr;
    int64_t job_cap = 0, cube_cap = 0;
    // proof logs of the last solve (proof_words > 0): per job, and the
    // caller's job index -> internal job (-1: no job, preprocessing decided it)
    int32_t *d_proof = nullptr;
    int64_t *d_proof_len = nullptr;
    int64_t proof_words = 0, proof_bytes = 0, proof_len_cap = 0;
    std::vector<int32_t> caller_job, job_verdict;
    unsigned int *d_counter = nullptr;
    // workspace
    cdcl::Params P{};
    int64_t ws_bytes = 0;
    int32_t ws_slots = 0, ws_N = 0, kind = gpsat::K_SMEM3;  // build of the solver kernel
    int64_t ws_W = 0, ws_A = 0, ws_C = 0;
    void *ws = nullptr;
    int max_len = 0, max_m = 0;
    int64_t max_words = 0;
};

namespace {

template <class T>
bool dalloc(T **p, size_t n)
{
    return cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T)) == cudaSuccess;
}
template <class T>
bool dup(T **p, const std::vector<T> &v)
{
    if (!dalloc(p, v.size())) return false;
    return v.empty() || cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

void batch_free(gpsat_batch *b)
{
    void *ptrs[] = {b->d_lits, b->d_cb, b->d_ce, b->d_nv, b->d_coff, b->d_var_off, b->d_olits, b->d_ocb,
                    b->d_oce, b->d_ocoff, b->d_model, b->d_state, b->d_verdict, b->d_ok, b->d_part,
                    b->d_seed_act, b->d_seed_phase, b->d_job_inst, b->d_job_cube_off, b->d_job_cube_len,
                    b->d_cubes, b->d_job_verdict, b->d_job_stats, b->d_counter, b->ws, b->d_proof,
                    b->d_proof_len, b->d_job_order};
    for (void *p : ptrs) cudaFree(p);
}

// Workspace sized for the largest formula of the batch and a launch of J jobs.
int ensure_workspace(gpsat_batch *b, const gpsat_solve_options *o, int32_t J)
{
    // (a multiple of 4: the shared-memory arrays stay 16-byte aligned)
    const int32_t N = (int32_t)((*std::max_element(b->n_vars.begin(), b->n_vars.end()) + 3) / 4 * 4);
    const int64_t lfirst = std::max<int64_t>(o->learnt_first, b->max_m / 2);
    const int64_t C = b->max_m + 3 * lfirst + 4 * (int64_t)o->learnt_inc + N + 64;
    // a multiple of 4 words: every slot's arena starts 16-byte aligned (the
    // replacement-watch search reads clause literals four at a time)
    const int64_t A = (b->max_words + (C - b->max_m) * 48 + 3) / 4 * 4;
    const int64_t W = 3 * C + 8 * (int64_t)N + 256;
    int sms = 0, per_sm = 0, smem_max = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    // Three builds of the kernel: with the per-variable arrays in shared
    // memory, 4 blocks/SM when four blocks of them fit and 3 when three do (no
    // fewer resident blocks than each build's registers allow); else 4
    // blocks/SM with the arrays in HBM.  The 4-block build leaves L1 little
    // room beside four blocks' shared memory, so it is the first choice only
    // for a launch with more jobs than three blocks per SM hold.
    int32_t smem_warp = (int32_t)cdcl::smem_bytes_per_warp(N);
    int kind = K_HBM;
    if (4 * (int64_t)smem_warp + 1024 > smem_max) smem_warp = 0;
    if (smem_warp > 0) {
        const bool many = (int64_t)J > (int64_t)sms * 3 * 4;
        const int order[2] = {many ? K_SMEM4 : K_SMEM3, many ? K_SMEM3 : K_SMEM4};
        for (int k : order) {
            const void *fn = k == K_SMEM4 ? (const void *)cdcl::cdcl_kernel_smem4 : (const void *)cdcl::cdcl_kernel_smem;
            int by_regs = 0, with_smem = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&by_regs, fn, 128, 0) == cudaSuccess &&
                cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * smem_warp) == cudaSuccess &&
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&with_smem, fn, 128, 4 * smem_warp) == cudaSuccess &&
                with_smem >= by_regs && by_regs >= (k == K_SMEM4 ? 4 : 3)) {
                kind = k;
                per_sm = by_regs;  // (shared memory allows at least as many)
                break;
            }
            cudaGetLastError();
        }
        if (kind == K_HBM) smem_warp = 0;
    }
    if (kind == K_HBM) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cdcl::cdcl_kernel_hbm, 128, 0);
    int32_t slots = o->max_slots > 0 ? o->max_slots : std::max(1, sms * std::max(per_sm, 1) * 4);
    // per-variable arrays in HBM only when they are not in shared memory
    const int64_t NV = smem_warp > 0 ? 0 : N;
    const int64_t per_slot =
        NV * (1 + 1 + 1 + 4 * 4) + 3 * (NV + 1) * 4 + 3 * 2 * NV * 4 + 4 * (NV / 16) + W * 8 + A * 4 + C * 8;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const int64_t budget = (int64_t)((free_b + (size_t)b->ws_bytes) * 0.5);
    if ((int64_t)slots * per_slot > budget) slots = (int32_t)std::max<int64_t>(1, budget / per_slot);
    if (b->ws && slots == b->ws_slots && N == b->ws_N && W == b->ws_W && A == b->ws_A && C == b->ws_C &&
        smem_warp == b->P.smem_per_warp && kind == b->kind)
        return GPSAT_OK;
    b->kind = kind;
    cudaFree(b->ws);
    b->ws = nullptr;
    const size_t S = slots;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o2 = off;
        off += (bytes + 255) / 256 * 256;
        return o2;
    };
    size_t o_val = take(S * NV), o_phase = take(S * NV), o_seen = take(S * NV), o_level = take(S * NV * 4),
           o_reason = take(S * NV * 4), o_trail = take(S * NV * 4), o_tlim = take(S * (NV + 1) * 4),
           o_learnt = take(S * (NV + 1) * 4), o_lstamp = take(S * (NV + 1) * 4), o_act = take(S * NV * 4),
           o_bmax = take(S * (NV / 16) * 4),
           o_ws = take(S * 2 * NV * 4), o_wz = take(S * 2 * NV * 4), o_wc = take(S * 2 * NV * 4),
           o_w = take(S * W * 8), o_a = take(S * A * 4), o_c = take(S * C * 4),
           o_t = take(S * C * 4);
    if (cudaMalloc(&b->ws, off) != cudaSuccess) {
        cudaGetLastError();
        return set_error(GPSAT_ERR_NOMEM, "solver workspace allocation failed");
    }
    char *base = (char *)b->ws;
    cdcl::Params &P = b->P;
    P.val = (int8_t *)(base + o_val);
    P.phase = (int8_t *)(base + o_phase);
    P.seen = (uint8_t *)(base + o_seen);
    P.level = (int32_t *)(base + o_level);
    P.reason = (int32_t *)(base + o_reason);
    P.trail = (int32_t *)(base + o_trail);
    P.tlim = (int32_t *)(base + o_tlim);
    P.learnt = (int32_t *)(base + o_learnt);
    P.lstamp = (int32_t *)(base + o_lstamp);
    P.act = (float *)(base + o_act);
    P.bmax = (float *)(base + o_bmax);
    P.wl_start = (int32_t *)(base + o_ws);
    P.wl_size = (int32_t *)(base + o_wz);
    P.wl_cap = (int32_t *)(base + o_wc);
    P.watches = (int2 *)(base + o_w);
    P.arena = (int32_t *)(base + o_a);
    P.crefs = (int32_t *)(base + o_c);
    P.tmp = (int32_t *)(base + o_t);
    P.n_slots = slots;
    P.N = N;
    P.smem_per_warp = smem_warp;
    P.WCAP = W;
    P.ACAP = A;
    P.CCAP = C;
    b->ws_bytes = (int64_t)off;
    b->ws_slots = slots;
    b->ws_N = N;
    b->ws_W = W;
    b->ws_A = A;
    b->ws_C = C;
    return GPSAT_OK;
}

}  // namespace

extern "C" int gpsat_solve_options_default(gpsat_solve_options *o)
{
    if (!o) return set_error(GPSAT_ERR_ARG, "null options");
    std::memset(o, 0, sizeof(*o));
    o->decide = GPSAT_DECIDE_VSIDS;
    o->restart = GPSAT_RESTART_LUBY;
    // Luby unit, VSIDS decay and clause-database limit from sweeps on the
    // 16,384-instance random 3-SAT batch (n 50-250, 10^5 conflicts): from
    // Luby 100, decay 0.95 and 2000 kept before the first reduction to the
    // values below, 15,640 decided in 18.2 s became 16,112 in 15.0 s
    o->restart_base = 400;
    o->restart_factor = 1.5f;
    o->var_decay = 0.99f;
    o->learnt_first = 6000;
    o->learnt_inc = 300;
    o->minimize = 1;
    o->conflict_budget = 100000;
    o->phase_init = 0;
    o->max_slots = 0;
    o->log_participation = 0;
    return GPSAT_OK;
}

extern "C" int gpsat_batch_create(const int32_t *lits, const int64_t *clause_offsets, const int64_t *formula_offsets,
                                  const int32_t *n_vars, int32_t n_formulas, gpsat_batch **out)
{
    if (!out || n_formulas <= 0 || !clause_offsets || !formula_offsets || !n_vars)
        return set_error(GPSAT_ERR_ARG, "gpsat_batch_create: bad argument");
    *out = nullptr;
    // every offset, before any formula's clauses are read through them (the
    // literals are checked as each formula is prepared)
    if (formula_offsets[0] < 0) return set_error(GPSAT_ERR_FORMULA, "formula_offsets[0] must be >= 0");
    for (int32_t f = 0; f < n_formulas; f++)
        if (formula_offsets[f + 1] < formula_offsets[f])
            return set_error(GPSAT_ERR_FORMULA, "formula offsets must be non-decreasing");
    if (clause_offsets[formula_offsets[0]] < 0) return set_error(GPSAT_ERR_FORMULA, "clause offsets must be >= 0");
    for (int64_t c = formula_offsets[0]; c < formula_offsets[n_formulas]; c++)
        if (clause_offsets[c + 1] < clause_offsets[c])
            return set_error(GPSAT_ERR_FORMULA, "clause offsets must be non-decreasing");
    if (clause_offsets[formula_offsets[n_formulas]] > clause_offsets[formula_offsets[0]] && !lits)
        return set_error(GPSAT_ERR_ARG, "null literal array");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_error(GPSAT_ERR_NODEVICE, "no CUDA device visible");
    }
    gpsat_batch *b = new gpsat_batch();
    cudaGetDevice(&b->device);
    b->n_formulas = n_formulas;
    b->prep.resize(n_formulas);
    b->n_vars.assign(n_vars, n_vars + n_formulas);
    std::vector<int> rcs(n_formulas, GPSAT_OK);
    std::vector<std::string> msgs(n_formulas);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int nt = (int)std::min<int64_t>(hw, std::max(1, n_formulas / 64));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        th.emplace_back([&, t] {
            for (int32_t f = t; f < n_formulas; f += nt) {
                const int64_t c0 = formula_offsets[f], c1 = formula_offsets[f + 1];
                std::vector<int64_t> off(c1 - c0 + 1);
                for (int64_t c = c0; c <= c1; c++) off[c - c0] = clause_offsets[c] - clause_offsets[c0];
                rcs[f] = prepare_formula(lits + clause_offsets[c0], off.data(), n_vars[f], c1 - c0, b->prep[f]);
                if (rcs[f] != GPSAT_OK) msgs[f] = gpsat_last_error();  // this worker thread's message
            }
        });
    }
    for (auto &x : th) x.join();
    for (int32_t f = 0; f < n_formulas; f++) {
        if (rcs[f] != GPSAT_OK) {
            delete b;
            return set_error(rcs[f], "formula " + std::to_string(f) + ": " + msgs[f]);
        }
    }
    // concatenate preprocessed and original clauses
    std::vector<int32_t> plits, pcb(n_formulas), pce(n_formulas);
    std::vector<uint32_t> pcoff;
    b->var_off.assign(n_formulas + 1, 0);
    b->ocb.resize(n_formulas);
    b->oce.resize(n_formulas);
    pcoff.push_back(0);
    b->ocoff.push_back(0);
    for (int32_t f = 0; f < n_formulas; f++) {
        const HostFormula &h = b->prep[f];
        pcb[f] = (int32_t)(pcoff.size() - 1);
        for (int64_t c = 0; c < h.n_clauses(); c++) {
            for (int64_t k = h.off[c]; k < h.off[c + 1]; k++) plits.push_back(h.lits[k]);
            pcoff.push_back((uint32_t)plits.size());
        }
        pce[f] = (int32_t)(pcoff.size() - 1);
        b->max_m = std::max<int>(b->max_m, (int)h.n_clauses());
        b->max_words = std::max<int64_t>(b->max_words, (int64_t)h.lits.size() + cdcl::HDR * h.n_clauses());
        b->ocb[f] = (int32_t)(b->ocoff.size() - 1);
        for (int64_t c = formula_offsets[f]; c < formula_offsets[f + 1]; c++) {
            for (int64_t k = clause_offsets[c]; k < clause_offsets[c + 1]; k++)
                b->olits.push_back(lit_of_dimacs(lits[k]));
            b->ocoff.push_back((uint32_t)b->olits.size());
        }
        b->oce[f] = (int32_t)(b->ocoff.size() - 1);
        b->var_off[f + 1] = b->var_off[f] + n_vars[f];
        if (plits.size() >= (size_t)UINT32_MAX / 2 || b->olits.size() >= (size_t)UINT32_MAX / 2) {
            delete b;
            return set_error(GPSAT_ERR_CAPACITY, "batch too large (2^31 literals)");
        }
    }
    const int64_t V = b->var_off[n_formulas];
    bool ok = dup(&b->d_lits, plits) && dup(&b->d_coff, pcoff) && dup(&b->d_cb, pcb) && dup(&b->d_ce, pce) &&
              dup(&b->d_nv, b->n_vars) && dup(&b->d_var_off, b->var_off) && dup(&b->d_olits, b->olits) &&
              dup(&b->d_ocoff, b->ocoff) && dup(&b->d_ocb, b->ocb) && dup(&b->d_oce, b->oce) &&
              dalloc(&b->d_model, V) && dalloc(&b->d_state, n_formulas) && dalloc(&b->d_verdict, n_formulas) &&
              dalloc(&b->d_ok, n_formulas) && dalloc(&b->d_counter, 4);
    if (!ok) {
        cudaGetLastError();
        batch_free(b);
        delete b;
        return set_error(GPSAT_ERR_NOMEM, "batch upload failed");
    }
    *out = b;
    return GPSAT_OK;
}

extern "C" int gpsat_batch_destroy(gpsat_batch *b)
{
    if (!b) return GPSAT_OK;
    cudaSetDevice(b->device);
    batch_free(b);
    delete b;
    return GPSAT_OK;
}

extern "C" int gpsat_batch_info(const gpsat_batch *b, int32_t *n_formulas, int64_t *total_vars, int32_t *slots,
                                int64_t *workspace_bytes)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null batch");
    if (n_formulas) *n_formulas = b->n_formulas;
    if (total_vars) *total_vars = b->var_off[b->n_formulas];
    if (slots) *slots = b->ws_slots;
    if (workspace_bytes) *workspace_bytes = b->ws_bytes;
    return GPSAT_OK;
}

extern "C" int gpsat_batch_set_seeds(gpsat_batch *b, const float *activity, const int8_t *phase)
{
    if (!b) return set_error(GPSAT_ERR_ARG, "null batch");
    cudaSetDevice(b->device);
    const int64_t V = b->var_off[b->n_formulas];
    cudaFree(b->d_seed_act);
    cudaFree(b->d_seed_phase);
    b->d_seed_act = nullptr;
    b->d_seed_phase = nullptr;
    if (activity) {
        if (!dalloc(&b->d_seed_act, V) ||
            cudaMemcpy(b->d_seed_act, activity, V * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return cuda_error(cudaGetLastError(), "seed upload");
    }
    if (phase) {
        if (!dalloc(&b->d_seed_phase, V) ||
            cudaMemcpy(b->d_seed_phase, phase, V, cudaMemcpyHostToDevice) != cudaSuccess)
            return cuda_error(cudaGetLastError(), "seed upload");
    }
    return GPSAT_OK;
}

extern "C" int gpsat_batch_solve(gpsat_batch *b, const gpsat_solve_options *opt, const int32_t *job_formula,
                                 const int64_t *cube_offsets, const int32_t *cube_lits, int32_t n_jobs,
                                 int32_t *verdicts, int8_t *models, int64_t *stats, int32_t *model_ok,
                                 int32_t *participation)
{
    if (!b || !verdicts || n_jobs < 0) return set_error(GPSAT_ERR_ARG, "gpsat_batch_solve: bad argument");
    gpsat_solve_options o;
    if (opt) o = *opt;
    else gpsat_solve_options_default(&o);
    if (o.log_participation < 0 || o.log_participation > 2)
        return set_error(GPSAT_ERR_ARG, "log_participation must be 0, 1 or 2");
    if (o.proof_words < 0) return set_error(GPSAT_ERR_ARG, "proof_words must be >= 0");
    if (o.phase_init < 0 || o.phase_init > 2) return set_error(GPSAT_ERR_ARG, "phase_init must be 0, 1 or 2");
    cudaError_t err = cudaSetDevice(b->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
    const int32_t F = b->n_formulas;
    // jobs: given, or one per formula; preprocessing-decided formulas get none.
    // A job's level-0 facts are the literals preprocessing fixed, then its cube.
    // (the previous solve's jobs are forgotten first: a call that fails
    // leaves no proof log to read)
    std::vector<int32_t> jinst, jcoff, jclen, cubes, caller_job;
    b->caller_job.clear();
    b->job_verdict.clear();
    auto add_job = [&](int32_t f, const int32_t *cube, int64_t clen) {
        if (b->prep[f].verdict != GPSAT_UNKNOWN) {
            caller_job.push_back(-1);
            return;
        }
        caller_job.push_back((int32_t)jinst.size());
        jinst.push_back(f);
        jcoff.push_back((int32_t)cubes.size());
        for (int32_t l : b->prep[f].solved) cubes.push_back(l);
        for (int64_t k = 0; k < clen; k++) cubes.push_back(lit_of_dimacs(cube[k]));
        jclen.push_back((int32_t)cubes.size() - jcoff.back());
    };
    if (job_formula) {
        for (int32_t j = 0; j < n_jobs; j++) {
            const int32_t f = job_formula[j];
            if (f < 0 || f >= F) return set_error(GPSAT_ERR_ARG, "job formula index out of range");
            const int64_t c0 = cube_offsets ? cube_offsets[j] : 0, c1 = cube_offsets ? cube_offsets[j + 1] : 0;
            if (c0 < 0 || c1 < c0 || (c1 > c0 && !cube_lits))
                return set_error(GPSAT_ERR_ARG, "bad cube offsets");
            for (int64_t k = c0; k < c1; k++) {
                const int32_t d = cube_lits[k];
                if (d == 0 || d > b->n_vars[f] || d < -b->n_vars[f])
                    return set_error(GPSAT_ERR_ARG, "cube literal out of range");
            }
            add_job(f, cube_lits ? cube_lits + c0 : nullptr, c1 - c0);
        }
    } else {
        for (int32_t f = 0; f < F; f++) add_job(f, nullptr, 0);
    }
    const int32_t J = (int32_t)jinst.size();
    int rc = ensure_workspace(b, &o, J);
    if (rc != GPSAT_OK) return rc;
    if (J > b->job_cap) {
        cudaFree(b->d_job_inst);
        cudaFree(b->d_job_cube_off);
        cudaFree(b->d_job_cube_len);
        cudaFree(b->d_job_order);
        cudaFree(b->d_job_verdict);
        cudaFree(b->d_job_stats);
        b->job_cap = 0;
        if (!dalloc(&b->d_job_inst, J) || !dalloc(&b->d_job_cube_off, J) || !dalloc(&b->d_job_cube_len, J) ||
            !dalloc(&b->d_job_order, J) || !dalloc(&b->d_job_verdict, J) ||
            !dalloc(&b->d_job_stats, (size_t)J * cdcl::NSTATS))
            return set_error(GPSAT_ERR_NOMEM, "job arrays");
        b->job_cap = J;
    }
    if ((int64_t)cubes.size() > b->cube_cap) {
        cudaFree(b->d_cubes);
        b->cube_cap = 0;
        if (!dalloc(&b->d_cubes, cubes.size())) return set_error(GPSAT_ERR_NOMEM, "cube array");
        b->cube_cap = (int64_t)cubes.size();
    }
    const int64_t V = b->var_off[F];
    const int64_t PV = o.log_participation >= 2 ? 2 * V : V;
    // proof logs: proof_words per job
    b->proof_words = o.proof_words;
    if (o.proof_words > 0 && J > 0) {
        const int64_t need = (int64_t)J * o.proof_words * 4;
        if (need > b->proof_bytes) {
            cudaFree(b->d_proof);
            b->d_proof = nullptr;
            b->proof_bytes = 0;
            if (cudaMalloc(&b->d_proof, need) != cudaSuccess) {
                cudaGetLastError();
                return set_error(GPSAT_ERR_NOMEM, "proof log allocation");
            }
            b->proof_bytes = need;
        }
        if (J > b->proof_len_cap) {
            cudaFree(b->d_proof_len);
            b->d_proof_len = nullptr;
            b->proof_len_cap = 0;
            if (!dalloc(&b->d_proof_len, J)) return set_error(GPSAT_ERR_NOMEM, "proof lengths");
            b->proof_len_cap = J;
        }
    }
    if (o.log_participation && b->part_cap < PV) {
        cudaFree(b->d_part);
        b->d_part = nullptr;
        b->part_cap = 0;
        if (!dalloc(&b->d_part, PV)) return set_error(GPSAT_ERR_NOMEM, "part");
        b->part_cap = PV;
    }
    // processing order: the jobs of the largest formulas first (the
    // persistent grid takes them in this order).  A batch lasts as long as
    // its slowest jobs, and at a fixed clause ratio the search grows with the
    // variables, so the likely-long jobs should not start in the last wave.
    // Each job's search and outputs do not depend on the order.
    std::vector<int32_t> jorder(J);
    for (int32_t j = 0; j < J; j++) jorder[j] = j;
    std::stable_sort(jorder.begin(), jorder.end(), [&](int32_t a, int32_t c) {
        const int32_t na = b->n_vars[jinst[a]], nc = b->n_vars[jinst[c]];
        if (na != nc) return na > nc;
        return b->prep[jinst[a]].n_clauses() > b->prep[jinst[c]].n_clauses();
    });
    cudaStream_t st = 0;
    bool ok = true;
    if (J) {
        ok = cudaMemcpyAsync(b->d_job_inst, jinst.data(), J * 4, cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(b->d_job_order, jorder.data(), J * 4, cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(b->d_job_cube_off, jcoff.data(), J * 4, cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(b->d_job_cube_len, jclen.data(), J * 4, cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (ok && !cubes.empty())
            ok = cudaMemcpyAsync(b->d_cubes, cubes.data(), cubes.size() * 4, cudaMemcpyHostToDevice, st) ==
                 cudaSuccess;
    }
    ok = ok && cudaMemsetAsync(b->d_state, 0, F * 4, st) == cudaSuccess &&
         cudaMemsetAsync(b->d_model, 0, V, st) == cudaSuccess &&
         cudaMemsetAsync(b->d_counter, 0, 4, st) == cudaSuccess;
    if (ok && o.log_participation) ok = cudaMemsetAsync(b->d_part, 0, PV * 4, st) == cudaSuccess;
    if (ok && o.proof_words > 0 && J > 0) ok = cudaMemsetAsync(b->d_proof_len, 0, (size_t)J * 8, st) == cudaSuccess;
    if (!ok) return cuda_error(cudaGetLastError(), "solve setup");
    cdcl::Params &P = b->P;
    P.o.decide = o.decide;
    P.o.restart = o.restart;
    P.o.restart_base = std::max(1, o.restart_base);
    P.o.restart_factor = o.restart_factor > 1.0f ? o.restart_factor : 1.5f;
    P.o.var_decay = (o.var_decay > 0.5f && o.var_decay < 1.0f) ? o.var_decay : 0.95f;
    P.o.learnt_first = std::max(100, o.learnt_first);
    P.o.learnt_inc = std::max(0, o.learnt_inc);
    P.o.minimize = o.minimize;
    P.o.conflict_budget = o.conflict_budget > 0 ? o.conflict_budget : INT64_MAX;
    P.o.phase_init = o.phase_init;
    P.o.log_participation = o.log_participation;
    P.o.check_every = 256;
    P.lits = b->d_lits;
    P.coff = b->d_coff;
    P.inst_cb = b->d_cb;
    P.inst_ce = b->d_ce;
    P.inst_nv = b->d_nv;
    P.seed_act = b->d_seed_act;
    P.seed_phase = b->d_seed_phase;
    P.var_off = b->d_var_off;
    P.job_inst = b->d_job_inst;
    P.job_cube_off = b->d_job_cube_off;
    P.job_cube_len = b->d_job_cube_len;
    P.job_order = b->d_job_order;
    P.cubes = b->d_cubes;
    P.n_jobs = J;
    P.next_job = b->d_counter;
    P.inst_state = b->d_state;
    P.job_verdict = b->d_job_verdict;
    P.job_stats = b->d_job_stats;
    P.model = b->d_model;
    P.part = o.log_participation ? b->d_part : nullptr;
    P.var_total = V;
    P.proof = o.proof_words > 0 ? b->d_proof : nullptr;
    P.proof_len = o.proof_words > 0 ? b->d_proof_len : nullptr;
    P.proof_cap = o.proof_words;
    if (J) {
        const int slots = std::min<int32_t>(b->ws_slots, J);
        P.n_slots = slots;
        if (b->kind == K_HBM)
            cdcl::cdcl_kernel_hbm<<<(slots + 3) / 4, 128, 0, st>>>(P);
        else if (b->kind == K_SMEM4)
            cdcl::cdcl_kernel_smem4<<<(slots + 3) / 4, 128, 4 * (size_t)P.smem_per_warp, st>>>(P);
        else
            cdcl::cdcl_kernel_smem<<<(slots + 3) / 4, 128, 4 * (size_t)P.smem_per_warp, st>>>(P);
        P.n_slots = b->ws_slots;
        err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_error(err, "solve kernel launch");
    }
    // verdicts and models: SAT if some job found a model; UNSAT if every job
    // of the formula refuted its cube; preprocessing verdicts pass through
    std::vector<int32_t> jv(J);
    std::vector<int64_t> js((size_t)J * cdcl::NSTATS);
    std::vector<int32_t> state(F);
    ok = (J == 0 || (cudaMemcpyAsync(jv.data(), b->d_job_verdict, J * 4, cudaMemcpyDeviceToHost, st) ==
                         cudaSuccess &&
                     cudaMemcpyAsync(js.data(), b->d_job_stats, js.size() * 8, cudaMemcpyDeviceToHost, st) ==
                         cudaSuccess)) &&
         cudaMemcpyAsync(state.data(), b->d_state, F * 4, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (!ok) return cuda_error(cudaGetLastError(), "result copy");
    err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return cuda_error(err, "solve");
    b->job_verdict = jv;
    b->caller_job = std::move(caller_job);
    std::vector<int32_t> n_unsat(F, 0), n_jobs_f(F, 0);
    if (stats) std::memset(stats, 0, sizeof(int64_t) * (size_t)F * GPSAT_SOLVE_NSTATS);
    for (int32_t j = 0; j < J; j++) {
        const int32_t f = jinst[j];
        n_jobs_f[f]++;
        n_unsat[f] += jv[j] == GPSAT_UNSAT;
        if (stats) {
            int64_t *s = stats + (size_t)f * GPSAT_SOLVE_NSTATS;
            for (int k = 0; k < cdcl::ST_FLAGS; k++) s[k] += js[(size_t)j * cdcl::NSTATS + k];
            s[cdcl::ST_FLAGS] |= js[(size_t)j * cdcl::NSTATS + cdcl::ST_FLAGS];
            s[GPSAT_SOLVE_NSTATS - 1] += 1;  // jobs
        }
    }
    std::vector<int8_t> hm;
    std::vector<int32_t> vd(F);
    bool any_pre_sat = false;
    for (int32_t f = 0; f < F; f++) {
        const HostFormula &h = b->prep[f];
        if (h.verdict != GPSAT_UNKNOWN) {
            vd[f] = h.verdict;
            any_pre_sat |= h.verdict == GPSAT_SAT;
        } else if (state[f] == 1) {
            vd[f] = GPSAT_SAT;
        } else if (n_jobs_f[f] > 0 && n_unsat[f] == n_jobs_f[f]) {
            vd[f] = GPSAT_UNSAT;
        } else {
            vd[f] = GPSAT_UNKNOWN;
        }
    }
    if (any_pre_sat) {
        // formulas decided by preprocessing: fixed literals, the rest positive
        for (int32_t f = 0; f < F; f++) {
            const HostFormula &h = b->prep[f];
            if (h.verdict != GPSAT_SAT) continue;
            std::vector<int8_t> m(b->n_vars[f], 1);
            for (int32_t l : h.solved) m[l >> 1] = (l & 1) ? 1 : -1;
            if (cudaMemcpyAsync(b->d_model + b->var_off[f], m.data(), m.size(), cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
                return cuda_error(cudaGetLastError(), "model upload");
        }
    }
    if (cudaMemcpyAsync(b->d_verdict, vd.data(), F * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "verdict upload");
    check_models_kernel<<<(F * 32 + 127) / 128, 128, 0, st>>>(b->d_olits, b->d_ocoff, b->d_ocb, b->d_oce,
                                                              b->d_var_off, b->d_model, b->d_verdict, F, b->d_ok);
    err = cudaGetLastError();
    if (err != cudaSuccess) return cuda_error(err, "model check launch");
    if (models && cudaMemcpyAsync(models, b->d_model, V, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "model copy");
    if (model_ok && cudaMemcpyAsync(model_ok, b->d_ok, F * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "check copy");
    if (participation && o.log_participation &&
        cudaMemcpyAsync(participation, b->d_part, PV * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "participation copy");
    err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return cuda_error(err, "model check");
    std::memcpy(verdicts, vd.data(), F * 4);
    if (models) {
        // eliminated variables: the solver never wrote them
        for (int32_t f = 0; f < F; f++)
            if (vd[f] == GPSAT_SAT) pad_model(models + b->var_off[f], b->n_vars[f]);
    }
    return GPSAT_OK;
}

extern "C" int gpsat_batch_proof(const gpsat_batch *b, int32_t job, int32_t *verdict, int32_t *words, int64_t cap,
                                 int64_t *len)
{
    if (!b || !len || cap < 0 || (cap > 0 && !words)) return set_error(GPSAT_ERR_ARG, "gpsat_batch_proof: bad argument");
    if (job < 0 || job >= (int32_t)b->caller_job.size())
        return set_error(GPSAT_ERR_ARG, "gpsat_batch_proof: job outside the last solve's jobs");
    const int32_t j = b->caller_job[job];
    *len = 0;
    if (j < 0) {   // decided by preprocessing: no search, nothing logged
        if (verdict) *verdict = GPSAT_UNKNOWN;
        return GPSAT_OK;
    }
    if (verdict) *verdict = b->job_verdict[j];
    if (b->proof_words <= 0) return GPSAT_OK;
    cudaError_t err = cudaSetDevice(b->device);
    if (err != cudaSuccess) return cuda_error(err, "cudaSetDevice");
    int64_t n = 0;
    if (cudaMemcpy(&n, b->d_proof_len + j, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return cuda_error(cudaGetLastError(), "proof length copy");
    *len = n;
    if (n <= 0 || cap <= 0) return GPSAT_OK;
    const int64_t k = std::min(n, cap);
    if (cudaMemcpy(words, b->d_proof + (size_t)j * (size_t)b->proof_words, (size_t)k * 4, cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return cuda_error(cudaGetLastError(), "proof copy");
    // literals to DIMACS, lengths as they are
    for (int64_t p = 0; p < k;) {
        const int64_t l = words[p];
        for (int64_t i = 1; i <= l && p + i < k; i++) words[p + i] = dimacs_of_lit(words[p + i]);
        p += 1 + l;
    }
    return GPSAT_OK;
}

extern "C" int gpsat_check_model(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, const int8_t *model,
                                 int32_t n_vars, int64_t *first_false_clause)
{
    if (n_clauses < 0 || (n_clauses > 0 && (!offsets || !lits)) || !model || n_vars <= 0)
        return set_error(GPSAT_ERR_ARG, "gpsat_check_model: bad argument");
    for (int64_t c = 0; c < n_clauses; c++) {
        if (offsets[c + 1] < offsets[c] || offsets[c] < 0)
            return set_error(GPSAT_ERR_FORMULA, "gpsat_check_model: offsets must be non-decreasing from >= 0");
        bool sat = false;
        for (int64_t k = offsets[c]; k < offsets[c + 1] && !sat; k++) {
            const int32_t d = lits[k];
            const int32_t v = (d > 0 ? d : -d) - 1;
            if (v < 0 || v >= n_vars) return set_error(GPSAT_ERR_FORMULA, "literal out of range");
            sat = d > 0 ? model[v] > 0 : model[v] < 0;
        }
        if (!sat) {
            if (first_false_clause) *first_false_clause = c;
            return 0;
        }
    }
    if (first_false_clause) *first_false_clause = -1;
    return 1;
}
