// Device CDCL solver shared declarations (host <-> device parameter blocks).
#pragma once

#include <cstdint>

namespace gpsat {
namespace cdcl {

constexpr int HDR = 2;                       // words before a clause's literals: [len|flags][lbd]
constexpr uint32_t LEN_MASK = 0x00FFFFFFu;
constexpr uint32_t F_LEARNT = 1u << 30;
constexpr uint32_t F_DELETED = 1u << 31;
constexpr int NSTATS = 8;                    // per-job counters (see JobStat)
enum JobStat { ST_CONFLICTS = 0, ST_DECISIONS, ST_PROPS, ST_RESTARTS, ST_LEARNTS, ST_REDUCES, ST_REBUILDS, ST_FLAGS };
// job flags (ST_FLAGS); FL_INTERNAL carries a check code in bits 8..15
constexpr int64_t FL_CANCELLED = 1, FL_RESOURCE = 2, FL_BUDGET = 4, FL_INTERNAL = 8;
// internal consistency checks (a failing one ends the job UNKNOWN instead of
// touching memory out of range)
enum CheckCode : int { CK_REASON = 1, CK_UIP = 2, CK_NO_CURRENT = 3, CK_TRAIL = 4, CK_ASSIGNED = 5, CK_CREF = 6 };
// which limit ended a job with FL_RESOURCE (bits 16..23 of ST_FLAGS)
enum ResourceCode : int { RS_INIT = 1, RS_WATCHES = 2, RS_CLAUSES = 3, RS_REBUILD_LOOP = 4, RS_DECISIONS = 5 };

enum Decide : int32_t { DECIDE_VSIDS = 0, DECIDE_LAST_FREE = 1 };
enum Restart : int32_t { RESTART_NONE = 0, RESTART_LUBY = 1, RESTART_GEOMETRIC = 2 };

struct Opts {
    int32_t decide = DECIDE_VSIDS;
    int32_t restart = RESTART_LUBY;
    int32_t restart_base = 100;
    float restart_factor = 1.5f;
    float var_decay = 0.95f;
    int32_t learnt_first = 2000;
    int32_t learnt_inc = 300;
    int32_t minimize = 1;
    int64_t conflict_budget = 100000;
    int32_t phase_init = 0;          // 0: negative first, 1: positive first, 2: majority sign of the occurrences
    int32_t log_participation = 0;   // 1: participation counts; 2: and learnt-clause occurrences
    int32_t check_every = 256;       // conflicts between cancellation checks
};

// Bytes of shared memory one warp needs to hold its job's per-variable and
// per-literal arrays for N variables (N a multiple of 4): level, reason,
// trail, activity (4N each); tlim, learnt, lstamp (4(N+4) each); the three
// watch-list header arrays start, size, capacity (8N each); value, phase,
// seen (N each); rounded up to 16 bytes.  (The activity block bounds serve
// formulas above 1024 variables, far more than shared memory holds.)
constexpr int64_t smem_bytes_per_warp(int64_t N)
{
    return (16 * N + 12 * (N + 4) + 24 * N + 3 * N + 15) / 16 * 16;
}

struct Params {
    Opts o;
    // instances: clauses of instance i are global clause ids [inst_cb[i], inst_ce[i])
    const int32_t *lits;         // internal literals
    const uint32_t *coff;        // per global clause, offset into lits (+1 sentinel)
    const int32_t *inst_cb, *inst_ce, *inst_nv;
    const float *seed_act;       // optional: initial VSIDS activity per (instance, var)
    const int8_t *seed_phase;    // optional: initial phase per (instance, var)
    const int64_t *var_off;      // per instance offset into per-var arrays (model, seeds, participation)
    // jobs
    const int32_t *job_inst, *job_cube_off, *job_cube_len, *cubes;
    const int32_t *job_order;    // jobs in processing order (largest formula first)
    int32_t n_jobs;
    unsigned int *next_job;
    int32_t *inst_state;         // 0 open, 1 a job found a model
    // outputs
    int32_t *job_verdict;
    int64_t *job_stats;          // NSTATS per job
    int8_t *model;               // per (instance, var): +1 / -1
    int32_t *part;               // per (instance, var): conflict participation (optional); with
                                 // log_participation 2 followed by learnt-clause occurrences
    int64_t var_total;           // variables of all instances (the second half's offset)
    // optional proof log: job j appends each learnt clause as [len, literals...]
    // (internal encoding) to proof[j * proof_cap ...]; proof_len[j] = words
    // written, or -1 when the clauses outgrew proof_cap
    int32_t *proof;
    int64_t *proof_len;
    int64_t proof_cap;
    // workspace
    int32_t n_slots;
    int32_t N;                   // max vars (padded to 16)
    int32_t smem_per_warp;       // > 0: the per-variable and per-literal arrays live in
                                 // dynamic shared memory (that many bytes per warp)
    int64_t WCAP, ACAP, CCAP;
    int8_t *val, *phase;
    uint8_t *seen;
    int32_t *level, *reason, *trail, *tlim, *learnt, *lstamp, *tmp;
    float *act;
    float *bmax;                 // per slot N/16 floats: activity bound per block of 32 variables
    int32_t *wl_start, *wl_size, *wl_cap;
    int2 *watches;
    int32_t *arena, *crefs;
};

}  // namespace cdcl
}  // namespace gpsat
