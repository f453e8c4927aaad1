/*
 * gpsat -- GB300-native CDCL SAT engine, C ABI.
 *
 * One shared library (libgpsat.so) holds the sm_103a kernels and the C++
 * host code around them.  Every entry point returns an int status code
 * (GPSAT_OK or a negative GPSAT_ERR_*); none of them exits the process.
 * The caller owns host buffers; handles own device memory.  A handle is used
 * by one host thread at a time and binds the CUDA device that was current
 * when it was created.  Work is ordered on the stream passed in (NULL = the
 * legacy default stream); the *_host entry points are synchronous.
 *
 * Literals at this boundary are DIMACS integers: +v / -v for variable v
 * (1-based).  Internally the library uses the reference's encoding
 * 2*(v-1) + sign with sign 1 = positive (reference SATSolver/SolverTypes.cu:6-42).
 *
 * Each declaration names the reference interface it replaces (paths inside
 * the reference project).
 */
#ifndef GPSAT_H
#define GPSAT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GPSAT_OK 0
#define GPSAT_ERR_ARG (-1)       /* bad argument (null pointer, negative size ...) */
#define GPSAT_ERR_CUDA (-2)      /* a CUDA call failed; gpsat_last_error() has the text */
#define GPSAT_ERR_NOMEM (-3)     /* host or device allocation failed */
#define GPSAT_ERR_FORMULA (-4)   /* literal out of range, bad offsets, ... */
#define GPSAT_ERR_PARSE (-5)     /* malformed DIMACS text */
#define GPSAT_ERR_CAPACITY (-6)  /* a size exceeds a documented limit */
#define GPSAT_ERR_NODEVICE (-7)  /* no CUDA device visible */
#define GPSAT_ERR_TIMEOUT (-8)   /* a device wait ran out of its budget */
#define GPSAT_ERR_STATE (-9)     /* handle used in the wrong state */

/* ---- verdicts (reference sat_status, SATSolver/SolverTypes.cuh:125) ----- */
#define GPSAT_UNKNOWN 0
#define GPSAT_SAT 10
#define GPSAT_UNSAT 20

/* ---- per-trail BCP status ---------------------------------------------- */
#define GPSAT_BCP_NO_CONFLICT 0
#define GPSAT_BCP_CONFLICT 1
#define GPSAT_BCP_OVERFLOW (-1)   /* implication / list capacity exceeded */
#define GPSAT_BCP_BAD_TRAIL (-2)  /* variable out of range, or assigned both ways */
#define GPSAT_BCP_BUDGET (-3)     /* per-trail iteration budget exhausted (never expected) */

/* number of int64 counters reported per trail by the BCP entry points:
 * [0] propagations (watch-list scans), [1] watch entries processed,
 * [2] clause literals of processed entries, [3] assignment lookups,
 * [4] implications, [5] trail literals assigned                          */
#define GPSAT_BCP_NCOUNTERS 6

/* ---- library ------------------------------------------------------------ */
/* Version string of this library.  (reference FileManager/Version.h) */
const char *gpsat_version(void);
/* Text for a status code. */
const char *gpsat_error_string(int code);
/* Detail of the last error raised on the calling host thread ("" if none).
 * (replaces the reference's print-and-exit check(),
 *  ErrorHandler/CudaMemoryErrorHandler.cu:3-10) */
const char *gpsat_last_error(void);
/* Number of visible CUDA devices (0 on a machine without a GPU). */
int gpsat_device_count(int32_t *count);

/* ---- formula ------------------------------------------------------------ */
typedef struct gpsat_formula gpsat_formula;

/* Builds a formula from clauses in CSR form: clause c is
 * lits[offsets[c] .. offsets[c+1]), DIMACS literals.  Runs the reference's
 * preprocessing (duplicate-literal and tautology removal, then unit-clause
 * propagation; reference Preprocessing/RepeatedLiteralsRemover.cu:25-62 and
 * Preprocessing/UnaryClausesRemover.cu:75-235, always on as in
 * FileManager/ParametersManager.cpp:176-182), computes the reference's initial
 * two watches per clause (BCPStrategy/ClauseListStructure.cu:101-148) and
 * uploads the clause arena and watch lists to the current device.
 * Replaces FormulaData::copy_host_clauses_to_dev (FileManager/FormulaData.cu:82-105)
 * and CUDAClauseVec::alloc_and_copy_to_dev (Utils/CUDAClauseVec.cu:85-118). */
int gpsat_formula_create(const int32_t *lits, const int64_t *offsets, int32_t n_vars,
                         int64_t n_clauses, gpsat_formula **out);
int gpsat_formula_destroy(gpsat_formula *f);
/* Sizes after preprocessing and the preprocessing verdict (GPSAT_UNKNOWN,
 * GPSAT_SAT when every clause was removed, GPSAT_UNSAT on a unit conflict or
 * an empty clause). */
int gpsat_formula_info(const gpsat_formula *f, int32_t *n_vars, int64_t *n_clauses,
                       int64_t *n_lits, int32_t *preproc_verdict, int64_t *n_solved);
/* Copies out the preprocessed clauses (DIMACS, CSR), the literals fixed by
 * preprocessing, and the initial watch indices (position inside the clause)
 * of every preprocessed clause.  Any pointer may be NULL to skip that part. */
int gpsat_formula_export(const gpsat_formula *f, int32_t *lits, int64_t *offsets,
                         int32_t *solved_lits, int32_t *watch1, int32_t *watch2);

/* ---- two-watched-literal BCP over a batch of partial trails --------------
 * Applies each trail exactly as the reference applies assumptions: every
 * trail literal is assigned first (SATSolver/VariablesStateHandler.cu:35-59),
 * then WatchedClausesList::new_decision runs for each trail literal in order
 * with one shared pending list, depth-first over new implications, stopping
 * at the first conflict (ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu:56-73,
 * BCPStrategy/WatchedClausesList.cu:46-314).  Outputs per trail t:
 *   status[t]          GPSAT_BCP_*
 *   conflict_clause[t] index of the conflicting preprocessed clause, or -1
 *   stop_index[t]      trail position whose propagation met the conflict, or -1
 *   n_impl[t]          implied literals, in the reference's order, written to
 *   impl_lit[t*impl_cap ...]     (DIMACS) and
 *   impl_reason[t*impl_cap ...]  (index of the implying clause)
 *   counters[t*GPSAT_BCP_NCOUNTERS ...]  (may be NULL)
 * Trail t is trail_lits[trail_offsets[t] .. trail_offsets[t+1]): the offsets
 * must be non-decreasing from >= 0 (gpsat_bcp_run_host refuses others with
 * GPSAT_ERR_ARG; the device entries read them as given).
 * Trails must not assign a variable both ways (GPSAT_BCP_BAD_TRAIL);
 * a variable repeated with the same sign is propagated twice, as in the
 * reference.  Clause length is limited to 2048 literals.                     */
typedef struct gpsat_bcp gpsat_bcp;

/* Allocates the device workspace: max_slots trails in flight (0 = as many as
 * the GPU keeps resident), impl_cap implied literals per trail, arena_cap
 * watch moves per trail (0 = default). */
int gpsat_bcp_create(const gpsat_formula *f, int32_t max_slots, int64_t impl_cap,
                     int64_t arena_cap, gpsat_bcp **out);
int gpsat_bcp_destroy(gpsat_bcp *b);
/* Device pointers, stream ordered, asynchronous. */
int gpsat_bcp_run_device(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets,
                         int32_t n_trails, int32_t *status, int32_t *conflict_clause,
                         int32_t *stop_index, int64_t *n_impl, int32_t *impl_lit,
                         int32_t *impl_reason, int64_t *counters, void *stream);
/* Host pointers: copies the trails in, runs, copies the results out, waits.
 * When every buffer is page-locked host memory (cudaHostAlloc, cudaHostRegister,
 * torch's pin_memory) the trails are copied in by DMA and the kernel writes the
 * results in place over the CPU-GPU link, with no output staging; the results
 * are the same. */
int gpsat_bcp_run_host(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets,
                       int32_t n_trails, int32_t *status, int32_t *conflict_clause,
                       int32_t *stop_index, int64_t *n_impl, int32_t *impl_lit,
                       int32_t *impl_reason, int64_t *counters);
/* Trails in flight and the device bytes the workspace holds (its slots, and
 * the per-trail assignment words and staging buffers earlier runs grew). */
int gpsat_bcp_info(const gpsat_bcp *b, int32_t *slots, int64_t *device_bytes);
/* Runs that follow use at most n of the workspace's slots (1 <= n <= slots;
 * 0 = all).  Outputs do not depend on it.  A launch lasts as long as its
 * longest trails, which wait on memory the other trails also load: with
 * trails of very unequal length fewer trails in flight can finish sooner,
 * with equal ones all slots can (no counterpart in the reference). */
int gpsat_bcp_set_active_slots(gpsat_bcp *b, int32_t n);
/* The processing order of the runs that follow, when a run has more trails
 * than it keeps in flight: trails whose literal count is nearest `pivot`
 * start first (0, the default: shortest first).  A run lasts as long as its
 * slowest trail; the slowest are those that reach their fixpoint without a
 * conflict, which is likelier the fewer literals a trail assigns, but such a
 * trail has fewer literals to propagate, so the slowest ones have a middling
 * length that depends on the formula (BCPBatch.tune picks the pivot among
 * quantiles of the caller's trail lengths).  Outputs do not depend on it.
 * No counterpart in the reference, which propagates one trail at a time. */
int gpsat_bcp_set_order_pivot(gpsat_bcp *b, int64_t pivot);

/* Watch entries one round of the two-watched-literal kernel evaluates per
 * trail (64, 128 or 256; default 128): one thread per entry, so the trail's
 * thread block has entries / 32 warps.  Wider windows need fewer rounds per
 * propagation but keep fewer trails in flight; outputs do not depend on it.
 * (No counterpart in the reference, whose BCP is one thread per solver.) */
int gpsat_bcp_set_window(gpsat_bcp *b, int32_t entries);
/* Trails a window width keeps in flight at most: its resident blocks, within
 * the workspace's slots. */
int gpsat_bcp_window_slots(const gpsat_bcp *b, int32_t entries, int32_t *slots);
/* The propagation strategy of the runs that follow (the reference chooses it at
 * compile time, SATSolver/Configs.cuh:27-33, CONFLICT_ANALYSIS_STRATEGY):
 *   GPSAT_BCP_WATCHED    two watched literals in the reference's order (default;
 *                        reference TWO_WATCHED_LITERALS, BCPStrategy/WatchedClausesList.cu)
 *   GPSAT_BCP_FULL_SCAN  full-scan clause evaluation (reference BASIC_SEARCH,
 *                        ConflictAnalysis/ConflictAnalyzer.cu:173-245): every trail
 *                        literal assigned, then sweeps over all clauses in index
 *                        order, a unit clause implying at once, until a conflict or
 *                        a sweep that implies nothing.  Outputs as above, except:
 *                        stop_index = the sweep (0-based) that met the conflict;
 *                        counters [0] sweeps, [1] clause evaluations, [2] and [3]
 *                        literals examined, [4] implications, [5] trail literals.
 * Trails run one per thread block; a formula of up to 196,608 variables keeps a
 * trail's assignment in shared memory.  gpsat_bcp_run_static always runs
 * GPSAT_BCP_WATCHED. */
#define GPSAT_BCP_WATCHED 0
#define GPSAT_BCP_FULL_SCAN 1
int gpsat_bcp_set_strategy(gpsat_bcp *b, int32_t strategy);

/* Allocation-free BCP (no counterpart in the reference, whose BCP allocates
 * its watch-node pool and graph up front): the same kernel and outputs as
 * gpsat_bcp_run_device, but the per-trail state lives in one fixed 64 MiB
 * device array inside the library (GPSAT_BCP_STATIC_SCRATCH_BYTES), and the
 * call makes no cudaMalloc, cudaFree or other allocating call.  It is for
 * callers that cannot allocate at propagation time: code capturing the call
 * into a CUDA graph (device allocation is not allowed on a capturing stream,
 * and a replayed graph needs fixed addresses), and hosts whose device memory
 * is reserved up front by their own pool.
 *   f      must already be resident on the device: gpsat_bcp_create on it
 *          uploads it (the upload allocates, so do it beforehand).
 *   impl_cap, arena_cap  as in gpsat_bcp_create (arena_cap 0 = default).
 * As many trails run at once as fit in the array (at most the resident warp
 * count); if one trail's state does not fit, the call returns
 * GPSAT_ERR_CAPACITY and launches nothing.  The state that must start at
 * zero is cleared on the stream by every call.
 * The first call on a device looks the array up (and may load the module):
 * make that first call before any stream capture begins.
 * One array per device: calls whose GPU work overlaps (e.g. on two streams)
 * race on it and give wrong results; order them on one stream. */
#define GPSAT_BCP_STATIC_SCRATCH_BYTES ((int64_t)64 << 20)
int gpsat_bcp_run_static(const gpsat_formula *f, int64_t impl_cap, int64_t arena_cap,
                         const int32_t *trail_lits, const int64_t *trail_offsets, int32_t n_trails,
                         int32_t *status, int32_t *conflict_clause, int32_t *stop_index,
                         int64_t *n_impl, int32_t *impl_lit, int32_t *impl_reason,
                         int64_t *counters, void *stream);

/* ---- CDCL solving on the device -------------------------------------------
 * One warp runs one complete CDCL search (two watched literals, first-UIP
 * learning, VSIDS, restarts) for one job; a persistent grid pulls jobs from a
 * global counter.  A job is a whole formula or a formula restricted to a cube
 * of assumption literals (the reference's JobChooser jobs).  Replaces the
 * reference's sequential kernel run_sequential and the relaunched
 * parallel_kernel (SATSolver/Parallelizer.cu:133-277, main.cu:197-310). */
#define GPSAT_DECIDE_VSIDS 0      /* DecisionStrategy: VSIDS (reference DecisionStrategy/VSIDS.cu) */
#define GPSAT_DECIDE_LAST_FREE 1  /* the reference's default rule (SATSolver/DecisionMaker.cu:45-55) */
#define GPSAT_RESTART_NONE 0
#define GPSAT_RESTART_LUBY 1
#define GPSAT_RESTART_GEOMETRIC 2 /* reference Restarts/GeometricRestartsManager.cu (100, x1.3) */

typedef struct {
    int32_t decide;            /* GPSAT_DECIDE_* */
    int32_t restart;           /* GPSAT_RESTART_* */
    int32_t restart_base;      /* conflicts: Luby unit or first geometric interval */
    float restart_factor;      /* geometric growth */
    float var_decay;           /* VSIDS activity decay per conflict */
    int32_t learnt_first;      /* ClauseLearning: learnt clauses kept before the first reduction */
    int32_t learnt_inc;        /* growth of that limit per reduction */
    int32_t minimize;          /* ConflictAnalysis: basic learnt-clause minimisation */
    int64_t conflict_budget;   /* per job; reaching it ends the job UNKNOWN (0 = none) */
    int32_t phase_init;        /* first polarity of an unseeded variable: 0 false, 1 true,
                                  2 the sign of most of its occurrences in the formula */
    int32_t max_slots;         /* jobs in flight (0 = as many as the GPU keeps resident) */
    int32_t log_participation; /* 1: count, per variable, the conflicts whose analysis saw it;
                                  2: also its occurrences in learnt clauses */
    int32_t proof_words;       /* > 0: every job logs its learnt clauses, in the order learnt,
                                  in a log of this many int32 words (see gpsat_batch_proof) */
    int32_t reserved[4];
} gpsat_solve_options;

/* per-formula statistics written by gpsat_batch_solve (summed over its jobs) */
#define GPSAT_SOLVE_NSTATS 9
/* [0] conflicts [1] decisions [2] propagations [3] restarts [4] learnt clauses
 * kept [5] reductions [6] watch rebuilds [7] flags (1 cancelled, 2 slot too
 * small, 4 conflict budget) [8] jobs                                        */

int gpsat_solve_options_default(gpsat_solve_options *o);

typedef struct gpsat_batch gpsat_batch;
/* Formulas f = 0..n_formulas-1: clauses formula_offsets[f] .. formula_offsets[f+1]
 * of the CSR (lits, clause_offsets); n_vars[f] variables each.  Every formula
 * goes through the reference's preprocessing on the host, then is uploaded. */
int gpsat_batch_create(const int32_t *lits, const int64_t *clause_offsets, const int64_t *formula_offsets,
                       const int32_t *n_vars, int32_t n_formulas, gpsat_batch **out);
int gpsat_batch_destroy(gpsat_batch *b);
int gpsat_batch_info(const gpsat_batch *b, int32_t *n_formulas, int64_t *total_vars, int32_t *slots,
                     int64_t *workspace_bytes);
/* Optional per-variable seeds (concatenated over formulas, NULL to clear):
 * initial VSIDS activity and initial phase (0 false, 1 true). */
int gpsat_batch_set_seeds(gpsat_batch *b, const float *activity, const int8_t *phase);
/* Solves every formula.  Jobs: job_formula[j] with cube literals
 * cube_lits[cube_offsets[j] .. cube_offsets[j+1]) (DIMACS); job_formula NULL =
 * one job per formula.  A formula is SAT when one of its jobs finds a model
 * (the other jobs of it are cancelled), UNSAT when all its jobs are refuted,
 * otherwise UNKNOWN.  Outputs per formula: verdicts, models (n_vars bytes each,
 * +1 true / -1 false, concatenated; may be NULL), stats (GPSAT_SOLVE_NSTATS
 * each; may be NULL), model_ok (device checker: 1 every original clause holds
 * a true literal, 0 not, -1 no model; may be NULL), participation (int32 per
 * variable, with log_participation; with log_participation 2 the array holds
 * twice the variables: participation, then learnt-clause occurrences; may be
 * NULL). */
int gpsat_batch_solve(gpsat_batch *b, const gpsat_solve_options *opt, const int32_t *job_formula,
                      const int64_t *cube_offsets, const int32_t *cube_lits, int32_t n_jobs, int32_t *verdicts,
                      int8_t *models, int64_t *stats, int32_t *model_ok, int32_t *participation);
/* The proof log of one job of the last gpsat_batch_solve made with
 * proof_words > 0 (no counterpart in the reference, which outputs no proof).
 * job is the caller's job index (the formula index when the solve was given no
 * job list).  The log is the job's learnt clauses in the order learnt, each as
 * [length, DIMACS literal...]; up to cap words are copied to words.  *len is the
 * log's size in words, 0 when nothing was logged (no search ran, or logging was
 * off) and -1 when the clauses outgrew proof_words (the log is then incomplete).
 * *verdict (may be NULL) is the job's own verdict.  A job's UNSAT is certified
 * by gpsat_check_rup over the original clauses, the job's cube and this log. */
int gpsat_batch_proof(const gpsat_batch *b, int32_t job, int32_t *verdict, int32_t *words, int64_t cap,
                      int64_t *len);
/* Host checker of UNSAT proofs by reverse unit propagation, independent of the
 * device solver (no counterpart in the reference): returns 1 when the formula
 * (clauses in CSR, DIMACS) with the assumption literals is refuted -- every
 * clause of the proof log ([length, literal...] per clause) follows from
 * everything before it by unit propagation, and unit propagation over the
 * formula, the assumptions and the log ends in a conflict -- 0 when a step
 * fails (*failed_step = its index, or the number of steps when the log ends
 * without a conflict), negative on bad input. */
int gpsat_check_rup(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, int32_t n_vars,
                    const int32_t *assumptions, int32_t n_assumptions, const int32_t *proof, int64_t proof_len,
                    int64_t *failed_step);
/* Independent host model check: 1 if every clause holds a true literal, 0 if
 * not (first_false_clause set), negative on bad input.
 * (the reference's own "verified" check, SATSolver/Results.cu:143-155,
 *  ignores literal signs; this one does not) */
int gpsat_check_model(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, const int8_t *model,
                      int32_t n_vars, int64_t *first_false_clause);

/* ---- DIMACS input (host) ---------------------------------------------------
 * Parses CNF text.  Call once with lits/offsets NULL for the sizes, then with
 * buffers of n_lits and n_clauses+1 entries.  n_vars is the highest variable
 * that occurs, as the reference's reader sets it; the header's counts are
 * returned for comparison.  Malformed text gives GPSAT_ERR_PARSE with the
 * line in gpsat_last_error().  (replaces CnfManager::read_cnf, reference
 * FileManager/CnfReader.cpp:30-135) */
int gpsat_dimacs_parse(const char *text, int64_t len, int32_t *n_vars, int64_t *n_clauses, int64_t *n_lits,
                       int32_t *header_vars, int64_t *header_clauses, int32_t *lits, int64_t *offsets);

/* ---- seeded synthetic inputs (host) ---------------------------------------
 * Generator: splitmix64, one independent stream per clause / per trail, so
 * outputs do not depend on thread count.  uniform(n) = high 64 bits of
 * (64-bit draw * n).                                                         */
/* Uniform random k-SAT: m clauses of k distinct variables, fair signs.
 * lits must hold m*k ints; clause c is lits[c*k .. c*k+k). */
int gpsat_gen_random_ksat(uint64_t seed, int32_t n_vars, int64_t n_clauses, int32_t k,
                          int32_t *lits);
/* Random partial trails: trail t assigns round(n*(fmin + (fmax-fmin)*u_t))
 * distinct variables (at least 1) in random order with fair signs.
 * Call with lits == NULL to get offsets (n_trails+1 entries) only. */
int gpsat_gen_trails(uint64_t seed, int32_t n_vars, int32_t n_trails, double fmin,
                     double fmax, int64_t *offsets, int32_t *lits);
/* Planted k-SAT with community structure: the variables form n_communities
 * equal contiguous blocks; clause c picks a block uniformly and each of its
 * k distinct variables comes from that block with probability p_in, else
 * from all variables.  A hidden assignment (planted[v] = +1/-1, optional
 * output) satisfies every clause: signs are drawn uniformly among the
 * patterns it satisfies.  lits holds m*k ints as in gpsat_gen_random_ksat.
 * (no counterpart in the reference, which reads CNF files only: this is the
 * structured-batch workload's generator) */
int gpsat_gen_planted(uint64_t seed, int32_t n_vars, int64_t n_clauses, int32_t k,
                      int32_t n_communities, double p_in, int32_t *lits, int8_t *planted);

/* ---- learned seeding: message-passing network kernels ----------------------
 * No counterpart in the reference (it has no learned component): a 3-layer,
 * 64-wide network over the variable-clause graph whose outputs seed the
 * solver's VSIDS activities and phases (gpsat_batch_set_seeds) and rank the
 * JobChooser's split variables.  Matrices are bf16, row-major, 16-byte
 * aligned, with row strides (ld*) in elements that are multiples of 8;
 * accumulation is fp32.  All calls are stream ordered and asynchronous;
 * device pointers only.  An edge is (row << 1) | positive, segments are CSR
 * (seg_off[segs+1], int64). */
/* Y[rows x N] = act(X[rows x K] . B^T + bias), B = N x K (row stride ldb),
 * act = relu when relu != 0; K in {64, 128, 192}, N in {64, 128, 192, 256};
 * tcgen05 tensor cores.  *err is set to 1 if a tile gave up waiting for its
 * data or its product. */
int gpsat_gnn_mm(const void *X, int32_t ldx, int64_t rows, int32_t K, const void *B, int32_t ldb,
                 int32_t N, const float *bias, int32_t relu, void *Y, int32_t ldy, int32_t *err,
                 void *stream);
/* dW[64 x N] += X[rows x 64]^T . dY[rows x N] (fp32 dW, N in {64, 128, 192});
 * tcgen05 tensor cores, the rows being the contraction axis.  *err (may be
 * NULL) is set to 1 if a block gave up waiting for its products. */
int gpsat_gnn_wgrad(const void *X, int32_t ldx, const void *dY, int32_t ldy, int64_t rows, int32_t N,
                    float *dW, int32_t *err, void *stream);
/* out[s] = act(seg_scale[s] * sum over edges e of s of (positive ? srcP : srcN)[row e] + Z[s]),
 * 64 channels; act = relu when relu != 0; seg_scale and Z may be NULL */
int gpsat_gnn_gather(const int64_t *seg_off, const int32_t *edges, int64_t segs, const void *srcP,
                     const void *srcN, int32_t lds, const float *seg_scale, const void *Z, int32_t ldz,
                     void *out, int32_t ldo, int32_t relu, void *stream);
/* outP[s] / outN[s] = sum of src_scale[row e] * src[row e] over the positive /
 * negative edges of s (src_scale may be NULL) */
int gpsat_gnn_gather_split(const int64_t *seg_off, const int32_t *edges, int64_t segs, const void *src,
                           int32_t lds, const float *src_scale, void *outP, void *outN, int32_t ldo,
                           void *stream);
/* dpre = dout where h > 0, else 0 (64 channels) */
int gpsat_gnn_relu_bwd(const void *dout, int32_t ldd, const void *h, int32_t ldh, int64_t rows, void *dpre,
                       int32_t ldp, void *stream);
/* out[64] += column sums of Y (fp32) */
int gpsat_gnn_colsum(const void *Y, int32_t ldy, int64_t rows, float *out, void *stream);
/* H[r] = vec (64 fp32 -> bf16) for every row */
int gpsat_gnn_broadcast(const float *vec, int64_t rows, void *H, int32_t ldh, void *stream);
/* Heads: score = H.ws + bs, phase = H.wp + bp with head = [ws(64), wp(64), bs, bp].
 * With y_act != NULL also the losses sum((sigmoid(score) - y_act)^2 * w_act) and
 * sum(BCE(sigmoid(phase), t_phase) * w_phase) into loss[0..1], their gradient
 * w.r.t. H into dH and w.r.t. head into ghead (accumulated).  score / phase
 * outputs may be NULL. */
int gpsat_gnn_head(const void *H, int32_t ldh, int64_t rows, const float *head, const float *y_act,
                   const float *w_act, const float *t_phase, const float *w_phase, float *score, float *phase,
                   void *dH, int32_t ldd, float *ghead, float *loss, void *stream);
/* Adam step (bias-corrected, step >= 1) on n fp32 parameters; zeroes g. */
int gpsat_gnn_adam(float *p, float *g, float *m, float *v, int64_t n, float lr, float beta1, float beta2,
                   float eps, int64_t step, void *stream);
/* W (K x N fp32) -> fwd = W^T (N x K bf16) and/or bwd = W (K x N bf16, row stride ldb) */
int gpsat_gnn_pack(const float *W, int32_t K, int32_t N, void *fwd, void *bwd, int32_t ldb, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GPSAT_H */
