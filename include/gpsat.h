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
#define GPSAT_ERR_FORMULA (-4)   /* literal out of range, empty clause, ... */
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
 * GPSAT_SAT when every clause was removed, GPSAT_UNSAT on a unit conflict). */
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
/* Host pointers: copies the trails in, runs, copies the results out, waits. */
int gpsat_bcp_run_host(gpsat_bcp *b, const int32_t *trail_lits, const int64_t *trail_offsets,
                       int32_t n_trails, int32_t *status, int32_t *conflict_clause,
                       int32_t *stop_index, int64_t *n_impl, int32_t *impl_lit,
                       int32_t *impl_reason, int64_t *counters);
/* Trails in flight and the device bytes the workspace holds. */
int gpsat_bcp_info(const gpsat_bcp *b, int32_t *slots, int64_t *device_bytes);

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

#ifdef __cplusplus
}
#endif

#endif /* GPSAT_H */
