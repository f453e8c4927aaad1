// Internal declarations shared by the host C++ and CUDA translation units of
// libgpsat.  Not part of the public ABI (include/gpsat.h is).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gpsat.h"

namespace gpsat {

// Internal literal encoding, the reference's: 2*var + sign, sign 1 = positive
// (reference SATSolver/SolverTypes.cu:6-42).
inline int32_t lit_of_dimacs(int32_t d) { return d > 0 ? 2 * (d - 1) + 1 : 2 * (-d - 1); }
inline int32_t dimacs_of_lit(int32_t l) { return (l & 1) ? (l >> 1) + 1 : -((l >> 1) + 1); }

// Records the detail of the last error on this host thread and returns code.
int set_error(int code, const std::string &msg);
int cuda_error(int cuda_code, const char *what);

// ---- host-side formula preparation (formula_host.cpp) --------------------
struct HostFormula {
    int32_t n_vars = 0;
    std::vector<int32_t> lits;      // internal encoding, preprocessed clauses
    std::vector<int64_t> off;       // n_clauses + 1
    std::vector<int32_t> solved;    // literals fixed by preprocessing (internal)
    int32_t verdict = GPSAT_UNKNOWN;
    std::vector<int32_t> w1, w2;    // initial watch positions per clause
    std::vector<uint32_t> w0off;    // per-var initial list offsets (n_vars + 1)
    std::vector<int32_t> w0cl;      // per-var initial lists, head first
    int32_t max_len = 0;
    int64_t n_clauses() const { return (int64_t)off.size() - 1; }
};

// Validates DIMACS input, converts to the internal encoding and runs the
// reference's preprocessing.  Fills lits/off/solved/verdict.
int prepare_formula(const int32_t *lits, const int64_t *offsets, int32_t n_vars,
                    int64_t n_clauses, HostFormula &out);
// The reference's initial watch choice and per-var list order.
void build_initial_watches(HostFormula &f);

}  // namespace gpsat

// Opaque handle behind gpsat_formula*.
struct gpsat_formula {
    int device = 0;
    gpsat::HostFormula h;
    // device copies
    int32_t *d_lits = nullptr;      // internal literals
    uint32_t *d_coff = nullptr;     // clause offsets (n_clauses + 1)
    uint32_t *d_w0off = nullptr;    // per-var initial watch list offsets
    int32_t *d_w0ent = nullptr;     // int4 per entry: clause, offset, length, packed watches
    int64_t device_bytes = 0;
    bool uploaded = false;
};

namespace gpsat {
int formula_upload(gpsat_formula *f);
}
