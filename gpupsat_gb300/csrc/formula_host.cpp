// Host-side formula preparation: input validation, the reference's
// preprocessing and its initial two-watch choice.
//
// The preprocessing is kept semantically identical to the reference's because
// it decides clause order and literal order, and the BCP batch reports clause
// indices of the preprocessed formula:
//   RepeatedLiteralsRemover  reference Preprocessing/RepeatedLiteralsRemover.cu:25-62
//   UnaryClausesRemover      reference Preprocessing/UnaryClausesRemover.cu:75-235
// The data structures (flat CSR arrays, a stamped per-var table instead of a
// per-clause std::fill over all variables) are this file's own.
#include <algorithm>
#include <climits>
#include <cstring>

#include "internal.h"

namespace gpsat {

namespace {

// One pass of duplicate-literal / tautology removal (reference
// RepeatedLiteralsRemover::process_clause): scanning left to right, a literal
// whose variable was already seen with the same sign is dropped; a variable
// seen with both signs removes the whole clause.
struct Cnf {
    std::vector<std::vector<int32_t>> cls;
};

void remove_repeated(Cnf &f, int32_t n_vars)
{
    std::vector<int32_t> stamp(n_vars, -1);
    std::vector<int8_t> sgn(n_vars, 0);
    std::vector<std::vector<int32_t>> kept;
    kept.reserve(f.cls.size());
    int32_t cid = 0;
    for (auto &c : f.cls) {
        std::vector<int32_t> out;
        out.reserve(c.size());
        bool taut = false;
        for (int32_t l : c) {
            int32_t v = l >> 1;
            int8_t s = (int8_t)(l & 1);
            if (stamp[v] != cid) {
                stamp[v] = cid;
                sgn[v] = s;
                out.push_back(l);
            } else if (sgn[v] != s) {
                taut = true;
                break;
            }
            // same sign: dropped
        }
        cid++;
        if (!taut) kept.push_back(std::move(out));
    }
    f.cls.swap(kept);
}

// Reference UnaryClausesRemover: unit clauses become solved literals (a
// repeated unit clause is kept in the formula, a contradicting one sets
// UNSAT), then passes of propagate_literals until no new literal is solved.
struct UnitRemover {
    Cnf &f;
    int32_t n_vars;
    std::vector<int32_t> solved;
    std::vector<int8_t> val;  // 0 unknown, 1 literal with sign 1 solved, 2 sign 0 solved
    int32_t status = GPSAT_UNKNOWN;

    UnitRemover(Cnf &f_, int32_t n) : f(f_), n_vars(n), val(n, 0) {}

    bool in_solved(int32_t l) const { return val[l >> 1] == ((l & 1) ? 1 : 2); }
    bool neg_in_solved(int32_t l) const { return val[l >> 1] == ((l & 1) ? 2 : 1); }

    // reference UnaryClausesRemover::add
    bool add(int32_t l)
    {
        if (in_solved(l)) return false;
        if (neg_in_solved(l)) {
            status = GPSAT_UNSAT;
            return false;
        }
        solved.push_back(l);
        val[l >> 1] = (l & 1) ? 1 : 2;
        return true;
    }

    void process_unary()
    {
        std::vector<std::vector<int32_t>> kept;
        kept.reserve(f.cls.size());
        for (auto &c : f.cls) {
            if (c.size() == 1 && add(c[0])) continue;  // removed
            kept.push_back(std::move(c));
        }
        f.cls.swap(kept);
    }

    // reference UnaryClausesRemover::propagate_literals
    void propagate()
    {
        std::vector<std::vector<int32_t>> kept;
        kept.reserve(f.cls.size());
        size_t i = 0;
        for (; i < f.cls.size(); i++) {
            auto &c = f.cls[i];
            size_t unsat = 0;
            bool sat = false;
            int32_t unit = -1;
            for (int32_t l : c) {
                if (in_solved(l)) {
                    sat = true;
                    break;
                }
                if (neg_in_solved(l)) unsat++;
                else unit = l;
            }
            if (sat) {
                unit = -1;
                continue;  // erased
            }
            if (unsat != c.size() - 1) unit = -1;
            if (unit != -1) {
                add(unit);
                if (status == GPSAT_UNSAT) {
                    // the reference returns here, leaving the rest untouched
                    kept.push_back(std::move(c));
                    for (size_t j = i + 1; j < f.cls.size(); j++) kept.push_back(std::move(f.cls[j]));
                    f.cls.swap(kept);
                    return;
                }
                continue;  // erased
            }
            if (unsat == c.size()) {
                status = GPSAT_UNSAT;
                kept.push_back(std::move(c));
                for (size_t j = i + 1; j < f.cls.size(); j++) kept.push_back(std::move(f.cls[j]));
                f.cls.swap(kept);
                return;
            }
            // clean_clause: drop literals whose negation is solved
            std::vector<int32_t> out;
            out.reserve(c.size());
            for (int32_t l : c)
                if (!neg_in_solved(l)) out.push_back(l);
            kept.push_back(std::move(out));
        }
        f.cls.swap(kept);
        if (f.cls.empty()) status = GPSAT_SAT;
    }

    void process()
    {
        process_unary();
        if (status != GPSAT_UNKNOWN) return;
        size_t last = 0, cur = solved.size();
        while (cur != last) {
            propagate();
            if (status != GPSAT_UNKNOWN) return;
            last = cur;
            cur = solved.size();
        }
    }
};

}  // namespace

int prepare_formula(const int32_t *lits, const int64_t *offsets, int32_t n_vars, int64_t n_clauses,
                    HostFormula &out)
{
    if (n_vars <= 0 || n_clauses < 0) return set_error(GPSAT_ERR_ARG, "n_vars must be > 0 and n_clauses >= 0");
    if (n_clauses > 0 && (!lits || !offsets)) return set_error(GPSAT_ERR_ARG, "null clause arrays");
    if (n_clauses >= INT32_MAX / 2) return set_error(GPSAT_ERR_CAPACITY, "too many clauses (limit 2^30)");
    if (offsets && offsets[0] != 0) return set_error(GPSAT_ERR_FORMULA, "offsets[0] must be 0");
    Cnf f;
    f.cls.reserve(n_clauses);
    bool has_empty = false;  // an empty clause: the formula is unsatisfiable
    for (int64_t c = 0; c < n_clauses; c++) {
        int64_t b = offsets[c], e = offsets[c + 1];
        if (e < b) return set_error(GPSAT_ERR_FORMULA, "offsets must be non-decreasing");
        if (e == b) {
            has_empty = true;
            continue;
        }
        f.cls.emplace_back();
        auto &cl = f.cls.back();
        cl.resize(e - b);
        for (int64_t i = b; i < e; i++) {
            int32_t d = lits[i];
            if (d == 0 || d > n_vars || d < -n_vars)
                return set_error(GPSAT_ERR_FORMULA, "literal " + std::to_string(d) + " out of range in clause " +
                                                        std::to_string(c));
            cl[i - b] = lit_of_dimacs(d);
        }
    }
    out = HostFormula();
    out.n_vars = n_vars;
    remove_repeated(f, n_vars);
    if (has_empty) out.verdict = GPSAT_UNSAT;
    else if (f.cls.empty()) out.verdict = GPSAT_SAT;
    if (out.verdict == GPSAT_UNKNOWN) {
        UnitRemover ur(f, n_vars);
        ur.process();
        out.verdict = ur.status;
        out.solved = ur.solved;
    }
    // the reference uploads the clause set only when preprocessing left it
    // undecided (FileManager/FormulaData.cu:99-101)
    out.off.push_back(0);
    if (out.verdict == GPSAT_UNKNOWN) {
        int64_t total = 0;
        for (auto &c : f.cls) total += (int64_t)c.size();
        if (total >= INT32_MAX) return set_error(GPSAT_ERR_CAPACITY, "too many literals (limit 2^31)");
        out.lits.reserve(total);
        for (auto &c : f.cls) {
            out.lits.insert(out.lits.end(), c.begin(), c.end());
            out.off.push_back((int64_t)out.lits.size());
            out.max_len = std::max<int32_t>(out.max_len, (int32_t)c.size());
        }
    }
    return GPSAT_OK;
}

// Initial watches (reference ClauseListStructure::watch_clause and
// get_two_literals_with_fewer_clauses, BCPStrategy/ClauseListStructure.cu:101-148,
// driven by WatchedClausesList::add_all_clauses, WatchedClausesList.cu:356-364):
// clauses are taken in order; each watches the two literals whose variables
// currently have the fewest watching clauses (strict '<', earlier literal wins
// ties) and is add_first'ed to both lists, so every list ends up in
// decreasing clause order.  Clauses of length 1 are never watched.
void build_initial_watches(HostFormula &f)
{
    const int64_t m = f.n_clauses();
    f.w1.assign(m, -1);
    f.w2.assign(m, -1);
    std::vector<uint32_t> size(f.n_vars, 0);
    for (int64_t c = 0; c < m; c++) {
        int64_t b = f.off[c], k = f.off[c + 1] - b;
        if (k < 2) continue;
        uint64_t sv = (uint64_t)INT32_MAX - 1, sv2 = (uint64_t)INT32_MAX;
        int32_t s1 = -1, s2 = -1;
        for (int64_t i = 0; i < k; i++) {
            uint64_t cur = size[f.lits[b + i] >> 1];
            if (cur < sv) {
                s2 = s1;
                sv2 = sv;
                sv = cur;
                s1 = (int32_t)i;
            } else if (cur < sv2) {
                sv2 = cur;
                s2 = (int32_t)i;
            }
        }
        f.w1[c] = s1;
        f.w2[c] = s2;
        size[f.lits[b + s1] >> 1]++;
        size[f.lits[b + s2] >> 1]++;
    }
    f.w0off.assign((size_t)f.n_vars + 1, 0);
    for (int32_t v = 0; v < f.n_vars; v++) f.w0off[v + 1] = f.w0off[v] + size[v];
    f.w0cl.assign(f.w0off[f.n_vars], 0);
    std::vector<uint32_t> fill(f.w0off.begin(), f.w0off.end() - 1);
    for (int64_t c = m - 1; c >= 0; c--) {
        if (f.w1[c] < 0) continue;
        int32_t v1 = f.lits[f.off[c] + f.w1[c]] >> 1, v2 = f.lits[f.off[c] + f.w2[c]] >> 1;
        f.w0cl[fill[v1]++] = (int32_t)c;
        f.w0cl[fill[v2]++] = (int32_t)c;
    }
}

}  // namespace gpsat
