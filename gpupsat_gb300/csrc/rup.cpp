// Host checker of UNSAT proofs: reverse unit propagation (RUP) over a clause
// log.  Independent of the device solver that wrote the log (its own data
// structures, its own propagation), it certifies that a formula, with a cube
// of assumption literals, is unsatisfiable: each logged clause must follow
// from the formula, the cube and the clauses logged before it by unit
// propagation alone (asserting the negation of every literal of the clause
// propagates to a conflict), and unit propagation over everything must end in
// a conflict.  The reference has no proof output (its UNSAT verdict is the
// search's word, SATSolver/SATSolver.cu:160-168); this checker is what lets a
// verdict the reference cannot reach within its iteration cap be certified.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace gpsat {
namespace {

// Two watched literals over a growing clause store; level-0 facts persist,
// a RUP check assigns above them and is undone.
struct Rup {
    int32_t n;
    std::vector<int32_t> lits;       // clause literals (internal encoding), CSR
    std::vector<int64_t> start;      // clause start in lits; size = clauses + 1
    std::vector<std::vector<int32_t>> watch;  // per literal: clauses watching it
    std::vector<int8_t> val;         // per variable: 0 free, 1 true, -1 false
    std::vector<int32_t> trail;
    size_t qhead = 0;

    explicit Rup(int32_t nv) : n(nv), start(1, 0), watch(2 * (size_t)nv), val(nv, 0) {}

    int value(int32_t l) const
    {
        const int v = val[l >> 1];
        return (l & 1) ? v : -v;
    }
    void assign(int32_t l)
    {
        val[l >> 1] = (l & 1) ? 1 : -1;
        trail.push_back(l);
    }
    // unit propagation from qhead; false on a conflict
    bool propagate()
    {
        while (qhead < trail.size()) {
            const int32_t p = trail[qhead++];
            const int32_t fl = p ^ 1;   // the literal that just became false
            std::vector<int32_t> &ws = watch[fl];
            size_t i = 0, j = 0;
            bool conflict = false;
            while (i < ws.size()) {
                const int32_t c = ws[i++];
                int32_t *L = &lits[start[c]];
                const int64_t len = start[c + 1] - start[c];
                if (L[0] == fl) std::swap(L[0], L[1]);
                if (value(L[0]) == 1) {
                    ws[j++] = c;
                    continue;
                }
                bool moved = false;
                for (int64_t k = 2; k < len; k++) {
                    if (value(L[k]) != -1) {
                        std::swap(L[1], L[k]);
                        watch[L[1]].push_back(c);
                        moved = true;
                        break;
                    }
                }
                if (moved) continue;
                ws[j++] = c;
                if (value(L[0]) == -1) {
                    conflict = true;
                    while (i < ws.size()) ws[j++] = ws[i++];
                    break;
                }
                assign(L[0]);
            }
            ws.resize(j);
            if (conflict) return false;
        }
        return true;
    }
    void undo_to(size_t mark)
    {
        while (trail.size() > mark) {
            val[trail.back() >> 1] = 0;
            trail.pop_back();
        }
        qhead = std::min(qhead, mark);
    }
    // Adds a clause at level 0 (nothing above level 0 is assigned).  Returns
    // false when it leaves level 0 in conflict.
    bool add(const int32_t *c, int64_t len)
    {
        // the two watches: literals not false at level 0 come first
        std::vector<int32_t> cl(c, c + len);
        std::stable_partition(cl.begin(), cl.end(), [&](int32_t l) { return value(l) != -1; });
        const int32_t id = (int32_t)start.size() - 1;
        lits.insert(lits.end(), cl.begin(), cl.end());
        start.push_back((int64_t)lits.size());
        if (len == 0) return false;
        if (len == 1 || value(cl[1]) == -1) {
            // at most one literal is not false: unit or conflicting at level 0
            if (value(cl[0]) == -1) return false;
            if (len >= 2) {
                watch[cl[0]].push_back(id);
                watch[cl[1]].push_back(id);
            }
            if (value(cl[0]) == 0) assign(cl[0]);
            return propagate();
        }
        watch[cl[0]].push_back(id);
        watch[cl[1]].push_back(id);
        return true;
    }
};

}  // namespace
}  // namespace gpsat

using namespace gpsat;

extern "C" int gpsat_check_rup(const int32_t *lits, const int64_t *offsets, int64_t n_clauses, int32_t n_vars,
                               const int32_t *assumptions, int32_t n_assumptions, const int32_t *proof,
                               int64_t proof_len, int64_t *failed_step)
{
    if (failed_step) *failed_step = -1;
    if (n_vars <= 0 || n_clauses < 0 || (n_clauses > 0 && (!lits || !offsets)) || n_assumptions < 0 ||
        (n_assumptions > 0 && !assumptions) || proof_len < 0 || (proof_len > 0 && !proof))
        return set_error(GPSAT_ERR_ARG, "gpsat_check_rup: bad argument");
    auto conv = [&](int32_t d, int32_t &out) {
        if (d == 0 || d > n_vars || d < -n_vars) return false;
        out = lit_of_dimacs(d);
        return true;
    };
    Rup R(n_vars);
    std::vector<int32_t> buf;
    bool refuted = false;
    for (int64_t c = 0; c < n_clauses && !refuted; c++) {
        if (offsets[c + 1] < offsets[c]) return set_error(GPSAT_ERR_FORMULA, "gpsat_check_rup: offsets go back");
        buf.clear();
        for (int64_t i = offsets[c]; i < offsets[c + 1]; i++) {
            int32_t l;
            if (!conv(lits[i], l)) return set_error(GPSAT_ERR_FORMULA, "gpsat_check_rup: literal out of range");
            buf.push_back(l);
        }
        // a tautology holds everywhere; a repeated literal counts once
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
        bool taut = false;
        for (size_t i = 1; i < buf.size(); i++) taut |= (buf[i] >> 1) == (buf[i - 1] >> 1);
        if (taut) continue;
        if (!R.add(buf.data(), (int64_t)buf.size())) refuted = true;
    }
    for (int32_t k = 0; k < n_assumptions && !refuted; k++) {
        int32_t l;
        if (!conv(assumptions[k], l)) return set_error(GPSAT_ERR_ARG, "gpsat_check_rup: assumption out of range");
        const int v = R.value(l);
        if (v == -1) refuted = true;
        else if (v == 0) {
            R.assign(l);
            if (!R.propagate()) refuted = true;
        }
    }
    if (!refuted && !R.propagate()) refuted = true;
    // the log: [len, literal...] per clause
    int64_t pos = 0, step = 0;
    while (!refuted && pos < proof_len) {
        const int64_t len = proof[pos];
        if (len < 0 || pos + 1 + len > proof_len)
            return set_error(GPSAT_ERR_FORMULA, "gpsat_check_rup: malformed proof log");
        buf.clear();
        for (int64_t i = 0; i < len; i++) {
            int32_t l;
            if (!conv(proof[pos + 1 + i], l))
                return set_error(GPSAT_ERR_FORMULA, "gpsat_check_rup: proof literal out of range");
            buf.push_back(l);
        }
        // RUP: the negation of the clause propagates to a conflict
        const size_t mark = R.trail.size();
        bool conflict = false;
        for (int32_t l : buf) {
            const int v = R.value(l);
            if (v == 1) {
                conflict = true;   // a literal true at level 0: its negation conflicts at once
                break;
            }
            if (v == 0) R.assign(l ^ 1);
        }
        if (!conflict) conflict = !R.propagate();
        R.undo_to(mark);
        if (!conflict) {
            if (failed_step) *failed_step = step;
            return 0;
        }
        if (!R.add(buf.data(), (int64_t)buf.size())) refuted = true;
        pos += 1 + len;
        step++;
    }
    if (refuted) return 1;
    if (failed_step) *failed_step = step;   // the log ended without a conflict at level 0
    return 0;
}
