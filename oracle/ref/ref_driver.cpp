/*
 * ORACLE -- test infrastructure only.
 *
 * C entry points over the reference's own solver classes, compiled for the
 * host by oracle/ref/build_ref.py (output in oracle/_ref/).  Nothing here is
 * shipped; tests use it to pin the C restatement (oracle/bcp_ref.c) and the
 * GPU path against the reference itself, and bench.py's reference arm times it.
 *
 * ref_solve mirrors the reference's sequential path: main() reading a formula
 * (SATSolver/main.cu:109-216) then run_sequential (SATSolver/Parallelizer.cu:230-277),
 * except that it calls solve() with an assumptions vector that outlives the
 * call -- the reference's solve() overload keeps a pointer to a stack vector
 * (SATSolver/SATSolver.cu:51-62) that get_results() later reads.
 *
 * ref_bcp mirrors the reference's trail application: assign every literal
 * (SATSolver/VariablesStateHandler.cu:334-341), then
 * WatchedClausesList::new_decision per literal with one shared pending list,
 * stopping at the first conflict (ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu:56-73).
 */
#include <chrono>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "BCPStrategy/WatchedClausesList.cuh"
#include "ConflictAnalysis/ConflictAnalyzer.cuh"
#include "FileManager/FormulaData.cuh"
#include "JobsManager/VariableChooser.cuh"
#include "SATSolver/SATSolver.cuh"
#include "SATSolver/VariablesStateHandler.cuh"
#include "Statistics/RuntimeStatistics.cuh"

namespace {

// Builds the reference's FormulaData from DIMACS CSR input (same calls as
// CnfManager::read_cnf, FileManager/CnfReader.cpp:86-135: add_clause per
// clause, n_vars = highest variable, then copy_host_clauses_to_dev, which runs
// the preprocessing).
FormulaData *make_formula(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses)
{
    FormulaData *fd = new FormulaData((int)n_clauses + 1, true);
    std::vector<Lit> buf;
    for (int64_t c = 0; c < n_clauses; c++) {
        buf.clear();
        for (int64_t i = off[c]; i < off[c + 1]; i++) {
            int32_t d = lits[i];
            buf.push_back(mkLit((d > 0 ? d : -d) - 1, d > 0));
        }
        fd->add_clause(buf.data(), (int)buf.size());
    }
    fd->set_n_vars(n_vars);
    fd->copy_host_clauses_to_dev();
    return fd;
}

}  // namespace

extern "C" {

/* Returns 10 (SAT), 20 (UNSAT), 0 (UNDEF: the reference's iteration cap),
 * negative on bad input.  model[v] = +1 / -1 for SAT, in the reference's
 * printed form (decisions, implications and preprocessing-fixed literals;
 * anything else printed positive, SATSolver/Results.cu:106-135). */
int ref_solve(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, int32_t *model)
{
    if (n_vars <= 0 || n_clauses < 0) return -1;
    FormulaData *fd = make_formula(lits, off, n_vars, n_clauses);
    std::vector<int32_t> asg(n_vars, 0);
    for (Lit l : fd->get_solved_literals()) asg[var(l)] = sign(l) ? 1 : -1;
    int verdict;
    sat_status pre = fd->get_status_after_preprocessing();
    if (pre != sat_status::UNDEF) {
        verdict = pre == sat_status::SAT ? 10 : 20;
    } else {
        CUDAClauseVec formula = fd->get_formula_dev();
        std::vector<Var> dead;
        for (Lit l : fd->get_solved_literals()) dead.push_back(var(l));
        GPUVecView<Var> dead_view(dead.data(), dead.size(), dead.size());
        RuntimeStatistics stats(1, 1, nullptr);
        auto *repo = new NodesRepository<GPULinkedList<WatchedClause *>::Node>(MAX_NUMBER_OF_NODES);
        std::vector<Var> fv(n_vars);
        std::vector<Decision> dec(n_vars), imp(n_vars);
        int mipv = std::max(fd->get_largest_clause_size(), MIN_IMPLICATION_PER_VAR);
        auto *solver = new SATSolver(&formula, n_vars, mipv, &dead_view, &stats, repo, fv.data(), dec.data(),
                                     imp.data());
        auto *no_assumptions = new GPUStaticVec<Lit>();
        sat_status st = solver->solve(no_assumptions);
        if (st == sat_status::SAT) {
            verdict = 10;
            std::vector<Lit> res(solver->get_results_size());
            solver->get_results(res.data());
            for (Lit l : res) asg[var(l)] = sign(l) ? 1 : -1;
        } else if (st == sat_status::UNSAT) {
            verdict = 20;
        } else {
            verdict = 0;
        }
        // the reference leaks its per-thread structures too; the process is short-lived
    }
    if (model)
        for (int32_t v = 0; v < n_vars; v++) model[v] = asg[v] == -1 ? -1 : 1;
    return verdict;
}

int ref_bcp_timed(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, const int32_t *trail,
                  int64_t trail_len, int64_t cap, int32_t *impl_lit, int32_t *impl_reason, int64_t *n_impl,
                  int32_t *conflict_clause, int32_t *stop_index, double *seconds);

/* Returns 0 (no conflict), 1 (conflict), -2 (a variable given both signs),
 * -3 (preprocessing decided the formula), -1 (implication capacity). */
int ref_bcp(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, const int32_t *trail,
            int64_t trail_len, int64_t cap, int32_t *impl_lit, int32_t *impl_reason, int64_t *n_impl,
            int32_t *conflict_clause, int32_t *stop_index)
{
    return ref_bcp_timed(lits, off, n_vars, n_clauses, trail, trail_len, cap, impl_lit, impl_reason, n_impl,
                         conflict_clause, stop_index, nullptr);
}

/* ref_bcp, and with seconds != NULL the wall time of the trail application
 * alone (the assignments and the new_decision calls), without the set-up of
 * the formula and the watch lists that precedes it. */
int ref_bcp_timed(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, const int32_t *trail,
                  int64_t trail_len, int64_t cap, int32_t *impl_lit, int32_t *impl_reason, int64_t *n_impl,
                  int32_t *conflict_clause, int32_t *stop_index, double *seconds)
{
    *n_impl = 0;
    *conflict_clause = -1;
    *stop_index = -1;
    FormulaData *fd = make_formula(lits, off, n_vars, n_clauses);
    if (fd->get_status_after_preprocessing() != sat_status::UNDEF) return -3;
    CUDAClauseVec formula = fd->get_formula_dev();
    std::unordered_map<const Lit *, int32_t> index;
    for (int i = 0; i < formula.size_of(); i++) index[formula.get_ptr(i)->literals] = i;
    std::vector<Var> dead;
    for (Lit l : fd->get_solved_literals()) dead.push_back(var(l));
    GPUVecView<Var> dead_view(dead.data(), dead.size(), dead.size());
    std::vector<Var> fv(n_vars);
    std::vector<Decision> dec(n_vars + trail_len), imp(n_vars);
    auto *handler = new VariablesStateHandler(n_vars, &dead_view, nullptr, fv.data(), dec.data(), imp.data());
    auto *repo = new NodesRepository<GPULinkedList<WatchedClause *>::Node>(MAX_NUMBER_OF_NODES);
    auto *wcl = new WatchedClausesList(n_vars, handler, repo, formula.size_of());
    wcl->add_all_clauses(formula);
    handler->set_decision_level(1);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<Decision> ds;
    for (int64_t i = 0; i < trail_len; i++) {
        int32_t d = trail[i];
        Decision x;
        x.literal = mkLit((d > 0 ? d : -d) - 1, d > 0);
        x.decision_level = 1;
        x.branched = false;
        sat_status cur = handler->literal_status(x.literal);
        if (cur == sat_status::UNSAT) return -2;
        handler->new_decision(x);
        ds.push_back(x);
    }
    GPULinkedList<found_implication> pending;
    int rc = 0;
    for (int64_t i = 0; i < trail_len; i++) {
        const Clause *confl = nullptr;
        sat_status st = wcl->new_decision(ds[i], &confl, pending);
        if (st == sat_status::UNSAT) {
            *conflict_clause = index.at(confl->literals);
            *stop_index = (int32_t)i;
            rc = 1;
            break;
        }
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    auto it = pending.get_iterator();
    int64_t k = 0;
    while (it.has_next()) {
        found_implication fi = it.get_next();
        if (k >= cap) return -1;
        Lit l = fi.implication.literal;
        impl_lit[k] = sign(l) ? var(l) + 1 : -(var(l) + 1);
        impl_reason[k] = index.at(fi.implicating_clause->literals);
        k++;
    }
    *n_impl = k;
    return rc;
}

/* The reference's split-variable ranking: VariableChooser::evaluate over the
 * preprocessed clauses, as MaxClauseJobChooser uses it (SATSolver/main.cu:221,
 * JobsManager/VariableChooser.cu:23-40).  order[i] = 1-based variable at rank
 * i, score[i] its evaluation; returns the number of ranked variables. */
int ref_rank_vars(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, int32_t *order,
                  int32_t *score)
{
    FormulaData *fd = make_formula(lits, off, n_vars, n_clauses);
    std::vector<Clause> const &formula = *fd->get_formula_host();
    VariableChooser vc(formula, (size_t)n_vars);
    vc.evaluate();
    // the evaluation of each variable, recomputed the way evaluate() sums it
    std::vector<int32_t> ev(n_vars, 0);
    for (Clause const &c : formula)
        for (size_t j = 0; j < c.n_lits; j++) ev[var(c.literals[j])] += var(c.literals[j]);
    int32_t k = 0;
    while (vc.has_next_var() && k < n_vars) {
        Var v = vc.next_var();
        order[k] = (int32_t)v + 1;
        score[k] = ev[v];
        k++;
    }
    return k;
}

namespace {
// The reference's full-scan clause evaluation (BASIC_SEARCH) is a protected
// member; a subclass calls it as the reference's own propagate() does.
struct FullScan : public ConflictAnalyzer {
    using ConflictAnalyzer::ConflictAnalyzer;
    sat_status sweep(Decision d, const Clause **confl) { return propagate_all_clauses(d, confl); }
};
}  // namespace

/* The reference's full-scan clause evaluation over a trail: every trail
 * literal assigned as ref_bcp does, then ConflictAnalyzer::propagate_all_clauses
 * (ConflictAnalysis/ConflictAnalyzer.cu:173-245).  Returns 0 (no conflict),
 * 1 (conflict, *conflict_clause set), -2 (a variable given both signs), -3
 * (preprocessing decided the formula), -1 (implication capacity); the implied
 * literals in the order the sweeps found them. */
int ref_scan(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, const int32_t *trail,
             int64_t trail_len, int64_t cap, int32_t *impl_lit, int64_t *n_impl, int32_t *conflict_clause)
{
    *n_impl = 0;
    *conflict_clause = -1;
    FormulaData *fd = make_formula(lits, off, n_vars, n_clauses);
    if (fd->get_status_after_preprocessing() != sat_status::UNDEF) return -3;
    CUDAClauseVec formula = fd->get_formula_dev();
    std::unordered_map<const Lit *, int32_t> index;
    for (int i = 0; i < formula.size_of(); i++) index[formula.get_ptr(i)->literals] = i;
    std::vector<Var> dead;
    for (Lit l : fd->get_solved_literals()) dead.push_back(var(l));
    GPUVecView<Var> dead_view(dead.data(), dead.size(), dead.size());
    std::vector<Var> fv(n_vars);
    std::vector<Decision> dec(n_vars + trail_len), imp(n_vars);
    auto *handler = new VariablesStateHandler(n_vars, &dead_view, nullptr, fv.data(), dec.data(), imp.data());
    handler->set_decision_level(1);
    Decision last;
    last.literal = mkLit(0, true);
    last.decision_level = 1;
    last.branched = false;
    last.implicated_from_formula = false;
    for (int64_t i = 0; i < trail_len; i++) {
        int32_t d = trail[i];
        Decision x;
        x.literal = mkLit((d > 0 ? d : -d) - 1, d > 0);
        x.decision_level = 1;
        x.branched = false;
        x.implicated_from_formula = false;
        sat_status cur = handler->literal_status(x.literal);
        if (cur == sat_status::UNSAT) return -2;
        if (cur == sat_status::UNDEF) handler->new_decision(x);
        last = x;
    }
    RuntimeStatistics stats(1, 1, nullptr);
    auto *fs = new FullScan(n_vars, &formula, handler, false, 1, nullptr, &stats);
    const Clause *confl = nullptr;
    sat_status st = fs->sweep(last, &confl);
    const int64_t k = (int64_t)handler->n_implications();
    if (k > cap) return -1;
    for (int64_t i = 0; i < k; i++) {
        Lit l = handler->get_implication(i)->literal;
        impl_lit[i] = sign(l) ? var(l) + 1 : -(var(l) + 1);
    }
    *n_impl = k;
    if (st == sat_status::UNSAT) {
        *conflict_clause = index.at(confl->literals);
        return 1;
    }
    return 0;
}

/* Clauses after the reference's preprocessing and its initial watches. */
int ref_preprocess(const int32_t *lits, const int64_t *off, int32_t n_vars, int64_t n_clauses, int32_t *out_lits,
                   int64_t *out_off, int64_t *out_n_clauses, int32_t *watch1, int32_t *watch2, int32_t *verdict)
{
    FormulaData *fd = make_formula(lits, off, n_vars, n_clauses);
    sat_status pre = fd->get_status_after_preprocessing();
    *verdict = pre == sat_status::UNDEF ? 0 : pre == sat_status::SAT ? 10 : 20;
    *out_n_clauses = 0;
    out_off[0] = 0;
    if (pre != sat_status::UNDEF) return 0;
    CUDAClauseVec formula = fd->get_formula_dev();
    int64_t p = 0;
    for (int i = 0; i < formula.size_of(); i++) {
        Clause c = formula.get(i);
        for (unsigned j = 0; j < c.n_lits; j++) {
            Lit l = c.literals[j];
            out_lits[p++] = sign(l) ? var(l) + 1 : -(var(l) + 1);
        }
        out_off[i + 1] = p;
    }
    *out_n_clauses = formula.size_of();
    // initial watches: read back from a freshly built watch structure
    std::vector<Var> dead;
    for (Lit l : fd->get_solved_literals()) dead.push_back(var(l));
    GPUVecView<Var> dead_view(dead.data(), dead.size(), dead.size());
    std::vector<Var> fv(n_vars);
    std::vector<Decision> dec(n_vars), imp(n_vars);
    auto *handler = new VariablesStateHandler(n_vars, &dead_view, nullptr, fv.data(), dec.data(), imp.data());
    auto *repo = new NodesRepository<GPULinkedList<WatchedClause *>::Node>(MAX_NUMBER_OF_NODES);
    auto *wcl = new WatchedClausesList(n_vars, handler, repo, formula.size_of());
    wcl->add_all_clauses(formula);
    // every clause is in the list of both watched vars; recover the watched
    // positions by membership (the lists hold each clause under exactly the
    // two vars it watches)
    for (int i = 0; i < formula.size_of(); i++) {
        Clause c = formula.get(i);
        int a = -1, b = -1;
        for (unsigned j = 0; j < c.n_lits; j++) {
            if (wcl->contains(var(c.literals[j]), c)) {
                if (a < 0) a = (int)j;
                else b = (int)j;
            }
        }
        watch1[i] = a;
        watch2[i] = b;
    }
    return 0;
}

}  // extern "C"
