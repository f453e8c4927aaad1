// gpsat C++ host interface (header-only, over the C ABI in gpsat.h).
//
// Keeps the roles of the reference solver's building blocks as C++ types so
// host code written against them reads the same; each strategy object writes
// its part of gpsat_solve_options, and the device runs the chosen variant
// inside one kernel (there are no per-operation host calls).
//
//   BCPStrategy, TrailPropagator
//                      reference BCPStrategy/WatchedClausesList.cuh:33-67
//   DecisionStrategy   reference SATSolver/DecisionMaker.cuh:11-29, DecisionStrategy/VSIDS.cuh
//   ConflictAnalysis   reference ConflictAnalysis/ConflictAnalyzer.cuh:24-62
//   ClauseLearning     reference ClauseLearning/LearntClausesManager.cuh:8-27
//   Restarts           reference Restarts/RestartsManager.cuh:4-9, GeometricRestartsManager.cuh
//   JobChooser, JobsQueue, MaxClauseJobChooser, SimpleJobChooser
//                      reference JobsManager/JobChooser.cuh:21-72, SimpleJobChooser.cuh,
//                      SATSolver/JobsQueue.cuh:19-45
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <memory>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpsat.h"

namespace gpsat {

class Error : public std::runtime_error {
public:
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc, const char *what)
{
    if (rc != GPSAT_OK)
        throw Error(rc, std::string(what) + ": " + gpsat_error_string(rc) + ": " + gpsat_last_error());
}

// ---------------------------------------------------------------- formula
struct Cnf {
    int32_t n_vars = 0;
    int32_t header_vars = 0;
    int64_t header_clauses = 0;
    std::vector<int32_t> lits;     // DIMACS literals
    std::vector<int64_t> offsets;  // n_clauses + 1
    int64_t n_clauses() const { return (int64_t)offsets.size() - 1; }
};

inline Cnf parse_dimacs(const std::string &text)
{
    Cnf f;
    int64_t nc = 0, nl = 0;
    check(gpsat_dimacs_parse(text.data(), (int64_t)text.size(), &f.n_vars, &nc, &nl, &f.header_vars,
                             &f.header_clauses, nullptr, nullptr),
          "parse");
    f.lits.resize(nl);
    f.offsets.resize(nc + 1);
    check(gpsat_dimacs_parse(text.data(), (int64_t)text.size(), &f.n_vars, &nc, &nl, &f.header_vars,
                             &f.header_clauses, f.lits.data(), f.offsets.data()),
          "parse");
    return f;
}

inline Cnf read_dimacs(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw Error(GPSAT_ERR_ARG, "cannot open " + path);
    std::stringstream ss;
    ss << in.rdbuf();
    return parse_dimacs(ss.str());
}

// A preprocessed formula held by the library (gpsat_formula).
class Formula {
public:
    explicit Formula(const Cnf &f)
    {
        check(gpsat_formula_create(f.lits.data(), f.offsets.data(), std::max(f.n_vars, 1), f.n_clauses(), &h_),
              "formula");
    }
    ~Formula() { gpsat_formula_destroy(h_); }
    Formula(const Formula &) = delete;
    Formula &operator=(const Formula &) = delete;
    const gpsat_formula *get() const { return h_; }

private:
    gpsat_formula *h_ = nullptr;
};

// ---------------------------------------------------------------- BCP over trails
// The outcome of applying one trail the way the reference applies
// assumptions: every literal assigned, then WatchedClausesList::new_decision
// per literal in order, depth-first over implications, until the first
// conflict (reference BCPStrategy/WatchedClausesList.cu:46-101,
// ConflictAnalysis/ConflictAnalyzerWithWatchedLits.cu:56-73).
struct TrailOutcome {
    int32_t status = GPSAT_BCP_NO_CONFLICT;  // GPSAT_BCP_*
    int32_t conflict_clause = -1;            // preprocessed clause index
    int32_t stop_index = -1;                 // trail position that met the conflict
    std::vector<int32_t> implied;            // DIMACS literals, in the reference's order
    std::vector<int32_t> reasons;            // implying clause of each
    int64_t counters[GPSAT_BCP_NCOUNTERS] = {};
};

// The BCPStrategy role over many partial trails at once (gpsat_bcp_*): the
// device runs each trail's propagation in the reference's order.
class TrailPropagator {
public:
    TrailPropagator(const Formula &f, int64_t impl_cap, int32_t max_slots = 0, int64_t arena_cap = 0)
        : cap_(impl_cap)
    {
        check(gpsat_bcp_create(f.get(), max_slots, impl_cap, arena_cap, &h_), "bcp");
    }
    ~TrailPropagator() { gpsat_bcp_destroy(h_); }
    TrailPropagator(const TrailPropagator &) = delete;
    TrailPropagator &operator=(const TrailPropagator &) = delete;

    // The reference's CONFLICT_ANALYSIS_STRATEGY (SATSolver/Configs.cuh:27-33):
    // two watched literals (default) or full-scan clause evaluation
    // (BASIC_SEARCH, ConflictAnalysis/ConflictAnalyzer.cu:173-245).
    void use_full_scan(bool on)
    {
        check(gpsat_bcp_set_strategy(h_, on ? GPSAT_BCP_FULL_SCAN : GPSAT_BCP_WATCHED), "bcp strategy");
    }
    // Launch shape of the two-watched-literal kernel (outputs do not depend
    // on it): watch entries per round (64, 128, 256), trails in flight (0:
    // all resident), and the processing order's length pivot (0: shortest first).
    void set_window(int32_t entries) { check(gpsat_bcp_set_window(h_, entries), "bcp window"); }
    void set_active_slots(int32_t n) { check(gpsat_bcp_set_active_slots(h_, n), "bcp slots"); }
    void set_order_pivot(int64_t pivot) { check(gpsat_bcp_set_order_pivot(h_, pivot), "bcp order pivot"); }

    std::vector<TrailOutcome> new_decisions(const std::vector<std::vector<int32_t>> &trails)
    {
        const int32_t T = (int32_t)trails.size();
        std::vector<int64_t> off(T + 1, 0);
        for (int32_t t = 0; t < T; t++) off[t + 1] = off[t] + (int64_t)trails[t].size();
        std::vector<int32_t> lits;
        lits.reserve(off[T]);
        for (const auto &tr : trails) lits.insert(lits.end(), tr.begin(), tr.end());
        std::vector<int32_t> st(T), cc(T), si(T), il((size_t)T * cap_), ir((size_t)T * cap_);
        std::vector<int64_t> ni(T), cn((size_t)T * GPSAT_BCP_NCOUNTERS);
        check(gpsat_bcp_run_host(h_, lits.data(), off.data(), T, st.data(), cc.data(), si.data(), ni.data(),
                                 il.data(), ir.data(), cn.data()),
              "bcp run");
        std::vector<TrailOutcome> out(T);
        for (int32_t t = 0; t < T; t++) {
            TrailOutcome &o = out[t];
            o.status = st[t];
            o.conflict_clause = cc[t];
            o.stop_index = si[t];
            const size_t b = (size_t)t * cap_, k = (size_t)std::max<int64_t>(0, std::min<int64_t>(ni[t], cap_));
            o.implied.assign(il.begin() + b, il.begin() + b + k);
            o.reasons.assign(ir.begin() + b, ir.begin() + b + k);
            std::copy(cn.begin() + (size_t)t * GPSAT_BCP_NCOUNTERS, cn.begin() + (size_t)(t + 1) * GPSAT_BCP_NCOUNTERS,
                      o.counters);
        }
        return out;
    }

private:
    gpsat_bcp *h_ = nullptr;
    int64_t cap_;
};

// ---------------------------------------------------------------- strategies
struct BCPStrategy {
    virtual ~BCPStrategy() = default;
    virtual void configure(gpsat_solve_options &o) const = 0;
    virtual const char *name() const = 0;
};
// per-literal watch lists with blocker literals, 32 watches per warp step
struct TwoWatchedLiterals : BCPStrategy {
    void configure(gpsat_solve_options &) const override {}
    const char *name() const override { return "two watched literals"; }
};

struct DecisionStrategy {
    virtual ~DecisionStrategy() = default;
    virtual void configure(gpsat_solve_options &o) const = 0;
    virtual const char *name() const = 0;
};
struct VSIDS : DecisionStrategy {
    float decay;
    explicit VSIDS(float d = 0.99f) : decay(d) {}
    void configure(gpsat_solve_options &o) const override
    {
        o.decide = GPSAT_DECIDE_VSIDS;
        o.var_decay = decay;
    }
    const char *name() const override { return "VSIDS"; }
};
// the reference's default when VSIDS is compiled out: last free variable, positive
struct LastFreeVariable : DecisionStrategy {
    void configure(gpsat_solve_options &o) const override { o.decide = GPSAT_DECIDE_LAST_FREE; }
    const char *name() const override { return "last free variable"; }
};

struct ConflictAnalysis {
    virtual ~ConflictAnalysis() = default;
    virtual void configure(gpsat_solve_options &o) const = 0;
    virtual const char *name() const = 0;
};
struct FirstUIP : ConflictAnalysis {
    bool minimize;
    explicit FirstUIP(bool m = true) : minimize(m) {}
    void configure(gpsat_solve_options &o) const override { o.minimize = minimize ? 1 : 0; }
    const char *name() const override { return minimize ? "first UIP, minimised" : "first UIP"; }
};

struct ClauseLearning {
    virtual ~ClauseLearning() = default;
    virtual void configure(gpsat_solve_options &o) const = 0;
    virtual const char *name() const = 0;
};
// keeps learnt clauses, halving the worst by LBD when the limit is reached
struct LearntClauseDatabase : ClauseLearning {
    int32_t first, inc;
    LearntClauseDatabase(int32_t f = 6000, int32_t i = 300) : first(f), inc(i) {}
    void configure(gpsat_solve_options &o) const override
    {
        o.learnt_first = first;
        o.learnt_inc = inc;
    }
    const char *name() const override { return "learnt clause database (LBD)"; }
};

struct Restarts {
    virtual ~Restarts() = default;
    virtual void configure(gpsat_solve_options &o) const = 0;
    virtual const char *name() const = 0;
};
struct GeometricRestarts : Restarts {  // reference defaults: 100 conflicts, x1.3
    int32_t first;
    float factor;
    GeometricRestarts(int32_t f = 100, float x = 1.3f) : first(f), factor(x) {}
    void configure(gpsat_solve_options &o) const override
    {
        o.restart = GPSAT_RESTART_GEOMETRIC;
        o.restart_base = first;
        o.restart_factor = factor;
    }
    const char *name() const override { return "geometric"; }
};
struct LubyRestarts : Restarts {
    int32_t unit;
    explicit LubyRestarts(int32_t u = 400) : unit(u) {}
    void configure(gpsat_solve_options &o) const override
    {
        o.restart = GPSAT_RESTART_LUBY;
        o.restart_base = unit;
    }
    const char *name() const override { return "Luby"; }
};
struct NoRestarts : Restarts {
    void configure(gpsat_solve_options &o) const override { o.restart = GPSAT_RESTART_NONE; }
    const char *name() const override { return "none"; }
};

// ---------------------------------------------------------------- jobs
struct Job {
    std::vector<int32_t> literals;  // DIMACS assumption literals (a cube)
};

class JobsQueue {
public:
    void add(const Job &j)
    {
        jobs_.push_back(j);
        largest_ = std::max(largest_, j.literals.size());
    }
    void close() { closed_ = true; }
    size_t n_jobs() const { return jobs_.size(); }
    size_t largest_job_size() const { return largest_; }
    const std::vector<Job> &jobs() const { return jobs_; }

private:
    std::vector<Job> jobs_;
    size_t largest_ = 0;
    bool closed_ = false;
};

enum class ChoosingStrategy { DISTRIBUTE_JOBS_PER_THREAD, UNIFORM, FIXED };

class JobChooser {
public:
    virtual ~JobChooser() = default;
    virtual void evaluate() = 0;
    virtual void getJobs(JobsQueue &queue) = 0;
    virtual size_t get_n_jobs() = 0;
    virtual bool is_evaluated() = 0;
};

// Splits on `depth` chosen variables and enumerates all 2^depth sign
// assignments, positive first, depth-first (reference MaxClauseJobChooser::addJobs,
// JobsManager/JobChooser.cu:75-100).
class CubeJobChooser : public JobChooser {
public:
    void getJobs(JobsQueue &queue) override
    {
        if (!evaluated_) evaluate();
        std::vector<int32_t> fixed;
        add(fixed, queue);
    }
    size_t get_n_jobs() override { return (size_t)1 << chosen_.size(); }
    bool is_evaluated() override { return evaluated_; }
    const std::vector<int32_t> &chosen() const { return chosen_; }

protected:
    std::vector<int32_t> chosen_;  // 1-based variables
    bool evaluated_ = false;

private:
    void add(std::vector<int32_t> &fixed, JobsQueue &q)
    {
        if (fixed.size() == chosen_.size()) {
            q.add(Job{fixed});
            return;
        }
        const int32_t v = chosen_[fixed.size()];
        fixed.push_back(v);
        add(fixed, q);
        fixed.back() = -v;
        add(fixed, q);
        fixed.pop_back();
    }
};

// Number of split variables from the launch shape, as the reference does
// (JobsManager/JobChooser.cu:115-135: DISTRIBUTE = log2(threads*blocks*10)+1,
// UNIFORM = 7, both capped at 15 and at the free variables minus 2).
inline size_t vars_per_job(ChoosingStrategy s, size_t n_working_vars, size_t threads, size_t blocks,
                           size_t fixed_depth)
{
    const size_t max_by_vars = std::max<size_t>(n_working_vars > 2 ? n_working_vars - 2 : 0, 1);
    size_t d;
    if (s == ChoosingStrategy::DISTRIBUTE_JOBS_PER_THREAD) {
        double expected = (double)threads * blocks * 10.0;
        expected = std::min(expected, std::pow(2.0, (double)std::min<size_t>(max_by_vars, 62)));
        d = (size_t)std::log2(expected) + 1;
    } else if (s == ChoosingStrategy::UNIFORM) {
        d = std::min<size_t>(7, max_by_vars);
    } else {
        d = fixed_depth;
    }
    return std::min<size_t>(std::min<size_t>(d, 15), n_working_vars);
}

// The reference's chooser: variables ranked by (variable index x occurrences),
// the score VariableChooser::evaluate computes (JobsManager/VariableChooser.cu:23-40).
class MaxClauseJobChooser : public CubeJobChooser {
public:
    MaxClauseJobChooser(const Cnf &f, size_t n_threads, size_t n_blocks,
                        ChoosingStrategy s = ChoosingStrategy::DISTRIBUTE_JOBS_PER_THREAD, size_t fixed_depth = 0)
        : f_(f), threads_(n_threads), blocks_(n_blocks), s_(s), fixed_(fixed_depth)
    {
    }
    void evaluate() override
    {
        std::vector<double> score(f_.n_vars + 1, 0.0);
        for (int32_t d : f_.lits) score[std::abs(d)] += (double)(std::abs(d) - 1);
        std::vector<int32_t> order(f_.n_vars);
        std::iota(order.begin(), order.end(), 1);
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return score[a] > score[b]; });
        const size_t k = vars_per_job(s_, f_.n_vars, threads_, blocks_, fixed_);
        chosen_.assign(order.begin(), order.begin() + std::min<size_t>(k, order.size()));
        evaluated_ = true;
    }

private:
    const Cnf &f_;
    size_t threads_, blocks_;
    ChoosingStrategy s_;
    size_t fixed_;
};

// Variables ranked by caller scores (occurrence counts by default, or the
// split scores of the learned model).
class ScoredJobChooser : public CubeJobChooser {
public:
    ScoredJobChooser(const Cnf &f, size_t depth, std::vector<float> scores = {})
        : f_(f), depth_(depth), scores_(std::move(scores))
    {
    }
    void evaluate() override
    {
        std::vector<double> s(f_.n_vars + 1, 0.0);
        if (scores_.size() == (size_t)f_.n_vars) {
            for (int32_t v = 1; v <= f_.n_vars; v++) s[v] = scores_[v - 1];
        } else {
            for (int32_t d : f_.lits) s[std::abs(d)] += 1.0;
        }
        std::vector<int32_t> order(f_.n_vars);
        std::iota(order.begin(), order.end(), 1);
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return s[a] > s[b]; });
        chosen_.assign(order.begin(), order.begin() + std::min<size_t>(depth_, order.size()));
        evaluated_ = true;
    }

private:
    const Cnf &f_;
    size_t depth_;
    std::vector<float> scores_;
};

// ---------------------------------------------------------------- solving
struct Result {
    int32_t verdict = GPSAT_UNKNOWN;
    std::vector<int8_t> model;     // +1 / -1 per variable (SAT only)
    int32_t device_check = -1;     // device model checker: 1 ok, 0 failed, -1 no model
    bool host_check = false;       // independent host model checker
    std::vector<int64_t> stats;    // GPSAT_SOLVE_NSTATS entries
    double ms = 0.0;
};

struct SolverConfig {
    std::shared_ptr<BCPStrategy> bcp = std::make_shared<TwoWatchedLiterals>();
    std::shared_ptr<DecisionStrategy> decision = std::make_shared<VSIDS>();
    std::shared_ptr<ConflictAnalysis> analysis = std::make_shared<FirstUIP>();
    std::shared_ptr<ClauseLearning> learning = std::make_shared<LearntClauseDatabase>();
    std::shared_ptr<Restarts> restarts = std::make_shared<LubyRestarts>();
    int64_t conflict_budget = 0;  // 0: none
    int32_t max_slots = 0;

    gpsat_solve_options options() const
    {
        gpsat_solve_options o;
        check(gpsat_solve_options_default(&o), "options");
        bcp->configure(o);
        decision->configure(o);
        analysis->configure(o);
        learning->configure(o);
        restarts->configure(o);
        o.conflict_budget = conflict_budget;
        o.max_slots = max_slots;
        return o;
    }
};

// Solves one formula on the device: one job, or the cubes of a JobChooser.
inline Result solve(const Cnf &f, const SolverConfig &cfg, JobChooser *chooser = nullptr)
{
    Result r;
    gpsat_batch *b = nullptr;
    const int64_t foff[2] = {0, f.n_clauses()};
    const int32_t nv = std::max(f.n_vars, 1);
    check(gpsat_batch_create(f.lits.data(), f.offsets.data(), foff, &nv, 1, &b), "batch");
    std::unique_ptr<gpsat_batch, int (*)(gpsat_batch *)> guard(b, gpsat_batch_destroy);
    gpsat_solve_options o = cfg.options();
    std::vector<int32_t> jf, cl;
    std::vector<int64_t> co{0};
    if (chooser) {
        JobsQueue q;
        chooser->getJobs(q);
        for (const Job &j : q.jobs()) {
            jf.push_back(0);
            cl.insert(cl.end(), j.literals.begin(), j.literals.end());
            co.push_back((int64_t)cl.size());
        }
    }
    r.model.assign(nv, 0);
    r.stats.assign(GPSAT_SOLVE_NSTATS, 0);
    check(gpsat_batch_solve(b, &o, chooser ? jf.data() : nullptr, chooser ? co.data() : nullptr,
                            chooser ? cl.data() : nullptr, (int32_t)jf.size(), &r.verdict, r.model.data(),
                            r.stats.data(), &r.device_check, nullptr),
          "solve");
    if (r.verdict == GPSAT_SAT)
        r.host_check = gpsat_check_model(f.lits.data(), f.offsets.data(), f.n_clauses(), r.model.data(), nv,
                                         nullptr) == 1;
    else
        r.model.clear();
    return r;
}

}  // namespace gpsat
