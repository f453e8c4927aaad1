// gpsat -- command-line drop-in for the reference's gpupsat binary.
//
// Same flags as the reference's code (reference FileManager/ParametersManager.cpp:48-61;
// its README disagrees, the code wins):
//   gpsat [-i] FILE [-b BLOCKS] [-t THREADS] [-v LEVEL] [-p] [-s distributed|uniform] [-l]
//         [-u] [-o FILE] [--help] [--version]
// -b/-t keep their meaning for the job split: with 1 block and 1 thread and no
// -p the formula is solved as one job (the reference's sequential path);
// otherwise it is split into cube jobs (JobChooser) and all jobs run in one
// persistent launch, one warp per job.  Output lines follow the reference
// (SATSolver/main.cu:312, Results.cu:62-155): "Total time on GPU: X ms", then
// SATISFIABLE + the model line + "Solution was verified" (checked by the
// device and host checkers, which the reference's check is not), or
// UNSATISFIABLE, or UNDEFINED.  A missing file exits with status 255 like the
// reference's exit(-1); errors print a message and exit 1.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "gpsat.hpp"

namespace {

struct Args {
    std::string input = "task.cnf";
    int threads = 32, blocks = 32, verbosity = 1;
    std::string strategy = "distributed";
    bool seq_as_parallel = false, write_log = false, help = false, version = false, any = false;
    long long budget = 0;
};

void usage()
{
    std::printf(
        "gpsat: gpsat <file> [options]\n"
        "  --help                         Displays this help message\n"
        "  --version                      Displays version number\n"
        "  -i [ --input-file ] arg        Input file\n"
        "  -o [ --output-file ] arg       Output file (accepted, unused, as in the reference)\n"
        "  -t [ --number-of-threads ] arg Number of threads (job split)\n"
        "  -b [ --number-of-blocks ] arg  Number of blocks (job split)\n"
        "  -v [ --verbosity-level ] arg   Set verbosity level\n"
        "  -s [ --strategy ] arg          Strategy for generating the jobs: distributed or uniform\n"
        "  -p [ --sequential-as-parallel ] Forces the parallel strategy with 1 thread and 1 block\n"
        "  -u [ --preprocess-unary-clauses ] Accepted (preprocessing is always on)\n"
        "  -l [ --write-log ]             Prints file,threads,blocks,ms to autolog.txt\n"
        "  --conflict-budget arg          Conflicts per job before UNDEFINED (default: none)\n");
}

bool parse(int argc, char **argv, Args &a)
{
    for (int i = 1; i < argc; i++) {
        std::string s = argv[i];
        auto val = [&](const char *name) -> const char * {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "the required argument for option '%s' is missing\n", name);
                return nullptr;
            }
            return argv[++i];
        };
        a.any = true;
        if (s == "--help") a.help = true;
        else if (s == "--version") a.version = true;
        else if (s == "-i" || s == "--input-file") {
            const char *v = val("--input-file");
            if (!v) return false;
            a.input = v;
        } else if (s == "-o" || s == "--output-file") {
            if (!val("--output-file")) return false;
        } else if (s == "-t" || s == "--number-of-threads") {
            const char *v = val("--number-of-threads");
            if (!v) return false;
            a.threads = std::atoi(v);
        } else if (s == "-b" || s == "--number-of-blocks") {
            const char *v = val("--number-of-blocks");
            if (!v) return false;
            a.blocks = std::atoi(v);
        } else if (s == "-v" || s == "--verbosity-level") {
            const char *v = val("--verbosity-level");
            if (!v) return false;
            a.verbosity = std::atoi(v);
        } else if (s == "-s" || s == "--strategy") {
            const char *v = val("--strategy");
            if (!v) return false;
            a.strategy = v;
        } else if (s == "-p" || s == "--sequential-as-parallel") a.seq_as_parallel = true;
        else if (s == "-u" || s == "--preprocess-unary-clauses") { /* always on */ }
        else if (s == "-l" || s == "--write-log") a.write_log = true;
        else if (s == "--conflict-budget") {
            const char *v = val("--conflict-budget");
            if (!v) return false;
            a.budget = std::atoll(v);
        } else if (!s.empty() && s[0] == '-') {
            std::fprintf(stderr, "unrecognised option '%s'\n", s.c_str());
            return false;
        } else a.input = s;
    }
    return true;
}

}  // namespace

int main(int argc, char **argv)
{
    Args a;
    if (!parse(argc, argv, a)) return 1;
    if (a.help || !a.any) {
        usage();
        return 0;
    }
    if (a.version) {
        std::printf("%s\n", gpsat_version());
        return 0;
    }
    if (a.blocks <= 0) {
        std::printf("Invalid number of blocks: %d\n", a.blocks);
        return 1;
    }
    if (a.threads <= 0) {
        std::printf("Invalid number of threads: %d\n", a.threads);
        return 1;
    }
    {
        std::ifstream probe(a.input);
        if (!probe) {
            std::printf("The specified CNF file (%s) was not found!\n", a.input.c_str());
            return 255;
        }
    }
    try {
        gpsat::Cnf f = gpsat::read_dimacs(a.input);
        if (f.header_vars >= 0 && f.n_vars > f.header_vars)
            std::printf("header claims %d vars, but highest var found is %d. Using %d...", f.header_vars, f.n_vars,
                        f.n_vars);
        if (f.header_clauses >= 0 && f.n_clauses() != f.header_clauses)
            std::printf("header claims %lld clauses, but found %lld clauses. Using %lld...",
                        (long long)f.header_clauses, (long long)f.n_clauses(), (long long)f.n_clauses());
        bool parallel = a.blocks > 1 || a.threads > 1 || a.seq_as_parallel;
        if (f.n_vars < 3 && parallel) {
            std::printf("Warning: There are %d vars in the formula and at least 3 are necessary to parallelize. "
                        "Forcing sequential execution!\n", f.n_vars);
            parallel = false;
            a.blocks = a.threads = 1;
            a.seq_as_parallel = false;
        }
        gpsat::SolverConfig cfg;
        cfg.conflict_budget = a.budget;
        gpsat::ChoosingStrategy strat = a.strategy == "uniform" ? gpsat::ChoosingStrategy::UNIFORM
                                                                : gpsat::ChoosingStrategy::DISTRIBUTE_JOBS_PER_THREAD;
        if (a.verbosity >= 1) {
            std::printf("Solver configuration:\n");
            std::printf("Input file: %s\n", a.input.c_str());
            std::printf("Formula has %d vars and %lld clauses\n", f.n_vars, (long long)f.n_clauses());
            if (!parallel) std::printf("Parallelization strategy: SEQUENTIAL RUN (one warp)\n");
            else {
                std::printf("Parallelization strategy: Divide and Conquer (cube jobs, one warp per job)\n");
                std::printf("Number of blocks: %d\nNumber of threads: %d\n", a.blocks, a.threads);
                std::printf("Job creation strategy: %s\n",
                            strat == gpsat::ChoosingStrategy::UNIFORM ? "uniform" : "distribution per thread");
            }
            std::printf("BCP: %s\nDecisions: %s\nConflict analysis: %s\nClause learning: %s\nRestarts: %s\n",
                        cfg.bcp->name(), cfg.decision->name(), cfg.analysis->name(), cfg.learning->name(),
                        cfg.restarts->name());
        }
        gpsat::MaxClauseJobChooser chooser(f, parallel ? a.threads : 1, parallel ? a.blocks : 1, strat);
        if (parallel) chooser.evaluate();
        const auto t0 = std::chrono::steady_clock::now();
        gpsat::Result r = gpsat::solve(f, cfg, parallel ? &chooser : nullptr);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (a.verbosity >= 1 && parallel)
            std::printf("There were %zu jobs created.\n", chooser.get_n_jobs());
        std::printf("Total time on GPU: %f ms\n", ms);
        if (r.verdict == GPSAT_SAT) {
            std::printf("SATISFIABLE\n");
            std::string line;
            for (int32_t v = 0; v < f.n_vars; v++) {
                line += (r.model[v] < 0 ? "-" : "") + std::to_string(v + 1) + " ";
            }
            std::printf("%s0\n", line.c_str());
            std::printf("Solution %s\n", (r.host_check && r.device_check == 1) ? "was verified" : "was not verified");
        } else if (r.verdict == GPSAT_UNSAT) {
            std::printf("UNSATISFIABLE\n");
        } else {
            std::printf("UNDEFINED\n");
        }
        if (a.write_log) {
            std::ofstream out("autolog.txt", std::ios_base::app);
            char buf[512];
            std::snprintf(buf, sizeof(buf), "%s,%d,%d,%f\n", a.input.c_str(), a.threads, a.blocks, ms);
            out << buf;
        }
        return 0;
    } catch (const gpsat::Error &e) {
        std::printf("Error: %s\n", e.what());
        return 1;
    }
}
