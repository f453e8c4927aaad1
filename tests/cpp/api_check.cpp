// Exercises the C++ host interface (include/gpsat.hpp) from a program that
// includes it, as a user of the library would.
//   api_check rank  <cnf> <depth>       chosen split variables of MaxClauseJobChooser
//   api_check trails <cnf> <trail file> [scan]
//                                       TrailPropagator over the trails (one per
//                                        line, DIMACS literals ending in 0): one
//                                        line per trail: status conflict stop
//                                        n_implied then (literal reason) pairs;
//                                        "scan": the full-scan strategy, with a
//                                        256-entry window and 8 trails in flight
//                                        set on the way (the watched kernel's
//                                        shape, which the full scan ignores)
//   api_check config                    the solve options of the default
//                                        SolverConfig, then of the reference's
//                                        roles (last free variable, geometric
//                                        restarts), then the library's defaults
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "gpsat.hpp"

static void print_options(const gpsat_solve_options &o)
{
    std::printf("%d %d %d %.6g %.6g %d %d %d %lld %d %d\n", o.decide, o.restart, o.restart_base,
                (double)o.restart_factor, (double)o.var_decay, o.learnt_first, o.learnt_inc, o.minimize,
                (long long)o.conflict_budget, o.phase_init, o.max_slots);
}

int main(int argc, char **argv)
{
    if (argc == 2 && std::string(argv[1]) == "config") {
        gpsat::SolverConfig c;
        print_options(c.options());
        gpsat::SolverConfig r;
        r.decision = std::make_shared<gpsat::LastFreeVariable>();
        r.restarts = std::make_shared<gpsat::GeometricRestarts>();
        r.conflict_budget = 5000;
        print_options(r.options());
        gpsat_solve_options d;
        if (gpsat_solve_options_default(&d) != GPSAT_OK) return 1;
        print_options(d);
        return 0;
    }
    if (argc < 4) {
        std::fprintf(stderr, "usage: api_check rank|trails <cnf> <arg>\n");
        return 2;
    }
    try {
        const std::string mode = argv[1];
        gpsat::Cnf f = gpsat::read_dimacs(argv[2]);
        if (mode == "rank") {
            gpsat::MaxClauseJobChooser ch(f, 1, 1, gpsat::ChoosingStrategy::FIXED, (size_t)std::atoi(argv[3]));
            ch.evaluate();
            gpsat::JobsQueue q;
            ch.getJobs(q);
            for (int32_t v : ch.chosen()) std::printf("%d ", v);
            std::printf("\n%zu\n", q.n_jobs());
            return 0;
        }
        if (mode == "trails") {
            std::ifstream in(argv[3]);
            std::vector<std::vector<int32_t>> trails;
            std::string line;
            while (std::getline(in, line)) {
                std::istringstream ls(line);
                std::vector<int32_t> t;
                int32_t x;
                while (ls >> x && x != 0) t.push_back(x);
                trails.push_back(t);
            }
            gpsat::Formula fo(f);
            gpsat::TrailPropagator bcp(fo, 4096);
            if (argc > 4 && std::string(argv[4]) == "scan") {
                bcp.set_window(256);
                bcp.set_active_slots(8);
                bcp.set_order_pivot(100);
                bcp.use_full_scan(true);
            }
            for (const gpsat::TrailOutcome &o : bcp.new_decisions(trails)) {
                std::printf("%d %d %d %zu", o.status, o.conflict_clause, o.stop_index, o.implied.size());
                for (size_t i = 0; i < o.implied.size(); i++) std::printf(" %d %d", o.implied[i], o.reasons[i]);
                std::printf("\n");
            }
            return 0;
        }
    } catch (const gpsat::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 2;
}
