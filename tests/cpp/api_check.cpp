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
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "gpsat.hpp"

int main(int argc, char **argv)
{
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
