// rift_sim_main.cpp -- command-line driver of the host drop-in layer, the
// counterpart of the reference's main.cc: open the simulation of a config
// file, run RunSimulation until t >= tf, close.
#include <cstdio>

#include "../../include/rift_host.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config file>\n", argv[0]);
        return 2;
    }
    rift_sim* sim = nullptr;
    if (rift_sim_open(argv[1], &sim) != RIFT_OK) {
        std::fprintf(stderr, "open failed: %s\n", rift_host_last_error());
        return 1;
    }
    double t = 0.0, dt = 0.0, tf = 0.0;
    rift_sim_time(sim, &t, &dt, &tf);
    std::printf("This will run for %g seconds\n", tf);
    int64_t steps = 0;
    int rc = rift_sim_run(sim, tf, &t, &steps);
    if (rc != RIFT_OK) std::fprintf(stderr, "run failed: %s\n", rift_sim_last_error(sim));
    const int rc2 = rift_sim_close(sim);
    if (rc == RIFT_OK && rc2 != RIFT_OK) std::fprintf(stderr, "close failed: %s\n", rift_host_last_error());
    std::printf("t = %.17g after %lld steps\n", t, (long long)steps);
    return (rc == RIFT_OK && rc2 == RIFT_OK) ? 0 : 1;
}
