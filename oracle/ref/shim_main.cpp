// shim_main.cpp -- driver for the compiled reference (oracle/_ref/mcref).
//
// Test infrastructure.  Usage:
//   mcref <io_dir> <seed> [<wr> <ws>] [--digest <file>]
// Runs the reference's Simulator(io_dir) (setup.cpp:30; cross sections from
// ./xs_library relative to the working directory, setup.cpp:326) through the
// shim's history loop and prints, as C99 hex floats, Ntrack and every
// estimator's tally mean / uncertainty (Estimator.cpp:424-432).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "simulator.h"

extern bool g_shim_wr_set;
extern double g_shim_wr, g_shim_ws;
extern uint64_t g_shim_seed;
extern std::vector<uint64_t> g_shim_digest;

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: mcref <io_dir> <seed> [wr ws] [--digest file]\n");
        return 2;
    }
    const std::string io_dir = std::string(argv[1]) + "/";
    g_shim_seed = std::strtoull(argv[2], nullptr, 0);
    const char *digest_file = nullptr;
    std::vector<const char *> pos;
    for (int i = 3; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--digest") && i + 1 < argc) { digest_file = argv[++i]; }
        else pos.push_back(argv[i]);
    }
    if (pos.size() >= 2) {
        g_shim_wr_set = true;
        g_shim_wr = std::strtod(pos[0], nullptr);
        g_shim_ws = std::strtod(pos[1], nullptr);
    }
    Simulator S(io_dir);
    S.start();
    std::printf("Ntrack %llu\n", (unsigned long long)S.Ntrack);
    std::printf("Nsample %llu\n", (unsigned long long)S.Nsample);
    std::printf("estimators %zu\n", S.Estimators.size());
    for (size_t e = 0; e < S.Estimators.size(); ++e) {
        const unsigned long long n = S.Estimators[e]->tally_size();
        std::printf("estimator %zu %llu\n", e, n);
        for (unsigned long long j = 0; j < n; ++j) {
            Tally t = S.Estimators[e]->tally((int)j);
            std::printf("%a %a\n", t.mean, t.uncer);
        }
    }
    if (digest_file) {
        FILE *f = std::fopen(digest_file, "wb");
        if (!f) return 4;
        std::fwrite(g_shim_digest.data(), sizeof(uint64_t), g_shim_digest.size(), f);
        std::fclose(f);
    }
    return 0;
}
