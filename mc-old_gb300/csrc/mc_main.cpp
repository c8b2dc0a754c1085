// mc_main.cpp -- mcgpu_run, the command-line driver over the C ABI and the
// counterpart of the reference's MC.exe (Main.cpp:8-31): reads
// <dir>/input.xml, runs the problem's samples, and writes the output.h5 tree
// as <dir>/output.json.  Cross sections come from ./xs_library, as the
// reference reads them (setup.cpp:326), unless --xs names a directory.
//
//   mcgpu_run <dir> [--mode replay|plain|event] [--xs <xs_dir>] [--seed <n>]
//
// Exit status: 0 on success; 1 for a usage error; 2 + the mc_status code
// when the library reports one (the message goes to stderr).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "mcgpu.h"

namespace {

int fail(mc_problem *p, mc_status st, const char *what)
{
    std::fprintf(stderr, "[ERROR] %s: %s: %s\n", what, mc_status_string(st), p ? mc_last_error(p) : "");
    if (p) mc_problem_free(p);
    return 2 + (int)st;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc == 1) {
        std::cout << "[ERROR] Please provide input.xml directory...\n";
        return 1;
    }
    const std::string io_dir = std::string(argv[1]) + "/";
    std::string xs_dir = "./xs_library";
    mc_mode mode = MC_MIXED_EVENT;
    uint64_t seed = 0x4D43;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--mode" && i + 1 < argc) {
            const std::string m = argv[++i];
            if (m == "replay") mode = MC_FP64_REPLAY;
            else if (m == "plain") mode = MC_FP64_PLAIN;
            else if (m == "event") mode = MC_MIXED_EVENT;
            else { std::cerr << "[ERROR] unknown mode " << m << "\n"; return 1; }
        } else if (a == "--xs" && i + 1 < argc) {
            xs_dir = argv[++i];
        } else if (a == "--seed" && i + 1 < argc) {
            seed = std::strtoull(argv[++i], nullptr, 0);
        } else {
            std::cerr << "[ERROR] unknown argument " << a << "\n";
            return 1;
        }
    }
    mc_problem *p = nullptr;
    mc_status st = mc_problem_load_xml(io_dir.c_str(), xs_dir.c_str(), &p);
    if (st != MC_OK) return fail(p, st, "setup");
    std::cout << "\nSimulation setup done,\nNow running the simulation...\n\n";
    uint64_t n = 0;
    mc_nsample(p, &n);
    if ((st = mc_run(p, 0, n, seed, mode, nullptr)) != MC_OK) return fail(p, st, "simulation");
    std::cout << "Simulation done!\n\nReporting simulation output...\n";
    if ((st = mc_report(p, (io_dir + "output.json").c_str())) != MC_OK) return fail(p, st, "report");
    std::cout << "Simulation output done!\n";
    mc_problem_free(p);
    return 0;
}
