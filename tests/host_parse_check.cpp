// Host-side input check (test infrastructure): loads each (input dir,
// cross-section dir) pair given on the command line through the library's
// XML reader and problem builder, and, when that succeeds, through the FP32
// table builder; prints "ok" or "err <message>" per pair.  The test suite
// builds it with AddressSanitizer and UndefinedBehaviorSanitizer, so a
// memory error or undefined behaviour in the readers stops it with a report.
#include <cstdio>
#include <string>

#include "mc_evtables.h"
#include "mc_problem.h"

int main(int argc, char **argv)
{
    for (int i = 1; i + 1 < argc; i += 2) {
        mc::Tables t;
        std::string err;
        bool ok = mc::load_problem(argv[i], argv[i + 1], t, err);
        if (ok) {
            mc::EvHost h;
            ok = mc::build_event_tables(t, h, err);
        }
        std::printf("%s %s\n", ok ? "ok" : "err", ok ? "" : err.c_str());
    }
    return 0;
}
