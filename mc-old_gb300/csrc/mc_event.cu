// mc_event.cu -- mixed-precision event-based engine (placeholder).
#include "mc_engine.h"

namespace mc {

struct EventState {};

void event_state_free(EventState *s) { delete s; }

mc_status run_event(const Tables &, DeviceProblem &, uint64_t, uint64_t, uint64_t, const mc_tune *,
                    std::string &err)
{
    err = "the mixed-precision event engine is not available in this build";
    return MC_ERR_ARG;
}

}  // namespace mc
