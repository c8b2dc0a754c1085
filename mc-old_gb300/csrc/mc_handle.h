// mc_handle.h -- the opaque mc_problem handle behind include/mcgpu.h.
#pragma once

#include <string>

#include "mc_engine.h"
#include "mc_problem.h"

struct mc_problem {
    mc::Tables t;
    mc::DeviceProblem dev;
    std::string err;
};
