// shim_random.cpp -- replaces the reference's src/Random.cpp.
//
// Test infrastructure (reference build for the CPU oracle).  The reference's
// Urand() (Random.cpp:121-126) advances one global LCG; here it draws from the
// Philox stream keyed by (seed, history, particle, event, draw) whose context
// the shim's history loop (shim_sim.cpp) keeps up to date, so the reference's
// own physics objects consume exactly the draws the oracle and the GPU path
// consume.
#include "shim_rng.h"
#include "Random.h"

orc_rng g_shim_rng;
uint64_t g_shim_draws = 0;

double Urand(void)
{
    g_shim_draws++;
    return orc_urand(&g_shim_rng);
}

void RN_init_particle(unsigned long long *) {}
