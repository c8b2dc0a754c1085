// shim_rng.h -- state shared by the reference shim's Urand() and history loop.
// Test infrastructure (reference build for the CPU oracle).
#ifndef ORC_SHIM_RNG_H
#define ORC_SHIM_RNG_H
#include <stdint.h>
extern "C" {
#include "../orc_philox.h"
}
extern orc_rng g_shim_rng;
extern uint64_t g_shim_draws;
#endif
