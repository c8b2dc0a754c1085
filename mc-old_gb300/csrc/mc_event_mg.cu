// mc_event_mg.cu -- the per-thread kernels (k_track) for multigroup problems without time filters.
// Their Philox refills beyond an event's first block go through one shared
// out-of-line copy (see Rng32 in mc_event_kernels.cuh): measured faster for
// these short, cheap events.
#define MC_EV_RNG_OUTLINE 1
#include "mc_event_kernels.cuh"

namespace mc {
namespace ev {

EvKernel pick_track_mg(int minb, bool batch) { return pick_track<FL_MG>(minb, batch); }

}  // namespace ev
}  // namespace mc
