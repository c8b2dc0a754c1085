// mc_event_ce.cu -- the per-thread kernels (k_track) for continuous-energy problems without time filters.
#include "mc_event_kernels.cuh"

namespace mc {
namespace ev {

EvKernel pick_track_ce(int minb, bool batch) { return pick_track<FL_CE>(minb, batch); }

}  // namespace ev
}  // namespace mc
