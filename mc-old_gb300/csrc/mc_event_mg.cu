// mc_event_mg.cu -- the per-thread kernels (k_track) for multigroup problems without time filters.
#include "mc_event_kernels.cuh"

namespace mc {
namespace ev {

EvKernel pick_track_mg(int minb, bool batch) { return pick_track<FL_MG>(minb, batch); }

}  // namespace ev
}  // namespace mc
