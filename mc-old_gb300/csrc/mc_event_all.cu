// mc_event_all.cu -- the per-thread kernels (k_track) for problems with time filters, and batches that mix continuous-energy and multigroup problems.
#include "mc_event_kernels.cuh"

namespace mc {
namespace ev {

EvKernel pick_track_all(int minb, bool batch) { return pick_track<FL_ALL>(minb, batch); }

}  // namespace ev
}  // namespace mc
