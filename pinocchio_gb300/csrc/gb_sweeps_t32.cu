// ABA-derivative and computeMinverse sweep kernels, a warp per configuration.
#include "gb_sweeps.cuh"

namespace gbi {
int sweeps_t32(const SweepCall& c) { return sweeps_for<32>(c); }
}  // namespace gbi
