// ABA-derivative and computeMinverse sweep kernels, a team of 8 lanes per configuration.
#include "gb_sweeps.cuh"

namespace gbi {
int sweeps_t8(const SweepCall& c) { return sweeps_for<8>(c); }
}  // namespace gbi
