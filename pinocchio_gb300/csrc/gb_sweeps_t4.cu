// ABA-derivative and computeMinverse sweep kernels, a team of 4 lanes per configuration.
#include "gb_sweeps.cuh"

namespace gbi {
int sweeps_t4(const SweepCall& c) { return sweeps_for<4>(c); }
}  // namespace gbi
