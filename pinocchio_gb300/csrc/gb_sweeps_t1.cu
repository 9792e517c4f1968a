// ABA-derivative and computeMinverse sweep kernels, one thread per configuration.
#include "gb_sweeps.cuh"

namespace gbi {
int sweeps_t1(const SweepCall& c) { return sweeps_for<1>(c); }
}  // namespace gbi
