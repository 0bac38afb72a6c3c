// Flux sweeps instantiated for the HLL Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hll(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLL>(e, invdt, fold_max); }
}  // namespace idfx
