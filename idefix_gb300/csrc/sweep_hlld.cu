// Flux sweeps instantiated for the HLLD Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hlld(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLLD>(e, invdt, fold_max); }
}  // namespace idfx
