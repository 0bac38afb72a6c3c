// Flux sweeps instantiated for the ROE Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_roe(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kROE>(e, invdt, fold_max); }
}  // namespace idfx
