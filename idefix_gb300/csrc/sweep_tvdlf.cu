// Flux sweeps instantiated for the TVDLF Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_tvdlf(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kTVDLF>(e, invdt, fold_max); }
}  // namespace idfx
