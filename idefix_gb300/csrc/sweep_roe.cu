// Flux sweeps instantiated for the ROE Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_roe(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kROE>(e, invdt, fold_max); }
void launch_ens_sweep_roe(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kROE>(e, dir, t, invdt, last);
}
}  // namespace idfx
