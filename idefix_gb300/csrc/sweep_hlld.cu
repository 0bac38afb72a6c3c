// Flux sweeps instantiated for the HLLD Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hlld(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLLD>(e, invdt, fold_max); }
void launch_ens_sweep_hlld(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kHLLD>(e, dir, t, invdt, last);
}
}  // namespace idfx
