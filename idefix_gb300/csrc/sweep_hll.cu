// Flux sweeps instantiated for the HLL Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hll(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLL>(e, invdt, fold_max); }
void launch_ens_sweep_hll(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kHLL>(e, dir, t, invdt, last);
}
}  // namespace idfx
