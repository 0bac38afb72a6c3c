// Flux sweeps instantiated for the HLL Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hll(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLL>(e, invdt, fold_max); }
void launch_ens_sweep_hll(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kHLL>(e, dir, t, invdt, last);
}
cudaError_t launch_ens_persist_hll(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kHLL>(e, ncyc, grid);
}
int ens_persist_blocks_hll(const EnsEngine& e) { return ens_persist_blocks_solver<kHLL>(e); }
}  // namespace idfx
