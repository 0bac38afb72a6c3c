// Flux sweeps instantiated for the HLLD Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_hlld(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kHLLD>(e, invdt, fold_max); }
void launch_ens_sweep_hlld(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kHLLD>(e, dir, t, invdt, last);
}
cudaError_t launch_ens_persist_hlld(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kHLLD>(e, ncyc, grid);
}
int ens_persist_blocks_hlld(const EnsEngine& e) { return ens_persist_blocks_solver<kHLLD>(e); }
}  // namespace idfx
