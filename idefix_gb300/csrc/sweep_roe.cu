// Flux sweeps instantiated for the ROE Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_roe(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kROE>(e, invdt, fold_max); }
void launch_ens_sweep_roe(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kROE>(e, dir, t, invdt, last);
}
cudaError_t launch_ens_persist_roe(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kROE>(e, ncyc, grid);
}
int ens_persist_blocks_roe(const EnsEngine& e) { return ens_persist_blocks_solver<kROE>(e); }
}  // namespace idfx
