// Persistent ensemble kernel instantiated for the ROE Riemann solver (its own
// translation unit, so that it compiles in parallel with the sweeps).
#include "sweeps.cuh"

namespace idfx {
cudaError_t launch_ens_persist_roe(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kROE>(e, ncyc, grid);
}
int ens_persist_blocks_roe(const EnsEngine& e) { return ens_persist_blocks_solver<kROE>(e); }
}  // namespace idfx
