// Persistent ensemble kernel instantiated for the HLLD Riemann solver (its own
// translation unit, so that it compiles in parallel with the sweeps).
#include "sweeps.cuh"

namespace idfx {
cudaError_t launch_ens_persist_hlld(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kHLLD>(e, ncyc, grid);
}
int ens_persist_blocks_hlld(const EnsEngine& e) { return ens_persist_blocks_solver<kHLLD>(e); }
}  // namespace idfx
