// Persistent ensemble kernel instantiated for the HLL Riemann solver (its own
// translation unit, so that it compiles in parallel with the sweeps).
#include "sweeps.cuh"

namespace idfx {
cudaError_t launch_ens_persist_hll(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kHLL>(e, ncyc, grid);
}
int ens_persist_blocks_hll(const EnsEngine& e) { return ens_persist_blocks_solver<kHLL>(e); }
}  // namespace idfx
