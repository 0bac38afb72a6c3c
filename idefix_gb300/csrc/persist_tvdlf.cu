// Persistent ensemble kernel instantiated for the TVDLF Riemann solver (its own
// translation unit, so that it compiles in parallel with the sweeps).
#include "sweeps.cuh"

namespace idfx {
cudaError_t launch_ens_persist_tvdlf(EnsEngine& e, int ncyc, int grid) {
  return launch_ens_persist_solver<kTVDLF>(e, ncyc, grid);
}
int ens_persist_blocks_tvdlf(const EnsEngine& e) { return ens_persist_blocks_solver<kTVDLF>(e); }
}  // namespace idfx
