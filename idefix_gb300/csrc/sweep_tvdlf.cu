// Flux sweeps instantiated for the TVDLF Riemann solver.
#include "sweeps.cuh"

namespace idfx {
void launch_sweeps_tvdlf(Engine& e, int invdt, int fold_max) { launch_sweeps_solver<kTVDLF>(e, invdt, fold_max); }
void launch_ens_sweep_tvdlf(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  launch_ens_sweep_solver<kTVDLF>(e, dir, t, invdt, last);
}
}  // namespace idfx
