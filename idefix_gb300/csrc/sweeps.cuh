// Launch of the flux sweeps for one Riemann solver (SOLVER), dispatching on
// dimensionality and reconstruction order.
#pragma once
#include "engine.hpp"

namespace idfx {

template <int D, int ORDER, int SOLVER>
void launch_sweeps_t(Engine& e, int invdt, int fold_max) {
  const Geo& g = e.g;
  // x: one block per kTX faces of each (j,k) row, rows include the CT extension
  {
    dim3 grid((g.n[0] + 1 + kTX - 1) / kTX, g.n[1] + 2 * g.ext, D == 3 ? g.n[2] + 2 * g.ext : 1);
    mark_begin(e, kKSweepX);
    k_sweep_x<D, ORDER, SOLVER><<<grid, kTX, 0, e.stream>>>(g, e.f, e.ctl, invdt, fold_max && D == 1);
    mark_end(e);
  }
  // y
  {
    const int nseg = (g.n[1] + e.seg[1] - 1) / e.seg[1];
    dim3 grid((g.n[0] + 2 * g.ext + kTM - 1) / kTM, nseg, D == 3 ? g.n[2] + 2 * g.ext : 1);
    mark_begin(e, kKSweepY);
    k_sweep_march<D, 1, ORDER, SOLVER><<<grid, kTM, 0, e.stream>>>(g, e.f, e.ctl, invdt == 0 ? 0 : 2,
                                                                   fold_max && D == 2, e.seg[1]);
    mark_end(e);
  }
  if constexpr (D == 3) {
    const int nseg = (g.n[2] + e.seg[2] - 1) / e.seg[2];
    dim3 grid((g.n[0] + 2 * g.ext + kTM - 1) / kTM, nseg, g.n[1] + 2 * g.ext);
    mark_begin(e, kKSweepZ);
    k_sweep_march<D, 2, ORDER, SOLVER><<<grid, kTM, 0, e.stream>>>(g, e.f, e.ctl, invdt == 0 ? 0 : 2,
                                                                   fold_max, e.seg[2]);
    mark_end(e);
  }
}

template <int SOLVER>
void launch_sweeps_solver(Engine& e, int invdt, int fold_max) {
  const int D = e.g.D, O = e.g.order;
#define IDFX_CASE(DD, OO)                                   \
  if (D == DD && O == OO) {                                 \
    launch_sweeps_t<DD, OO, SOLVER>(e, invdt, fold_max);    \
    return;                                                 \
  }
  IDFX_CASE(2, 1) IDFX_CASE(2, 2) IDFX_CASE(2, 3) IDFX_CASE(2, 4)
  IDFX_CASE(3, 1) IDFX_CASE(3, 2) IDFX_CASE(3, 3) IDFX_CASE(3, 4)
#undef IDFX_CASE
}

}  // namespace idfx
