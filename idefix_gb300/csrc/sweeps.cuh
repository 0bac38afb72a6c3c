// Launch of the flux sweeps for one Riemann solver (SOLVER), dispatching on
// dimensionality and reconstruction order.
#pragma once
#include "engine.hpp"

namespace idfx {

template <int D, int DIR, int ORDER, int SOLVER, typename T>
void launch_dir(Engine& e, int invdt, int last) {
  const Geo& g = e.g;
  constexpr int A = (DIR == 0) ? 1 : 0;
  constexpr int B = (DIR == 2) ? 1 : 2;
  const int nseg = (g.n[DIR] + e.seg[DIR] - 1) / e.seg[DIR];
  const long long cols = (long long)(g.n[A] + 2 * g.ext) * (D == 3 ? g.n[B] + 2 * g.ext : 1);
  dim3 grid((unsigned)((cols + kTM - 1) / kTM), nseg, 1);
  mark_begin(e, kKSweepX + DIR);
  k_sweep_march<D, DIR, ORDER, SOLVER, T><<<grid, kTM, 0, e.stream>>>(g, e.f, e.ctl, invdt, last, e.seg[DIR]);
  mark_end(e);
}

// invdt: 0 none, 1 first contribution of the cycle (InvDt reset), 2 accumulate
template <int D, int ORDER, int SOLVER, typename T>
void launch_sweeps_tt(Engine& e, int invdt, int fold_max) {
  launch_dir<D, 0, ORDER, SOLVER, T>(e, invdt, 0);
  launch_dir<D, 1, ORDER, SOLVER, T>(e, invdt == 0 ? 0 : 2, fold_max && D == 2);
  if constexpr (D == 3) launch_dir<D, 2, ORDER, SOLVER, T>(e, invdt == 0 ? 0 : 2, fold_max);
}

// precision: FP64 (bit-exact) or mixed (FP32 reconstruction + Riemann)
template <int D, int ORDER, int SOLVER>
void launch_sweeps_t(Engine& e, int invdt, int fold_max) {
  if (e.precision == 1) launch_sweeps_tt<D, ORDER, SOLVER, float>(e, invdt, fold_max);
  else launch_sweeps_tt<D, ORDER, SOLVER, double>(e, invdt, fold_max);
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
