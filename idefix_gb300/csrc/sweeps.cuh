// Launch of the flux sweeps for one Riemann solver (SOLVER), dispatching on
// dimensionality and reconstruction order.
#pragma once
#include "engine.hpp"
#include "ensemble.hpp"

namespace idfx {

template <int D, int DIR, int ORDER, int SOLVER, typename T>
void launch_dir(Engine& e, int invdt, int last) {
  const Geo& g = e.g;
  constexpr int A = (DIR == 0) ? 1 : 0;
  constexpr int B = (DIR == 2) ? 1 : 2;
  const int nseg = (g.n[DIR] + e.seg[DIR] - 1) / e.seg[DIR];
  const long long cols = (long long)(g.n[A] + 2 * g.ext) * (D == 3 ? g.n[B] + 2 * g.ext : 1);
  mark_begin(e, kKSweepX + DIR);
  if constexpr (DIR == 0 && sizeof(T) == 4 && ORDER <= 4) {
    // FP32 x sweep: warp chunks along each row (coalesced); staged by bulk
    // copies when rows and arrays are 16-byte aligned
    const unsigned blocks = (unsigned)((cols + kXW - 1) / kXW);
    const bool aligned = g.nt[0] % 4 == 0 && (reinterpret_cast<uintptr_t>(e.f.Vc32) & 15) == 0 &&
                         (reinterpret_cast<uintptr_t>(e.f.Uc) & 15) == 0;
    if (aligned) {
      const size_t smem = (size_t)kXW * xb_warp_bytes(Var<D>::NV, Var<D>::BX1);
      k_sweep_xbulk<D, ORDER, SOLVER, T><<<blocks, 32 * kXW, smem, e.stream>>>(g, e.f, e.ctl, invdt, last);
    } else {
      k_sweep_xwarp<D, ORDER, SOLVER, T><<<blocks, 32 * kXW, 0, e.stream>>>(g, e.f, e.ctl, invdt, last);
    }
  } else {
    dim3 grid((unsigned)((cols + kTM - 1) / kTM), nseg, 1);
    k_sweep_march<D, DIR, ORDER, SOLVER, T><<<grid, kTM, 0, e.stream>>>(g, e.f, e.ctl, invdt, last, e.seg[DIR]);
  }
  mark_end(e);
}

// invdt: 0 none, 1 first contribution of the cycle (InvDt reset), 2 accumulate
template <int D, int ORDER, int SOLVER, typename T>
void launch_sweeps_tt(Engine& e, int invdt, int fold_max) {
  // e.only_dir >= 0 (autotuner): that direction alone
  if (e.only_dir < 0 || e.only_dir == 0) launch_dir<D, 0, ORDER, SOLVER, T>(e, invdt, 0);
  if (e.only_dir < 0 || e.only_dir == 1)
    launch_dir<D, 1, ORDER, SOLVER, T>(e, invdt == 0 ? 0 : 2, fold_max && D == 2);
  if constexpr (D == 3)
    if (e.only_dir < 0 || e.only_dir == 2) launch_dir<D, 2, ORDER, SOLVER, T>(e, invdt == 0 ? 0 : 2, fold_max);
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
  if constexpr (SOLVER == kHLLD)  // learned reconstruction: 3-D, HLLD, FP64 (learned.cu)
    if (D == 3 && O == 5) launch_learned_sweeps(e, invdt, fold_max);
}

// ---------------------------------------------------------------------------
// ensemble: one launch covers the sweep blocks of every box
// ---------------------------------------------------------------------------
template <int D, int DIR, int ORDER, int SOLVER, typename T>
__global__ void __launch_bounds__(kTM) ke_sweep_march(const EnsBox* boxes, const int4* items, int invdt,
                                                      int last) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_sweep_march<D, DIR, ORDER, SOLVER, T>(B.g, B.f, B.ctl, invdt, last, B.seg[DIR], dim3(it.y, it.z, it.w));
}

template <int D, int ORDER, int SOLVER, typename T>
void launch_ens_dir(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  if (t.n == 0) return;
  if (dir == 0) ke_sweep_march<D, 0, ORDER, SOLVER, T><<<t.n, kTM, 0, e.stream>>>(e.d_boxes, t.items, invdt, last);
  if (dir == 1) ke_sweep_march<D, 1, ORDER, SOLVER, T><<<t.n, kTM, 0, e.stream>>>(e.d_boxes, t.items, invdt, last);
  if constexpr (D == 3)
    if (dir == 2) ke_sweep_march<D, 2, ORDER, SOLVER, T><<<t.n, kTM, 0, e.stream>>>(e.d_boxes, t.items, invdt, last);
}

template <int SOLVER>
void launch_ens_sweep_solver(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  const int D = e.D, O = e.order;
  const bool mixed = e.precision == 1;
#define IDFX_ECASE(DD, OO)                                                            \
  if (D == DD && O == OO) {                                                           \
    if (mixed) launch_ens_dir<DD, OO, SOLVER, float>(e, dir, t, invdt, last);         \
    else launch_ens_dir<DD, OO, SOLVER, double>(e, dir, t, invdt, last);              \
    return;                                                                           \
  }
  IDFX_ECASE(2, 1) IDFX_ECASE(2, 2) IDFX_ECASE(2, 3) IDFX_ECASE(2, 4)
  IDFX_ECASE(3, 1) IDFX_ECASE(3, 2) IDFX_ECASE(3, 3) IDFX_ECASE(3, 4)
#undef IDFX_ECASE
}

}  // namespace idfx
