// Launch of the flux sweeps for one Riemann solver (SOLVER), dispatching on
// dimensionality and reconstruction order.
#pragma once
#include "engine.hpp"
#include "ensemble.hpp"
#include "sweep_tile.cuh"

namespace idfx {

// the FP32 y or z sweep of a 3-D block as the tile sweep
template <int DIR, int ORDER, int SOLVER>
void launch_tile(Engine& e, int invdt, int last, const SweepTileMaps* tm) {
  const Geo& g = e.g;
  constexpr int B = (DIR == 2) ? 1 : 2;
  constexpr int smem = tile_smem<ORDER>();
  static const bool smem_set =
      cudaFuncSetAttribute(k_sweep_tile<DIR, ORDER, SOLVER>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) ==
      cudaSuccess;
  (void)smem_set;
  dim3 grid((unsigned)((g.end[0] + g.ext + kTX - 1) / kTX), (unsigned)((g.n[B] + 2 * g.ext + kTB - 1) / kTB),
            (unsigned)((g.n[DIR] + e.seg[DIR] - 1) / e.seg[DIR]));
  k_sweep_tile<DIR, ORDER, SOLVER><<<grid, 32 * kTW, smem, e.stream>>>(
      g, e.f, e.ctl, invdt, last, e.seg[DIR], tm->vc[DIR - 1], tm->uc[DIR - 1], tm->inv[DIR - 1]);
}

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
    const SweepTileMaps* tm = nullptr;
    if constexpr (D == 3 && DIR >= 1 && sizeof(T) == 4 && ORDER >= 2 && ORDER <= 4)
      if (e.tile[DIR]) tm = sweep_tile_maps(e);
    if (tm) {
      if constexpr (D == 3 && DIR >= 1 && sizeof(T) == 4 && ORDER >= 2 && ORDER <= 4)
        launch_tile<DIR, ORDER, SOLVER>(e, invdt, last, tm);
    } else {
      dim3 grid((unsigned)((cols + kTM - 1) / kTM), nseg, 1);
      k_sweep_march<D, DIR, ORDER, SOLVER, T><<<grid, kTM, 0, e.stream>>>(g, e.f, e.ctl, invdt, last, e.seg[DIR]);
    }
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

// ---------------------------------------------------------------------------
// Persistent ensemble kernel: `ncyc` cycles of every box in ONE launch.
// The blocks (64 threads, all co-resident: cooperative launch) walk the same
// per-phase work lists as the batched launches - each item one block of the
// single-box device body (d_* of mhd_kernels.cuh) for one box - and meet at
// a grid-wide barrier between dependent phases, so every box evolves
// exactly as in the batched launches (and as alone).  Every barrier wait is
// bounded (kBarrierNs of %globaltimer): a block that gives up marks the
// barrier failed, every block stops, and each box's control block reports a
// CUDA-side failure; nothing waits without bound.
// ---------------------------------------------------------------------------
constexpr unsigned long long kBarrierNs = 5000000000ull;  // 5 s per barrier

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool grid_barrier(GridBar* b) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* gen = &b->gen;
    volatile int* failed = &b->failed;
    const unsigned g0 = *gen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {  // the last block to arrive opens it
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const unsigned long long deadline = global_ns() + kBarrierNs;
      while (*gen == g0) {
        if (*failed || global_ns() > deadline) {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (!ok) atomicExch(&b->failed, 1);
    ok_s = ok && !*failed;
  }
  __syncthreads();
  return ok_s != 0;
}

__device__ __forceinline__ bool any_due(const EnsBox* boxes, int nbox, int period) {
  if (period <= 0) return false;
  for (int b = 0; b < nbox; b++)
    if (boxes[b].ctl->ncycles % period == 0) return true;
  return false;
}

template <int D, int ORDER, int SOLVER, typename T>
__global__ void __launch_bounds__(kTM) ke_persistent(const EnsBox* boxes, EnsPersist P, int ncyc, GridBar* bar) {
  using E = T;  // EMF buffers in the arithmetic type of the sweeps
  const int stride = (int)gridDim.x;
  const int tstride = stride * (int)blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  auto dd = [](const int4& it) { return dim3(it.y, it.z, it.w); };
  auto due_box = [](const Ctl* c, int period) { return period > 0 && c->ncycles % period == 0; };
  for (int cyc = 0; cyc < ncyc && ok; cyc++) {
    for (int b = t0; b < P.nbox; b += tstride) d_cycle_begin(boxes[b].g, boxes[b].ctl, 1);
    if (!(ok = grid_barrier(bar))) break;
    // divB of the boxes whose own cycle count makes it due (uniform decision:
    // the counters change only in the cycle end)
    if (any_due(boxes, P.nbox, P.log_period)) {
      for (int b = t0; b < P.nbox; b += tstride)
        if (due_box(boxes[b].ctl, P.log_period)) boxes[b].ctl->divb_bits = 0ull;
      if (!(ok = grid_barrier(bar))) break;
      for (int i = blockIdx.x; i < P.nactive; i += stride) {
        const int4 it = P.active[i];
        const EnsBox& B = boxes[it.x];
        if (due_box(B.ctl, P.log_period)) d_divb<D>(B.g, B.f, B.ctl, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
      for (int b = t0; b < P.nbox; b += tstride)
        if (due_box(boxes[b].ctl, P.log_period)) d_check_divb(boxes[b].ctl);
      if (!(ok = grid_barrier(bar))) break;
    }
    const bool nan_due = any_due(boxes, P.nbox, P.check_nan_period);
    for (int stage = 0; stage < P.nstages && ok; stage++) {
      const int save = (P.nstages > 1 && stage == 0);
      for (int i = blockIdx.x; i < P.nfill; i += stride) {
        const int4 it = P.fill[i];
        d_fill_faces<D>(boxes[it.x].g, boxes[it.x].f, boxes[it.x].ctl, save, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
      const int flags = kSbCons | (P.keep_cons ? kSbKeepCons : 0) | (save ? kSbSaveBegin : 0) |
                        (P.cell_emf ? kSbCellEmf : 0);
      for (int i = blockIdx.x; i < P.nbegin; i += stride) {
        const int4 it = P.begin[i];
        d_stage_begin<D, E>(boxes[it.x].g, boxes[it.x].f, boxes[it.x].ctl, flags, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
      if (P.shock) {
        for (int i = blockIdx.x; i < P.nbegin; i += stride) {
          const int4 it = P.begin[i];
          d_find_shock<D>(boxes[it.x].g, boxes[it.x].f, boxes[it.x].ctl, dd(it));
        }
        if (!(ok = grid_barrier(bar))) break;
      }
      for (int d = 0; d < D && ok; d++) {
        const int invdt = stage == 0 ? (d == 0 ? 1 : 2) : 0;
        const int last = stage == 0 && d == D - 1;
        for (int i = blockIdx.x; i < P.nsweep[d]; i += stride) {
          const int4 it = P.sweep[d][i];
          const EnsBox& B = boxes[it.x];
          if (d == 0) d_sweep_march<D, 0, ORDER, SOLVER, T>(B.g, B.f, B.ctl, invdt, last, B.seg[0], dd(it));
          if (d == 1) d_sweep_march<D, 1, ORDER, SOLVER, T>(B.g, B.f, B.ctl, invdt, last, B.seg[1], dd(it));
          if constexpr (D == 3)
            if (d == 2) d_sweep_march<D, 2, ORDER, SOLVER, T>(B.g, B.f, B.ctl, invdt, last, B.seg[2], dd(it));
        }
        ok = grid_barrier(bar);
      }
      if (!ok) break;
      const int combine = stage > 0;
      const double wc = combine ? P.wc[stage - 1] : 1.0, w0 = combine ? P.w0[stage - 1] : 0.0;
      for (int i = blockIdx.x; i < P.nedges; i += stride) {
        const int4 it = P.edges[i];
        d_ct_corner<D, E>(boxes[it.x].g, boxes[it.x].f, boxes[it.x].ctl, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
      for (int i = blockIdx.x; i < P.nedges; i += stride) {
        const int4 it = P.edges[i];
        const EnsBox& B = boxes[it.x];
        // a box with a NaN check this cycle combines its faces after the count
        const int cmb = combine && !due_box(B.ctl, P.check_nan_period);
        d_ct_faces<D, E>(B.g, B.f, B.ctl, cmb, cmb ? wc : 1.0, cmb ? w0 : 0.0, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
      if (nan_due) {
        for (int b = t0; b < P.nbox; b += tstride)
          if (due_box(boxes[b].ctl, P.check_nan_period)) boxes[b].ctl->nan_count = 0ull;
        if (!(ok = grid_barrier(bar))) break;
        for (int i = blockIdx.x; i < P.nedges; i += stride) {
          const int4 it = P.edges[i];
          const EnsBox& B = boxes[it.x];
          if (due_box(B.ctl, P.check_nan_period)) d_nan_count<D>(B.g, B.f, B.ctl, dd(it));
        }
        if (!(ok = grid_barrier(bar))) break;
        for (int b = t0; b < P.nbox; b += tstride)
          if (due_box(boxes[b].ctl, P.check_nan_period)) d_check_nan(boxes[b].ctl);
        if (!(ok = grid_barrier(bar))) break;
        if (combine) {
          for (int i = blockIdx.x; i < P.nfill; i += stride) {
            const int4 it = P.fill[i];
            const EnsBox& B = boxes[it.x];
            if (B.ctl->done || !due_box(B.ctl, P.check_nan_period)) continue;
            const long long tid = (long long)it.y * blockDim.x + threadIdx.x;
            if (tid >= B.g.nface) continue;
            const long long q = (long long)it.z * B.g.nface + tid;
            B.f.Vs[q] = rk_combine<E>(B.f.Vs[q], B.f.Vs0[q], wc, w0);
          }
          if (!(ok = grid_barrier(bar))) break;
        }
      }
      for (int i = blockIdx.x; i < P.nactive; i += stride) {
        const int4 it = P.active[i];
        d_stage_end<D, E>(boxes[it.x].g, boxes[it.x].f, boxes[it.x].ctl, combine, wc, w0, dd(it));
      }
      if (!(ok = grid_barrier(bar))) break;
    }
    if (!ok) break;
    for (int b = t0; b < P.nbox; b += tstride) d_cycle_end(boxes[b].ctl);
    if (!(ok = grid_barrier(bar))) break;
  }
  if (!ok) {  // a bounded barrier wait gave up: every box reports it and stops
    for (int b = t0; b < P.nbox; b += tstride) report_wait_timeout(boxes[b].ctl);
  }
}

template <int D, int ORDER, int SOLVER, typename T>
int persist_blocks_t() {
  int dev = 0, sms = 148, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ke_persistent<D, ORDER, SOLVER, T>, kTM, 0) != cudaSuccess)
    return 0;
  return per * sms;
}

template <int D, int ORDER, int SOLVER, typename T>
cudaError_t launch_persist_t(EnsEngine& e, int ncyc, int grid) {
  EnsPersist P = ens_persist_args(e);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kTM);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = e.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // every block co-resident: the grid barrier is safe
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, ke_persistent<D, ORDER, SOLVER, T>, (const EnsBox*)e.d_boxes, P, ncyc, e.d_bar);
}

template <int SOLVER>
int ens_persist_blocks_solver(const EnsEngine& e) {
  const int D = e.D, O = e.order;
  const bool mixed = e.precision == 1;
#define IDFX_PCASE(DD, OO)                                                         \
  if (D == DD && O == OO) return mixed ? persist_blocks_t<DD, OO, SOLVER, float>()  \
                                       : persist_blocks_t<DD, OO, SOLVER, double>();
  IDFX_PCASE(2, 1) IDFX_PCASE(2, 2) IDFX_PCASE(2, 3) IDFX_PCASE(2, 4)
  IDFX_PCASE(3, 1) IDFX_PCASE(3, 2) IDFX_PCASE(3, 3) IDFX_PCASE(3, 4)
#undef IDFX_PCASE
  return 0;
}

template <int SOLVER>
cudaError_t launch_ens_persist_solver(EnsEngine& e, int ncyc, int grid) {
  const int D = e.D, O = e.order;
  const bool mixed = e.precision == 1;
#define IDFX_PCASE(DD, OO)                                                                      \
  if (D == DD && O == OO) return mixed ? launch_persist_t<DD, OO, SOLVER, float>(e, ncyc, grid)  \
                                       : launch_persist_t<DD, OO, SOLVER, double>(e, ncyc, grid);
  IDFX_PCASE(2, 1) IDFX_PCASE(2, 2) IDFX_PCASE(2, 3) IDFX_PCASE(2, 4)
  IDFX_PCASE(3, 1) IDFX_PCASE(3, 2) IDFX_PCASE(3, 3) IDFX_PCASE(3, 4)
#undef IDFX_PCASE
  return cudaErrorInvalidValue;
}

}  // namespace idfx
