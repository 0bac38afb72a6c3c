// C ABI and host driver of the GB300 ideal-MHD stage (see include/idefix_gb300.h).
//
// The driver mirrors TimeIntegrator::Cycle (timeIntegrator.cpp:246-414) with
// the time-step state kept on the device, so that successive cycles are
// queued without host synchronisation; the host mirrors only the cycle count
// (to schedule the divB / NaN diagnostics exactly when the reference does).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/idefix_gb300.h"
#include "ct_tile.cuh"
#include "engine.hpp"
#include "sweep_tile.cuh"

using namespace idfx;

namespace idfx {

cudaEvent_t take_event(Engine& e) {
  if (!e.free_events.empty()) {
    cudaEvent_t ev = e.free_events.back();
    e.free_events.pop_back();
    return ev;
  }
  cudaEvent_t ev;
  cudaEventCreate(&ev);
  return ev;
}

void mark_begin(Engine& e, int cls) {
  if (!e.profile) return;
  Engine::Mark m;
  m.cls = cls;
  m.a = take_event(e);
  m.b = take_event(e);
  cudaEventRecord(m.a, e.stream);
  e.marks.push_back(m);
}

void mark_end(Engine& e) {
  if (!e.profile || e.marks.empty()) return;
  cudaEventRecord(e.marks.back().b, e.stream);
}

}  // namespace idfx

namespace {

constexpr int kThreads = 256;

inline unsigned nblocks(long long n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

int fail(Engine& e, int code, const std::string& msg) {
  e.err = msg;
  return code;
}

int cuda_check(Engine& e, cudaError_t rc, const char* what) {
  if (rc != cudaSuccess) return fail(e, IDFX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(rc));
  return IDFX_OK;
}

#define IDFX_CK(call)                                        \
  do {                                                       \
    int idfx_rc_ = cuda_check(e, (call), #call);             \
    if (idfx_rc_ != IDFX_OK) return idfx_rc_;                \
  } while (0)

// ---------------------------------------------------------------------------
// auxiliary whole-block kernels used by the building-block entry points
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_prim_to_cons_all(Geo g, Fields f) {
  using v = Var<D>;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  double V[v::NV], U[v::NV];
  for (int n = 0; n < v::NV; n++) V[n] = f.Vc[n * g.ncell + c];
  prim_to_cons<D, true>(g.gm1, U, V);
  for (int n = 0; n < v::NV; n++) f.Uc[n * g.ncell + c] = U[n];
}

// ReconstructVcField on Uc (boundary.hpp:388-404), optionally followed by
// ConvertConsToPrim (convertConsToPrim.hpp:104-149), over the whole block
template <int D>
__global__ void k_uc_field_all(Geo g, Fields f, int to_prim) {
  using v = Var<D>;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const int i = (int)(c % g.nt[0]);
  const long long r = c / g.nt[0];
  const int j = (int)(r % g.nt[1]);
  const int k = (int)(r / g.nt[1]);
  const long long fc = fidx(g, k, j, i);
  double U[v::NV], V[v::NV];
  for (int n = 0; n < v::BX1; n++) U[n] = f.Uc[n * g.ncell + c];
  for (int d = 0; d < D; d++) {
    const double* vs = f.Vs + d * g.nface;
    U[v::BX1 + d] = 0.5 * (vs[fc] + vs[fc + g.fs[d]]);
    f.Uc[(v::BX1 + d) * g.ncell + c] = U[v::BX1 + d];
  }
  if (!to_prim) return;
  cons_to_prim<D, true>(g.gm1, V, U);
  for (int n = 0; n < v::NV; n++) f.Vc[n * g.ncell + c] = V[n];
}

// the cell-centred field of Uc from the faces over the active cells, as the
// stage end forms it (mixed path, whose stage ends do not store it)
template <int D>
__global__ void k_uc_field_active(Geo g, Fields f) {
  using v = Var<D>;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)g.n[0] * g.n[1] * (D == 3 ? g.n[2] : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % g.n[0]);
  const long long r = tid / g.n[0];
  const int j = g.beg[1] + (int)(r % g.n[1]);
  const int k = (D == 3) ? g.beg[2] + (int)(r / g.n[1]) : 0;
  const long long c = cidx(g, k, j, i), fc = fidx(g, k, j, i);
  for (int d = 0; d < D; d++) {
    const double* vs = f.Vs + d * g.nface;
    f.Uc[(v::BX1 + d) * g.ncell + c] = 0.5 * (vs[fc] + vs[fc + g.fs[d]]);
  }
}

// E: type of the EMF buffers (FP32 on the mixed path)
template <int D, typename E>
__global__ void k_cell_emf_all(Geo g, Fields f) {
  using v = Var<D>;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  auto V = [&](int n) { return from_f64<E>(f.Vc[n * g.ncell + c]); };
  const E vx1 = V(v::MX1), vx2 = V(v::MX2);
  const E Bx1 = V(v::BX1), Bx2 = V(v::BX2);
  if constexpr (D == 3) {
    const E vx3 = V(v::MX3), Bx3 = V(v::BX3);
    emf<E>(f.Ex1)[c] = (vx3 * Bx2 - vx2 * Bx3);
    emf<E>(f.Ex2)[c] = (vx1 * Bx3 - vx3 * Bx1);
  }
  emf<E>(f.Ex3)[c] = (vx2 * Bx1 - vx1 * Bx2);
}

// FP32 copy of the primitives for the mixed-precision sweeps (the building
// blocks run the sweeps without a stage begin)
__global__ void k_vc32(Geo g, Fields f, int nv) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  for (int n = 0; n < nv; n++) f.Vc32[n * g.ncell + c] = d2f_rn(f.Vc[n * g.ncell + c]);
}

template <int D>
__global__ void k_invdt_max(Geo g, Fields f, Ctl* ctl) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)g.n[0] * g.n[1] * (D == 3 ? g.n[2] : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % g.n[0]);
  const long long r = tid / g.n[0];
  const int j = g.beg[1] + (int)(r % g.n[1]);
  const int k = (D == 3) ? g.beg[2] + (int)(r / g.n[1]) : 0;
  atomic_max_pos(&ctl->invdt_max_bits, f.InvDt[cidx(g, k, j, i)]);
}

// Control-block traffic and device-side state copies by kernels rather
// than cudaMemcpyAsync / cudaMemsetAsync: those go to the copy engines,
// where a control read of a few hundred bytes waits behind whatever
// gigabyte-sized host transfer a caller has queued on another stream (the
// pipelined loop that overlaps the next step's input and the previous
// step's result with a cycle).  A kernel writes the pinned host mirror
// directly, and a Ctl passed by value is taken at launch.
__global__ void k_ctl_put(Ctl* ctl, Ctl v) { *ctl = v; }
__global__ void k_ctl_get(const Ctl* ctl, Ctl* host) { *host = *ctl; }
enum { kClrUcFresh = 1, kClrDone = 2, kClrNan = 4, kClrDivB = 8, kClrInvDt = 16 };
__global__ void k_ctl_clear(Ctl* ctl, int what) {
  if (what & kClrUcFresh) ctl->uc_fresh = 0;
  if (what & kClrDone) ctl->done = 0;
  if (what & kClrNan) ctl->nan_count = 0ull;
  if (what & kClrDivB) ctl->divb_bits = 0ull;
  if (what & kClrInvDt) ctl->invdt_max_bits = 0ull;
}
// n doubles from src to dst (device memory), 16-byte vectors where both
// addresses allow it
__global__ void k_copy_f64(double* __restrict__ dst, const double* __restrict__ src, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
    const long long n2 = n / 2;
    double2* d2 = reinterpret_cast<double2*>(dst);
    const double2* s2 = reinterpret_cast<const double2*>(src);
    for (long long q = t; q < n2; q += stride) d2[q] = s2[q];
    if (t == 0 && (n & 1)) dst[n - 1] = src[n - 1];
  } else {
    for (long long q = t; q < n; q += stride) dst[q] = src[q];
  }
}

// Bounded-wait probe: the wait of the bulk-copy staged sweep (mbar_wait)
// and its give-up path (report_wait_timeout) on an mbarrier whose phase
// never completes (mode 0: nothing arrives, as when a copy never lands) or
// completes at once (mode 1: its one expected arrival is made).
__global__ void k_wait_probe(Ctl* ctl, int mode, long long limit, int* gave_up) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (mode == 1) mbar_arrive(&bar);
  const bool ok = mbar_wait(&bar, 0u, limit);
  *gave_up = ok ? 0 : 1;
  if (!ok) report_wait_timeout(ctl);
}

__global__ void k_set_stage_dt(Geo g, Ctl* ctl, double dt) {
  double dV = g.dx[0] * g.dx[1];
  if (g.D == 3) dV = dV * g.dx[2];
  ctl->dtdV = dt / dV;
  for (int d = 0; d < 3; d++) ctl->dtdx[d] = dt / g.dx[d];
}

template <typename E>
__global__ void k_faces_combine(Geo g, Fields f, Ctl* ctl, double wc, double w0) {
  if (ctl->done) return;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = g.nface * g.D;
  if (tid >= tot) return;
  f.Vs[tid] = rk_combine<E>(f.Vs[tid], f.Vs0[tid], wc, w0);  // as k_ct_faces combines
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
// A profiler range named as the reference's region for the same work
// (idfx::pushRegion / popRegion, which reach NVTX through Kokkos' profiling
// hooks): Nsight shows the library's launches under the reference's names.
// Host-side ranges around the launches they queue; no cost without a tool.
struct Region {
  explicit Region(const char* name) { nvtxRangePushA(name); }
  ~Region() { nvtxRangePop(); }
  Region(const Region&) = delete;
  Region& operator=(const Region&) = delete;
};

void launch_sweeps(Engine& e, int invdt, int fold_max) {
  switch (e.g.solver) {
    case kHLLD: launch_sweeps_hlld(e, invdt, fold_max); break;
    case kHLL: launch_sweeps_hll(e, invdt, fold_max); break;
    case kROE: launch_sweeps_roe(e, invdt, fold_max); break;
    default: launch_sweeps_tvdlf(e, invdt, fold_max); break;
  }
}

long long n_active(const Geo& g) { return (long long)g.n[0] * g.n[1] * g.n[2]; }
long long n_edges(const Geo& g) {
  return (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.D == 3 ? g.n[2] + 1 : 1);
}

#define IDFX_DISPATCH_D(K, GRID, BLOCK, ...)                                \
  do {                                                                      \
    if (e.g.D == 2) K<2><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);        \
    else K<3><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);                   \
  } while (0)

// dimension and EMF type (FP32 EMF buffers on the mixed path)
#define IDFX_DISPATCH_DE(K, GRID, BLOCK, ...)                                              \
  do {                                                                                     \
    const bool f32 = (e.precision == IDFX_MIXED);                                          \
    if (e.g.D == 2) {                                                                      \
      if (f32) K<2, float><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);                     \
      else K<2, double><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);                        \
    } else {                                                                               \
      if (f32) K<3, float><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);                     \
      else K<3, double><<<GRID, BLOCK, 0, e.stream>>>(__VA_ARGS__);                        \
    }                                                                                      \
  } while (0)

void launch_fill_faces(Engine& e, int save_begin) {
  dim3 grid(nblocks(e.g.nface), e.g.D);
  mark_begin(e, kKFillFaces);
  IDFX_DISPATCH_D(k_fill_faces, grid, kThreads, e.g, e.f, e.ctl, save_begin);
  mark_end(e);
}
// the ghost faces alone (periodic block, no Runge-Kutta begin copy due)
void launch_fill_face_ghosts(Engine& e) {
  long long slab = 0;
  for (int comp = 0; comp < e.g.D; comp++)
    for (int dir = 0; dir < e.g.D; dir++) {
      long long n = 2LL * e.g.ng;
      for (int d = 0; d < e.g.D; d++)
        if (d != dir) n *= (d == comp) ? e.g.nt[d] + 1 : e.g.nt[d];
      if (n > slab) slab = n;
    }
  mark_begin(e, kKFillFaces);
  IDFX_DISPATCH_D(k_fill_face_ghosts, dim3(nblocks(slab), e.g.D * e.g.D), kThreads, e.g, e.f, e.ctl);
  mark_end(e);
}
// Boundary::SetBoundaries of a block with a reflective or outflow direction
void launch_boundaries(Engine& e) {
  if (!e.g.nonper) return;
  for (int dir = 0; dir < e.g.D; dir++) {
    const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;
    mark_begin(e, kKFillFaces);
    dim3 grid(nblocks(2LL * e.g.ng * e.g.ntv[a] * e.g.ntv[b]), 1 + e.g.D);
    IDFX_DISPATCH_D(k_bc_slab, grid, kThreads, e.g, e.f, e.ctl, dir);
    mark_end(e);
    if (e.g.bc[dir][0] != 0) {
      mark_begin(e, kKFillFaces);
      IDFX_DISPATCH_D(k_normal_field, nblocks((long long)e.g.nt[a] * e.g.nt[b]), kThreads, e.g, e.f, e.ctl, dir);
      mark_end(e);
    }
  }
}
void launch_stage_begin(Engine& e, int flags) {
  mark_begin(e, kKStageBegin);
  IDFX_DISPATCH_DE(k_stage_begin, nblocks(e.g.ncell), kThreads, e.g, e.f, e.ctl, flags);
  mark_end(e);
}
// the ghost cells alone (mixed path, periodic block, after a stage end that
// wrote the active cells' outputs)
void launch_stage_ghosts(Engine& e, int flags) {
  long long slab = 0;
  for (int d = 0; d < e.g.D; d++) {
    const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
    const long long n = 2LL * e.g.ng * e.g.nt[a] * e.g.nt[b];
    if (n > slab) slab = n;
  }
  mark_begin(e, kKStageBegin);
  IDFX_DISPATCH_DE(k_stage_ghosts, dim3(nblocks(slab), e.g.D), kThreads, e.g, e.f, e.ctl, flags);
  mark_end(e);
}
void launch_ct(Engine& e, int combine, double wc, double w0) {
  // mixed path: corner EMFs and face update in one pass (the corner EMFs
  // stay on chip) - for the averages that do not read the face field; the
  // uct_hll / uct_hlld corner EMFs reconstruct it, and the fused pass
  // updates it while other tiles still read it
  if (e.precision == IDFX_MIXED && e.g.emf != kEmfUctHll && e.g.emf != kEmfUctHlld) {
    const Geo& g = e.g;
    dim3 grid((unsigned)((g.n[0] + 1 + kCtTI - 1) / kCtTI), (unsigned)((g.n[1] + 1 + kCtTJ - 1) / kCtTJ),
              (unsigned)(g.D == 3 ? (g.n[2] + 1 + kCtKSeg - 1) / kCtKSeg : 1));
    // (the corner EMFs are computed inside the face update's pass)
    const Region r("ConstrainedTransport::EvolveMagField");
    mark_begin(e, kKCtFaces);
    const CtTileMap* cm = (g.D == 3) ? ct_tile_map(e) : nullptr;
    if (cm) {
      // the corner EMFs' inputs staged by tensor-map copies (ct_tile.cuh)
      static const bool smem_set = cudaFuncSetAttribute(k_ct_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        ct_tile_smem()) == cudaSuccess;
      (void)smem_set;
      k_ct_tile<<<grid, dim3(kCtTI, kCtTJ), ct_tile_smem(), e.stream>>>(g, e.f, e.ctl, combine, wc, w0, cm->emf);
    } else if (g.D == 2) {
      k_ct_fused<2, float><<<grid, dim3(kCtTI, kCtTJ), 0, e.stream>>>(g, e.f, e.ctl, combine, wc, w0);
    } else {
      k_ct_fused<3, float><<<grid, dim3(kCtTI, kCtTJ), 0, e.stream>>>(g, e.f, e.ctl, combine, wc, w0);
    }
    mark_end(e);
    return;
  }
  {
    const Region r("ConstrainedTransport::CalcCornerEMF");
    mark_begin(e, kKCtCorner);
    IDFX_DISPATCH_DE(k_ct_corner, nblocks(n_edges(e.g)), kThreads, e.g, e.f, e.ctl);
    mark_end(e);
  }
  const Region r("ConstrainedTransport::EvolveMagField");
  mark_begin(e, kKCtFaces);
  IDFX_DISPATCH_DE(k_ct_faces, nblocks(n_edges(e.g)), kThreads, e.g, e.f, e.ctl, combine, wc, w0);
  mark_end(e);
}
void launch_find_shock(Engine& e) {
  const long long m = (long long)(e.g.n[0] + 2) * (e.g.n[1] + 2) * (e.g.D == 3 ? e.g.n[2] + 2 : 1);
  mark_begin(e, kKStageBegin);
  IDFX_DISPATCH_D(k_find_shock, nblocks(m), kThreads, e.g, e.f, e.ctl);
  mark_end(e);
}

void ctl_clear(Engine& e, int what) { k_ctl_clear<<<1, 1, 0, e.stream>>>(e.ctl, what); }
void ctl_push(Engine& e) { k_ctl_put<<<1, 1, 0, e.stream>>>(e.ctl, *e.ctl_host); }

// device -> device copy of n doubles on the engine's stream (SMs, not a copy engine)
void copy_f64(Engine& e, double* dst, const double* src, long long n) {
  if (n <= 0) return;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n / 2 + kThreads - 1) / kThreads;
  const unsigned blocks = (unsigned)(want < (long long)sms * 8 ? (want > 0 ? want : 1) : (long long)sms * 8);
  k_copy_f64<<<blocks, kThreads, 0, e.stream>>>(dst, src, n);
}

void launch_nan_check(Engine& e) {
  ctl_clear(e, kClrNan);
  IDFX_DISPATCH_D(k_nan_count, nblocks(n_edges(e.g)), kThreads, e.g, e.f, e.ctl);
  k_check_nan<<<1, 1, 0, e.stream>>>(e.ctl);
}
void launch_divb_check(Engine& e) {
  ctl_clear(e, kClrDivB);
  IDFX_DISPATCH_D(k_divb, nblocks(n_active(e.g)), kThreads, e.g, e.f, e.ctl);
  k_check_divb<<<1, 1, 0, e.stream>>>(e.ctl);
}

// queue one TimeIntegrator::Cycle
void queue_cycle(Engine& e, int use_tstop) {
  const Region cycle_region("TimeIntegrator::Cycle");
  const Geo& g = e.g;
  const bool cell_emf = (g.emf == kEmfContact || g.emf == kEmfUct0);
  const bool fused = (e.precision == IDFX_MIXED) && !g.nonper;
  k_cycle_begin<<<1, 1, 0, e.stream>>>(g, e.ctl, use_tstop);
  if (e.log_period > 0 && e.ncycles % e.log_period == 0) launch_divb_check(e);
  const bool nan_check = e.check_nan_period > 0 && e.ncycles % e.check_nan_period == 0;
  for (int stage = 0; stage < e.nstages; stage++) {
    const int save = (e.nstages > 1 && stage == 0);
    {
      const Region r("Boundary::SetBoundaries");
      launch_boundaries(e);
      // periodic block: a Runge-Kutta begin copy of the faces that the
      // previous cycle's last face update already wrote leaves the ghosts
      if (!g.nonper && (!save || e.faces_saved)) launch_fill_face_ghosts(e);
      else launch_fill_faces(e, save);
    }
    // mixed path: Uc carried over from the previous stage end when it is
    // still the state Vc came from (Ctl::uc_fresh); the FP64 path rebuilds it
    // as the reference does
    const int cons = kSbCons | (e.precision == IDFX_MIXED ? kSbKeepCons : 0);
    const int sb_flags = cons | (save ? kSbSaveBegin : 0) | (cell_emf ? kSbCellEmf : 0);
    // mixed path, periodic block: once a stage end of this run has written
    // the active cells' FP32 primitives, cell EMF and Runge-Kutta begin copy,
    // the stage begin fills the ghost cells alone
    {
      const Region r("Fluid::ConvertPrimToCons");
      if (fused && e.stage_outputs) launch_stage_ghosts(e, sb_flags);
      else launch_stage_begin(e, sb_flags);
    }
    const int combine = stage > 0;
    const double wc = combine ? e.wc[stage - 1] : 1.0, w0 = combine ? e.w0[stage - 1] : 0.0;
    {
      const Region stage_region("Fluid::EvolveStage");
      {
        const Region r("RiemannSolver::CalcFlux");
        if (e.f.shock) launch_find_shock(e);  // RiemannSolver::CalcFlux (calcFlux.hpp:33)
        launch_sweeps(e, stage == 0 ? 1 : 0, stage == 0);
      }
      if (nan_check) {
        launch_ct(e, 0, 1.0, 0.0);
        {
          const Region rn("Fluid::CheckNan");
          launch_nan_check(e);
        }
        if (combine) {
          if (e.precision == IDFX_MIXED)
            k_faces_combine<float><<<nblocks(g.nface * g.D), kThreads, 0, e.stream>>>(g, e.f, e.ctl, wc, w0);
          else
            k_faces_combine<double><<<nblocks(g.nface * g.D), kThreads, 0, e.stream>>>(g, e.f, e.ctl, wc, w0);
        }
        e.faces_saved = false;
      } else {
        // periodic block: the last stage's face update also writes the next
        // cycle's Runge-Kutta begin copy of the faces
        const bool save_next = !g.nonper && e.nstages > 1 && stage == e.nstages - 1;
        launch_ct(e, (combine ? kCtCombine : 0) | (save_next ? kCtSaveBegin : 0), wc, w0);
        if (save_next) e.faces_saved = true;
      }
    }
    const int out = fused ? (kSeOutputs | kSeNoUcField | (cell_emf ? kSbCellEmf : 0) |
                             (e.nstages > 1 && stage == e.nstages - 1 ? kSeSaveBegin : 0))
                          : 0;
    if (fused) e.uc_field_stale = true;
    {
      const Region r("Fluid::ConvertConsToPrim");
      mark_begin(e, kKStageEnd);
      IDFX_DISPATCH_DE(k_stage_end, nblocks(n_active(g)), kThreads, g, e.f, e.ctl, combine, wc, w0, out);
      mark_end(e);
    }
    if (fused) e.stage_outputs = true;
  }
  k_cycle_end<<<1, 1, 0, e.stream>>>(e.ctl);
  e.ncycles++;
}

int read_ctl(Engine& e) {
  k_ctl_get<<<1, 1, 0, e.stream>>>(e.ctl, e.ctl_host_dev);
  IDFX_CK(cudaGetLastError());
  IDFX_CK(cudaStreamSynchronize(e.stream));
  return IDFX_OK;
}

const char* status_text(int s) {
  switch (s) {
    case kErrNan: return "Nan found after integration cycle";
    case kErrDivB: return "divB too large, check your calculation";
    case kErrDtSmall: return "dt is too small";
    case kErrFirstDt: return "Your guessed first_dt is too large. Try to reduce first_dt.";
    default: return "error";
  }
}

}  // namespace

// Boundary types per direction: IDFX_BC_* on both sides, periodic on both or
// on neither; a mirror (reflective) needs as many active cells as ghosts.
static bool boundaries_valid(const idfx_gpu_config* cfg) {
  const int ng = (cfg->order == 4) ? 3 : 2;
  for (int d = 0; d < cfg->dims; d++) {
    const int l = cfg->lbound[d], r = cfg->rbound[d];
    if (l < IDFX_BC_PERIODIC || l > IDFX_BC_OUTFLOW || r < IDFX_BC_PERIODIC || r > IDFX_BC_OUTFLOW) return false;
    if ((l == IDFX_BC_PERIODIC) != (r == IDFX_BC_PERIODIC)) return false;
    if ((l == IDFX_BC_REFLECTIVE || r == IDFX_BC_REFLECTIVE) && cfg->n[d] < ng) return false;
  }
  return true;
}

namespace idfx {

// the staged fused CT pass: a 4-D tensor map (x, y, z, array) over the
// twelve FP32 EMF inputs of the corner EMFs, consecutive arrays of the pool;
// null where the block does not allow it (then the unstaged fused pass runs)
const CtTileMap* ct_tile_map(Engine& e) {
  if (e.ct_map_tried) return e.ct_map;
  e.ct_map_tried = true;
  const Geo& g = e.g;
  const Fields& f = e.f;
  if (g.D != 3 || e.precision != IDFX_MIXED || g.nt[0] % 4 != 0) return nullptr;
  const double* arr[kEaN] = {f.ezi, f.ezj, f.exj, f.exk, f.eyi, f.eyk, f.svx, f.svy, f.svz, f.Ex1, f.Ex2, f.Ex3};
  for (int q = 0; q < kEaN; q++)
    if (arr[q] != f.ezi + (long long)q * g.ncell) return nullptr;  // evenly spaced, in this order
  if ((reinterpret_cast<uintptr_t>(f.ezi) & 15) || (g.ncell * 8) % 16) return nullptr;
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return nullptr;
  }
  const Encode enc = reinterpret_cast<Encode>(fn);
  auto* m = new (std::nothrow) CtTileMap();
  if (!m) return nullptr;
  const cuuint64_t n0 = (cuuint64_t)g.nt[0], n1 = (cuuint64_t)g.nt[1], n2 = (cuuint64_t)g.nt[2];
  const cuuint64_t dims[4] = {n0, n1, n2, (cuuint64_t)kEaN};
  // FP32 values in the arrays' FP64-sized slots: rows of nt0 floats, arrays
  // ncell doubles apart
  const cuuint64_t strides[3] = {n0 * 4, n0 * n1 * 4, (cuuint64_t)g.ncell * 8};
  const cuuint32_t box[4] = {kCsX, kCsY, 1, kEaN};
  const cuuint32_t unit[4] = {1, 1, 1, 1};
  if (enc(&m->emf, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<double*>(f.ezi), dims, strides, box, unit,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    delete m;
    return nullptr;
  }
  e.ct_map = m;
  return m;
}

const SweepTileMaps* sweep_tile_maps(Engine& e) {
  if (e.tile_maps_tried) return e.tile_maps;
  e.tile_maps_tried = true;
  const Geo& g = e.g;
  if (g.D != 3 || e.precision != IDFX_MIXED || g.nt[0] % 4 != 0 || !e.f.Vc32) return nullptr;
  if ((reinterpret_cast<uintptr_t>(e.f.Vc32) | reinterpret_cast<uintptr_t>(e.f.Uc) |
       reinterpret_cast<uintptr_t>(e.f.InvDt)) & 15)
    return nullptr;
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return nullptr;
  }
  const Encode enc = reinterpret_cast<Encode>(fn);
  auto* m = new (std::nothrow) SweepTileMaps();
  if (!m) return nullptr;
  const cuuint64_t n0 = (cuuint64_t)g.nt[0], n1 = (cuuint64_t)g.nt[1], n2 = (cuuint64_t)g.nt[2];
  const cuuint64_t nc = (cuuint64_t)g.ncell;
  const cuuint32_t unit[4] = {1, 1, 1, 1};
  bool ok = true;
  for (int d = 0; d < 2; d++) {
    // y sweep: a box of one y row and kTB z rows; z sweep: kTB y rows and one z row
    const cuuint32_t by = (d == 0) ? 1 : kTB, bz = (d == 0) ? kTB : 1;
    const cuuint64_t dims[4] = {n0, n1, n2, 8};
    const cuuint64_t s4[3] = {n0 * 4, n0 * n1 * 4, nc * 4};
    const cuuint32_t bv[4] = {kTX, by, bz, 8};
    ok = ok && enc(&m->vc[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, e.f.Vc32, dims, s4, bv, unit,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    const cuuint64_t s8[3] = {n0 * 8, n0 * n1 * 8, nc * 8};
    const cuuint32_t bu[4] = {kTX, by, bz, 5};
    ok = ok && enc(&m->uc[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, e.f.Uc, dims, s8, bu, unit,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    const cuuint32_t bi[3] = {kTX, by, bz};
    ok = ok && enc(&m->inv[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, e.f.InvDt, dims, s8, bi, unit,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  if (!ok) {
    delete m;
    return nullptr;
  }
  e.tile_maps = m;
  return m;
}

bool tile_sweep_eligible(Engine& e, int dir) {
  return (dir == 1 || dir == 2) && e.g.D == 3 && e.precision == IDFX_MIXED && e.g.order >= 2 && e.g.order <= 4 &&
         sweep_tile_maps(e) != nullptr;
}

// Validation of a block configuration and the block's grid and geometry:
// ghost zones (grid.cpp:60-65), cell widths (gridHost.cpp:80-86), face
// areas (makeGeometry.cpp:146-147,178-179,201-202), the correctly rounded
// reciprocals of the exact quotient forms, and the CT extension of the
// sweeps.  Shared by the handle (idfx_gpu_create) and the allocation-free
// stage, so that both set up a block identically.
int block_geometry(const idfx_gpu_config* cfg, Geo& g) {
  if (!cfg) return IDFX_ERR_STATE;
  if (cfg->dims != 2 && cfg->dims != 3) return IDFX_ERR_CONFIG;
  if (cfg->order < 1 || cfg->order > 5 || cfg->solver < 0 || cfg->solver > 3) return IDFX_ERR_CONFIG;
  // the learned reconstruction: 3-D, HLLD, FP64 arithmetic around the network
  if (cfg->order == IDFX_LEARNED &&
      (cfg->dims != 3 || cfg->solver != IDFX_HLLD || cfg->precision != IDFX_FP64 || cfg->shock_flattening))
    return IDFX_ERR_CONFIG;
  if (cfg->emf < 0 || cfg->emf > 4 || cfg->nstages < 1 || cfg->nstages > 3) return IDFX_ERR_CONFIG;
  if (cfg->precision != IDFX_FP64 && cfg->precision != IDFX_MIXED) return IDFX_ERR_CONFIG;
  // constrainedTransport.hpp:256-261
  if (cfg->emf == IDFX_EMF_UCT_HLLD && (cfg->solver == IDFX_HLL || cfg->solver == IDFX_TVDLF))
    return IDFX_ERR_CONFIG;
  for (int d = 0; d < cfg->dims; d++)
    if (cfg->n[d] < 2 || !(cfg->xend[d] > cfg->xbeg[d])) return IDFX_ERR_CONFIG;
  if (!boundaries_valid(cfg)) return IDFX_ERR_CONFIG;
  g.D = cfg->dims;
  g.order = cfg->order;
  g.solver = cfg->solver;
  g.emf = cfg->emf;
  g.nstages = cfg->nstages;
  g.ng = (cfg->order == 4) ? 3 : 2;  // grid.cpp:60-65
  for (int d = 0; d < 3; d++) {
    const bool act = d < g.D;
    const int gd = act ? g.ng : 0;
    g.n[d] = act ? cfg->n[d] : 1;
    g.nt[d] = g.n[d] + 2 * gd;
    g.ntv[d] = g.nt[d] + (act ? 1 : 0);
    g.beg[d] = gd;
    g.end[d] = gd + g.n[d];
    const double xb = act ? cfg->xbeg[d] : 0.0, xe = act ? cfg->xend[d] : 1.0;
    g.dx[d] = (xe - xb) / (g.n[d]);  // gridHost.cpp:80-86
  }
  g.s[0] = 1;
  g.s[1] = g.nt[0];
  g.s[2] = (long long)g.nt[0] * g.nt[1];
  g.fs[0] = 1;
  g.fs[1] = g.ntv[0];
  g.fs[2] = (long long)g.ntv[0] * g.ntv[1];
  g.ncell = (long long)g.nt[0] * g.nt[1] * g.nt[2];
  g.nface = (long long)g.ntv[0] * g.ntv[1] * g.ntv[2];
  if (g.D == 2) {  // makeGeometry.cpp (Cartesian): D_EXPAND products
    g.A[0] = 1.0 * g.dx[1];
    g.A[1] = g.dx[0] * 1.0;
    g.A[2] = 1.0;
  } else {
    g.A[0] = 1.0 * g.dx[1] * g.dx[2];
    g.A[1] = g.dx[0] * 1.0 * g.dx[2];
    g.A[2] = g.dx[0] * g.dx[1] * 1.0;
  }
  g.gamma = cfg->gamma;
  g.gm1 = cfg->gamma - 1.0;
  g.rgm1 = 1.0 / g.gm1;  // correctly rounded reciprocals (Markstein quotients)
  for (int d = 0; d < 3; d++) {
    g.rdx[d] = 1.0 / g.dx[d];
    const double e = 0.1 * g.dx[d];  // LimO3's r dx, squared as the limiter does
    g.l3b[d] = e * e;
    g.l3y[d] = 1.0 / g.l3b[d];
  }
  g.ext = 1;  // hlldMHD.hpp:30-49: uct_hll(d) with HLLD/HLL needs nghost cells
  if ((g.emf == kEmfUctHll || g.emf == kEmfUctHlld) && (g.solver == kHLLD || g.solver == kHLL)) g.ext = g.ng;
  g.shock_smoothing = cfg->shock_smoothing;
  g.nonper = 0;
  for (int d = 0; d < 3; d++) {
    g.bc[d][0] = d < g.D ? cfg->lbound[d] : 0;
    g.bc[d][1] = d < g.D ? cfg->rbound[d] : 0;
    if (g.bc[d][0] || g.bc[d][1]) g.nonper = 1;
  }
  return IDFX_OK;
}

// March segment length per direction: enough marching columns x segments to
// fill the GPU (>= ~512 threads per SM)
void choose_segments(Engine& e) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (long long)sms * 512;
  for (int d = 0; d < e.g.D; d++) {
    // marching columns: the two other directions (with the CT extension)
    const int a = (d == 0) ? 1 : 0, b = (d == 2) ? 1 : 2;
    const long long cols = (long long)(e.g.n[a] + 2 * e.g.ext) * (e.g.D == 3 ? e.g.n[b] + 2 * e.g.ext : 1);
    int s = 64;
    while (s > 2 && cols * ((e.g.n[d] + s - 1) / s) < want) s /= 2;
    e.seg[d] = s;
  }
}

}  // namespace idfx

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void idfx_gpu_default_config(idfx_gpu_config* c, int dims, int nx, int ny, int nz) {
  std::memset(c, 0, sizeof(*c));
  c->dims = dims;
  c->n[0] = nx;
  c->n[1] = ny;
  c->n[2] = dims == 3 ? nz : 1;
  for (int d = 0; d < 3; d++) {
    c->xbeg[d] = 0.0;
    c->xend[d] = 1.0;
  }
  c->order = IDFX_PLM;
  c->solver = IDFX_HLLD;
  c->emf = IDFX_EMF_UCT_CONTACT;
  c->nstages = 2;
  c->gamma = 5.0 / 3.0;
  c->cfl = 0.9;
  c->cfl_max_var = 1.1;   // timeIntegrator.cpp:40
  c->first_dt = 1.0e-10;  // timeIntegrator.cpp:41
  c->maxdivb = 1e-6;      // timeIntegrator.cpp:56
  c->log_period = 100;    // timeIntegrator.cpp:44
  c->check_nan_period = 100;
  c->precision = IDFX_FP64;
}

int idfx_gpu_create(const idfx_gpu_config* cfg, void* stream, idfx_gpu** out) {
  if (!cfg || !out) return IDFX_ERR_STATE;
  *out = nullptr;
  Geo geo{};
  const int grc = block_geometry(cfg, geo);
  if (grc != IDFX_OK) return grc;
  idfx_gpu* h = new (std::nothrow) idfx_gpu();
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  Geo& g = e.g;
  g = geo;
  e.nstages = cfg->nstages;
  e.precision = cfg->precision;
  if (e.nstages == 2) {  // timeIntegrator.cpp:62-71
    e.wc[0] = 0.5;
    e.w0[0] = 0.5;
  }
  if (e.nstages == 3) {
    e.wc[0] = 0.25;
    e.w0[0] = 0.75;
    e.wc[1] = 2.0 / 3.0;
    e.w0[1] = 1.0 / 3.0;
  }
  e.log_period = cfg->log_period;
  e.check_nan_period = cfg->check_nan_period;

  // device buffers: one pool, zero-initialised like Kokkos views
  const int NV = 2 * g.D + 2;
  const size_t nc = (size_t)g.ncell, nf = (size_t)g.nface;
  const bool hll_emf = (g.emf == kEmfUctHll || g.emf == kEmfUctHlld);
  size_t len = 3 * NV * nc + 2 * g.D * nf + nc  // Vc, Uc, Uc0, Vs, Vs0, InvDt
               + 6 * nc + 3 * nc + 3 * nc + 3 * nc  // face EMFs, sv, cell EMFs, corner EMFs
               + (hll_emf ? 12 * nc : 0)
               + (cfg->precision == IDFX_MIXED ? (NV * nc + 1) / 2 : 0)   // FP32 primitives
               + (cfg->shock_flattening ? (nc + 7) / 8 : 0);               // shock flags
  int rc = IDFX_OK;
  if (stream) {
    e.stream = (cudaStream_t)stream;
  } else {
    rc = cuda_check(e, cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    e.own_stream = (rc == IDFX_OK);
  }
  if (rc == IDFX_OK) rc = cuda_check(e, cudaMalloc(&e.pool, len * sizeof(double)), "cudaMalloc(fields)");
  if (rc == IDFX_OK) rc = cuda_check(e, cudaMemsetAsync(e.pool, 0, len * sizeof(double), e.stream), "cudaMemset");
  if (rc == IDFX_OK) rc = cuda_check(e, cudaMalloc(&e.ctl, sizeof(Ctl)), "cudaMalloc(ctl)");
  if (rc == IDFX_OK) rc = cuda_check(e, cudaMallocHost(&e.ctl_host, sizeof(Ctl)), "cudaMallocHost(ctl)");
  if (rc == IDFX_OK)
    rc = cuda_check(e, cudaHostGetDevicePointer((void**)&e.ctl_host_dev, e.ctl_host, 0), "cudaHostGetDevicePointer(ctl)");
  if (rc != IDFX_OK) {
    std::fprintf(stderr, "idfx_gpu_create: %s\n", e.err.c_str());
    idfx_gpu_destroy(h);
    return rc;
  }
  e.pool_len = len;
  double* p = e.pool;
  auto take = [&](size_t n) { double* q = p; p += n; return q; };
  Fields& f = e.f;
  f.Vc = take(NV * nc);
  f.Uc = take(NV * nc);
  f.Uc0 = take(NV * nc);
  f.Vs = take(g.D * nf);
  f.Vs0 = take(g.D * nf);
  f.InvDt = take(nc);
  f.ezi = take(nc); f.ezj = take(nc); f.exj = take(nc); f.exk = take(nc); f.eyi = take(nc); f.eyk = take(nc);
  f.svx = take(nc); f.svy = take(nc); f.svz = take(nc);
  f.Ex1 = take(nc); f.Ex2 = take(nc); f.Ex3 = take(nc);
  f.ex = take(nc); f.ey = take(nc); f.ez = take(nc);
  for (int d = 0; d < 3; d++) {
    f.aL[d] = hll_emf ? take(nc) : nullptr;
    f.aR[d] = hll_emf ? take(nc) : nullptr;
    f.dL[d] = hll_emf ? take(nc) : nullptr;
    f.dR[d] = hll_emf ? take(nc) : nullptr;
  }
  f.Vc32 = (cfg->precision == IDFX_MIXED) ? reinterpret_cast<float*>(take((NV * nc + 1) / 2)) : nullptr;
  f.shock = cfg->shock_flattening ? reinterpret_cast<unsigned char*>(take((nc + 7) / 8)) : nullptr;
  Ctl c{};
  c.t = 0.0;
  c.dt = cfg->first_dt;
  c.tstop = -1.0;
  c.cfl = cfg->cfl;
  c.cflmax = cfg->cfl_max_var;
  c.maxdivb = cfg->maxdivb;
  *e.ctl_host = c;
  ctl_push(e);
  rc = cuda_check(e, cudaGetLastError(), "ctl");
  if (rc == IDFX_OK) rc = cuda_check(e, cudaStreamSynchronize(e.stream), "sync");
  if (rc != IDFX_OK) {
    idfx_gpu_destroy(h);
    return rc;
  }
  choose_segments(e);
  *out = h;
  return IDFX_OK;
}

// Autotuner of the march segment length per direction: the sweeps of each
// direction are timed alone for every candidate (min over reps launches);
// they accumulate into Uc, InvDt and the EMF arrays, so the whole field pool
// and the control block are saved first and put back afterwards.  Results
// do not depend on the segment length (each face is solved once either way).
int idfx_gpu_autotune(idfx_gpu* h, int reps) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  if (e.g.order == IDFX_LEARNED && !e.learned)
    return fail(e, IDFX_ERR_STATE, "the learned reconstruction needs idfx_gpu_set_learned first");
  if (reps < 1) reps = 1;
  double* backup = nullptr;
  IDFX_CK(cudaMalloc(&backup, e.pool_len * sizeof(double)));
  int rc = read_ctl(e);
  const Ctl saved = *e.ctl_host;
  if (!rc) rc = cuda_check(e, cudaMemcpyAsync(backup, e.pool, e.pool_len * sizeof(double),
                                              cudaMemcpyDeviceToDevice, e.stream), "autotune backup");
  if (!rc) {
    e.ctl_host->done = 0;
    ctl_push(e);
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const bool prof = e.profile;
  e.profile = false;
  for (int d = 0; d < e.g.D && !rc; d++) {
    e.only_dir = d;
    // candidates timed in two passes (ascending, then descending), the best
    // of every launch kept per candidate, so that a drift of the clocks or
    // of the cache state during the search favours no candidate
    // candidates: march segments 4..64, and for the FP32 y / z sweeps of a
    // 3-D block the tile sweep with segments 16..256
    int cand[16], kind[16], nc = 0;
    float cand_ms[16];
    for (int s = 4; s <= 64 && s <= e.g.n[d] && nc < 16; s *= 2) {
      cand[nc] = s;
      kind[nc] = 0;
      cand_ms[nc++] = 1e30f;
    }
    if (tile_sweep_eligible(e, d))
      for (int s = 16; s <= 256 && (s <= e.g.n[d] || s == 16) && nc < 16; s *= 2) {
        cand[nc] = s;
        kind[nc] = 1;
        cand_ms[nc++] = 1e30f;
      }
    for (int pass = 0; pass < 2; pass++) {
      for (int q = 0; q < nc; q++) {
        const int c = pass == 0 ? q : nc - 1 - q;
        e.seg[d] = cand[c];
        e.tile[d] = kind[c];
        launch_sweeps(e, 2, 0);  // warm-up
        for (int r = 0; r < reps; r++) {
          cudaEventRecord(a, e.stream);
          launch_sweeps(e, 2, 0);
          cudaEventRecord(b, e.stream);
          cudaEventSynchronize(b);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, a, b);
          if (ms < cand_ms[c]) cand_ms[c] = ms;
        }
      }
    }
    int best = 0;
    for (int c = 1; c < nc; c++)
      if (cand_ms[c] < cand_ms[best]) best = c;
    if (nc > 0) {
      e.seg[d] = cand[best];
      e.tile[d] = kind[best];
    }
  }
  e.only_dir = -1;
  e.profile = prof;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!rc) rc = cuda_check(e, cudaGetLastError(), "autotune");
  cudaMemcpyAsync(e.pool, backup, e.pool_len * sizeof(double), cudaMemcpyDeviceToDevice, e.stream);
  *e.ctl_host = saved;
  ctl_push(e);
  const cudaError_t se = cudaStreamSynchronize(e.stream);
  cudaFree(backup);
  if (!rc) rc = cuda_check(e, se, "autotune restore");
  return rc;
}

int idfx_gpu_set_segments(idfx_gpu* h, const int* seg) {
  if (!h || !seg) return IDFX_ERR_STATE;
  for (int d = 0; d < h->e.g.D; d++)
    if (seg[d] < 1 || seg[d] > 1024) return IDFX_ERR_CONFIG;
  for (int d = 0; d < h->e.g.D; d++) h->e.seg[d] = seg[d];
  return IDFX_OK;
}

int idfx_gpu_get_segments(const idfx_gpu* h, int* seg) {
  if (!h || !seg) return IDFX_ERR_STATE;
  for (int d = 0; d < 3; d++) seg[d] = h->e.seg[d];
  return IDFX_OK;
}

int idfx_gpu_get_sweep_kernels(const idfx_gpu* h, int* kind) {
  if (!h || !kind) return IDFX_ERR_STATE;
  for (int d = 0; d < 3; d++) kind[d] = h->e.tile[d] ? IDFX_SWEEP_TILE : IDFX_SWEEP_MARCH;
  return IDFX_OK;
}

int idfx_gpu_set_sweep_kernels(idfx_gpu* h, const int* kind) {
  if (!h || !kind) return IDFX_ERR_STATE;
  Engine& e = h->e;
  for (int d = 0; d < e.g.D; d++) {
    if (kind[d] != IDFX_SWEEP_MARCH && kind[d] != IDFX_SWEEP_TILE) return IDFX_ERR_CONFIG;
    if (kind[d] == IDFX_SWEEP_TILE && !tile_sweep_eligible(e, d))
      return fail(e, IDFX_ERR_CONFIG, "the tile sweep serves the y and z sweeps of 3-D mixed-precision blocks "
                                      "with PLM, LimO3 or PPM and nt0 a multiple of 4");
  }
  for (int d = 0; d < e.g.D; d++) e.tile[d] = kind[d] == IDFX_SWEEP_TILE ? 1 : 0;
  return IDFX_OK;
}

int idfx_gpu_profile(idfx_gpu* h, int enable) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  IDFX_CK(cudaStreamSynchronize(e.stream));
  for (auto& m : e.marks) {
    e.free_events.push_back(m.a);
    e.free_events.push_back(m.b);
  }
  e.marks.clear();
  e.profile = enable != 0;
  return IDFX_OK;
}

int idfx_gpu_profile_read(idfx_gpu* h, double* ms, long long* launches, int nclasses) {
  if (!h || !ms || !launches) return IDFX_ERR_STATE;
  Engine& e = h->e;
  IDFX_CK(cudaStreamSynchronize(e.stream));
  for (int c = 0; c < nclasses; c++) {
    ms[c] = 0.0;
    launches[c] = 0;
  }
  for (auto& m : e.marks) {
    float t = 0.f;
    IDFX_CK(cudaEventElapsedTime(&t, m.a, m.b));
    if (m.cls < nclasses) {
      ms[m.cls] += t;
      launches[m.cls] += 1;
    }
  }
  return IDFX_OK;
}

int idfx_gpu_destroy(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  if (e.stream) cudaStreamSynchronize(e.stream);
  for (auto& m : e.marks) {
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  for (auto ev : e.free_events) cudaEventDestroy(ev);
  free_learned(e);
  delete e.tile_maps;
  delete e.ct_map;
  if (e.pool) cudaFree(e.pool);
  if (e.ctl) cudaFree(e.ctl);
  if (e.ctl_host) cudaFreeHost(e.ctl_host);
  if (e.own_stream && e.stream) cudaStreamDestroy(e.stream);
  delete h;
  return IDFX_OK;
}

int idfx_gpu_last_error(const idfx_gpu* h, char* buf, size_t len) {
  if (!h || !buf || len == 0) return IDFX_ERR_STATE;
  std::snprintf(buf, len, "%s", h->e.err.c_str());
  return IDFX_OK;
}

int idfx_gpu_sizes(const idfx_gpu* h, int* nvar, int* nghost, long long* vc_len, long long* vs_len) {
  if (!h) return IDFX_ERR_STATE;
  const Geo& g = h->e.g;
  if (nvar) *nvar = 2 * g.D + 2;
  if (nghost) *nghost = g.ng;
  if (vc_len) *vc_len = (2 * g.D + 2) * g.ncell;
  if (vs_len) *vs_len = g.D * g.nface;
  return IDFX_OK;
}

static int copy_state(idfx_gpu* h, const double* Vc, const double* Vs, cudaMemcpyKind kind, bool up) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  const size_t bc = sizeof(double) * (2 * e.g.D + 2) * e.g.ncell;
  const size_t bs = sizeof(double) * e.g.D * e.g.nface;
  const bool d2d = (kind == cudaMemcpyDeviceToDevice);  // by a kernel (see k_copy_f64)
  if (up) {
    ctl_clear(e, kClrUcFresh);  // Uc no longer Vc's
    if (d2d) {
      if (Vc) copy_f64(e, e.f.Vc, Vc, (long long)(bc / sizeof(double)));
      if (Vs) copy_f64(e, e.f.Vs, Vs, (long long)(bs / sizeof(double)));
    } else {
      if (Vc) IDFX_CK(cudaMemcpyAsync(e.f.Vc, Vc, bc, kind, e.stream));
      if (Vs) IDFX_CK(cudaMemcpyAsync(e.f.Vs, Vs, bs, kind, e.stream));
    }
  } else if (d2d) {
    if (Vc) copy_f64(e, (double*)Vc, e.f.Vc, (long long)(bc / sizeof(double)));
    if (Vs) copy_f64(e, (double*)Vs, e.f.Vs, (long long)(bs / sizeof(double)));
  } else {
    if (Vc) IDFX_CK(cudaMemcpyAsync((void*)Vc, e.f.Vc, bc, kind, e.stream));
    if (Vs) IDFX_CK(cudaMemcpyAsync((void*)Vs, e.f.Vs, bs, kind, e.stream));
  }
  IDFX_CK(cudaGetLastError());
  IDFX_CK(cudaStreamSynchronize(e.stream));
  return IDFX_OK;
}

int idfx_gpu_upload_prim(idfx_gpu* h, const double* Vc, const double* Vs) {
  return copy_state(h, Vc, Vs, cudaMemcpyHostToDevice, true);
}
int idfx_gpu_download_prim(idfx_gpu* h, double* Vc, double* Vs) {
  return copy_state(h, Vc, Vs, cudaMemcpyDeviceToHost, false);
}
int idfx_gpu_upload_prim_device(idfx_gpu* h, const double* Vc, const double* Vs) {
  return copy_state(h, Vc, Vs, cudaMemcpyDeviceToDevice, true);
}
int idfx_gpu_download_prim_device(idfx_gpu* h, double* Vc, double* Vs) {
  return copy_state(h, Vc, Vs, cudaMemcpyDeviceToDevice, false);
}
int idfx_gpu_download_cons(idfx_gpu* h, double* Uc) {
  if (!h || !Uc) return IDFX_ERR_STATE;
  Engine& e = h->e;
  if (e.uc_field_stale) {  // mixed path: the field part of Uc from the faces
    IDFX_DISPATCH_D(k_uc_field_active, nblocks(n_active(e.g)), kThreads, e.g, e.f);
    e.uc_field_stale = false;
  }
  IDFX_CK(cudaMemcpyAsync(Uc, e.f.Uc, sizeof(double) * (2 * e.g.D + 2) * e.g.ncell, cudaMemcpyDeviceToHost,
                          e.stream));
  IDFX_CK(cudaStreamSynchronize(e.stream));
  return IDFX_OK;
}

int idfx_gpu_set_time(idfx_gpu* h, double t, double dt, long long ncycles) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  int rc = read_ctl(e);
  if (rc) return rc;
  e.ctl_host->t = t;
  e.ctl_host->dt = dt;
  e.ctl_host->ncycles = ncycles;
  e.ctl_host->done = 0;
  e.ctl_host->status = 0;
  e.ncycles = ncycles;
  ctl_push(e);
  IDFX_CK(cudaGetLastError());
  IDFX_CK(cudaStreamSynchronize(e.stream));
  return IDFX_OK;
}

int idfx_gpu_get_time(idfx_gpu* h, double* t, double* dt, long long* ncycles) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  int rc = read_ctl(e);
  if (rc) return rc;
  if (t) *t = e.ctl_host->t;
  if (dt) *dt = e.ctl_host->dt;
  if (ncycles) *ncycles = e.ctl_host->ncycles;
  return IDFX_OK;
}

// run cycles; the device flags `done` when t reaches tstop or on error
static int run_cycles(idfx_gpu* h, double tstop, long long max_cycles) {
  Engine& e = h->e;
  if (e.g.order == IDFX_LEARNED && !e.learned)
    return fail(e, IDFX_ERR_STATE, "the learned reconstruction needs idfx_gpu_set_learned first");
  int rc = read_ctl(e);
  if (rc) return rc;
  e.ctl_host->tstop = tstop;
  e.ctl_host->done = 0;
  e.ctl_host->status = 0;
  e.ncycles = e.ctl_host->ncycles;
  ctl_push(e);
  e.stage_outputs = false;  // the run's first stage begin rebuilds from the stored state
  e.faces_saved = false;    // and its first face fill takes the Runge-Kutta begin copy
  const int use_tstop = tstop >= 0.0;
  long long done = 0;
  const long long chunk = 64;  // host polls t / status every chunk of queued cycles
  while (max_cycles < 0 || done < max_cycles) {
    long long n = chunk;
    if (max_cycles >= 0 && max_cycles - done < n) n = max_cycles - done;
    for (long long q = 0; q < n; q++) queue_cycle(e, use_tstop);
    done += n;
    IDFX_CK(cudaGetLastError());
    rc = read_ctl(e);
    if (rc) return rc;
    e.ncycles = e.ctl_host->ncycles;
    if (e.ctl_host->status) return fail(e, e.ctl_host->status, status_text(e.ctl_host->status));
    if (e.ctl_host->done) break;
    if (!use_tstop && max_cycles < 0) break;
  }
  return IDFX_OK;
}

int idfx_gpu_cycle(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  return run_cycles(h, -1.0, 1);
}

int idfx_gpu_run(idfx_gpu* h, double tstop, long long max_cycles) {
  if (!h) return IDFX_ERR_STATE;
  if (tstop < 0.0 && max_cycles < 0) return fail(h->e, IDFX_ERR_CONFIG, "run needs tstop or max_cycles");
  return run_cycles(h, tstop, max_cycles);
}

// ---------------------------------------------------------------------------
// building blocks
// ---------------------------------------------------------------------------
// the building blocks run whatever the time-integrator control says; after
// any of them the next cycle rebuilds the conserved state from Vc
static void clear_done(Engine& e) { ctl_clear(e, kClrUcFresh | kClrDone); }

static int sync_status(Engine& e) {
  IDFX_CK(cudaGetLastError());
  IDFX_CK(cudaStreamSynchronize(e.stream));
  return IDFX_OK;
}

int idfx_gpu_set_boundaries(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  clear_done(e);
  launch_boundaries(e);
  launch_fill_faces(e, 0);
  launch_stage_begin(e, 0);
  return sync_status(e);
}

int idfx_gpu_prim_to_cons(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  clear_done(e);
  IDFX_DISPATCH_D(k_prim_to_cons_all, nblocks(e.g.ncell), kThreads, e.g, e.f);
  return sync_status(e);
}

int idfx_gpu_cons_to_prim(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  clear_done(e);
  IDFX_DISPATCH_D(k_uc_field_all, nblocks(e.g.ncell), kThreads, e.g, e.f, 1);
  return sync_status(e);
}

int idfx_gpu_reset_stage(idfx_gpu* h) {
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  IDFX_CK(cudaMemsetAsync(e.f.InvDt, 0, sizeof(double) * e.g.ncell, e.stream));
  return sync_status(e);
}

int idfx_gpu_evolve_stage(idfx_gpu* h, double t, double dt) {
  (void)t;
  if (!h) return IDFX_ERR_STATE;
  Engine& e = h->e;
  clear_done(e);
  if (e.g.order == IDFX_LEARNED && !e.learned)
    return fail(e, IDFX_ERR_STATE, "the learned reconstruction needs idfx_gpu_set_learned first");
  k_set_stage_dt<<<1, 1, 0, e.stream>>>(e.g, e.ctl, dt);
  if (e.f.Vc32) k_vc32<<<nblocks(e.g.ncell), kThreads, 0, e.stream>>>(e.g, e.f, 2 * e.g.D + 2);
  if (e.f.shock) launch_find_shock(e);
  if (e.g.emf == kEmfContact || e.g.emf == kEmfUct0)
    IDFX_DISPATCH_DE(k_cell_emf_all, nblocks(e.g.ncell), kThreads, e.g, e.f);
  launch_sweeps(e, 2, 0);
  launch_ct(e, 0, 1.0, 0.0);
  IDFX_DISPATCH_D(k_uc_field_all, nblocks(e.g.ncell), kThreads, e.g, e.f, 0);
  return sync_status(e);
}

int idfx_gpu_compute_timestep(idfx_gpu* h, double* dt) {
  if (!h || !dt) return IDFX_ERR_STATE;
  Engine& e = h->e;
  ctl_clear(e, kClrInvDt);
  IDFX_DISPATCH_D(k_invdt_max, nblocks(n_active(e.g)), kThreads, e.g, e.f, e.ctl);
  int rc = sync_status(e);
  if (rc) return rc;
  rc = read_ctl(e);
  if (rc) return rc;
  unsigned long long b = e.ctl_host->invdt_max_bits;
  double m;
  std::memcpy(&m, &b, sizeof(m));
  *dt = 1.0 / m;
  return IDFX_OK;
}

int idfx_gpu_check_divb(idfx_gpu* h, double* divb) {
  if (!h || !divb) return IDFX_ERR_STATE;
  Engine& e = h->e;
  ctl_clear(e, kClrDivB);
  IDFX_DISPATCH_D(k_divb, nblocks(n_active(e.g)), kThreads, e.g, e.f, e.ctl);
  int rc = read_ctl(e);
  if (rc) return rc;
  unsigned long long b = e.ctl_host->divb_bits;
  std::memcpy(divb, &b, sizeof(double));
  return IDFX_OK;
}

int idfx_check_wait_timeout(int mode, long long limit, int* gave_up, int* status, int* done) {
  if ((mode != 0 && mode != 1) || limit < 1 || !gave_up || !status || !done) return IDFX_ERR_STATE;
  Ctl* ctl = nullptr;
  int* flag = nullptr;
  if (cudaMalloc(&ctl, sizeof(Ctl)) != cudaSuccess) return IDFX_ERR_CUDA;
  if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) {
    cudaFree(ctl);
    return IDFX_ERR_CUDA;
  }
  Ctl c{};
  c.status = kOk;
  c.done = 0;
  Ctl back{};
  int gu = -1;
  bool ok = cudaMemcpy(ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    k_wait_probe<<<1, 32>>>(ctl, mode, limit, flag);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  }
  ok = ok && cudaMemcpy(&back, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost) == cudaSuccess;
  ok = ok && cudaMemcpy(&gu, flag, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(ctl);
  cudaFree(flag);
  if (!ok) return IDFX_ERR_CUDA;
  *gave_up = gu;
  *status = back.status;
  *done = back.done;
  return IDFX_OK;
}

int idfx_gpu_check_nan(idfx_gpu* h, long long* count) {
  if (!h || !count) return IDFX_ERR_STATE;
  Engine& e = h->e;
  ctl_clear(e, kClrNan);
  IDFX_DISPATCH_D(k_nan_count, nblocks(n_edges(e.g)), kThreads, e.g, e.f, e.ctl);
  int rc = read_ctl(e);
  if (rc) return rc;
  *count = (long long)e.ctl_host->nan_count;
  return IDFX_OK;
}

}  // extern "C"
