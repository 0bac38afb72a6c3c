// Allocation-free variant of Fluid::EvolveStage (idfx_evolve_stage_noalloc).
//
// Who needs it: callers that must not allocate GPU memory while they step —
// for example a host code that owns every device buffer through its own
// memory pool or arena (Kokkos views, a framework allocator), or one that
// runs inside a region where cudaMalloc is forbidden or would synchronise the
// device.  They pass their own device arrays for the state; everything the
// stage needs besides that (face and corner EMFs, upwind flags, cell EMFs,
// InvDt, the small control block) lives in one file-scope static device array
// of fixed size, so this entry point calls no cudaMalloc, cudaFree or any
// other allocating routine.
//
// Limits and sharing:
//  * the scratch array holds IDFX_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB) on
//    every GPU that loads the library, until the process exits; a block whose
//    work arrays do not fit is rejected with IDFX_ERR_CONFIG and a message;
//  * every call on a device uses the same scratch and leaves its contents
//    behind; the parts that must start at zero are cleared by each call;
//  * calls whose GPU work overlaps (e.g. on two streams at once) race on the
//    scratch: serialise them;
//  * each call looks up the scratch address of the current device
//    (cudaGetSymbolAddress, which allocates nothing), so a device reset or a
//    new primary context between calls leaves no stale address behind; the
//    first call on a device may load the library's device code there - make
//    that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/idefix_gb300.h"
#include "engine.hpp"

using namespace idfx;

static __device__ __align__(256) double g_noalloc_scratch[IDFX_NOALLOC_SCRATCH_DOUBLES];

namespace {

// the scratch array as the current device addresses it: in host code the
// symbol g_noalloc_scratch is a host-side stand-in, never a device address
int scratch_for_current_device(double** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return IDFX_ERR_CUDA;
  *out = static_cast<double*>(p);
  return IDFX_OK;
}

void report(char* err, size_t errlen, const char* msg) {
  if (err && errlen) std::snprintf(err, errlen, "%s", msg);
}

// cell-centred EMF from the primitive state (calcCornerEmf.hpp:84-126)
template <int D>
__global__ void k_na_cell_emf(Geo g, Fields f) {
  using v = Var<D>;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const double vx1 = f.Vc[v::MX1 * g.ncell + c], vx2 = f.Vc[v::MX2 * g.ncell + c];
  const double Bx1 = f.Vc[v::BX1 * g.ncell + c], Bx2 = f.Vc[v::BX2 * g.ncell + c];
  if constexpr (D == 3) {
    const double vx3 = f.Vc[v::MX3 * g.ncell + c], Bx3 = f.Vc[v::BX3 * g.ncell + c];
    f.Ex1[c] = (vx3 * Bx2 - vx2 * Bx3);
    f.Ex2[c] = (vx1 * Bx3 - vx3 * Bx1);
  }
  f.Ex3[c] = (vx2 * Bx1 - vx1 * Bx2);
}

// Uc(BX) from the faces over the whole block (boundary.hpp:388-404)
template <int D>
__global__ void k_na_uc_field(Geo g, Fields f) {
  using v = Var<D>;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const int i = (int)(c % g.nt[0]);
  const long long r = c / g.nt[0];
  const int j = (int)(r % g.nt[1]);
  const int k = (int)(r / g.nt[1]);
  const long long fc = fidx(g, k, j, i);
  for (int d = 0; d < D; d++) {
    const double* vs = f.Vs + d * g.nface;
    f.Uc[(v::BX1 + d) * g.ncell + c] = 0.5 * (vs[fc] + vs[fc + g.fs[d]]);
  }
}

__global__ void k_na_set_dt(Geo g, Ctl* ctl, double dt) {
  double dV = g.dx[0] * g.dx[1];
  if (g.D == 3) dV = dV * g.dx[2];
  ctl->dtdV = dt / dV;
  for (int d = 0; d < 3; d++) ctl->dtdx[d] = dt / g.dx[d];
}

// geometry of the block, set up exactly as idfx_gpu_create sets it up
// (block_geometry), for the configurations this entry point supports:
// periodic FP64 blocks of the plain reconstructions, no shock flattening
int na_geometry(const idfx_gpu_config* cfg, Geo& g) {
  if (!cfg) return IDFX_ERR_STATE;
  if (cfg->order > 4 || cfg->shock_flattening || cfg->precision != IDFX_FP64) return IDFX_ERR_CONFIG;
  for (int d = 0; d < 3; d++)  // periodic blocks only
    if (cfg->lbound[d] || cfg->rbound[d]) return IDFX_ERR_CONFIG;
  return block_geometry(cfg, g);
}

}  // namespace

extern "C" int idfx_evolve_stage_noalloc(const idfx_gpu_config* cfg, const double* Vc, double* Uc,
                                         double* Vs, double t, double dt, void* stream, char* err,
                                         size_t errlen) {
  (void)t;
  Engine e;  // launch context only: every buffer below is the caller's or the static scratch
  int rc = na_geometry(cfg, e.g);
  if (rc != IDFX_OK) {
    report(err, errlen, "idfx_evolve_stage_noalloc: invalid configuration");
    return rc;
  }
  if (!Vc || !Uc || !Vs) {
    report(err, errlen, "idfx_evolve_stage_noalloc: null state pointer");
    return IDFX_ERR_STATE;
  }
  const Geo& g = e.g;
  const bool hll_emf = (g.emf == kEmfUctHll || g.emf == kEmfUctHlld);
  const long long nc = g.ncell;
  const long long ctl_doubles = (long long)((sizeof(Ctl) + sizeof(double) - 1) / sizeof(double));
  // InvDt, 6 face EMFs, 3 flags, 3 cell EMFs, 3 corner EMFs (+12 weights)
  const long long need = (16 + (hll_emf ? 12 : 0)) * nc + ctl_doubles;
  if (need > (long long)IDFX_NOALLOC_SCRATCH_DOUBLES) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "idfx_evolve_stage_noalloc: block needs %lld scratch doubles, the static scratch "
                  "holds %lld (IDFX_NOALLOC_SCRATCH_DOUBLES); use the handle API for larger blocks",
                  need, (long long)IDFX_NOALLOC_SCRATCH_DOUBLES);
    report(err, errlen, msg);
    return IDFX_ERR_CONFIG;
  }
  double* scratch = nullptr;
  rc = scratch_for_current_device(&scratch);
  if (rc != IDFX_OK) {
    report(err, errlen, "idfx_evolve_stage_noalloc: cudaGetSymbolAddress of the scratch failed");
    return rc;
  }
  e.stream = (cudaStream_t)stream;
  // work arrays and control block inside the scratch
  double* p = scratch;
  auto take = [&](long long n) { double* q = p; p += n; return q; };
  Fields& f = e.f;
  f.Vc = const_cast<double*>(Vc);  // read only in this stage
  f.Uc = Uc;
  f.Vs = Vs;
  f.Uc0 = nullptr;
  f.Vs0 = nullptr;
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
  e.ctl = reinterpret_cast<Ctl*>(p);
  // everything the stage reads before writing starts at zero: InvDt, the
  // EMF arrays (never-written positions read as zero, as in the handle
  // path), and the control block (done = 0)
  if (cudaMemsetAsync(scratch, 0, (size_t)need * sizeof(double), e.stream) != cudaSuccess) {
    report(err, errlen, "idfx_evolve_stage_noalloc: cudaMemsetAsync failed");
    return IDFX_ERR_CUDA;
  }
  // segment length of the marching sweeps, as the handle path chooses it
  choose_segments(e);
  const int threads = 256;
  const unsigned cell_blocks = (unsigned)((nc + threads - 1) / threads);
  const long long edges = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.D == 3 ? g.n[2] + 1 : 1);
  const unsigned edge_blocks = (unsigned)((edges + threads - 1) / threads);
  k_na_set_dt<<<1, 1, 0, e.stream>>>(g, e.ctl, dt);
  if (g.emf == kEmfContact || g.emf == kEmfUct0) {
    if (g.D == 2) k_na_cell_emf<2><<<cell_blocks, threads, 0, e.stream>>>(g, f);
    else k_na_cell_emf<3><<<cell_blocks, threads, 0, e.stream>>>(g, f);
  }
  switch (g.solver) {
    case kHLLD: launch_sweeps_hlld(e, 2, 0); break;
    case kHLL: launch_sweeps_hll(e, 2, 0); break;
    case kROE: launch_sweeps_roe(e, 2, 0); break;
    default: launch_sweeps_tvdlf(e, 2, 0); break;
  }
  if (g.D == 2) {
    k_ct_corner<2><<<edge_blocks, threads, 0, e.stream>>>(g, f, e.ctl);
    k_ct_faces<2><<<edge_blocks, threads, 0, e.stream>>>(g, f, e.ctl, 0, 1.0, 0.0);
    k_na_uc_field<2><<<cell_blocks, threads, 0, e.stream>>>(g, f);
  } else {
    k_ct_corner<3><<<edge_blocks, threads, 0, e.stream>>>(g, f, e.ctl);
    k_ct_faces<3><<<edge_blocks, threads, 0, e.stream>>>(g, f, e.ctl, 0, 1.0, 0.0);
    k_na_uc_field<3><<<cell_blocks, threads, 0, e.stream>>>(g, f);
  }
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) {
    report(err, errlen, cudaGetErrorString(le));
    return IDFX_ERR_CUDA;
  }
  report(err, errlen, "");
  return IDFX_OK;
}
