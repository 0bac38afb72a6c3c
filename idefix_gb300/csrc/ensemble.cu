// Ensemble of independent periodic boxes (see ensemble.hpp) and its C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <numeric>

#include "../../include/idefix_gb300.h"
#include "ensemble.hpp"

using namespace idfx;

struct idfx_ens {
  EnsEngine e;
};

namespace {

constexpr int kT = 256;

// ---------------------------------------------------------------------------
// batched phase kernels: block -> (box, block index) from the work list
// ---------------------------------------------------------------------------
template <int D>
__global__ void ke_fill_faces(const EnsBox* boxes, const int4* items, int save) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_fill_faces<D>(B.g, B.f, B.ctl, save, dim3(it.y, it.z, it.w));
}
// E: type of the EMF buffers (FP32 on the mixed path)
template <int D, typename E>
__global__ void ke_stage_begin(const EnsBox* boxes, const int4* items, int flags) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_stage_begin<D, E>(B.g, B.f, B.ctl, flags, dim3(it.y, it.z, it.w));
}
template <int D>
__global__ void ke_find_shock(const EnsBox* boxes, const int4* items) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_find_shock<D>(B.g, B.f, B.ctl, dim3(it.y, it.z, it.w));
}
template <int D, typename E>
__global__ void ke_ct_corner(const EnsBox* boxes, const int4* items) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_ct_corner<D, E>(B.g, B.f, B.ctl, dim3(it.y, it.z, it.w));
}
// diagnostics are due for a box when its own cycle count is a multiple of
// the period (timeIntegrator.cpp:268-279 and 393-399 on the host mirror)
__device__ __forceinline__ bool due(const Ctl* c, int period) { return period > 0 && c->ncycles % period == 0; }

template <int D, typename E>
__global__ void ke_ct_faces(const EnsBox* boxes, const int4* items, int combine, double wc, double w0,
                            int nan_period) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  // a box with a NaN check this cycle combines its faces after the count
  const int cmb = combine && !due(B.ctl, nan_period);
  d_ct_faces<D, E>(B.g, B.f, B.ctl, cmb, cmb ? wc : 1.0, cmb ? w0 : 0.0, dim3(it.y, it.z, it.w));
}
template <int D, typename E>
__global__ void ke_stage_end(const EnsBox* boxes, const int4* items, int combine, double wc, double w0) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  d_stage_end<D, E>(B.g, B.f, B.ctl, combine, wc, w0, dim3(it.y, it.z, it.w));
}
template <int D>
__global__ void ke_divb(const EnsBox* boxes, const int4* items, int period) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  if (!due(B.ctl, period)) return;
  d_divb<D>(B.g, B.f, B.ctl, dim3(it.y, it.z, it.w));
}
template <int D>
__global__ void ke_nan_count(const EnsBox* boxes, const int4* items, int period) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  if (!due(B.ctl, period)) return;
  d_nan_count<D>(B.g, B.f, B.ctl, dim3(it.y, it.z, it.w));
}
// RK combination of the faces of the boxes that ran a NaN check this stage
template <typename E>
__global__ void ke_faces_combine(const EnsBox* boxes, const int4* items, double wc, double w0, int period) {
  const int4 it = items[blockIdx.x];
  const EnsBox& B = boxes[it.x];
  if (B.ctl->done || !due(B.ctl, period)) return;
  const long long tid = (long long)it.y * blockDim.x + threadIdx.x;  // fill-table layout
  if (tid >= B.g.nface) return;
  const long long q = (long long)it.z * B.g.nface + tid;
  B.f.Vs[q] = rk_combine<E>(B.f.Vs[q], B.f.Vs0[q], wc, w0);  // as d_ct_faces combines
}
// per-box control: one thread per box
__global__ void ke_cycle_begin(const EnsBox* boxes, int nbox) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox) d_cycle_begin(boxes[b].g, boxes[b].ctl, 1);
}
__global__ void ke_cycle_end(const EnsBox* boxes, int nbox) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox) d_cycle_end(boxes[b].ctl);
}
__global__ void ke_reset_nan(const EnsBox* boxes, int nbox, int period) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox && due(boxes[b].ctl, period)) boxes[b].ctl->nan_count = 0ull;
}
__global__ void ke_reset_divb(const EnsBox* boxes, int nbox, int period) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox && due(boxes[b].ctl, period)) boxes[b].ctl->divb_bits = 0ull;
}
__global__ void ke_check_divb(const EnsBox* boxes, int nbox, int period) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox && due(boxes[b].ctl, period)) d_check_divb(boxes[b].ctl);
}
__global__ void ke_check_nan(const EnsBox* boxes, int nbox, int period) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbox && due(boxes[b].ctl, period)) d_check_nan(boxes[b].ctl);
}

#define IDFX_ENS_D(K, N, ...)                                                   \
  do {                                                                          \
    if ((N) > 0) {                                                              \
      if (e.D == 2) K<2><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                \
      else K<3><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                         \
    }                                                                           \
  } while (0)

// dimension and EMF type (FP32 EMF buffers on the mixed path)
#define IDFX_ENS_DE(K, N, ...)                                                       \
  do {                                                                               \
    if ((N) > 0) {                                                                   \
      const bool f32 = (e.precision == IDFX_MIXED);                                  \
      if (e.D == 2) {                                                                \
        if (f32) K<2, float><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                 \
        else K<2, double><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                    \
      } else {                                                                       \
        if (f32) K<3, float><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                 \
        else K<3, double><<<(N), kT, 0, e.stream>>>(__VA_ARGS__);                    \
      }                                                                              \
    }                                                                                \
  } while (0)

inline unsigned per_box_blocks(const EnsEngine& e) { return (unsigned)((e.nbox + kT - 1) / kT); }

long long active_cells(const Geo& g) { return (long long)g.n[0] * g.n[1] * g.n[2]; }
long long edge_count(const Geo& g) { return (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.D == 3 ? g.n[2] + 1 : 1); }
long long sweep_cols(const Geo& g, int dir) {
  const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;
  return (long long)(g.n[a] + 2 * g.ext) * (g.D == 3 ? g.n[b] + 2 * g.ext : 1);
}

// boxes in decreasing work order: the largest boxes' blocks are issued first
std::vector<int> schedule(const EnsEngine& e) {
  std::vector<int> order(e.nbox);
  std::iota(order.begin(), order.end(), 0);
  if (e.schedule == 1) return order;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return active_cells(e.boxes[a].g) > active_cells(e.boxes[b].g);
  });
  return order;
}

int upload_table(EnsEngine& e, EnsTable& t, const std::vector<int4>& items) {
  if (t.items) cudaFree(t.items);
  t.items = nullptr;
  t.n = (int)items.size();
  if (t.n == 0) return IDFX_OK;
  if (cudaMalloc(&t.items, items.size() * sizeof(int4)) != cudaSuccess) return IDFX_ERR_CUDA;
  if (cudaMemcpy(t.items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
    return IDFX_ERR_CUDA;
  return IDFX_OK;
}

std::vector<int4> sweep_items(const EnsEngine& e, int dir, const std::vector<int>& boxes) {
  std::vector<int4> v;
  for (int b : boxes) {
    const Geo& g = e.boxes[b].g;
    const long long nx = (sweep_cols(g, dir) + kTM - 1) / kTM;
    const int seg = e.boxes[b].seg[dir];
    const int nseg = (g.n[dir] + seg - 1) / seg;
    for (int y = 0; y < nseg; y++)
      for (long long x = 0; x < nx; x++) v.push_back(make_int4(b, (int)x, y, 0));
  }
  return v;
}

// the per-box phases' work lists for blocks of bt threads
void phase_items(const EnsEngine& e, const std::vector<int>& order, int bt, std::vector<int4>& fill,
                 std::vector<int4>& begin, std::vector<int4>& edges, std::vector<int4>& active) {
  for (int b : order) {
    const Geo& g = e.boxes[b].g;
    const long long nf = (g.nface + bt - 1) / bt;
    for (int comp = 0; comp < g.D; comp++)
      for (long long x = 0; x < nf; x++) fill.push_back(make_int4(b, (int)x, comp, 0));
    for (long long x = 0; x < (g.ncell + bt - 1) / bt; x++) begin.push_back(make_int4(b, (int)x, 0, 0));
    for (long long x = 0; x < (edge_count(g) + bt - 1) / bt; x++) edges.push_back(make_int4(b, (int)x, 0, 0));
    for (long long x = 0; x < (active_cells(g) + bt - 1) / bt; x++) active.push_back(make_int4(b, (int)x, 0, 0));
  }
}

int build_tables(EnsEngine& e) {
  const std::vector<int> order = schedule(e);
  std::vector<int4> fill, begin, edges, active, fill64, begin64, edges64, active64;
  phase_items(e, order, kT, fill, begin, edges, active);
  phase_items(e, order, kTM, fill64, begin64, edges64, active64);
  int rc = upload_table(e, e.fill, fill);
  if (!rc) rc = upload_table(e, e.begin, begin);
  if (!rc) rc = upload_table(e, e.edges, edges);
  if (!rc) rc = upload_table(e, e.active, active);
  if (!rc) rc = upload_table(e, e.fill64, fill64);
  if (!rc) rc = upload_table(e, e.begin64, begin64);
  if (!rc) rc = upload_table(e, e.edges64, edges64);
  if (!rc) rc = upload_table(e, e.active64, active64);
  for (int d = 0; d < e.D && !rc; d++) rc = upload_table(e, e.sweep[d], sweep_items(e, d, order));
  return rc;
}

void launch_sweep(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last) {
  switch (e.solver) {
    case kHLLD: launch_ens_sweep_hlld(e, dir, t, invdt, last); break;
    case kHLL: launch_ens_sweep_hll(e, dir, t, invdt, last); break;
    case kROE: launch_ens_sweep_roe(e, dir, t, invdt, last); break;
    default: launch_ens_sweep_tvdlf(e, dir, t, invdt, last); break;
  }
}

// one TimeIntegrator::Cycle of every box (timeIntegrator.cpp:246-414).
// checks: also queue the divB / NaN diagnostics, which every box runs only
// in the cycles its own counter makes due.
void queue_cycle(EnsEngine& e, bool checks) {
  const bool cell_emf = (e.emf == kEmfContact || e.emf == kEmfUct0);
  const int lp = checks ? e.log_period : 0, np = checks ? e.check_nan_period : 0;
  ke_cycle_begin<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox);
  if (lp > 0) {
    ke_reset_divb<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox, lp);
    IDFX_ENS_D(ke_divb, e.active.n, e.d_boxes, e.active.items, lp);
    ke_check_divb<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox, lp);
  }
  for (int stage = 0; stage < e.nstages; stage++) {
    const int save = (e.nstages > 1 && stage == 0);
    IDFX_ENS_D(ke_fill_faces, e.fill.n, e.d_boxes, e.fill.items, save);
    IDFX_ENS_DE(ke_stage_begin, e.begin.n, e.d_boxes, e.begin.items,
               kSbCons | (e.precision == IDFX_MIXED ? kSbKeepCons : 0) | (save ? kSbSaveBegin : 0) |
                   (cell_emf ? kSbCellEmf : 0));
    // shock flags: the stage-begin table covers (n + 2)^D cells of every box
    if (e.shock) IDFX_ENS_D(ke_find_shock, e.begin.n, e.d_boxes, e.begin.items);
    for (int d = 0; d < e.D; d++)
      launch_sweep(e, d, e.sweep[d], stage == 0 ? (d == 0 ? 1 : 2) : 0, stage == 0 && d == e.D - 1);
    const int combine = stage > 0;
    const double wc = combine ? e.wc[stage - 1] : 1.0, w0 = combine ? e.w0[stage - 1] : 0.0;
    IDFX_ENS_DE(ke_ct_corner, e.edges.n, e.d_boxes, e.edges.items);
    IDFX_ENS_DE(ke_ct_faces, e.edges.n, e.d_boxes, e.edges.items, combine, wc, w0, np);
    if (np > 0) {
      ke_reset_nan<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox, np);
      IDFX_ENS_D(ke_nan_count, e.edges.n, e.d_boxes, e.edges.items, np);
      ke_check_nan<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox, np);
      if (combine && e.fill.n)
        if (e.precision == IDFX_MIXED)
          ke_faces_combine<float><<<e.fill.n, kT, 0, e.stream>>>(e.d_boxes, e.fill.items, wc, w0, np);
        else
          ke_faces_combine<double><<<e.fill.n, kT, 0, e.stream>>>(e.d_boxes, e.fill.items, wc, w0, np);
    }
    IDFX_ENS_DE(ke_stage_end, e.active.n, e.d_boxes, e.active.items, combine, wc, w0);
  }
  ke_cycle_end<<<per_box_blocks(e), kT, 0, e.stream>>>(e.d_boxes, e.nbox);
}

int capture_one(EnsEngine& e, bool checks, cudaGraphExec_t* exec) {
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return IDFX_ERR_CUDA;
  queue_cycle(e, checks);
  if (cudaStreamEndCapture(e.stream, &graph) != cudaSuccess) return IDFX_ERR_CUDA;
  const cudaError_t rc = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  return rc == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
}

int capture_graph(EnsEngine& e) {
  int rc = capture_one(e, false, &e.exec);
  if (!rc && (e.log_period > 0 || e.check_nan_period > 0)) rc = capture_one(e, true, &e.exec_checks);
  if (e.exec_persist) {  // the persistent graph is captured again on its next use
    cudaGraphExecDestroy(e.exec_persist);
    e.exec_persist = nullptr;
    e.persist_chunk = 0;
  }
  return rc;
}

int persist_blocks(const EnsEngine& e) {
  switch (e.solver) {
    case kHLLD: return ens_persist_blocks_hlld(e);
    case kHLL: return ens_persist_blocks_hll(e);
    case kROE: return ens_persist_blocks_roe(e);
    default: return ens_persist_blocks_tvdlf(e);
  }
}

__global__ void ke_bar_reset(GridBar* b) { *b = GridBar{0u, 0u, 0, 0}; }

// ncyc cycles of every box as one persistent launch (the barrier reset first)
cudaError_t queue_persist(EnsEngine& e, int ncyc) {
  const int grid = persist_blocks(e);
  if (grid < 1) return cudaErrorInvalidConfiguration;
  ke_bar_reset<<<1, 1, 0, e.stream>>>(e.d_bar);
  switch (e.solver) {
    case kHLLD: return launch_ens_persist_hlld(e, ncyc, grid);
    case kHLL: return launch_ens_persist_hll(e, ncyc, grid);
    case kROE: return launch_ens_persist_roe(e, ncyc, grid);
    default: return launch_ens_persist_tvdlf(e, ncyc, grid);
  }
}

// the persistent launch of `ncyc` cycles replayed from a CUDA graph (captured
// once per chunk length); where the capture of a cooperative launch is not
// available, the launch goes to the stream directly
cudaError_t run_persist(EnsEngine& e, int ncyc) {
  if (e.persist_graph && e.exec_persist && e.persist_chunk == ncyc) return cudaGraphLaunch(e.exec_persist, e.stream);
  if (e.exec_persist) {
    cudaGraphExecDestroy(e.exec_persist);
    e.exec_persist = nullptr;
  }
  cudaGraph_t graph = nullptr;
  e.persist_graph = false;
  if (cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const cudaError_t lr = queue_persist(e, ncyc);
    const cudaError_t cr = cudaStreamEndCapture(e.stream, &graph);
    if (lr == cudaSuccess && cr == cudaSuccess && graph &&
        cudaGraphInstantiate(&e.exec_persist, graph, 0) == cudaSuccess) {
      e.persist_graph = true;
      e.persist_chunk = ncyc;
    }
    if (graph) cudaGraphDestroy(graph);
  }
  cudaGetLastError();  // a refused capture leaves no error behind
  if (e.persist_graph) return cudaGraphLaunch(e.exec_persist, e.stream);
  return queue_persist(e, ncyc);
}

int ens_fail(EnsEngine& e, int code, const std::string& msg) {
  e.err = msg;
  return code;
}

int read_ctl(EnsEngine& e) {
  if (cudaMemcpyAsync(e.h_ctl, e.d_ctl, sizeof(Ctl) * e.nbox, cudaMemcpyDeviceToHost, e.stream) != cudaSuccess)
    return IDFX_ERR_CUDA;
  return cudaStreamSynchronize(e.stream) == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
}

// geometry of one box, set up as idfx_gpu_create sets it up (the boxes are
// periodic)
bool box_geometry(const idfx_gpu_config* cfg, Geo& g) {
  for (int d = 0; d < 3; d++)
    if (cfg->lbound[d] || cfg->rbound[d]) return false;
  return block_geometry(cfg, g) == IDFX_OK;
}

// first guess of the march segment (the autotuner refines it)
int default_seg(const Geo& g, int dir, int sms) {
  const long long want = (long long)sms * 128;  // ensemble launches hold many boxes
  int s = 64;
  while (s > 2 && sweep_cols(g, dir) * ((g.n[dir] + s - 1) / s) < want) s /= 2;
  return s;
}

}  // namespace

namespace {

int upload_boxes(EnsEngine& e) {
  if (cudaMemcpyAsync(e.d_boxes, e.boxes.data(), sizeof(EnsBox) * e.nbox, cudaMemcpyHostToDevice, e.stream) !=
      cudaSuccess)
    return IDFX_ERR_CUDA;
  return cudaStreamSynchronize(e.stream) == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
}

// times `reps` launches of one batched sweep (ms, minimum over launches)
float time_sweep(EnsEngine& e, int dir, const EnsTable& t, int reps, cudaEvent_t a, cudaEvent_t b) {
  launch_sweep(e, dir, t, 2, 0);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < reps; r++) {
    cudaEventRecord(a, e.stream);
    launch_sweep(e, dir, t, 2, 0);
    cudaEventRecord(b, e.stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    best = std::min(best, ms);
  }
  return best;
}

// Autotuner: for every box size and sweep direction, the march segment
// length with the fastest batched sweep over the boxes of that size.  The
// sweeps accumulate into Uc, InvDt and the EMF arrays, so the whole state is
// saved first and put back afterwards.
int autotune(EnsEngine& e, int reps) {
  double* backup = nullptr;
  if (cudaMalloc(&backup, e.pool_len * sizeof(double)) != cudaSuccess)
    return ens_fail(e, IDFX_ERR_CUDA, "autotune: no room for the state backup");
  std::vector<Ctl> ctl_save(e.nbox);
  int rc = read_ctl(e);
  if (!rc) std::copy(e.h_ctl, e.h_ctl + e.nbox, ctl_save.begin());
  if (!rc && cudaMemcpyAsync(backup, e.pool, e.pool_len * sizeof(double), cudaMemcpyDeviceToDevice, e.stream) !=
                 cudaSuccess)
    rc = IDFX_ERR_CUDA;
  if (!rc) {  // every box live for the trial launches
    for (int b = 0; b < e.nbox; b++) e.h_ctl[b].done = 0;
    if (cudaMemcpyAsync(e.d_ctl, e.h_ctl, sizeof(Ctl) * e.nbox, cudaMemcpyHostToDevice, e.stream) != cudaSuccess)
      rc = IDFX_ERR_CUDA;
  }
  std::map<std::vector<int>, std::vector<int>> classes;  // box size -> boxes
  for (int b = 0; b < e.nbox; b++) classes[{e.boxes[b].g.n[0], e.boxes[b].g.n[1], e.boxes[b].g.n[2]}].push_back(b);
  cudaEvent_t ea, eb;
  cudaEventCreate(&ea);
  cudaEventCreate(&eb);
  EnsTable trial;
  for (auto& kv : classes) {
    if (rc) break;
    const std::vector<int>& members = kv.second;
    for (int d = 0; d < e.D && !rc; d++) {
      int best_seg = e.boxes[members[0]].seg[d];
      float best_ms = 1e30f;
      for (int s = 2; s <= 64; s *= 2) {
        if (s > kv.first[d]) break;
        for (int b : members) e.boxes[b].seg[d] = s;
        rc = upload_boxes(e);
        if (!rc) rc = upload_table(e, trial, sweep_items(e, d, members));
        if (rc) break;
        const float ms = time_sweep(e, d, trial, reps, ea, eb);
        if (ms < best_ms) {
          best_ms = ms;
          best_seg = s;
        }
      }
      for (int b : members) e.boxes[b].seg[d] = best_seg;
    }
  }
  if (trial.items) cudaFree(trial.items);
  cudaEventDestroy(ea);
  cudaEventDestroy(eb);
  if (cudaGetLastError() != cudaSuccess && !rc) rc = IDFX_ERR_CUDA;
  // restore the state and the control blocks
  cudaMemcpyAsync(e.pool, backup, e.pool_len * sizeof(double), cudaMemcpyDeviceToDevice, e.stream);
  std::copy(ctl_save.begin(), ctl_save.end(), e.h_ctl);
  cudaMemcpyAsync(e.d_ctl, e.h_ctl, sizeof(Ctl) * e.nbox, cudaMemcpyHostToDevice, e.stream);
  if (cudaStreamSynchronize(e.stream) != cudaSuccess && !rc) rc = IDFX_ERR_CUDA;
  cudaFree(backup);
  if (!rc) rc = upload_boxes(e);
  if (!rc) rc = build_tables(e);
  if (!rc) rc = capture_graph(e);
  if (rc && e.err.empty()) e.err = "autotune: CUDA failure";
  return rc;
}

const char* ens_status_text(int s) {
  switch (s) {
    case kErrNan: return "Nan found after integration cycle";
    case kErrDivB: return "divB too large, check your calculation";
    case kErrDtSmall: return "dt is too small";
    case kErrFirstDt: return "Your guessed first_dt is too large. Try to reduce first_dt.";
    default: return "error";
  }
}

void release(EnsEngine& e) {
  if (e.stream) cudaStreamSynchronize(e.stream);
  if (e.exec) cudaGraphExecDestroy(e.exec);
  if (e.exec_checks) cudaGraphExecDestroy(e.exec_checks);
  if (e.exec_persist) cudaGraphExecDestroy(e.exec_persist);
  if (e.d_bar) cudaFree(e.d_bar);
  for (EnsTable* t : e.tables())
    if (t->items) cudaFree(t->items);
  if (e.d_boxes) cudaFree(e.d_boxes);
  if (e.d_ctl) cudaFree(e.d_ctl);
  if (e.h_ctl) cudaFreeHost(e.h_ctl);
  if (e.pool) cudaFree(e.pool);
  if (e.own_stream && e.stream) cudaStreamDestroy(e.stream);
}

}  // namespace

namespace idfx {

EnsPersist ens_persist_args(const EnsEngine& e) {
  EnsPersist P{};
  P.fill = e.fill64.items;
  P.nfill = e.fill64.n;
  P.begin = e.begin64.items;
  P.nbegin = e.begin64.n;
  P.edges = e.edges64.items;
  P.nedges = e.edges64.n;
  P.active = e.active64.items;
  P.nactive = e.active64.n;
  for (int d = 0; d < 3; d++) {
    P.sweep[d] = e.sweep[d].items;
    P.nsweep[d] = d < e.D ? e.sweep[d].n : 0;
  }
  P.nbox = e.nbox;
  P.nstages = e.nstages;
  P.log_period = e.log_period;
  P.check_nan_period = e.check_nan_period;
  P.shock = e.shock ? 1 : 0;
  P.keep_cons = e.precision == IDFX_MIXED ? 1 : 0;
  P.cell_emf = (e.emf == kEmfContact || e.emf == kEmfUct0) ? 1 : 0;
  for (int k = 0; k < 2; k++) {
    P.wc[k] = e.wc[k];
    P.w0[k] = e.w0[k];
  }
  return P;
}

}  // namespace idfx

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int idfx_ens_create(int nbox, const idfx_gpu_config* cfgs, void* stream, idfx_ens** out) {
  if (!cfgs || !out || nbox < 1) return IDFX_ERR_STATE;
  *out = nullptr;
  const idfx_gpu_config& c0 = cfgs[0];
  for (int b = 0; b < nbox; b++) {
    const idfx_gpu_config& c = cfgs[b];
    // the scheme is shared (one launch per phase); grids, gamma and the
    // time-step parameters are per box
    if (c.dims != c0.dims || c.order != c0.order || c.solver != c0.solver || c.emf != c0.emf ||
        c.nstages != c0.nstages || c.precision != c0.precision || c.log_period != c0.log_period ||
        c.check_nan_period != c0.check_nan_period || (c.shock_flattening != 0) != (c0.shock_flattening != 0))
      return IDFX_ERR_CONFIG;
    if (c.order < 1 || c.order > 4 || c.solver < 0 || c.solver > 3) return IDFX_ERR_CONFIG;
    if (c.emf < 0 || c.emf > 4 || c.nstages < 1 || c.nstages > 3) return IDFX_ERR_CONFIG;
    if (c.precision != IDFX_FP64 && c.precision != IDFX_MIXED) return IDFX_ERR_CONFIG;
    if (c.emf == IDFX_EMF_UCT_HLLD && (c.solver == IDFX_HLL || c.solver == IDFX_TVDLF)) return IDFX_ERR_CONFIG;
    Geo g{};
    if (!box_geometry(&c, g)) return IDFX_ERR_CONFIG;
  }
  idfx_ens* h = new (std::nothrow) idfx_ens();
  if (!h) return IDFX_ERR_STATE;
  EnsEngine& e = h->e;
  e.nbox = nbox;
  e.D = c0.dims;
  e.order = c0.order;
  e.solver = c0.solver;
  e.emf = c0.emf;
  e.nstages = c0.nstages;
  e.precision = c0.precision;
  e.log_period = c0.log_period;
  e.check_nan_period = c0.check_nan_period;
  e.shock = c0.shock_flattening != 0;
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
  e.boxes.resize(nbox);
  const bool hll_emf = (e.emf == kEmfUctHll || e.emf == kEmfUctHlld);
  const int NV = 2 * e.D + 2;
  // every array of every box starts on a 256-byte boundary
  auto up32 = [](size_t n) { return (n + 31) / 32 * 32; };
  std::vector<size_t> box_len(nbox);
  size_t len = 0;
  for (int b = 0; b < nbox; b++) {
    Geo& g = e.boxes[b].g;
    box_geometry(&cfgs[b], g);
    const size_t nc = up32((size_t)g.ncell), nf = up32((size_t)g.nface);
    box_len[b] = 3 * NV * nc + 2 * g.D * nf + nc + 15 * nc + (hll_emf ? 12 * nc : 0) +
                 (e.precision == IDFX_MIXED ? up32((NV * nc + 1) / 2) : 0) +  // FP32 primitives
                 (e.shock ? up32((nc + 7) / 8) : 0);                          // shock flags
    len += box_len[b];
  }
  int rc = IDFX_OK;
  if (stream) {
    e.stream = (cudaStream_t)stream;
  } else {
    rc = cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) == cudaSuccess ? IDFX_OK : IDFX_ERR_CUDA;
    e.own_stream = (rc == IDFX_OK);
  }
  if (!rc && cudaMalloc(&e.pool, len * sizeof(double)) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (!rc && cudaMemsetAsync(e.pool, 0, len * sizeof(double), e.stream) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (!rc && cudaMalloc(&e.d_ctl, sizeof(Ctl) * nbox) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (!rc && cudaMallocHost(&e.h_ctl, sizeof(Ctl) * nbox) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (!rc && cudaMalloc(&e.d_boxes, sizeof(EnsBox) * nbox) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (!rc && cudaMalloc(&e.d_bar, sizeof(GridBar)) != cudaSuccess) rc = IDFX_ERR_CUDA;
  if (rc) {
    std::fprintf(stderr, "idfx_ens_create: CUDA allocation failed (%.3f GB of fields)\n", len * 8.0 / 1e9);
    release(e);
    delete h;
    return rc;
  }
  e.pool_len = len;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* p = e.pool;
  for (int b = 0; b < nbox; b++) {
    EnsBox& B = e.boxes[b];
    const Geo& g = B.g;
    const size_t nc = up32((size_t)g.ncell), nf = up32((size_t)g.nface);
    auto take = [&](size_t n) { double* q = p; p += n; return q; };
    Fields& f = B.f;
    f = Fields{};
    // variables of a field are g.ncell apart (the reference layout); the
    // padding goes after the last one
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
    f.Vc32 = (e.precision == IDFX_MIXED) ? reinterpret_cast<float*>(take(up32((NV * nc + 1) / 2))) : nullptr;
    f.shock = e.shock ? reinterpret_cast<unsigned char*>(take(up32((nc + 7) / 8))) : nullptr;
    B.ctl = e.d_ctl + b;
    for (int d = 0; d < 3; d++) B.seg[d] = d < e.D ? default_seg(g, d, sms) : 1;
    Ctl c{};
    c.dt = cfgs[b].first_dt;
    c.tstop = DBL_MAX;
    c.cfl = cfgs[b].cfl;
    c.cflmax = cfgs[b].cfl_max_var;
    c.maxdivb = cfgs[b].maxdivb;
    e.h_ctl[b] = c;
  }
  if (cudaMemcpyAsync(e.d_ctl, e.h_ctl, sizeof(Ctl) * nbox, cudaMemcpyHostToDevice, e.stream) != cudaSuccess)
    rc = IDFX_ERR_CUDA;
  if (!rc) rc = upload_boxes(e);
  if (!rc) rc = build_tables(e);
  if (!rc) rc = capture_graph(e);
  if (rc) {
    std::fprintf(stderr, "idfx_ens_create: CUDA setup failed\n");
    release(e);
    delete h;
    return rc;
  }
  *out = h;
  return IDFX_OK;
}

int idfx_ens_destroy(idfx_ens* h) {
  if (!h) return IDFX_ERR_STATE;
  release(h->e);
  delete h;
  return IDFX_OK;
}

int idfx_ens_last_error(const idfx_ens* h, char* buf, size_t len) {
  if (!h || !buf || len == 0) return IDFX_ERR_STATE;
  std::snprintf(buf, len, "%s", h->e.err.c_str());
  return IDFX_OK;
}

int idfx_ens_sizes(const idfx_ens* h, int box, int* nvar, int* nghost, long long* vc_len, long long* vs_len) {
  if (!h || box < 0 || box >= h->e.nbox) return IDFX_ERR_STATE;
  const Geo& g = h->e.boxes[box].g;
  if (nvar) *nvar = 2 * g.D + 2;
  if (nghost) *nghost = g.ng;
  if (vc_len) *vc_len = (2 * g.D + 2) * g.ncell;
  if (vs_len) *vs_len = g.D * g.nface;
  return IDFX_OK;
}

static int ens_copy(idfx_ens* h, int box, const double* Vc, const double* Vs, bool up, bool device = false) {
  if (!h || box < 0 || box >= h->e.nbox) return IDFX_ERR_STATE;
  EnsEngine& e = h->e;
  const EnsBox& B = e.boxes[box];
  const size_t bc = sizeof(double) * (2 * B.g.D + 2) * B.g.ncell;
  const size_t bs = sizeof(double) * B.g.D * B.g.nface;
  cudaError_t rc = cudaSuccess;
  if (up) {
    rc = cudaMemsetAsync(&B.ctl->uc_fresh, 0, sizeof(int), e.stream);  // Uc no longer Vc's
    if (Vc && rc == cudaSuccess) rc = cudaMemcpyAsync(B.f.Vc, Vc, bc, cudaMemcpyHostToDevice, e.stream);
    if (Vs && rc == cudaSuccess) rc = cudaMemcpyAsync(B.f.Vs, Vs, bs, cudaMemcpyHostToDevice, e.stream);
  } else {
    const cudaMemcpyKind k = device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (Vc && rc == cudaSuccess) rc = cudaMemcpyAsync((void*)Vc, B.f.Vc, bc, k, e.stream);
    if (Vs && rc == cudaSuccess) rc = cudaMemcpyAsync((void*)Vs, B.f.Vs, bs, k, e.stream);
  }
  if (rc == cudaSuccess) rc = cudaStreamSynchronize(e.stream);
  if (rc != cudaSuccess) return ens_fail(e, IDFX_ERR_CUDA, std::string("copy: ") + cudaGetErrorString(rc));
  return IDFX_OK;
}

int idfx_ens_upload_prim(idfx_ens* h, int box, const double* Vc, const double* Vs) {
  return ens_copy(h, box, Vc, Vs, true);
}
int idfx_ens_download_prim(idfx_ens* h, int box, double* Vc, double* Vs) {
  return ens_copy(h, box, Vc, Vs, false);
}
int idfx_ens_download_prim_device(idfx_ens* h, int box, double* Vc, double* Vs) {
  return ens_copy(h, box, Vc, Vs, false, true);
}

int idfx_ens_get_time(idfx_ens* h, int box, double* t, double* dt, long long* ncycles, int* status) {
  if (!h || box < 0 || box >= h->e.nbox) return IDFX_ERR_STATE;
  EnsEngine& e = h->e;
  if (read_ctl(e)) return ens_fail(e, IDFX_ERR_CUDA, "get_time: CUDA failure");
  const Ctl& c = e.h_ctl[box];
  if (t) *t = c.t;
  if (dt) *dt = c.dt;
  if (ncycles) *ncycles = c.ncycles;
  if (status) *status = c.status;
  return IDFX_OK;
}

// Cycles every box until its time reaches tstop (tstop < 0: no limit) and at
// most max_cycles cycles (< 0: no limit); boxes that reach tstop or fail stop
// while the others go on.  Returns IDFX_OK when no box failed, else the
// status of the first failed box (idfx_ens_get_time gives every box's).
// mode: IDFX_ENS_LAUNCHES, IDFX_ENS_GRAPH, IDFX_ENS_PERSISTENT.
int idfx_ens_run(idfx_ens* h, double tstop, long long max_cycles, int mode) {
  if (!h) return IDFX_ERR_STATE;
  EnsEngine& e = h->e;
  if (tstop < 0.0 && max_cycles < 0) return ens_fail(e, IDFX_ERR_CONFIG, "run needs tstop or max_cycles");
  if (mode < IDFX_ENS_LAUNCHES || mode > IDFX_ENS_PERSISTENT) return ens_fail(e, IDFX_ERR_CONFIG, "run: unknown mode");
  if (read_ctl(e)) return ens_fail(e, IDFX_ERR_CUDA, "run: CUDA failure");
  std::vector<long long> nc(e.nbox);
  std::vector<char> live(e.nbox);
  for (int b = 0; b < e.nbox; b++) {
    Ctl& c = e.h_ctl[b];
    c.tstop = tstop < 0.0 ? DBL_MAX : tstop;
    c.done = c.status ? 1 : 0;  // a failed box stays stopped
  }
  if (cudaMemcpyAsync(e.d_ctl, e.h_ctl, sizeof(Ctl) * e.nbox, cudaMemcpyHostToDevice, e.stream) != cudaSuccess)
    return ens_fail(e, IDFX_ERR_CUDA, "run: CUDA failure");
  auto is_due = [](long long n, int p) { return p > 0 && n % p == 0; };
  long long done = 0;
  const long long chunk = 64;  // the host polls the control blocks every chunk of cycles
  while (max_cycles < 0 || done < max_cycles) {
    bool any_live = false;
    for (int b = 0; b < e.nbox; b++) {
      nc[b] = e.h_ctl[b].ncycles;
      live[b] = !e.h_ctl[b].done;
      any_live = any_live || live[b];
    }
    if (!any_live) break;
    long long n = chunk;
    if (max_cycles >= 0 && max_cycles - done < n) n = max_cycles - done;
    if (mode == IDFX_ENS_PERSISTENT) {
      const cudaError_t pr = run_persist(e, (int)n);
      if (pr != cudaSuccess)
        return ens_fail(e, IDFX_ERR_CUDA, std::string("persistent launch: ") + cudaGetErrorString(pr));
    }
    for (long long q = 0; q < n && mode != IDFX_ENS_PERSISTENT; q++) {
      bool checks = false;  // some live box runs a diagnostic this cycle
      for (int b = 0; b < e.nbox && !checks; b++)
        checks = live[b] && (is_due(nc[b] + q, e.log_period) || is_due(nc[b] + q, e.check_nan_period));
      if (mode == IDFX_ENS_GRAPH) {
        cudaGraphExec_t g = checks ? e.exec_checks : e.exec;
        if (cudaGraphLaunch(g, e.stream) != cudaSuccess) return ens_fail(e, IDFX_ERR_CUDA, "cudaGraphLaunch failed");
      } else {
        queue_cycle(e, checks);
      }
    }
    done += n;
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return ens_fail(e, IDFX_ERR_CUDA, std::string("run: ") + cudaGetErrorString(le));
    if (read_ctl(e)) return ens_fail(e, IDFX_ERR_CUDA, "run: CUDA failure");
    if (tstop < 0.0 && max_cycles < 0) break;
  }
  for (int b = 0; b < e.nbox; b++)
    if (e.h_ctl[b].status) {
      char msg[160];
      std::snprintf(msg, sizeof(msg), "box %d: %s", b, ens_status_text(e.h_ctl[b].status));
      return ens_fail(e, e.h_ctl[b].status, msg);
    }
  return IDFX_OK;
}

int idfx_ens_autotune(idfx_ens* h, int reps) {
  if (!h) return IDFX_ERR_STATE;
  return autotune(h->e, reps < 1 ? 1 : reps);
}

int idfx_ens_get_segments(const idfx_ens* h, int box, int* seg) {
  if (!h || !seg || box < 0 || box >= h->e.nbox) return IDFX_ERR_STATE;
  for (int d = 0; d < 3; d++) seg[d] = h->e.boxes[box].seg[d];
  return IDFX_OK;
}

int idfx_ens_persistent_info(idfx_ens* h, int* blocks, int* graph) {
  if (!h) return IDFX_ERR_STATE;
  if (blocks) *blocks = persist_blocks(h->e);
  if (graph) *graph = h->e.persist_graph ? 1 : 0;
  return IDFX_OK;
}

int idfx_ens_set_schedule(idfx_ens* h, int schedule) {
  if (!h || schedule < 0 || schedule > 1) return IDFX_ERR_STATE;
  EnsEngine& e = h->e;
  e.schedule = schedule;
  int rc = build_tables(e);
  if (!rc) rc = capture_graph(e);
  return rc ? ens_fail(e, rc, "set_schedule: CUDA failure") : IDFX_OK;
}

}  // extern "C"
