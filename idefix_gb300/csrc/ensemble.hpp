// Batched ensemble of independent periodic boxes (uneven sizes) advanced
// together: every phase of a stage is one launch over a work list that
// covers the blocks of every box, each box keeps its own time-step control
// block (per-box CFL dt), and one cycle of launches is captured in a CUDA
// graph and replayed.  The per-box arithmetic is the single-box code
// (the d_* device bodies of mhd_kernels.cuh), so every box evolves exactly
// as the same box run alone.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "engine.hpp"

namespace idfx {

struct EnsBox {
  Geo g;
  Fields f;
  Ctl* ctl;    // device control block of this box
  int seg[3];  // march segment length per direction (autotuned)
};

// one entry per CUDA block of a phase: {box, block.x, block.y, block.z}
struct EnsTable {
  int4* items = nullptr;
  int n = 0;
};

// grid-wide barrier of the persistent ensemble kernel (device memory)
struct GridBar {
  unsigned count;  // blocks arrived at the current barrier
  unsigned gen;    // barriers completed
  int failed;      // a block gave up waiting (bounded wait): every block stops
  int pad;
};

// work lists of the persistent ensemble kernel: the phase tables at the
// granularity of its 64-thread blocks, and the scheme
struct EnsPersist {
  const int4 *fill, *begin, *edges, *active, *sweep[3];
  int nfill, nbegin, nedges, nactive, nsweep[3];
  int nbox, nstages, log_period, check_nan_period, shock, keep_cons, cell_emf;
  double wc[2], w0[2];
};

struct EnsEngine {
  int nbox = 0;
  int D = 2, order = 2, solver = 0, emf = 0, nstages = 2, precision = 0;
  int log_period = 0, check_nan_period = 0;
  bool shock = false;  // shock flattening (flags per box)
  double wc[2] = {0, 0}, w0[2] = {0, 0};
  long long ncycles = 0;  // host mirror (all boxes cycle together)
  std::vector<EnsBox> boxes;
  EnsBox* d_boxes = nullptr;
  Ctl* d_ctl = nullptr;
  Ctl* h_ctl = nullptr;  // pinned mirror of all control blocks
  double* pool = nullptr;
  size_t pool_len = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  EnsTable fill, begin, sweep[3], edges, active;
  EnsTable fill64, begin64, edges64, active64;  // the same phases at 64 threads per item (persistent kernel)
  std::vector<EnsTable*> tables() {
    return {&fill, &begin, &sweep[0], &sweep[1], &sweep[2], &edges, &active, &fill64, &begin64, &edges64, &active64};
  }
  GridBar* d_bar = nullptr;
  cudaGraphExec_t exec_persist = nullptr;  // one chunk of cycles as one persistent launch
  int persist_chunk = 0;                   // cycles of that graph
  bool persist_graph = false;              // the persistent launch replays from a graph
  cudaGraphExec_t exec = nullptr;         // one cycle without diagnostics
  cudaGraphExec_t exec_checks = nullptr;  // one cycle with the divB / NaN checks
  int schedule = 0;                        // block order: 0 largest box first, 1 box order
  std::string err;
};

// the persistent kernel: ncyc cycles of every box in one cooperative launch
// of grid blocks (one per solver translation unit; 0 or a CUDA error)
cudaError_t launch_ens_persist_hlld(EnsEngine& e, int ncyc, int grid);
cudaError_t launch_ens_persist_hll(EnsEngine& e, int ncyc, int grid);
cudaError_t launch_ens_persist_roe(EnsEngine& e, int ncyc, int grid);
cudaError_t launch_ens_persist_tvdlf(EnsEngine& e, int ncyc, int grid);
// co-resident blocks of the persistent kernel on the whole device
int ens_persist_blocks_hlld(const EnsEngine& e);
int ens_persist_blocks_hll(const EnsEngine& e);
int ens_persist_blocks_roe(const EnsEngine& e);
int ens_persist_blocks_tvdlf(const EnsEngine& e);
EnsPersist ens_persist_args(const EnsEngine& e);

// batched sweep launch for one solver (one per translation unit)
void launch_ens_sweep_hlld(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_hll(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_roe(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_tvdlf(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);

}  // namespace idfx
