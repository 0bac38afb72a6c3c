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
  std::vector<EnsTable*> tables() { return {&fill, &begin, &sweep[0], &sweep[1], &sweep[2], &edges, &active}; }
  cudaGraphExec_t exec = nullptr;         // one cycle without diagnostics
  cudaGraphExec_t exec_checks = nullptr;  // one cycle with the divB / NaN checks
  int schedule = 0;                        // block order: 0 largest box first, 1 box order
  std::string err;
};

// batched sweep launch for one solver (one per translation unit)
void launch_ens_sweep_hlld(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_hll(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_roe(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);
void launch_ens_sweep_tvdlf(EnsEngine& e, int dir, const EnsTable& t, int invdt, int last);

}  // namespace idfx
