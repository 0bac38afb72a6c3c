// Host side of one GPU block: device buffers, control block and the
// TimeIntegrator::Cycle driver (timeIntegrator.cpp:246-414) behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/idefix_gb300.h"
#include "mhd_kernels.cuh"

namespace idfx {

struct SweepTileMaps;  // tensor maps of the tile sweeps (sweep_tile.cuh)
struct CtTileMap;      // tensor map of the staged fused CT pass (ct_tile.cuh)

struct Engine {
  Geo g{};
  Fields f{};
  Ctl* ctl = nullptr;        // device control block
  Ctl* ctl_host = nullptr;   // pinned mirror for reads
  Ctl* ctl_host_dev = nullptr;  // the same mirror as the device addresses it
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int nstages = 2;
  int precision = 0;         // 0: FP64 bit-exact, 1: mixed (FP32 recon + Riemann)
  double wc[2] = {0, 0}, w0[2] = {0, 0};
  int log_period = 0, check_nan_period = 0;
  long long ncycles = 0;     // host mirror of the cycle counter
  int seg[3] = {32, 32, 32}; // marching segment per direction
  int only_dir = -1;         // >= 0: sweeps launch that direction alone (autotuner)
  bool stage_outputs = false;  // mixed path: a stage end queued in this run wrote the next stage's inputs
  bool faces_saved = false;    // periodic block: the last face update queued wrote the next cycle's Vs0
  bool uc_field_stale = false; // mixed path: stage ends queued without the field part of Uc
  std::string err;
  double* pool = nullptr;    // one allocation for every field
  size_t pool_len = 0;
  // optional per-kernel timing: CUDA events around every launch of a class
  bool profile = false;
  struct Mark {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> free_events;
  void* learned = nullptr;   // network of the learned reconstruction (ORDER 5)
  int tile[3] = {0, 0, 0};   // 1: the y / z sweep runs as the tile sweep (mixed 3-D), else the march
  SweepTileMaps* tile_maps = nullptr;
  bool tile_maps_tried = false;
  CtTileMap* ct_map = nullptr;
  bool ct_map_tried = false;
};

// kernel classes reported by the per-kernel timing
enum KernelClass {
  kKFillFaces = 0,
  kKStageBegin,
  kKSweepX,
  kKSweepY,
  kKSweepZ,
  kKCtCorner,
  kKCtFaces,
  kKStageEnd,
  kKControl,
  kKChecks,
  kKLearned,
  kKNumClasses
};

// validation of a block configuration and its grid / geometry; march
// segment lengths for the block's size (both shared by every entry point
// that sets up a block)
int block_geometry(const idfx_gpu_config* cfg, Geo& g);
void choose_segments(Engine& e);

cudaEvent_t take_event(Engine& e);
void mark_begin(Engine& e, int cls);
void mark_end(Engine& e);

// tensor maps of the tile sweeps, made on first use; null when the block
// does not qualify (3-D mixed precision, nt0 a multiple of 4, 16-byte
// aligned arrays) or the driver offers no tensor-map encoder
const SweepTileMaps* sweep_tile_maps(Engine& e);
const CtTileMap* ct_tile_map(Engine& e);
// the y / z sweeps of this block can run as tile sweeps
bool tile_sweep_eligible(Engine& e, int dir);

// learned sweeps of one stage (ORDER 5: reconstruction with the network's
// correction, Riemann solve and flux difference in one kernel per
// direction) and the release of the network
void launch_learned_sweeps(Engine& e, int invdt, int fold_max);
void free_learned(Engine& e);

// launches the D flux sweeps of one stage (one function per Riemann solver,
// each in its own translation unit)
void launch_sweeps_hlld(Engine& e, int invdt, int fold_max);
void launch_sweeps_hll(Engine& e, int invdt, int fold_max);
void launch_sweeps_roe(Engine& e, int invdt, int fold_max);
void launch_sweeps_tvdlf(Engine& e, int invdt, int fold_max);

}  // namespace idfx

struct idfx_gpu {
  idfx::Engine e;
};
