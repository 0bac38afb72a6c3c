/*
 * idefix_gb300.hpp — C++ facade of the C ABI with the reference's class and
 * method names, for Idefix code that drives the hot path through its own
 * objects:
 *
 *   DataBlock             dataBlock.hpp:142,150   EvolveStage, ComputeTimestep
 *   DataBlock::hydro      fluid.hpp:57-67         ConvertPrimToCons, ConvertConsToPrim,
 *                                                 ResetStage, EvolveStage, CheckDivB, CheckNan
 *   hydro->boundary       boundary.hpp:240-282    SetBoundaries (ReconstructVcField included)
 *   TimeIntegrator        timeIntegrator.hpp:25   Cycle(DataBlock&), GetNCycles
 *
 * so that `Tint.Cycle(data)`, `data.hydro->EvolveStage(t, dt)` or
 * `data.hydro->boundary->SetBoundaries(t)` read as they do in the reference.
 * The corner EMFs and the face-field update of ConstrainedTransport
 * (CalcCornerEMF, EvolveMagField) run inside Fluid::EvolveStage, as the
 * reference's EvolveStage calls them (evolveStage.hpp:70-88); they have no
 * separate entry point.
 *
 * Errors: every non-zero status throws idefix_gb300::Error, a
 * std::runtime_error carrying the status and the library's message.  The
 * reference throws std::runtime_error for the numerical failures of a cycle
 * (NaN, divB, dt too small), which main.cpp:192-211 catches to write an
 * emergency dump; those reach the same catch here (Error::numerical() tells
 * them apart from setup and CUDA failures, which the reference reports
 * through IDEFIX_ERROR).
 *
 * Header-only over include/idefix_gb300.h; link with -lidefix_gb300.
 */
#ifndef IDEFIX_GB300_HPP_
#define IDEFIX_GB300_HPP_

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include "idefix_gb300.h"

namespace idefix_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }
  // a failure of the integration itself (main.cpp:192-211 catches these)
  bool numerical() const {
    return status_ == IDFX_ERR_NAN || status_ == IDFX_ERR_DIVB || status_ == IDFX_ERR_DT_SMALL;
  }

 private:
  int status_;
};

inline const char* status_name(int st) {
  switch (st) {
    case IDFX_OK: return "ok";
    case IDFX_ERR_CONFIG: return "invalid setup";
    case IDFX_ERR_NAN: return "Nan found after integration cycle";
    case IDFX_ERR_DIVB: return "divB too large, check your calculation";
    case IDFX_ERR_DT_SMALL: return "dt is too small";
    case IDFX_ERR_FIRST_DT: return "Your guessed first_dt is too large";
    case IDFX_ERR_CUDA: return "CUDA runtime failure";
    case IDFX_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

namespace detail {
// throws for a non-zero status, with the handle's last message when it has one
inline void check(int st, const idfx_gpu* h, const char* where) {
  if (st == IDFX_OK) return;
  std::string what = std::string("idefix_gb300: ") + where + ": " + status_name(st);
  if (h) {
    char buf[512] = {0};
    if (idfx_gpu_last_error(h, buf, sizeof(buf)) == IDFX_OK && buf[0]) what += std::string(" (") + buf + ")";
  }
  throw Error(st, what);
}
}  // namespace detail

// One device-resident block: owns the idfx_gpu handle and every device buffer.
class Block {
 public:
  explicit Block(const idfx_gpu_config& cfg, void* stream = nullptr) {
    idfx_gpu* h = nullptr;
    detail::check(idfx_gpu_create(&cfg, stream, &h), nullptr, "idfx_gpu_create");
    h_ = h;
  }
  ~Block() {
    if (h_) idfx_gpu_destroy(h_);
  }
  Block(const Block&) = delete;
  Block& operator=(const Block&) = delete;
  Block(Block&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  Block& operator=(Block&& o) noexcept {
    if (this != &o) {
      if (h_) idfx_gpu_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }

  idfx_gpu* handle() const { return h_; }
  void check(int st, const char* where) const { detail::check(st, h_, where); }

  // host arrays in the reference layout, ghosts included (DataBlockHost::SyncToDevice)
  void UploadPrim(const double* Vc, const double* Vs) { check(idfx_gpu_upload_prim(h_, Vc, Vs), "upload_prim"); }
  void DownloadPrim(double* Vc, double* Vs) { check(idfx_gpu_download_prim(h_, Vc, Vs), "download_prim"); }
  void DownloadCons(double* Uc) { check(idfx_gpu_download_cons(h_, Uc), "download_cons"); }
  // device pointers, same layout (a Kokkos CUDA build's Vc.data(), Vs.data())
  void UploadPrimDevice(const double* Vc, const double* Vs) {
    check(idfx_gpu_upload_prim_device(h_, Vc, Vs), "upload_prim_device");
  }
  void DownloadPrimDevice(double* Vc, double* Vs) {
    check(idfx_gpu_download_prim_device(h_, Vc, Vs), "download_prim_device");
  }

  void SetTime(double t, double dt, long long ncycles) { check(idfx_gpu_set_time(h_, t, dt, ncycles), "set_time"); }
  void GetTime(double* t, double* dt, long long* ncycles) const {
    check(idfx_gpu_get_time(h_, t, dt, ncycles), "get_time");
  }

 private:
  idfx_gpu* h_ = nullptr;
};

// Boundary (boundary.hpp): ghost cells and faces of Vc / Vs, then Vc(B) from the faces.
class Boundary {
 public:
  explicit Boundary(Block& b) : b_(&b) {}
  void SetBoundaries(double /*t: unused for periodic, reflective and outflow*/) {
    b_->check(idfx_gpu_set_boundaries(b_->handle()), "SetBoundaries");
  }

 private:
  Block* b_;
};

// Fluid<DefaultPhysics> (fluid.hpp): the stage and its companions.
class Fluid {
 public:
  explicit Fluid(Block& b) : b_(&b), boundary(std::make_unique<Boundary>(b)) {}

  void ConvertPrimToCons() { b_->check(idfx_gpu_prim_to_cons(b_->handle()), "ConvertPrimToCons"); }
  void ConvertConsToPrim() { b_->check(idfx_gpu_cons_to_prim(b_->handle()), "ConvertConsToPrim"); }
  void ResetStage() { b_->check(idfx_gpu_reset_stage(b_->handle()), "ResetStage"); }
  // fluxes, flux-difference update, corner EMFs and face update of one stage
  void EvolveStage(double t, double dt) { b_->check(idfx_gpu_evolve_stage(b_->handle(), t, dt), "EvolveStage"); }
  double CheckDivB() {
    double v = 0.0;
    b_->check(idfx_gpu_check_divb(b_->handle(), &v), "CheckDivB");
    return v;
  }
  int CheckNan() {
    long long n = 0;
    b_->check(idfx_gpu_check_nan(b_->handle(), &n), "CheckNan");
    return static_cast<int>(n);
  }

 private:
  Block* b_;

 public:
  std::unique_ptr<Boundary> boundary;
};

// DataBlock (dataBlock.hpp): the block, its Fluid, its time.
class DataBlock {
 public:
  explicit DataBlock(const idfx_gpu_config& cfg, void* stream = nullptr)
      : block(cfg, stream), hydro(std::make_unique<Fluid>(block)) {}

  // dataBlock.cpp:333-364: min over active cells of 1 / InvDt
  double ComputeTimestep() {
    double dt = 0.0;
    block.check(idfx_gpu_compute_timestep(block.handle(), &dt), "ComputeTimestep");
    return dt;
  }
  // evolveStage.cpp:13-35: the stage at the block's current t and dt
  void EvolveStage() {
    double t = 0.0, dt = 0.0;
    block.GetTime(&t, &dt, nullptr);
    hydro->EvolveStage(t, dt);
  }

  Block block;
  std::unique_ptr<Fluid> hydro;
};

// TimeIntegrator (timeIntegrator.hpp): RK cycles with the reference's dt logic.
class TimeIntegrator {
 public:
  TimeIntegrator() = default;
  // one cycle: boundaries, stages, RK combination, CFL dt (timeIntegrator.cpp:246-414)
  void Cycle(DataBlock& data) { data.block.check(idfx_gpu_cycle(data.block.handle()), "Cycle"); }
  // cycles until t reaches tstop or max_cycles have run (a negative value: no limit)
  void Run(DataBlock& data, double tstop, long long max_cycles = -1) {
    data.block.check(idfx_gpu_run(data.block.handle(), tstop, max_cycles), "Run");
  }
  long long GetNCycles(const DataBlock& data) const {
    long long n = 0;
    data.block.GetTime(nullptr, nullptr, &n);
    return n;
  }
};

}  // namespace idefix_gb300

#endif  // IDEFIX_GB300_HPP_
