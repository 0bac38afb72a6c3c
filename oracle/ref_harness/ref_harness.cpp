// TEST INFRASTRUCTURE ONLY — builds oracle/_ref/libofx_ref_d<D>_o<ORDER>.so.
//
// Compiles the reference's own hot-path method bodies, from the reference
// source tree where it lies, for a serial host build, and serves them through
// the same C entry points as the plain-C oracle (oracle/ofx.h).  The tests use
// it to pin the oracle bit for bit, and to generate the golden fixtures.
//
// Reference files compiled here (unmodified, by #include):
//   src/idefix.hpp, src/macros.hpp, src/real_types.hpp, src/physics.hpp,
//   src/fluid/fluid_defs.hpp, src/fluid/eos/eos.hpp (eos_adiabatic.hpp),
//   src/fluid/RiemannSolver/slopeLimiter.hpp, extrapolateToFaces.hpp,
//   flux.hpp, MHDsolvers/{storeFlux,hlldMHD,hllMHD,roeMHD,tvdlfMHD}.hpp,
//   src/fluid/convertConsToPrim.hpp, src/fluid/calcRightHandSide.hpp,
//   src/fluid/constrainedTransport/{calcCornerEmf,calcRiemannEmf,
//   evolveMagField}.hpp
// Kokkos is not available here, so the classes those bodies belong to
// (Fluid, DataBlock, RiemannSolver, ConstrainedTransport, Boundary, ...) are
// declared below with just the members the bodies touch, and idefix_for /
// IdefixArrayND are provided by a serial host implementation.  The stage
// driver (TimeIntegrator::Cycle), the periodic ghost copy
// (Boundary::EnforcePeriodic) and ReconstructVcField are restated below from
// src/timeIntegrator.cpp:246-414 and src/fluid/boundary/boundary.hpp:388-404,
// 576-673, since their classes pull in MPI, I/O and input parsing.
//
// Build: oracle/Makefile (needs the reference tree; -DORDER and
// -DDEFINITIONS_FILE select the variant, exactly like the reference's CMake
// options Idefix_RECONSTRUCTION and the problem's definitions.hpp).

#include <array>
#include <limits>
#include <cmath>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "Kokkos_Core.hpp"

// Reference headers replaced by the declarations in this file.
#define GLOBAL_HPP_
#define ERROR_HPP_
#define LOOP_HPP_
#define REDUCE_HPP_
#define ARRAYS_HPP_
#define GRID_HPP_
#define GRIDHOST_HPP_
#define INPUT_HPP_
#define FLUID_FLUID_HPP_
#define DATABLOCK_DATABLOCK_HPP_
#define FLUID_RIEMANNSOLVER_RIEMANNSOLVER_HPP_
#define FLUID_CONSTRAINEDTRANSPORT_CONSTRAINEDTRANSPORT_HPP_
#define FLUID_BOUNDARY_AXIS_HPP_
#define FLUID_TRACER_TRACER_HPP_
#define GRAVITY_GRAVITY_HPP_
#define DATABLOCK_FARGO_HPP_
#define UTILS_NPY_HPP_

#include "idefix.hpp"  // NOLINT  (variable indices, EXPAND/D_EXPAND, enums)

// ----------------------------------------------------------------------------
// Host arrays with the IdefixArrayND interface (shared, zero-initialised,
// LayoutRight), and the serial loop / region helpers.
// ----------------------------------------------------------------------------
template <typename T, int R>
class HostView {
 public:
  HostView() = default;
  HostView(const std::string&, int n0, int n1 = 1, int n2 = 1, int n3 = 1) {
    int n[4] = {n0, n1, n2, n3};
    size_t tot = 1;
    for (int d = 0; d < 4; d++) {
      ext_[d] = d < R ? n[d] : 1;
      tot *= static_cast<size_t>(ext_[d]);
    }
    mem_ = std::shared_ptr<T>(new T[tot ? tot : 1](), std::default_delete<T[]>());
    p_ = mem_.get();
    size_ = tot;
  }
  T& operator()(int i) const { return p_[i]; }
  T& operator()(int j, int i) const { return p_[static_cast<size_t>(j) * ext_[1] + i]; }
  T& operator()(int k, int j, int i) const {
    return p_[(static_cast<size_t>(k) * ext_[1] + j) * ext_[2] + i];
  }
  T& operator()(int n, int k, int j, int i) const {
    return p_[((static_cast<size_t>(n) * ext_[1] + k) * ext_[2] + j) * ext_[3] + i];
  }
  int extent(int d) const { return ext_[d]; }
  T* data() const { return p_; }
  size_t size() const { return size_; }

 private:
  std::shared_ptr<T> mem_;
  T* p_{nullptr};
  int ext_[4]{1, 1, 1, 1};
  size_t size_{0};
};

template <typename T> using IdefixArray1D = HostView<T, 1>;
template <typename T> using IdefixArray2D = HostView<T, 2>;
template <typename T> using IdefixArray3D = HostView<T, 3>;
template <typename T> using IdefixArray4D = HostView<T, 4>;
template <typename T> using IdefixHostArray1D = HostView<T, 1>;
template <typename T> using IdefixHostArray3D = HostView<T, 3>;
template <typename T> using IdefixHostArray4D = HostView<T, 4>;

template <typename F>
inline void idefix_for(const std::string&, int ib, int ie, F f) {
  for (int i = ib; i < ie; i++) f(i);
}
template <typename F>
inline void idefix_for(const std::string&, int jb, int je, int ib, int ie, F f) {
  for (int j = jb; j < je; j++)
    for (int i = ib; i < ie; i++) f(j, i);
}
template <typename F>
inline void idefix_for(const std::string&, int kb, int ke, int jb, int je, int ib, int ie, F f) {
  for (int k = kb; k < ke; k++)
    for (int j = jb; j < je; j++)
      for (int i = ib; i < ie; i++) f(k, j, i);
}
template <typename F>
inline void idefix_for(const std::string&, int nb, int ne, int kb, int ke, int jb, int je, int ib,
                       int ie, F f) {
  for (int n = nb; n < ne; n++)
    for (int k = kb; k < ke; k++)
      for (int j = jb; j < je; j++)
        for (int i = ib; i < ie; i++) f(n, k, j, i);
}

namespace Kokkos {
template <typename T>
struct Min {
  using value_type = T;
  T& r;
  explicit Min(T& x) : r(x) {}
  static T init() { return std::numeric_limits<T>::max(); }
};
template <typename T>
struct Max {
  using value_type = T;
  T& r;
  explicit Max(T& x) : r(x) {}
  static T init() { return std::numeric_limits<T>::lowest(); }
};
template <typename T>
struct Sum {
  using value_type = T;
  T& r;
  explicit Sum(T& x) : r(x) {}
  static T init() { return T(0); }
};
}  // namespace Kokkos

// serial reduction: the lambda folds every point into one accumulator
template <typename F, typename R>
inline void idefix_reduce(const std::string&, int kb, int ke, int jb, int je, int ib, int ie, F f,
                          R red) {
  typename R::value_type v = R::init();
  for (int k = kb; k < ke; k++)
    for (int j = jb; j < je; j++)
      for (int i = ib; i < ie; i++) f(k, j, i, v);
  red.r = v;
}
template <typename F, typename R>
inline void idefix_reduce(const std::string&, int nb, int ne, int kb, int ke, int jb, int je, int ib,
                          int ie, F f, R red) {
  typename R::value_type v = R::init();
  for (int n = nb; n < ne; n++)
    for (int k = kb; k < ke; k++)
      for (int j = jb; j < je; j++)
        for (int i = ib; i < ie; i++) f(n, k, j, i, v);
  red.r = v;
}

namespace idfx {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
inline std::ostream& cout = std::cout;
}  // namespace idfx

struct OfxRefError {
  std::string msg;
};
// messages are strings or string streams (both forms appear in the bodies)
inline std::string ofx_msg(const std::stringstream& m) { return m.str(); }
template <typename T>
inline const T& ofx_msg(const T& m) { return m; }
#define IDEFIX_ERROR(m)                \
  do {                                 \
    std::stringstream ofx_ss;          \
    ofx_ss << ofx_msg(m);              \
    throw OfxRefError{ofx_ss.str()};   \
  } while (0)
#define IDEFIX_WARNING(m) do {} while (0)

#include "physics.hpp"     // NOLINT
#include "fluid_defs.hpp"  // NOLINT

template <typename Phys> class Fluid;
template <typename Phys> class RiemannSolver;
template <typename Phys> class ConstrainedTransport;
template <typename Phys> class Boundary;
template <typename Phys> class ShockFlattening;

// ----------------------------------------------------------------------------
// Declarations of the surrounding classes (members used by the bodies only)
// ----------------------------------------------------------------------------
class Input {
 public:
  std::vector<std::pair<std::string, double>> vals;
  template <typename T>
  T GetOrSet(const std::string&, const std::string& key, int, T def) {
    for (auto& kv : vals)
      if (kv.first == key) return static_cast<T>(kv.second);
    return def;
  }
};

struct Grid {
  bool isRegularCartesian{true};
  std::array<real, 3> xbeg{{0, 0, 0}}, xend{{1, 1, 1}};
  std::array<int, 3> np_int{{1, 1, 1}};
  std::array<int, 3> nproc{{1, 1, 1}};
  std::array<int, 3> xproc{{0, 0, 0}};
};

class Fargo {
 public:
  enum FargoType { userdef, shearingbox };
  FargoType type{userdef};
  IdefixArray2D<real> meanVelocity;
  void GetFargoVelocity(real) {}
};

class Gravity {
 public:
  IdefixArray3D<real> phiP;
  bool havePotential{false};
  IdefixArray4D<real> bodyForceVector;
  bool haveBodyForce{false};
};

class DataBlock {
 public:
  int np_tot[3], np_int[3], nghost[3], beg[3], end[3];
  IdefixArray1D<real> x[3], xr[3], xl[3], dx[3], xgc[3];
  IdefixArray3D<real> dV;
  IdefixArray3D<real> A[3];
  IdefixArray1D<real> rt, dmu, sinx2, tanx2, sinx2m, tanx2m;
  std::array<IdefixArray2D<int>, 3> coarseningLevel;
  std::array<bool, 3> coarseningDirection{{false, false, false}};
  bool haveGridCoarsening{false};
  Grid* mygrid{nullptr};
  bool haveFargo{false};
  std::unique_ptr<Fargo> fargo;
  bool haveGravity{false};
  std::unique_ptr<Gravity> gravity;
  real t{0};  // read by ShockFlattening::FindShock's user hook (not used here)
  std::array<BoundaryType, 3> lbound{{periodic, periodic, periodic}};
  std::array<BoundaryType, 3> rbound{{periodic, periodic, periodic}};
  bool haveAxis{false};
};

#include "eos.hpp"  // NOLINT  (adiabatic EquationOfState)

#include "shockFlattening.hpp"  // NOLINT  (FindShock, real functor)

#include "slopeLimiter.hpp"        // NOLINT
#include "extrapolateToFaces.hpp"  // NOLINT

template <typename Phys>
class RiemannSolver {
 public:
  enum Solver { TVDLF_MHD, HLL_MHD, HLLD_MHD, ROE_MHD, TVDLF, HLL, HLLC, ROE, HLL_DUST };
  template <const int> void HlldMHD(IdefixArray4D<real>&);
  template <const int> void HllMHD(IdefixArray4D<real>&);
  template <const int> void RoeMHD(IdefixArray4D<real>&);
  template <const int> void TvdlfMHD(IdefixArray4D<real>&);
  template <int dir>
  ExtrapolateToFaces<Phys, dir>* GetExtrapolator() {
    if constexpr (dir == IDIR) return slopeLimIDIR.get();
    if constexpr (dir == JDIR) return slopeLimJDIR.get();
    if constexpr (dir == KDIR) return slopeLimKDIR.get();
  }
  std::unique_ptr<ShockFlattening<Phys>> shockFlattening;
  IdefixArray4D<real> Vc;
  IdefixArray4D<real> Vs;
  IdefixArray4D<real> Flux;
  IdefixArray3D<real> cMax;
  Fluid<Phys>* hydro;
  DataBlock* data;
  Solver mySolver;
  std::unique_ptr<ExtrapolateToFaces<Phys, IDIR>> slopeLimIDIR;
  std::unique_ptr<ExtrapolateToFaces<Phys, JDIR>> slopeLimJDIR;
  std::unique_ptr<ExtrapolateToFaces<Phys, KDIR>> slopeLimKDIR;
  bool haveShockFlattening{false};
};

template <typename Phys>
class ConstrainedTransport {
 public:
  enum AveragingType { none, arithmetic, uct0, uct_contact, uct_hll, uct_hlld };
  AveragingType averaging{none};
  IdefixArray3D<real> exj, exk, eyi, eyk, ezi, ezj, ex, ey, ez, svx, svy, svz;
  IdefixArray3D<real> axL, axR, ayL, ayR, azL, azR, dxL, dxR, dyL, dyR, dzL, dzR;
  IdefixArray3D<real> Ex1, Ex2, Ex3;
  void EvolveMagField(real, real, IdefixArray4D<real>&);
  void CalcCornerEMF(real);
  void CalcRiemannAverage();
  void CalcArithmeticAverage();
  void CalcCellCenteredEMF();
  void CalcUCT0Average();
  void CalcContactAverage();
  DataBlock* data;
  Fluid<Phys>* hydro;
};

// the axis is never used here (Cartesian): the members Boundary names
class Axis {
 public:
  template <typename B>
  explicit Axis(B*) {}
  bool haveLeftAxis() { return false; }
  bool haveRightAxis() { return false; }
  void EnforceAxisBoundary(int) {}
  void RegularizeBX2s() {}
  void RegularizeEMFs() {}
};

#include "boundary.hpp"  // NOLINT  (Boundary<Phys>: SetBoundaries, Enforce*, ReconstructNormalField)

class Tracer {
 public:
  void ConvertConsToPrim() {}
  void ConvertPrimToCons() {}
};
class Viscosity {
 public:
  IdefixArray4D<real> viscSrc;
};
class BragViscosity {
 public:
  IdefixArray4D<real> bragViscSrc;
};

template <typename Phys>
class Fluid {
 public:
  void ConvertConsToPrim();
  void ConvertPrimToCons();
  template <int> void CalcRightHandSide(real, real);
  real CheckDivB();
  std::unique_ptr<Boundary<Phys>> boundary;
  std::unique_ptr<EquationOfState> eos;
  bool haveExplicitParabolicTerms{false};
  ParabolicModuleStatus resistivityStatus, ambipolarStatus, hallStatus;
  ParabolicModuleStatus viscosityStatus;
  std::unique_ptr<Viscosity> viscosity;
  ParabolicModuleStatus bragViscosityStatus;
  std::unique_ptr<BragViscosity> bragViscosity;
  bool haveAxis{false};
  bool haveRotation{false};
  real OmegaZ{0};
  bool haveShearingBox{false};
  real sbS{0};
  std::unique_ptr<Tracer> tracer;
  bool haveTracer{false};
  int nTracer{0};
  std::string prefix{"Hydro"};
  IdefixArray4D<real> Vc, Vs, Uc, J;
  std::unique_ptr<ConstrainedTransport<Phys>> emf;
  IdefixArray3D<real> InvDt;
  IdefixArray4D<real> FluxRiemann;
  IdefixArray3D<real> dMax;
  std::unique_ptr<RiemannSolver<Phys>> rSolver;
  DataBlock* data;
  real etaO{0}, xH{0}, xA{0};
  IdefixArray3D<real> cMax;
  IdefixArray3D<real> xHall;
};

#include "flux.hpp"               // NOLINT
#include "convertConsToPrim.hpp"  // NOLINT
#include "storeFlux.hpp"          // NOLINT
#include "hlldMHD.hpp"            // NOLINT
#include "hllMHD.hpp"             // NOLINT
#include "roeMHD.hpp"             // NOLINT
#include "tvdlfMHD.hpp"           // NOLINT
#include "calcRightHandSide.hpp"  // NOLINT
#include "calcCornerEmf.hpp"      // NOLINT
#include "calcRiemannEmf.hpp"     // NOLINT
#include "evolveMagField.hpp"     // NOLINT
#include "checkDivB.hpp"          // NOLINT

// ----------------------------------------------------------------------------
// Harness state and the oracle C API (same entry points as oracle/ofx.h)
// ----------------------------------------------------------------------------
using Phys = DefaultPhysics;

struct ofx {
  DataBlock data;
  Grid grid;
  Fluid<Phys> fluid;
  IdefixArray4D<real> Uc0, Vs0;
  int solver, emf, nstages;
  real cfl, cflmax, maxdivb, t, dt;
  long ncycles{0};
  int log_period{0}, check_nan_period{0};
};

#include "ofx.h"  // NOLINT

static void ofx_ref_alloc(ofx* o, const int n[3], const double xb[3], const double xe[3]) {
  DataBlock& d = o->data;
  const int ng = (ORDER == 4) ? 3 : 2;  // grid.cpp:60-65
  for (int dir = 0; dir < 3; dir++) {
    const bool active = dir < DIMENSIONS;
    d.nghost[dir] = active ? ng : 0;
    d.np_int[dir] = active ? n[dir] : 1;
    d.np_tot[dir] = d.np_int[dir] + 2 * d.nghost[dir];
    d.beg[dir] = d.nghost[dir];
    d.end[dir] = d.nghost[dir] + d.np_int[dir];
    const int nt = d.np_tot[dir];
    d.x[dir] = IdefixArray1D<real>("x", nt);
    d.xl[dir] = IdefixArray1D<real>("xl", nt);
    d.xr[dir] = IdefixArray1D<real>("xr", nt);
    d.dx[dir] = IdefixArray1D<real>("dx", nt);
    d.xgc[dir] = IdefixArray1D<real>("xgc", nt);
    const double xs = active ? xb[dir] : 0.0, xend = active ? xe[dir] : 1.0;
    for (int i = -d.nghost[dir]; i < d.np_int[dir] + d.nghost[dir]; i++) {  // gridHost.cpp:80-86
      const int ii = i + d.nghost[dir];
      d.dx[dir](ii) = (xend - xs) / (d.np_int[dir]);
      d.x[dir](ii) = xs + (i + HALF_F) * d.dx[dir](ii);
      d.xl[dir](ii) = xs + i * d.dx[dir](ii);
      d.xr[dir](ii) = xs + (i + 1) * d.dx[dir](ii);
      d.xgc[dir](ii) = d.x[dir](ii);
    }
  }
  const int nk = d.np_tot[KDIR], nj = d.np_tot[JDIR], ni = d.np_tot[IDIR];
  d.dV = IdefixArray3D<real>("dV", nk, nj, ni);
  d.A[IDIR] = IdefixArray3D<real>("A1", nk, nj, ni + IOFFSET);
  d.A[JDIR] = IdefixArray3D<real>("A2", nk, nj + JOFFSET, ni);
  d.A[KDIR] = IdefixArray3D<real>("A3", nk + KOFFSET, nj, ni);
  auto dx1 = d.dx[IDIR];
  auto dx2 = d.dx[JDIR];
  auto dx3 = d.dx[KDIR];
  (void)dx3;
  auto dV = d.dV;
  auto Ax1 = d.A[IDIR];
  auto Ax2 = d.A[JDIR];
  auto Ax3 = d.A[KDIR];
  // Cartesian geometry, as makeGeometry.cpp:67-70,146-147,178-179,201-202
  idefix_for("Volumes", 0, nk, 0, nj, 0, ni, KOKKOS_LAMBDA(int k, int j, int i) {
    dV(k, j, i) = D_EXPAND(dx1(i), *dx2(j), *dx3(k));
  });
  idefix_for("AreaX1", 0, nk, 0, nj, 0, ni + IOFFSET, KOKKOS_LAMBDA(int k, int j, int i) {
    Ax1(k, j, i) = D_EXPAND(1.0, *dx2(j), *dx3(k));
    (void)i;
  });
  idefix_for("AreaX2", 0, nk, 0, nj + JOFFSET, 0, ni, KOKKOS_LAMBDA(int k, int j, int i) {
    Ax2(k, j, i) = D_EXPAND(dx1(i), *ONE_F, *dx3(k));
    (void)j;
  });
  idefix_for("AreaX3", 0, nk + KOFFSET, 0, nj, 0, ni, KOKKOS_LAMBDA(int k, int j, int i) {
    Ax3(k, j, i) = D_EXPAND(dx1(i), *dx2(j), *ONE_F);
    (void)k;
  });
  d.rt = IdefixArray1D<real>("rt", d.np_tot[IDIR]);
  d.dmu = IdefixArray1D<real>("dmu", d.np_tot[JDIR]);
  d.sinx2 = IdefixArray1D<real>("sinx2", d.np_tot[JDIR]);
  d.sinx2m = IdefixArray1D<real>("sinx2m", d.np_tot[JDIR]);
  d.mygrid = &o->grid;

  Fluid<Phys>& f = o->fluid;
  f.data = &d;
  f.Vc = IdefixArray4D<real>("Vc", Phys::nvar, nk, nj, ni);
  f.Uc = IdefixArray4D<real>("Uc", Phys::nvar, nk, nj, ni);
  f.InvDt = IdefixArray3D<real>("InvDt", nk, nj, ni);
  f.cMax = IdefixArray3D<real>("cMax", nk, nj, ni);
  f.dMax = IdefixArray3D<real>("dMax", nk, nj, ni);
  f.FluxRiemann = IdefixArray4D<real>("Flux", Phys::nvar, nk, nj, ni);
  f.Vs = IdefixArray4D<real>("Vs", DIMENSIONS, nk + KOFFSET, nj + JOFFSET, ni + IOFFSET);
  o->Uc0 = IdefixArray4D<real>("Uc0", Phys::nvar, nk, nj, ni);
  o->Vs0 = IdefixArray4D<real>("Vs0", DIMENSIONS, nk + KOFFSET, nj + JOFFSET, ni + IOFFSET);
  f.boundary = std::make_unique<Boundary<Phys>>(&f);  // boundary.hpp:128-190
  f.tracer = std::make_unique<Tracer>();
  f.viscosity = std::make_unique<Viscosity>();
  f.bragViscosity = std::make_unique<BragViscosity>();

  auto* ct = new ConstrainedTransport<Phys>();
  f.emf.reset(ct);
  ct->data = &d;
  ct->hydro = &f;
  IdefixArray3D<real>* emfs[] = {&ct->exj, &ct->exk, &ct->eyi, &ct->eyk, &ct->ezi, &ct->ezj,
                                 &ct->ex,  &ct->ey,  &ct->ez,  &ct->svx, &ct->svy, &ct->svz,
                                 &ct->axL, &ct->axR, &ct->ayL, &ct->ayR, &ct->azL, &ct->azR,
                                 &ct->dxL, &ct->dxR, &ct->dyL, &ct->dyR, &ct->dzL, &ct->dzR,
                                 &ct->Ex1, &ct->Ex2, &ct->Ex3};
  for (auto* a : emfs) *a = IdefixArray3D<real>("emf", nk, nj, ni);
  static const typename ConstrainedTransport<Phys>::AveragingType avg[] = {
      ConstrainedTransport<Phys>::uct_contact, ConstrainedTransport<Phys>::arithmetic,
      ConstrainedTransport<Phys>::uct0, ConstrainedTransport<Phys>::uct_hll,
      ConstrainedTransport<Phys>::uct_hlld};
  ct->averaging = avg[o->emf];

  auto* rs = new RiemannSolver<Phys>();
  f.rSolver.reset(rs);
  rs->Vc = f.Vc;
  rs->Vs = f.Vs;
  rs->Flux = f.FluxRiemann;
  rs->cMax = f.cMax;
  rs->hydro = &f;
  rs->data = &d;
  static const typename RiemannSolver<Phys>::Solver sol[] = {
      RiemannSolver<Phys>::HLLD_MHD, RiemannSolver<Phys>::HLL_MHD, RiemannSolver<Phys>::ROE_MHD,
      RiemannSolver<Phys>::TVDLF_MHD};
  rs->mySolver = sol[o->solver];
  rs->slopeLimIDIR = std::make_unique<ExtrapolateToFaces<Phys, IDIR>>(rs);
#if DIMENSIONS >= 2
  rs->slopeLimJDIR = std::make_unique<ExtrapolateToFaces<Phys, JDIR>>(rs);
#endif
#if DIMENSIONS == 3
  rs->slopeLimKDIR = std::make_unique<ExtrapolateToFaces<Phys, KDIR>>(rs);
#endif
}

extern "C" {

ofx* ofx_create(int dims, int nx, int ny, int nz, double xb0, double xe0, double xb1, double xe1,
                double xb2, double xe2, int order, int solver, int emf, int nstages, double gamma,
                double cfl, double cfl_max_var, double first_dt) {
  if (dims != DIMENSIONS || order != ORDER) return nullptr;
  if (solver < 0 || solver > 3 || emf < 0 || emf > 4 || nstages < 1 || nstages > 3) return nullptr;
  if (emf == OFX_UCT_HLLD && (solver == OFX_HLL || solver == OFX_TVDLF)) return nullptr;
  ofx* o = new ofx();
  o->solver = solver;
  o->emf = emf;
  o->nstages = nstages;
  o->cfl = cfl;
  o->cflmax = cfl_max_var;
  o->maxdivb = 1e-6;
  o->t = 0;
  o->dt = first_dt;
  int n[3] = {nx, ny, nz};
  double xb[3] = {xb0, xb1, xb2}, xe[3] = {xe0, xe1, xe2};
  ofx_ref_alloc(o, n, xb, xe);
  Input in;
  in.vals.push_back({"gamma", gamma});
  o->fluid.eos = std::make_unique<EquationOfState>(in, &o->data, std::string("Hydro"));
  return o;
}

void ofx_destroy(ofx* o) { delete o; }
int ofx_nvar(const ofx*) { return Phys::nvar; }
int ofx_nghost(const ofx* o) { return o->data.nghost[IDIR]; }
long ofx_ncell(const ofx* o) {
  return static_cast<long>(o->data.np_tot[0]) * o->data.np_tot[1] * o->data.np_tot[2];
}
long ofx_nface(const ofx* o) { return static_cast<long>(o->fluid.Vs.size() / DIMENSIONS); }
void ofx_set_threads(ofx*, int) {}

void ofx_set_prim(ofx* o, const double* Vc, const double* Vs) {
  std::memcpy(o->fluid.Vc.data(), Vc, sizeof(double) * o->fluid.Vc.size());
  std::memcpy(o->fluid.Vs.data(), Vs, sizeof(double) * o->fluid.Vs.size());
}
void ofx_get_prim(const ofx* o, double* Vc, double* Vs) {
  if (Vc) std::memcpy(Vc, o->fluid.Vc.data(), sizeof(double) * o->fluid.Vc.size());
  if (Vs) std::memcpy(Vs, o->fluid.Vs.data(), sizeof(double) * o->fluid.Vs.size());
}
void ofx_get_cons(const ofx* o, double* Uc) {
  std::memcpy(Uc, o->fluid.Uc.data(), sizeof(double) * o->fluid.Uc.size());
}
void ofx_set_time(ofx* o, double t, double dt, long ncycles) {
  o->t = t;
  o->dt = dt;
  o->ncycles = ncycles;
}
void ofx_get_time(const ofx* o, double* t, double* dt, long* ncycles) {
  if (t) *t = o->t;
  if (dt) *dt = o->dt;
  if (ncycles) *ncycles = o->ncycles;
}
void ofx_set_shock(ofx* o, int enabled, double smoothing) {
  // RiemannSolver constructor (riemannSolver.hpp:153-159), then the
  // extrapolators, which read the flag array when they are built
  RiemannSolver<Phys>* rs = o->fluid.rSolver.get();
  rs->haveShockFlattening = enabled != 0;
  rs->shockFlattening.reset();
  if (rs->haveShockFlattening) rs->shockFlattening = std::make_unique<ShockFlattening<Phys>>(&o->fluid, smoothing);
  rs->slopeLimIDIR = std::make_unique<ExtrapolateToFaces<Phys, IDIR>>(rs);
#if DIMENSIONS >= 2
  rs->slopeLimJDIR = std::make_unique<ExtrapolateToFaces<Phys, JDIR>>(rs);
#endif
#if DIMENSIONS == 3
  rs->slopeLimKDIR = std::make_unique<ExtrapolateToFaces<Phys, KDIR>>(rs);
#endif
}

void ofx_set_checks(ofx* o, int log_period, int check_nan_period, double maxdivb) {
  o->log_period = log_period;
  o->check_nan_period = check_nan_period;
  o->maxdivb = maxdivb;
}

// Boundary::SetBoundaries for periodic boxes: EnforcePeriodic per direction,
// left then right, then ReconstructVcField (restated from
// src/fluid/boundary/boundary.hpp:240-282,576-673,969-1099)
void ofx_set_boundaries(ofx* o) {  // Boundary::SetBoundaries (boundary.hpp:240-280)
  o->fluid.boundary->SetBoundaries(o->t);
}

// [Boundary] X?-beg / X?-end: 0 periodic, 1 reflective, 2 outflow
int ofx_set_bc(ofx* o, int dir, int left, int right) {
  static const BoundaryType map[] = {periodic, reflective, outflow};
  if (dir < 0 || dir >= DIMENSIONS || left < 0 || left > 2 || right < 0 || right > 2) return OFX_ERR_CONFIG;
  if ((left == 0) != (right == 0)) return OFX_ERR_CONFIG;  // periodic on both sides or neither
  o->data.lbound[dir] = map[left];
  o->data.rbound[dir] = map[right];
  return OFX_OK;
}

void ofx_prim_to_cons(ofx* o) { o->fluid.ConvertPrimToCons(); }
void ofx_cons_to_prim(ofx* o) { o->fluid.ConvertConsToPrim(); }
void ofx_reset_stage(ofx* o) {  // Fluid::ResetStage (enroll.hpp:116-129)
  auto InvDt = o->fluid.InvDt;
  idefix_for("HydroResetStage", 0, o->data.np_tot[KDIR], 0, o->data.np_tot[JDIR], 0,
             o->data.np_tot[IDIR], KOKKOS_LAMBDA(int k, int j, int i) { InvDt(k, j, i) = ZERO_F; });
}

}  // extern "C"

template <int dir>
static void ofx_ref_loopdir(ofx* o, real t, real dt) {
  // Fluid::LoopDir (evolveStage.hpp:13-35) with the RiemannSolver::CalcFlux
  // dispatch of calcFlux.hpp:26-85 (MHD solvers)
  RiemannSolver<Phys>* rs = o->fluid.rSolver.get();
  if (rs->haveShockFlattening) rs->shockFlattening->FindShock();  // calcFlux.hpp:33
  switch (rs->mySolver) {
    case RiemannSolver<Phys>::TVDLF_MHD: rs->template TvdlfMHD<dir>(o->fluid.FluxRiemann); break;
    case RiemannSolver<Phys>::HLL_MHD: rs->template HllMHD<dir>(o->fluid.FluxRiemann); break;
    case RiemannSolver<Phys>::HLLD_MHD: rs->template HlldMHD<dir>(o->fluid.FluxRiemann); break;
    case RiemannSolver<Phys>::ROE_MHD: rs->template RoeMHD<dir>(o->fluid.FluxRiemann); break;
    default: break;
  }
  o->fluid.template CalcRightHandSide<dir>(t, dt);
  if constexpr (dir + 1 < DIMENSIONS) ofx_ref_loopdir<dir + 1>(o, t, dt);
}

extern "C" {

void ofx_evolve_stage(ofx* o, double t, double dt) {  // Fluid::EvolveStage (evolveStage.hpp:40-90)
  ofx_ref_loopdir<IDIR>(o, t, dt);
  o->fluid.emf->CalcCornerEMF(t);
  o->fluid.emf->EvolveMagField(t, dt, o->fluid.Vs);
  o->fluid.boundary->ReconstructVcField(o->fluid.Uc);
}

double ofx_compute_timestep(ofx* o) {  // DataBlock::ComputeTimestep (dataBlock.cpp:333-364)
  auto InvDt = o->fluid.InvDt;
  real dt;
  DataBlock& d = o->data;
  idefix_reduce("Timestep_reduction", d.beg[KDIR], d.end[KDIR], d.beg[JDIR], d.end[JDIR],
                d.beg[IDIR], d.end[IDIR],
                KOKKOS_LAMBDA(int k, int j, int i, real& dtmin) {
                  dtmin = FMIN(ONE_F / InvDt(k, j, i), dtmin);
                },
                Kokkos::Min<real>(dt));
  return dt;
}

double ofx_check_divb(ofx* o) { return o->fluid.CheckDivB(); }
// Fluid::CheckNan counting part (checkNan.hpp:17-45), restated: its report
// path needs the host mirror classes
long ofx_check_nan(ofx* o) {
  DataBlock& d = o->data;
  auto Vc = o->fluid.Vc;
  auto Vs = o->fluid.Vs;
  long n = 0;
  for (int v = 0; v < Phys::nvar; v++)
    for (int k = d.beg[KDIR]; k < d.end[KDIR]; k++)
      for (int j = d.beg[JDIR]; j < d.end[JDIR]; j++)
        for (int i = d.beg[IDIR]; i < d.end[IDIR]; i++)
          if (std::isnan(Vc(v, k, j, i))) n++;
  for (int c = 0; c < DIMENSIONS; c++)
    for (int k = d.beg[KDIR]; k < d.end[KDIR] + KOFFSET; k++)
      for (int j = d.beg[JDIR]; j < d.end[JDIR] + JOFFSET; j++)
        for (int i = d.beg[IDIR]; i < d.end[IDIR] + IOFFSET; i++)
          if (std::isnan(Vs(c, k, j, i))) n++;
  return n;
}

int ofx_cycle(ofx* o) {  // TimeIntegrator::Cycle (timeIntegrator.cpp:246-414)
  real wc[2] = {0, 0}, w0[2] = {0, 0};
  if (o->nstages == 2) {
    wc[0] = 0.5;
    w0[0] = 0.5;
  }
  if (o->nstages == 3) {
    wc[0] = 0.25;
    w0[0] = 0.75;
    wc[1] = 2.0 / 3.0;
    w0[1] = 1.0 / 3.0;
  }
  try {
    if (o->log_period > 0 && o->ncycles % o->log_period == 0) {
      if (o->fluid.CheckDivB() > o->maxdivb) return OFX_ERR_DIVB;
    }
    const real t0 = o->t;
    real newdt = 0;
    ofx_reset_stage(o);
    for (int stage = 0; stage < o->nstages; stage++) {
      ofx_set_boundaries(o);
      ofx_prim_to_cons(o);
      if (o->nstages > 1 && stage == 0) {
        std::memcpy(o->Uc0.data(), o->fluid.Uc.data(), sizeof(double) * o->Uc0.size());
        std::memcpy(o->Vs0.data(), o->fluid.Vs.data(), sizeof(double) * o->Vs0.size());
      }
      ofx_evolve_stage(o, o->t, o->dt);
      o->t += o->dt;
      if (o->check_nan_period > 0 && o->ncycles % o->check_nan_period == 0) {
        if (ofx_check_nan(o) > 0) return OFX_ERR_NAN;
      }
      if (stage == 0) newdt = o->cfl * ofx_compute_timestep(o);
      if (stage > 0) {  // StateContainer::AddAndStore (stateContainer.cpp:75-104)
        const real wcs = wc[stage - 1], w0s = w0[stage - 1];
        for (size_t a = 0; a < o->Uc0.size(); a++)
          o->fluid.Uc.data()[a] = wcs * o->fluid.Uc.data()[a] + w0s * o->Uc0.data()[a];
        for (size_t a = 0; a < o->Vs0.size(); a++)
          o->fluid.Vs.data()[a] = wcs * o->fluid.Vs.data()[a] + w0s * o->Vs0.data()[a];
        o->t = wcs * o->t + w0s * t0;
      }
      ofx_cons_to_prim(o);
    }
    o->t = t0 + o->dt;
    if (newdt > o->cflmax * o->dt) {
      o->dt = o->cflmax * o->dt;
    } else {
      if (o->ncycles == 0 && newdt < 0.5 * o->dt) return OFX_ERR_FIRST_DT;
      o->dt = newdt;
    }
    if (o->dt < 1e-15) return OFX_ERR_DT_SMALL;
    o->ncycles++;
  } catch (const OfxRefError& e) {
    std::fprintf(stderr, "reference harness: %s\n", e.msg.c_str());
    return OFX_ERR_CONFIG;
  }
  return OFX_OK;
}

int ofx_run(ofx* o, double tstop, long max_cycles) {  // main.cpp:190-225
  long done = 0;
  while (true) {
    if (tstop >= 0 && !(o->t < tstop)) break;
    if (max_cycles >= 0 && done >= max_cycles) break;
    if (tstop >= 0 && tstop - o->t < o->dt) o->dt = tstop - o->t;
    int st = ofx_cycle(o);
    if (st) return st;
    done++;
  }
  return OFX_OK;
}

}  // extern "C"
