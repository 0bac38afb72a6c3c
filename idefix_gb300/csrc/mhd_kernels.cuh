// Kernels of one Runge-Kutta stage of the ideal-MHD Godunov step on a
// Cartesian block (periodic, reflective or outflow boundaries): FP64,
// bit-identical to the reference, or mixed precision (T = float).
//
// Device state keeps the reference layout (LayoutRight, ghost zones,
// face arrays padded by one in every active dimension) so that the C-ABI
// moves host arrays in and out unchanged:
//   Vc[nvar][nt2][nt1][nt0]   Vs[D][ntv2][ntv1][ntv0]
//
// Stage = fill_faces -> stage_begin -> sweep x, y(, z) -> ct_corner ->
// ct_faces -> stage_end.  Each face's Riemann problem is solved once and
// each cell's reconstruction is evaluated once per direction; fluxes never
// leave the registers of the thread that marches the column.
#pragma once
#include <cstdint>

#include "fpconv.cuh"
#include "mhd_math.cuh"

namespace idfx {

enum EmfMode { kEmfContact = 0, kEmfArithmetic = 1, kEmfUct0 = 2, kEmfUctHll = 3, kEmfUctHlld = 4 };
enum Status {
  kOk = 0,
  kErrConfig = 1,
  kErrNan = 2,
  kErrDivB = 3,
  kErrDtSmall = 4,
  kErrFirstDt = 5,
  kErrCuda = 6,
  kErrState = 7
};

// Geometry and scheme of one block (passed by value to every kernel).
struct Geo {
  int D, ng, order, solver, emf, nstages;
  int n[3], nt[3], ntv[3], beg[3], end[3];
  long long ncell, nface;
  long long s[3];   // cell strides
  long long fs[3];  // face strides
  double dx[3];
  double A[3];  // face areas (makeGeometry.cpp:146-147,178-179,201-202)
  double gamma, gm1;
  int ext;  // perpendicular extension of the flux sweeps for CT
  double shock_smoothing;  // [Hydro] shockFlattening value (flags in Fields::shock)
  double rgm1;    // RN(1 / gm1), for the FP64 Riemann solvers
  double rdx[3];  // RN(1 / dx[d]), for the InvDt quotient
  double l3b[3], l3y[3];  // LimO3: (0.1 dx[d])^2 and RN(1 / that)
  int bc[3][2];  // boundary type per direction and side (IDFX_BC_*: 0 periodic)
  int nonper;    // some direction is not periodic: ghosts filled by k_bc_* first
};

// Device-resident time-integrator control block.
struct Ctl {
  double t, dt, t0, tstop;
  double dtdV;        // dt / dV
  double dtdx[3];     // dt / dx[d]
  double cfl, cflmax, maxdivb;
  unsigned long long invdt_max_bits;  // max over active cells of InvDt (stage 0)
  unsigned long long divb_bits;       // max of the divB estimator
  unsigned long long nan_count;
  long long ncycles;
  int done;    // 1: every kernel returns at entry
  int status;  // Status
  int uc_fresh;  // 1: Uc (active cells) is the state the last stage end left
                 // and Vc was derived from it; 0 after any write from outside
};

// The EMF buffers (face EMFs ezi..eyk, upwind weights sv*, cell EMFs Ex*,
// corner EMFs ex/ey/ez, uct_hll(d) weights aL..dR) hold FP64 values on the
// FP64 path and FP32 values on the mixed path, in the same storage (emf<E>).
struct Fields {
  double *Vc, *Uc, *Uc0, *Vs, *Vs0, *InvDt;
  double *ezi, *ezj, *exj, *exk, *eyi, *eyk;
  double *svx, *svy, *svz;
  double *Ex1, *Ex2, *Ex3;
  double *ex, *ey, *ez;
  double *aL[3], *aR[3], *dL[3], *dR[3];
  float* Vc32;  // FP32 copy of Vc read by the mixed-precision sweeps (else null)
  unsigned char* shock;  // FlagShock per cell when shock flattening is on (else null)
};

// an EMF buffer in the arithmetic type of its producer
template <typename E>
__device__ __forceinline__ E* emf(double* p) {
  return reinterpret_cast<E*>(p);
}
template <typename E>
__device__ __forceinline__ const E* emf(const double* p) {
  return reinterpret_cast<const E*>(p);
}
// FP32 <-> FP64 on the integer pipe (fpconv.cuh); identity for doubles
template <typename T>
__device__ __forceinline__ double to_f64(T x) {
  if constexpr (sizeof(T) == 4) {
    return f2d_exact(x);
  } else {
    return x;
  }
}
template <typename T>
__device__ __forceinline__ T from_f64(double x) {
  if constexpr (sizeof(T) == 4) {
    return d2f_rn(x);
  } else {
    return x;
  }
}

__device__ __forceinline__ long long cidx(const Geo& g, int k, int j, int i) {
  return ((long long)k * g.nt[1] + j) * g.nt[0] + i;
}
__device__ __forceinline__ long long fidx(const Geo& g, int k, int j, int i) {
  return ((long long)k * g.ntv[1] + j) * g.ntv[0] + i;
}
// periodic image of a ghost index (boundary.hpp:588-606); n active cells
__device__ __forceinline__ int wrap(int i, int g, int n) { return g + (i + g * (n - 1)) % n; }

// non-negative doubles order like their bit patterns
__device__ __forceinline__ void atomic_max_pos(unsigned long long* p, double v) {
  if (!(v >= 0.0)) return;  // NaN ignored, like fmin/fmax in the reference reduction
  atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// hint: bring the line holding p into L2 (no register, no fault)
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
constexpr int kPrefetch = 4;  // steps ahead of the FP32 march

// ---------------------------------------------------------------------------
// Ghost faces of Vs (Boundary::EnforcePeriodic on Vs, boundary.hpp:608-670),
// plus the Runge-Kutta "begin" copy of the active faces at stage 0.
// One thread per location of the padded face box of one component.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void d_fill_faces(const Geo& g, const Fields& f, const Ctl* ctl, int save_begin, dim3 bid) {
  if (ctl->done) return;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const int comp = bid.y;
  if (tid >= g.nface) return;
  int i = (int)(tid % g.ntv[0]);
  long long r = tid / g.ntv[0];
  int j = (int)(r % g.ntv[1]);
  int k = (int)(r / g.ntv[1]);
  const int idx3[3] = {i, j, k};
  int src[3] = {i, j, k};
  bool ghost = false;
  for (int d = 0; d < D; d++) {
    const int v = idx3[d];
    const int hi = (d == comp) ? g.end[d] : g.end[d] - 1;  // last evolved face / cell
    if (d != comp && v == g.nt[d]) return;                 // padding, never used
    if (v < g.beg[d] || v > hi) {
      ghost = true;
      src[d] = wrap(v, g.ng, g.n[d]);
    }
  }
  double* vs = f.Vs + (long long)comp * g.nface;
  const long long fi = fidx(g, k, j, i);
  if (ghost) {
    if (!g.nonper) vs[fi] = vs[fidx(g, src[2], src[1], src[0])];
  } else if (save_begin) {
    f.Vs0[(long long)comp * g.nface + fi] = vs[fi];
  }
}

template <int D>
__global__ void k_fill_faces(Geo g, Fields f, const Ctl* ctl, int save_begin) {
  d_fill_faces<D>(g, f, ctl, save_begin, blockIdx);
}

// The ghost faces alone (periodic blocks, when no Runge-Kutta begin copy is
// due here: later stages, or a first stage whose copy the previous cycle's
// last face update wrote): the two ghost slabs of direction dir for
// component comp, bid.y = comp * D + dir, each over the full face box of the
// other two directions.  Every source is an active face (wrapped in every
// ghost direction, as k_fill_faces wraps), so no thread reads what another
// writes; faces in two slabs get the same value from both.
template <int D>
__device__ __forceinline__ void d_fill_face_ghosts(const Geo& g, const Fields& f, const Ctl* ctl, dim3 bid) {
  if (ctl->done) return;
  const int comp = (int)bid.y / D, dir = (int)bid.y % D;
  const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;
  int ext[3];  // the face box of component comp without its padding
  for (int d = 0; d < 3; d++) ext[d] = (d < D) ? (d == comp ? g.nt[d] + 1 : g.nt[d]) : 1;
  const long long per_side = (long long)g.ng * ext[a] * ext[b];
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  if (tid >= 2 * per_side) return;
  const int side = (int)(tid / per_side);
  long long r = tid % per_side;
  const int layer = (int)(r % g.ng);
  r /= g.ng;
  int idx[3];
  idx[a] = (int)(r % ext[a]);
  idx[b] = (int)(r / ext[a]);
  // right ghosts start past the last evolved face (end along comp, end - 1 across)
  idx[dir] = side ? g.end[dir] + (dir == comp ? 1 : 0) + layer : layer;
  int src[3] = {idx[0], idx[1], idx[2]};
  for (int d = 0; d < D; d++) {
    const int hi = (d == comp) ? g.end[d] : g.end[d] - 1;
    if (idx[d] < g.beg[d] || idx[d] > hi) src[d] = wrap(idx[d], g.ng, g.n[d]);
  }
  double* vs = f.Vs + (long long)comp * g.nface;
  vs[fidx(g, idx[2], idx[1], idx[0])] = vs[fidx(g, src[2], src[1], src[0])];
}

template <int D>
__global__ void k_fill_face_ghosts(Geo g, Fields f, const Ctl* ctl) {
  d_fill_face_ghosts<D>(g, f, ctl, blockIdx);
}

// ---------------------------------------------------------------------------
// Stage begin: ghost cells of Vc (periodic image), cell-centred field from
// the faces (ReconstructVcField, boundary.hpp:388-404), conservative state of
// the active cells (ConvertPrimToCons), RK begin copy, and the cell-centred
// EMF E = -v x B used by uct_contact / uct0 (calcCornerEmf.hpp:84-126).
// ---------------------------------------------------------------------------
// kSbKeepCons (mixed path): while Ctl::uc_fresh says that the conserved
// state of the active cells is the one the previous stage end left (Vc was
// derived from it), it is kept instead of being rebuilt from Vc; with
// kSbSaveBegin it is copied to Uc0.
enum { kSbCons = 1, kSbSaveBegin = 2, kSbCellEmf = 4, kSbKeepCons = 8 };

// the cell-centred EMF E = -v x B from the primitives W (in the EMF type)
template <int D, typename E>
__device__ __forceinline__ void cell_emf_store(const Fields& f, long long c, const E* W) {
  using v = Var<D>;
  const E vx1 = W[v::MX1], vx2 = W[v::MX2];
  const E Bx1 = W[v::BX1], Bx2 = W[v::BX2];
  if constexpr (D == 3) {
    const E vx3 = W[v::MX3], Bx3 = W[v::BX3];
    emf<E>(f.Ex1)[c] = (vx3 * Bx2 - vx2 * Bx3);
    emf<E>(f.Ex2)[c] = (vx1 * Bx3 - vx3 * Bx1);
  }
  emf<E>(f.Ex3)[c] = (vx2 * Bx1 - vx1 * Bx2);
}

// the primitives of cell c in the EMF type, their FP32 copy for the
// mixed-precision sweeps and the cell EMF
template <int D, typename E>
__device__ __forceinline__ void cell_outputs(const Fields& f, const Geo& g, long long c, const double* V,
                                             bool cell_emf) {
  constexpr int NV = Var<D>::NV;
  E W[NV];
#pragma unroll
  for (int n = 0; n < NV; n++) W[n] = from_f64<E>(V[n]);
  if (cell_emf) cell_emf_store<D, E>(f, c, W);
  if (f.Vc32) {  // mixed precision: the sweeps read the primitives in FP32
#pragma unroll
    for (int n = 0; n < NV; n++) f.Vc32[n * g.ncell + c] = (sizeof(E) == 4) ? (float)W[n] : d2f_rn(V[n]);
  }
}

// E: type of the EMF buffers (float on the mixed path: the cell EMF is then
// computed in FP32 from the FP32 primitives that the sweeps read)
template <int D, typename E = double>
__device__ __forceinline__ void stage_begin_cell(const Geo& g, const Fields& f, const Ctl* ctl, int flags, int i,
                                                 int j, int k) {
  using v = Var<D>;
  constexpr int NV = v::NV;
  const long long c = cidx(g, k, j, i);
  int src[3] = {i, j, k};
  bool ghost = false;
  const int idx3[3] = {i, j, k};
  for (int d = 0; d < D; d++) {
    if (idx3[d] < g.beg[d] || idx3[d] >= g.end[d]) {
      ghost = true;
      if (!g.nonper) src[d] = wrap(idx3[d], g.ng, g.n[d]);
    }
  }
  const bool copy = ghost && !g.nonper;  // else the ghosts are already filled
  double V[NV];
  const long long cs = cidx(g, src[2], src[1], src[0]);
#pragma unroll
  for (int n = 0; n < v::BX1; n++) V[n] = f.Vc[n * g.ncell + cs];
  const long long fc = fidx(g, k, j, i);
#pragma unroll
  for (int d = 0; d < D; d++) {
    const double* vs = f.Vs + d * g.nface;
    V[v::BX1 + d] = 0.5 * (vs[fc] + vs[fc + g.fs[d]]);
  }
  if (copy) {
#pragma unroll
    for (int n = 0; n < v::BX1; n++) f.Vc[n * g.ncell + c] = V[n];
  }
#pragma unroll
  for (int d = 0; d < D; d++) f.Vc[(v::BX1 + d) * g.ncell + c] = V[v::BX1 + d];
  const bool keep = (flags & kSbKeepCons) && ctl->uc_fresh;
  if (!ghost && !keep && (flags & kSbCons)) {
    double U[NV];
    prim_to_cons<D, true>(g.gm1, U, V);
#pragma unroll
    for (int n = 0; n < NV; n++) f.Uc[n * g.ncell + c] = U[n];
    if (flags & kSbSaveBegin) {
#pragma unroll
      for (int n = 0; n < NV; n++) f.Uc0[n * g.ncell + c] = U[n];
    }
  } else if (!ghost && keep && (flags & kSbSaveBegin)) {
    // the Runge-Kutta combination reads the non-field variables of Uc0
#pragma unroll
    for (int n = 0; n < v::BX1; n++) f.Uc0[n * g.ncell + c] = f.Uc[n * g.ncell + c];
  }
  cell_outputs<D, E>(f, g, c, V, (flags & kSbCellEmf) != 0);
}

template <int D, typename E = double>
__device__ __forceinline__ void d_stage_begin(const Geo& g, const Fields& f, const Ctl* ctl, int flags, dim3 bid) {
  if (ctl->done) return;
  const long long c = (long long)bid.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const int i = (int)(c % g.nt[0]);
  const long long r = c / g.nt[0];
  const int j = (int)(r % g.nt[1]);
  const int k = (int)(r / g.nt[1]);
  stage_begin_cell<D, E>(g, f, ctl, flags, i, j, k);
}

// Stage begin of the ghost cells only (periodic blocks, mixed path, when the
// previous stage end left Uc, Vc, the FP32 primitives and the cell EMF of
// every active cell): the two ghost slabs of direction bid.y, each over the
// full extent of the other two directions (cells in two slabs get the same
// values from both).
template <int D, typename E = double>
__device__ __forceinline__ void d_stage_ghosts(const Geo& g, const Fields& f, const Ctl* ctl, int flags, dim3 bid) {
  if (ctl->done) return;
  const int dir = bid.y;
  if (dir >= D) return;
  const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long per_side = (long long)g.ng * g.nt[a] * g.nt[b];
  if (tid >= 2 * per_side) return;
  const int side = (int)(tid / per_side);
  long long r = tid % per_side;
  const int layer = (int)(r % g.ng);
  r /= g.ng;
  const int ia = (int)(r % g.nt[a]);
  const int ib = (int)(r / g.nt[a]);
  int idx[3];
  idx[dir] = side ? g.end[dir] + layer : layer;
  idx[a] = ia;
  idx[b] = ib;
  stage_begin_cell<D, E>(g, f, ctl, flags, idx[0], idx[1], idx[2]);
}

template <int D, typename E = double>
__global__ void k_stage_ghosts(Geo g, Fields f, const Ctl* ctl, int flags) {
  d_stage_ghosts<D, E>(g, f, ctl, flags, blockIdx);
}

template <int D, typename E = double>
__global__ void k_stage_begin(Geo g, Fields f, const Ctl* ctl, int flags) {
  d_stage_begin<D, E>(g, f, ctl, flags, blockIdx);
}

// ---------------------------------------------------------------------------
// Non-periodic blocks: Boundary::SetBoundaries (boundary.hpp:240-280) one
// direction after the other, each direction's pass reading what the passes
// of the previous directions wrote (its loops span their ghosts too):
//   k_bc_slab(dir)     ghost cells of the non-field variables and ghost faces
//                      (both sides; boundary.hpp:575-809, loop ranges of
//                      BoundaryForAll / BoundaryForX?s, boundary.hpp:971-1100)
//   k_normal_field(dir) the normal field in the ghost faces of a reflective or
//                      outflow direction from div B = 0, marching outwards
//                      (ReconstructNormalField, boundary.hpp:408-532)
// then fill_faces / stage_begin run without the periodic copy.  The cell-
// centred field of the ghosts is not copied: stage_begin rebuilds it from the
// faces everywhere (ReconstructVcField, boundary.hpp:388-404).
// ---------------------------------------------------------------------------
// source index of ghost idx along a direction: periodic image, mirror
// (2 ibound - i - 1) or the last active cell (boundary.hpp:582-600, 687-689,
// 750-752); n active cells, side 0 left / 1 right
__device__ __forceinline__ int bc_src(int type, int idx, int ng, int n, int side) {
  if (type == 0) return wrap(idx, ng, n);
  if (type == 1) return 2 * (ng + side * n) - idx - 1;
  return ng + side * (n - 1);
}

// One thread per location of the two ghost slabs of dir (side, depth, and the
// full extent of the two other directions); blockIdx.y = 0 the cells, 1 + c
// the faces of component c.
template <int D>
__device__ __forceinline__ void d_bc_slab(const Geo& g, const Fields& f, const Ctl* ctl, int dir, dim3 bid) {
  if (ctl->done) return;
  using v = Var<D>;
  const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;  // the two other directions
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long per_side = (long long)g.ng * g.ntv[a] * g.ntv[b];
  if (tid >= 2 * per_side) return;
  const int side = (int)(tid / per_side);
  long long r = tid - side * per_side;
  const int depth = (int)(r % g.ng);
  r /= g.ng;
  const int ia = (int)(r % g.ntv[a]);
  const int ib = (int)(r / g.ntv[a]);
  const int type = g.bc[dir][side];
  const int comp = (int)bid.y - 1;  // -1: cells
  // extents of the array along a and b (faces: one more along their own direction)
  const int ea = g.nt[a] + (comp == a ? 1 : 0), eb = g.nt[b] + (comp == b ? 1 : 0);
  if (ia >= ea || ib >= eb) return;
  // along dir: ghosts [0, ng) on the left; on the right [ng + n, 2 ng + n) for
  // cells and tangential faces, one further for the normal faces
  const int shift = (comp == dir) ? 1 : 0;
  if (comp == dir && type != 0) return;  // rebuilt by k_normal_field
  const int id = side ? g.ng + g.n[dir] + shift + depth : depth;
  const int is = bc_src(type, id, g.ng, g.n[dir], side);
  int dst[3], src[3];
  dst[dir] = id;
  src[dir] = is;
  dst[a] = src[a] = ia;
  dst[b] = src[b] = ib;
  if (comp < 0) {
    const long long cd = cidx(g, dst[2], dst[1], dst[0]), cs = cidx(g, src[2], src[1], src[0]);
    const double sg = (double)(1 - 2 * side);
#pragma unroll
    for (int n = 0; n < v::BX1; n++) {
      const double x = f.Vc[n * g.ncell + cs];
      double y = x;
      if (type == 1) {
        if (n == v::MX1 + dir) y = -x;  // only the normal velocity: no field here
      } else if (type == 2) {
        if (n == v::MX1 + dir && sg * x >= 0.0) y = 0.0;  // no inflow (boundary.hpp:757-762)
      }
      f.Vc[n * g.ncell + cd] = y;
    }
  } else {
    double* vs = f.Vs + (long long)comp * g.nface;
    const double x = vs[fidx(g, src[2], src[1], src[0])];
    vs[fidx(g, dst[2], dst[1], dst[0])] = (type == 1) ? -x : x;
  }
}

template <int D>
__global__ void k_bc_slab(Geo g, Fields f, const Ctl* ctl, int dir) {
  d_bc_slab<D>(g, f, ctl, dir, blockIdx);
}

// One thread per line along dir (all locations of the two other directions);
// the recurrence runs outwards from the boundary face, each step reading the
// face it wrote before.  Face areas are uniform on a Cartesian grid.
template <int D>
__device__ __forceinline__ void d_normal_field(const Geo& g, const Fields& f, const Ctl* ctl, int dir, dim3 bid) {
  if (ctl->done) return;
  const int a = (dir == 0) ? 1 : 0, b = (dir == 2) ? 1 : 2;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)g.nt[a] * g.nt[b]) return;
  const int ia = (int)(tid % g.nt[a]), ib = (int)(tid / g.nt[a]);
  const bool left = g.bc[dir][0] != 0, right = g.bc[dir][1] != 0;
  double* V1 = f.Vs;
  double* V2 = f.Vs + g.nface;
  double* V3 = f.Vs + 2 * g.nface;  // read only when D == 3
  const double A1 = g.A[0], A2 = g.A[1], A3 = g.A[2];
  const long long s0 = g.fs[0], s1 = g.fs[1], s2 = g.fs[2];
  const int nb = g.beg[dir] - 1, ne = g.end[dir], nt = g.nt[dir];
  if (dir == 0) {
    const int j = ia, k = ib;
    if (left)
      for (int i = nb; i >= 0; i--) {
        const long long q = fidx(g, k, j, i);
        double t = 0.0 + A2 * V2[q + s1] - A2 * V2[q];
        if constexpr (D == 3) t = t + A3 * V3[q + s2] - A3 * V3[q];
        V1[q] = 1.0 / A1 * (A1 * V1[q + s0] + (t));
      }
    if (right)
      for (int i = ne; i < nt; i++) {
        const long long q = fidx(g, k, j, i);
        double t = 0.0 + A2 * V2[q + s1] - A2 * V2[q];
        if constexpr (D == 3) t = t + A3 * V3[q + s2] - A3 * V3[q];
        V1[q + s0] = 1.0 / A1 * (A1 * V1[q] - (t));
      }
  } else if (dir == 1) {
    const int i = ia, k = ib;
    if (left)
      for (int j = nb; j >= 0; j--) {
        const long long q = fidx(g, k, j, i);
        double t = A1 * V1[q + s0] - A1 * V1[q];
        if constexpr (D == 3) t = t + 1 * (A3 * V3[q + s2] - A3 * V3[q]);
        V2[q] = 1.0 / A2 * (A2 * V2[q + s1] + (t));
      }
    if (right)
      for (int j = ne; j < nt; j++) {
        const long long q = fidx(g, k, j, i);
        double t = A1 * V1[q + s0] - A1 * V1[q];
        if constexpr (D == 3) t = t + 1 * (A3 * V3[q + s2] - A3 * V3[q]);
        V2[q + s1] = 1.0 / A2 * (A2 * V2[q] - (t));
      }
  } else if constexpr (D == 3) {
    const int i = ia, j = ib;
    if (left)
      for (int k = nb; k >= 0; k--) {
        const long long q = fidx(g, k, j, i);
        V3[q] = 1.0 / A3 * (A3 * V3[q + s2] + (A1 * V1[q + s0] - A1 * V1[q] + A2 * V2[q + s1] - A2 * V2[q]));
      }
    if (right)
      for (int k = ne; k < nt; k++) {
        const long long q = fidx(g, k, j, i);
        V3[q + s2] = 1.0 / A3 * (A3 * V3[q] - (A1 * V1[q + s0] - A1 * V1[q] + A2 * V2[q + s1] - A2 * V2[q]));
      }
  }
}

template <int D>
__global__ void k_normal_field(Geo g, Fields f, const Ctl* ctl, int dir) {
  d_normal_field<D>(g, f, ctl, dir, blockIdx);
}

// ---------------------------------------------------------------------------
// ShockFlattening::FindShock (shockFlattening.hpp:82-168, 185-201): a cell of
// [beg-1, end] is flagged when div v < 0 and the pressure jump across it
// exceeds smoothing x the smallest pressure of its stencil; the sweeps then
// give it the minmod slope.  One thread per cell of that range.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void d_find_shock(const Geo& g, const Fields& f, const Ctl* ctl, dim3 bid) {
  if (ctl->done) return;
  using v = Var<D>;
  const int m0 = g.n[0] + 2, m1 = g.n[1] + 2, m2 = (D == 3) ? g.n[2] + 2 : 1;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)m0 * m1 * m2) return;
  const int i = g.beg[0] - 1 + (int)(tid % m0);
  const int j = g.beg[1] - 1 + (int)((tid / m0) % m1);
  const int k = (D == 3) ? g.beg[2] - 1 + (int)(tid / ((long long)m0 * m1)) : 0;
  const long long c = cidx(g, k, j, i);
  const long long si = 1, sj = g.s[1], sk = g.s[2];
  const double* vx = f.Vc + v::MX1 * g.ncell;
  const double* vy = f.Vc + v::MX2 * g.ncell;
  const double* p = f.Vc + v::PRS * g.ncell;
  double divV = (vx[c + si] - vx[c - si]) / (2 * g.dx[0]) + (vy[c + sj] - vy[c - sj]) / (2 * g.dx[1]);
  if constexpr (D == 3) {
    const double* vz = f.Vc + v::MX3 * g.ncell;
    divV = divV + (vz[c + sk] - vz[c - sk]) / (2 * g.dx[2]);
  }
  unsigned char flag = 0;
  if (divV < 0.0) {
    double pmin = p[c];
    pmin = fmin(pmin, p[c + si]);
    pmin = fmin(pmin, p[c - si]);
    double gradP = fabs(p[c + si] - p[c - si]);
    pmin = fmin(pmin, p[c + sj]);
    pmin = fmin(pmin, p[c - sj]);
    gradP += fabs(p[c + sj] - p[c - sj]);
    if constexpr (D == 3) {
      pmin = fmin(pmin, p[c + sk]);
      pmin = fmin(pmin, p[c - sk]);
      gradP += fabs(p[c + sk] - p[c - sk]);
    }
    if (gradP > g.shock_smoothing * pmin) flag = 1;
  }
  f.shock[c] = flag;
}

template <int D>
__global__ void k_find_shock(Geo g, Fields f, const Ctl* ctl) {
  d_find_shock<D>(g, f, ctl, blockIdx);
}

// ---------------------------------------------------------------------------
// EMF side outputs of a face (storeFlux.hpp:14-208)
// ---------------------------------------------------------------------------
template <int D, int DIR, typename T>
__device__ __forceinline__ void store_emf(const Geo& g, const Fields& f, long long c,
                                          const RiemannOut<D, T>& r, const T* vL, const T* vR) {
  using d = Dir<D, DIR>;
  using vv = Var<D>;
  // the EMF buffers take the arithmetic type T of the sweep
  T st, sb;
  T *Et, *Eb, *SV;
  if constexpr (DIR == 0) {
    st = T(-1); sb = T(+1); Et = emf<T>(f.ezi); Eb = emf<T>(f.eyi); SV = emf<T>(f.svx);
  } else if constexpr (DIR == 1) {
    st = T(+1); sb = T(-1); Et = emf<T>(f.ezj); Eb = emf<T>(f.exj); SV = emf<T>(f.svy);
  } else {
    st = T(-1); sb = T(+1); Et = emf<T>(f.eyk); Eb = emf<T>(f.exk); SV = emf<T>(f.svz);
  }
  if (g.emf == kEmfContact || g.emf == kEmfArithmetic || g.emf == kEmfUct0) {
    Et[c] = st * r.F[d::BXt];
    if constexpr (D == 3) Eb[c] = sb * r.F[d::BXb];
    if (g.emf == kEmfContact) {
      T s = T(0.5);
      if (r.F[vv::RHO] > T(kEpsUctContact)) s = T(1);
      if (r.F[vv::RHO] < T(-kEpsUctContact)) s = T(0);
      SV[c] = s;
    }
    return;
  }
  T* aL = emf<T>(f.aL[DIR]);
  T* aR = emf<T>(f.aR[DIR]);
  T* dL = emf<T>(f.dL[DIR]);
  T* dR = emf<T>(f.dR[DIR]);
  const T sl = r.sl, sr = r.sr;
  if (g.emf == kEmfUctHll) {
    const T ar = fmax(T(0), sr);
    const T al = fmin(T(0), sl);
    const T scrh = rcp(ar - al);
    Et[c] = -st * (ar * vL[d::Xt] - al * vR[d::Xt]) * scrh;
    if constexpr (D == 3) Eb[c] = -sb * (ar * vL[d::Xb] - al * vR[d::Xb]) * scrh;
    aL[c] = ar * scrh;
    aR[c] = -al * scrh;
    const T dr = -al * ar * scrh;
    dR[c] = dr;
    dL[c] = dr;
    return;
  }
  // uct_hlld (K_StoreHLLD, energy branch)
  const T* uL = r.uL;
  const T* uR = r.uR;
  const T ptL = vL[vv::PRS] + half_b2<D>(vL);
  const T ptR = vR[vv::PRS] + half_b2<D>(vR);
  int revert_to_hll = 0;
  const T Bn = dv(sr * vR[d::BXn] - sl * vL[d::BXn], sr - sl);
  const T duL = sl - vL[d::Xn];
  const T duR = sr - vR[d::Xn];
  T scrh = rcp(duR * uR[vv::RHO] - duL * uL[vv::RHO]);
  const T Sc = (duR * uR[d::Xn] - duL * uL[d::Xn] - ptR + ptL) * scrh;
  const T usLRHO = dv(uL[vv::RHO] * duL, sl - Sc);
  const T usRRHO = dv(uR[vv::RHO] * duR, sr - Sc);
  const T sqrL = sqr(usLRHO);
  const T sqrR = sqr(usRRHO);
  const T SaL = Sc - dv(fabs(Bn), sqrL);
  const T SaR = Sc + dv(fabs(Bn), sqrR);
  if ((SaL - sl) < T(1e-4) * (Sc - sl)) revert_to_hll = 1;
  if ((SaR - sr) > T(-1e-4) * (sr - Sc)) revert_to_hll = 1;
  const T chiL = dv((vL[d::Xn] - Sc) * (sl - Sc), SaL + sl - T(2) * Sc);
  const T chiR = dv((vR[d::Xn] - Sc) * (sr - Sc), SaR + sr - T(2) * Sc);
  const T nuL = dv(SaL + sl, fabs(SaL) + fabs(sl));
  const T nuR = dv(SaR + sr, fabs(SaR) + fabs(sr));
  const T nuLR = dv(SaL + SaR, fabs(SaL) + fabs(SaR));
  T a_l, a_r, d_l, d_r;
  if (fabs(SaR - SaL) > T(1.e-9) * fabs(sr - sl)) {
    d_l = T(0.5) * (chiL * nuL - chiL * nuLR) + T(0.5) * (fabs(SaL) - nuLR * SaL);
    d_r = T(0.5) * (chiR * nuR - chiR * nuLR) + T(0.5) * (fabs(SaR) - nuLR * SaR);
    a_l = T(0.5) * (T(1) + nuLR);
    a_r = T(0.5) * (T(1) - nuLR);
  } else {
    d_l = T(0.5) * chiL * nuL + T(0.5) * fabs(SaL);
    d_r = T(0.5) * chiR * nuR + T(0.5) * fabs(SaR);
    a_l = T(0.5);
    a_r = T(0.5);
  }
  const T ar = fmax(T(0), sr);
  const T al = fmin(T(0), sl);
  scrh = rcp(ar - al);
  if (revert_to_hll) {
    a_l = ar * scrh;
    a_r = -al * scrh;
    d_r = -al * ar * scrh;
    d_l = d_r;
  }
  aL[c] = a_l;
  aR[c] = a_r;
  dL[c] = d_l;
  dR[c] = d_r;
  Et[c] = -st * (ar * vL[d::Xt] - al * vR[d::Xt]) * scrh;
  if constexpr (D == 3) Eb[c] = -sb * (ar * vL[d::Xb] - al * vR[d::Xb]) * scrh;
}

// ---------------------------------------------------------------------------
// Flux sweeps (RiemannSolver::CalcFlux<DIR> + Fluid_CorrectFluxFunctor +
// Fluid_CalcRHSFunctor, calcRightHandSide.hpp:84-195,333-550): each thread
// owns one column (a line of cells along DIR) and marches a segment of `seg`
// cells, keeping the reconstruction stencil, the left face state and the
// previous face flux in registers.  Every cell is reconstructed once and
// every face solved once (plus one face and two cells per segment).
// Thread index -> coordinate A (j for the x sweep, i otherwise); blockIdx.z
// -> coordinate B (k, or j for the z sweep); both include the CT extension.
// invdt: 0 = no InvDt work, 1 = first contribution of a cycle (InvDt was
// reset to 0), 2 = accumulate onto the stored InvDt.  last_dir: fold the
// completed InvDt into the device maximum used for the next dt.
// ---------------------------------------------------------------------------
constexpr int kTM = 64;

// T: arithmetic of the reconstruction and the Riemann solve (double: the
// bit-exact path; float: the mixed-precision path).  The state is read in
// FP64 and converted once per cell; the flux difference, the conserved
// update and InvDt are FP64 in both.
template <int D, int DIR, int ORDER, int SOLVER, typename T>
__device__ __forceinline__ void d_sweep_march(const Geo& g, const Fields& f, const Ctl* ctl, int invdt,
                                              int last_dir, int seg, dim3 bid) {
  if (ctl->done) return;
  using v = Var<D>;
  using dd = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int H = Recon<ORDER>::H;
  constexpr int W = 2 * H + 1;
  constexpr int A = (DIR == 0) ? 1 : 0;
  constexpr int B = (DIR == 2) ? 1 : 2;
  // FP32 sweeps are load-latency bound: issue the next step's loads before
  // the current step's arithmetic.  FP64 sweeps are FP64-issue bound and
  // keep their registers for the arithmetic.
  constexpr bool PF = (sizeof(T) == 4);
  // flattened column index over the (A, B) plane, CT extension included
  const int nA = g.n[A] + 2 * g.ext;
  const int nB = (D == 3) ? g.n[B] + 2 * g.ext : 1;
  const long long col = (long long)bid.x * kTM + threadIdx.x;
  if (col >= (long long)nA * nB) return;
  const int ca = g.beg[A] - g.ext + (int)(col % nA);
  const int cb = (D == 3) ? g.beg[B] - g.ext + (int)(col / nA) : 0;
  const int m0 = g.beg[DIR] + bid.y * seg;
  const int m1 = min(m0 + seg, g.end[DIR]);
  bool active_col = (ca >= g.beg[A] && ca < g.end[A]);
  if constexpr (D == 3) active_col = active_col && cb >= g.beg[B] && cb < g.end[B];
  int idx[3];
  idx[DIR] = m0;
  idx[A] = ca;
  idx[B] = cb;
  const long long sd = g.s[DIR];
  const long long fsd = g.fs[DIR];
  const long long c0 = cidx(g, idx[2], idx[1], idx[0]);  // cell m0 of this column
  const long long f0 = fidx(g, idx[2], idx[1], idx[0]);
  const double* vs = f.Vs + DIR * g.nface;
  const T dxd = (T)g.dx[DIR];
  const Recip l3{g.l3b[DIR], g.l3y[DIR]};
  const T gam = (T)g.gamma;
  T w[NV][W];
  T vrp[NV];            // right-face state of the previous cell
  T Fp[v::BX1];         // flux x A of the previous face
  T cp = T(0);          // cmax of the previous face
  T nx[NV];             // prefetched stencil value of the next step
  // primitives in the arithmetic type: the FP32 copy for the mixed path
  const T* vcT;
  if constexpr (sizeof(T) == 4) {
    vcT = f.Vc32;
  } else {
    vcT = f.Vc;
  }
  double nbn = 0.0;     // prefetched normal face field of the next face
  double nU[v::BX1];    // prefetched conserved state of the next cell to update
  double nI = 0.0;      // prefetched InvDt of that cell
  // prime the window with cells m0-1-H .. m0-2+H
#pragma unroll
  for (int n = 0; n < NV; n++) {
    if (n == dd::BXn) continue;
#pragma unroll
    for (int m = 0; m < W - 1; m++) w[n][m + 1] = vcT[n * g.ncell + c0 + (m - 1 - H) * sd];
    if constexpr (PF) nx[n] = vcT[n * g.ncell + c0 + (H - 1) * sd];
  }
  if constexpr (PF) nbn = vs[f0];
  const T dtdVT = (T)ctl->dtdV;
  const T areaT = (T)g.A[DIR];
  const T invdxT = T(1) / (T)g.dx[DIR];  // FP32 path only
  double run_max = 0.0;                  // max of InvDt over this thread's cells
  for (int c = m0 - 1; c <= m1; c++) {
    const long long cc = c0 + (long long)(c - m0) * sd;
    const bool more = c < m1;
    double curU[v::BX1];
    double curI = 0.0;
    if constexpr (!PF && DIR != 0) {
      // FP64: the same L2 prefetch along y and z, kPrefetch steps ahead (the
      // step's loads are otherwise issued right before their use; measured:
      // y and z sweeps 35.15 -> 34.90 ms per 256^3 cycle, an L1 prefetch
      // no better)
      if (c + kPrefetch + H + 1 < g.nt[DIR]) {
#pragma unroll
        for (int n = 0; n < NV; n++)
          if (n != dd::BXn) prefetch_l2(vcT + n * g.ncell + cc + (kPrefetch + H + 1) * sd);
        prefetch_l2(vs + f0 + (long long)(c + 1 + kPrefetch - m0) * fsd);
        if (active_col) {
#pragma unroll
          for (int n = 0; n < v::BX1; n++) prefetch_l2(f.Uc + n * g.ncell + cc + kPrefetch * sd);
        }
      }
    }
    if constexpr (PF) {
      // L2 prefetch kPrefetch steps ahead along y (measured: +11 % on the
      // FP32 y sweep; along x consecutive steps share cache lines and the
      // extra requests cost more than they save, along z no gain); only
      // in-bounds cells of the ghosted arrays are touched
      if (DIR == 1 && c + kPrefetch + H + 1 < g.nt[DIR]) {
#pragma unroll
        for (int n = 0; n < NV; n++)
          if (n != dd::BXn) prefetch_l2(vcT + n * g.ncell + cc + (kPrefetch + H + 1) * sd);
        prefetch_l2(vs + f0 + (long long)(c + 1 + kPrefetch - m0) * fsd);
        if (active_col) {
#pragma unroll
          for (int n = 0; n < v::BX1; n++) prefetch_l2(f.Uc + n * g.ncell + cc + kPrefetch * sd);
        }
      }
      // conserved state (and InvDt) of cell c-1, loaded one step ago
      if (active_col && c > m0) {
#pragma unroll
        for (int n = 0; n < v::BX1; n++) curU[n] = nU[n];
        curI = nI;
      }
      if (active_col && c >= m0 && more) {
#pragma unroll
        for (int n = 0; n < v::BX1; n++) nU[n] = f.Uc[n * g.ncell + cc];
        if (invdt == 2) nI = f.InvDt[cc];
      }
    }
    T vl[NV], vr[NV];
    const bool shk = f.shock && f.shock[cc];  // shock flag of cell c
#pragma unroll
    for (int n = 0; n < NV; n++) {
      if (n == dd::BXn) continue;
#pragma unroll
      for (int m = 0; m < W - 1; m++) w[n][m] = w[n][m + 1];
      if constexpr (PF) {
        w[n][W - 1] = nx[n];
        if (more) nx[n] = vcT[n * g.ncell + cc + (H + 1) * sd];
      } else {
        w[n][W - 1] = vcT[n * g.ncell + cc + H * sd];
      }
      // FP64: odd variables' limiter quotient on the integer pipe
      Recon<ORDER>::cell(w[n], dxd, n == v::RHO || n == v::PRS, vl[n], vr[n], shk, l3,
                         sizeof(T) == 8 && (n & 1));
    }
    if (c >= m0) {
      T vL[NV], vR[NV];
#pragma unroll
      for (int n = 0; n < NV; n++) {
        if (n == dd::BXn) continue;
        vL[n] = vrp[n];
        vR[n] = vl[n];
      }
      T bn;
      if constexpr (PF) {
        bn = from_f64<T>(nbn);
        if (more) nbn = vs[f0 + (long long)(c + 1 - m0) * fsd];
      } else {
        bn = from_f64<T>(vs[f0 + (long long)(c - m0) * fsd]);
      }
      vL[dd::BXn] = bn;
      vR[dd::BXn] = bn;
      RiemannOut<D, T> r;
      riemann<D, DIR, SOLVER>(gam, (T)g.rgm1, vL, vR, r);
      store_emf<D, DIR>(g, f, cc, r, vL, vR);
      if (active_col) {
        // flux x area and the flux difference in the arithmetic type T; the
        // conserved state accumulates in FP64 (for T = double this is the
        // reference's expression, operation for operation)
        T FA[v::BX1];
#pragma unroll
        for (int n = 0; n < v::BX1; n++) FA[n] = r.F[n] * areaT;
        if (c > m0) {
          const long long cu = cc - sd;  // cell c-1
#pragma unroll
          for (int n = 0; n < v::BX1; n++) {
            const T rhs = -dtdVT * (FA[n] - Fp[n]);
            const double u = PF ? curU[n] : f.Uc[n * g.ncell + cu];
            f.Uc[n * g.ncell + cu] = u + to_f64(rhs);
          }
          if (invdt) {
            const double prev = (invdt == 1) ? 0.0 : (PF ? curI : f.InvDt[cu]);
            double inv;
            if constexpr (sizeof(T) == 8) {
              inv = prev + div_r(0.5 * (r.cmax + cp), Recip{g.dx[DIR], g.rdx[DIR]});
            } else {
              inv = prev + to_f64(T(0.5) * (r.cmax + cp) * invdxT);
            }
            f.InvDt[cu] = inv;
            if (inv > run_max) run_max = inv;  // NaN never compares greater
          }
        }
#pragma unroll
        for (int n = 0; n < v::BX1; n++) Fp[n] = FA[n];
        cp = r.cmax;
      }
    }
#pragma unroll
    for (int n = 0; n < NV; n++) vrp[n] = vr[n];
  }
  // CFL maximum of the last direction: one atomic per thread, not per cell
  // (a per-cell atomic on one address serialises the whole z sweep)
  if (last_dir && invdt && active_col) atomic_max_pos((unsigned long long*)&((Ctl*)ctl)->invdt_max_bits, run_max);
}

// ---------------------------------------------------------------------------
// x sweep by warp chunks (FP32 path).  The march above gives every lane its
// own x row, so a warp's loads touch 32 rows: one sector each, reused over
// the next steps only while it survives in L1 - at 256^3 the FP32 x march
// runs from DRAM at a fraction of the y march's speed.  Here a warp owns one
// row and walks it in chunks of 32 consecutive cells: lane l holds cell
// base + 32 k + l, so every load and store of the warp is contiguous; the
// reconstruction stencil comes from the neighbouring lanes by shuffles (the
// previous and the next chunk stay in registers), lane l solves the face on
// the left of its cell and updates the cell on its left, and the values that
// cross a chunk boundary (the right state, flux and wave speed of the last
// lane) are carried to lane 0 of the next chunk.  Arithmetic per face and
// per cell is the march's, term for term.
// One warp per column (y, z incl. the CT extension); blocks of kXW warps.
// ---------------------------------------------------------------------------
constexpr int kXW = 4;

template <typename T>
__device__ __forceinline__ T lane_from(T cur, T other, int src, bool use_other) {
  const T a = __shfl_sync(0xffffffffu, cur, src & 31);
  const T b = __shfl_sync(0xffffffffu, other, src & 31);
  return use_other ? b : a;
}

template <int D, int ORDER, int SOLVER, typename T>
__device__ __forceinline__ void d_sweep_xwarp(const Geo& g, const Fields& f, const Ctl* ctl, int invdt, int last_dir,
                                              dim3 bid) {
  if (ctl->done) return;
  using v = Var<D>;
  using dd = Dir<D, 0>;
  constexpr int NV = v::NV;
  constexpr int H = Recon<ORDER>::H;
  static_assert(ORDER >= 1 && ORDER <= 4, "warp-chunk x sweep: reconstruction orders 1-4");
  const int lane = threadIdx.x & 31;
  const int nA = g.n[1] + 2 * g.ext;
  const int nB = (D == 3) ? g.n[2] + 2 * g.ext : 1;
  const long long col = (long long)bid.x * kXW + (threadIdx.x >> 5);
  if (col >= (long long)nA * nB) return;  // whole warp
  const int ca = g.beg[1] - g.ext + (int)(col % nA);
  const int cb = (D == 3) ? g.beg[2] - g.ext + (int)(col / nA) : 0;
  bool active_col = (ca >= g.beg[1] && ca < g.end[1]);
  if constexpr (D == 3) active_col = active_col && cb >= g.beg[2] && cb < g.end[2];
  const long long row = cidx(g, cb, ca, 0);   // cell (0, ca, cb)
  const long long frow = fidx(g, cb, ca, 0);  // x face (0, ca, cb)
  const double* vs = f.Vs;                    // x component
  const T* vcT;
  if constexpr (sizeof(T) == 4) {
    vcT = f.Vc32;
  } else {
    vcT = f.Vc;
  }
  const int nx = g.nt[0];
  const int beg = g.beg[0], end = g.end[0];
  const int base = beg - 1;  // first cell reconstructed (left state of face beg)
  const T gam = (T)g.gamma;
  const T dxd = (T)g.dx[0];
  const Recip l3{g.l3b[0], g.l3y[0]};
  const T dtdVT = (T)ctl->dtdV;
  const T areaT = (T)g.A[0];
  const T invdxT = T(1) / (T)g.dx[0];
  auto load = [&](int n, int i) -> T { return (i >= 0 && i < nx) ? vcT[n * g.ncell + row + i] : T(0); };
  T prv[NV], cur[NV], nxt[NV];
#pragma unroll
  for (int n = 0; n < NV; n++) {
    prv[n] = load(n, base - 32 + lane);
    cur[n] = load(n, base + lane);
    nxt[n] = load(n, base + 32 + lane);
  }
  // carried from lane 31 of the previous chunk
  T cvr[NV];
  T cFA[v::BX1];
  T ccp = T(0);
#pragma unroll
  for (int n = 0; n < NV; n++) cvr[n] = T(0);
#pragma unroll
  for (int n = 0; n < v::BX1; n++) cFA[n] = T(0);
  const int nchunks = (end - base + 1 + 31) / 32;  // cells base .. end
  double run_max = 0.0;
  // conserved state (and InvDt) of the cell this lane updates in a chunk,
  // loaded one chunk ahead: the update is the chunk's last step and its
  // loads would otherwise wait on memory right at the point of use
  auto upd = [&](int kk) { return base + 32 * kk + lane - 1; };  // cell updated in chunk kk
  auto upd_ok = [&](int kk) { const int u = upd(kk); return active_col && u >= beg && u < end; };
  double nU[v::BX1], nI = 0.0;
  if (upd_ok(0)) {
#pragma unroll
    for (int n = 0; n < v::BX1; n++) nU[n] = f.Uc[n * g.ncell + row + upd(0)];
    if (invdt == 2) nI = f.InvDt[row + upd(0)];
  }
  for (int k = 0; k < nchunks; k++) {
    const int i = base + 32 * k + lane;  // this lane's cell
    double cU[v::BX1], cI = nI;
#pragma unroll
    for (int n = 0; n < v::BX1; n++) cU[n] = nU[n];
    if (upd_ok(k + 1)) {
#pragma unroll
      for (int n = 0; n < v::BX1; n++) nU[n] = f.Uc[n * g.ncell + row + upd(k + 1)];
      if (invdt == 2) nI = f.InvDt[row + upd(k + 1)];
    }
    // reconstruction of cell i from the lanes around it
    T vl[NV], vr[NV];
    const bool shk = f.shock && i >= 0 && i < nx && f.shock[row + i];
#pragma unroll
    for (int n = 0; n < NV; n++) {
      if (n == dd::BXn) continue;
      T w[2 * H + 1];
#pragma unroll
      for (int m = -H; m <= H; m++) {
        const int src = lane + m;
        if (m == 0) {
          w[H] = cur[n];
        } else if (m < 0) {
          w[H + m] = lane_from(cur[n], prv[n], src, src < 0);
        } else {
          w[H + m] = lane_from(cur[n], nxt[n], src, src > 31);
        }
      }
      Recon<ORDER>::cell(w, dxd, n == v::RHO || n == v::PRS, vl[n], vr[n], shk, l3);
    }
    // face on the left of cell i: left state = right state of cell i-1
    T vL[NV], vR[NV];
#pragma unroll
    for (int n = 0; n < NV; n++) {
      if (n == dd::BXn) continue;
      const T up = __shfl_up_sync(0xffffffffu, vr[n], 1);
      vL[n] = lane == 0 ? cvr[n] : up;
      vR[n] = vl[n];
    }
    const bool face = (i >= beg && i <= end);
    const long long cc = row + i;
    T FA[v::BX1];
    T cm = T(0);
#pragma unroll
    for (int n = 0; n < v::BX1; n++) FA[n] = T(0);
    if (face) {
      const T bn = from_f64<T>(vs[frow + i]);
      vL[dd::BXn] = bn;
      vR[dd::BXn] = bn;
      RiemannOut<D, T> r;
      riemann<D, 0, SOLVER>(gam, (T)g.rgm1, vL, vR, r);
      store_emf<D, 0>(g, f, cc, r, vL, vR);
#pragma unroll
      for (int n = 0; n < v::BX1; n++) FA[n] = r.F[n] * areaT;
      cm = r.cmax;
    }
    // update of cell i-1 with the faces i-1 (left) and i (right)
    T FAp[v::BX1];
#pragma unroll
    for (int n = 0; n < v::BX1; n++) {
      const T up = __shfl_up_sync(0xffffffffu, FA[n], 1);
      FAp[n] = lane == 0 ? cFA[n] : up;
    }
    const T cpu = __shfl_up_sync(0xffffffffu, cm, 1);
    const T cp = lane == 0 ? ccp : cpu;
    if (active_col && face && i - 1 >= beg) {
      const long long cu = cc - 1;
#pragma unroll
      for (int n = 0; n < v::BX1; n++) {
        const T rhs = -dtdVT * (FA[n] - FAp[n]);
        f.Uc[n * g.ncell + cu] = cU[n] + to_f64(rhs);
      }
      if (invdt) {
        const double prev = (invdt == 1) ? 0.0 : cI;
        double inv;
        if constexpr (sizeof(T) == 8) {
          inv = prev + div_r(0.5 * (cm + cp), Recip{g.dx[0], g.rdx[0]});
        } else {
          inv = prev + to_f64(T(0.5) * (cm + cp) * invdxT);
        }
        f.InvDt[cu] = inv;
        if (inv > run_max) run_max = inv;
      }
    }
    // carry lane 31 to the next chunk and shift the register window
#pragma unroll
    for (int n = 0; n < NV; n++) cvr[n] = __shfl_sync(0xffffffffu, vr[n], 31);
#pragma unroll
    for (int n = 0; n < v::BX1; n++) cFA[n] = __shfl_sync(0xffffffffu, FA[n], 31);
    ccp = __shfl_sync(0xffffffffu, cm, 31);
#pragma unroll
    for (int n = 0; n < NV; n++) {
      prv[n] = cur[n];
      cur[n] = nxt[n];
      nxt[n] = load(n, base + 32 * (k + 2) + lane);
    }
  }
  if (last_dir && invdt && active_col) atomic_max_pos((unsigned long long*)&((Ctl*)ctl)->invdt_max_bits, run_max);
}

template <int D, int ORDER, int SOLVER, typename T>
__global__ void __launch_bounds__(32 * kXW, 5) k_sweep_xwarp(Geo g, Fields f, const Ctl* ctl, int invdt, int last_dir) {
  d_sweep_xwarp<D, ORDER, SOLVER, T>(g, f, ctl, invdt, last_dir, blockIdx);
}

// ---------------------------------------------------------------------------
// x sweep by warp chunks with bulk-copy staging (FP32 path).  The same
// arithmetic as d_sweep_xwarp, lane for lane; only the data movement
// differs: each warp keeps a ring of kXB chunk slots in shared memory and
// its lane 0 fetches whole chunks - the 32 FP32 primitives of every
// variable and the 32 FP64 conserved values of every hydro variable, each a
// contiguous row piece - with the bulk-copy engine (cp.async.bulk, tracked
// by one mbarrier per slot), kXB - 2 chunks ahead of the stencil.  Lanes read
// their stencil and their conserved state straight from the ring (no
// register window, no shuffles for the stencil).  Needs 16-byte aligned rows
// and arrays (nt0 a multiple of 4); the host falls back to d_sweep_xwarp
// otherwise.  Every wait is bounded: on a timeout the kernel records a CUDA
// error status, stops the cycle, waits (bounded) for its copies in flight
// and returns.
// ---------------------------------------------------------------------------
constexpr int kXB = 4;                                        // ring slots per warp
// shared memory per warp: FP32 primitives (nv), FP64 hydro state (nu),
// mbarriers; a multiple of 128 bytes so that every warp's ring (the bulk
// copies' destinations) stays 16-byte aligned
__host__ __device__ constexpr int xb_warp_bytes(int nv, int nu) {
  return (kXB * 32 * (nv * 4 + nu * 8) + kXB * 8 + 127) / 128 * 128;
}
static_assert(xb_warp_bytes(6, 4) % 128 == 0 && xb_warp_bytes(8, 5) % 128 == 0, "ring alignment");
static_assert((32 * 4) % 16 == 0 && (32 * 8) % 16 == 0, "slot alignment");
constexpr long long kXBSpin = 1ll << 22;                      // try_wait attempts before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  uint64_t gsrc;
  asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_done(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase of the given parity, at most `limit` try_wait attempts;
// false when it gave up
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kXBSpin) {
  for (long long it = 0; it < limit; it++)
    if (mbar_done(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// a bounded wait gave up: the stage reports a CUDA-side failure and the
// cycle stops (every later kernel returns at entry; the host maps the status)
__device__ __forceinline__ void report_wait_timeout(const Ctl* ctl) {
  ((Ctl*)ctl)->status = kErrCuda;
  ((Ctl*)ctl)->done = 1;
}

template <int D, int ORDER, int SOLVER, typename T>
__device__ __forceinline__ void d_sweep_xbulk(const Geo& g, const Fields& f, const Ctl* ctl, int invdt, int last_dir,
                                              dim3 bid, unsigned char* smem) {
  if (ctl->done) return;
  static_assert(sizeof(T) == 4, "bulk-staged x sweep: FP32 path");
  using v = Var<D>;
  using dd = Dir<D, 0>;
  constexpr int NV = v::NV;
  constexpr int NU = v::BX1;  // hydro variables updated by the sweep
  constexpr int H = Recon<ORDER>::H;
  constexpr int RING = 32 * kXB;
  static_assert(ORDER >= 1 && ORDER <= 4, "bulk-staged x sweep: reconstruction orders 1-4");
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int nA = g.n[1] + 2 * g.ext;
  const int nB = (D == 3) ? g.n[2] + 2 * g.ext : 1;
  const long long col = (long long)bid.x * kXW + w;
  if (col >= (long long)nA * nB) return;  // whole warp
  // this warp's ring: float vr[NV][RING], double ur[NU][RING], mbarriers[kXB]
  unsigned char* base_w = smem + (size_t)w * xb_warp_bytes(NV, NU);
  double* ur = reinterpret_cast<double*>(base_w);
  float* vr = reinterpret_cast<float*>(base_w + (size_t)NU * RING * 8);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base_w + (size_t)NU * RING * 8 + (size_t)NV * RING * 4);
  const int ca = g.beg[1] - g.ext + (int)(col % nA);
  const int cb = (D == 3) ? g.beg[2] - g.ext + (int)(col / nA) : 0;
  bool active_col = (ca >= g.beg[1] && ca < g.end[1]);
  if constexpr (D == 3) active_col = active_col && cb >= g.beg[2] && cb < g.end[2];
  const long long row = cidx(g, cb, ca, 0);
  const long long frow = fidx(g, cb, ca, 0);
  const double* vs = f.Vs;
  const float* vc = f.Vc32;
  const int nx = g.nt[0];
  const int beg = g.beg[0], end = g.end[0];
  const T gam = (T)g.gamma;
  const T dxd = (T)g.dx[0];
  const Recip l3{g.l3b[0], g.l3y[0]};
  const T dtdVT = (T)ctl->dtdV;
  const T areaT = (T)g.A[0];
  const T invdxT = T(1) / (T)g.dx[0];
  const int nchunks = (end + 1 + 31) / 32;        // chunks of cells 0 .. end
  const int last = min(nchunks, (nx - 1) / 32);    // last chunk with data the stencil may read
  // lane 0 fetches chunk c into slot c % kXB
  // bulk copies need 16-byte aligned addresses and sizes: with nt0 a
  // multiple of 4 (so ncell and every row start are) and 16-byte aligned
  // Vc32 and Uc, checked by the host before it launches this kernel, every
  // chunk's source is; the ring's slots are by construction (xb_warp_bytes)
  auto fetch = [&](int c) {
    uint64_t* b = bar + (c % kXB);
    const int ne = min(32, nx - 32 * c);          // a multiple of 4 (nt0 is)
    const int s = (c % kXB) * 32;
    mbar_expect(b, (uint32_t)ne * (NV * 4 + NU * 8));
#pragma unroll
    for (int n = 0; n < NV; n++)
      bulk_to_smem(vr + (size_t)n * RING + s, vc + n * g.ncell + row + 32 * c, (uint32_t)ne * 4, b);
#pragma unroll
    for (int n = 0; n < NU; n++)
      bulk_to_smem(ur + (size_t)n * RING + s, f.Uc + n * g.ncell + row + 32 * c, (uint32_t)ne * 8, b);
  };
  if (lane == 0) {
    for (int s = 0; s < kXB; s++) mbar_init(bar + s);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int c = 0; c <= min(last, kXB - 1); c++) fetch(c);
  }
  __syncwarp();
  int fetched = min(last, kXB - 1);  // chunks 0 .. fetched are issued
  int waited = -1;                   // chunks 0 .. waited have landed
  bool ok = true;
  auto wait_upto = [&](int c) {
    c = min(c, last);
    while (ok && waited < c) {
      const int q = waited + 1;
      ok = mbar_wait(bar + (q % kXB), (uint32_t)((q / kXB) & 1));
      if (ok) waited = q;
    }
  };
  auto V = [&](int n, int i) -> T { return vr[(size_t)n * RING + ((i + RING) % RING)]; };
  auto U = [&](int n, int i) -> double { return ur[(size_t)n * RING + ((i + RING) % RING)]; };
  T cvr[NV];
  T cFA[NU];
  T ccp = T(0);
#pragma unroll
  for (int n = 0; n < NV; n++) cvr[n] = T(0);
#pragma unroll
  for (int n = 0; n < NU; n++) cFA[n] = T(0);
  double run_max = 0.0;
  for (int k = 0; k < nchunks; k++) {
    wait_upto(k + 1);
    ok = __all_sync(0xffffffffu, ok);  // the warp stops together
    if (!ok) break;
    const int i = 32 * k + lane;  // this lane's cell
    T vl[NV], vrr[NV];
    const bool shk = f.shock && i < nx && f.shock[row + i];
#pragma unroll
    for (int n = 0; n < NV; n++) {
      if (n == dd::BXn) continue;
      T wv[2 * H + 1];
#pragma unroll
      for (int m = -H; m <= H; m++) wv[H + m] = (i + m >= 0 && i + m < nx) ? V(n, i + m) : T(0);
      Recon<ORDER>::cell(wv, dxd, n == v::RHO || n == v::PRS, vl[n], vrr[n], shk, l3);
    }
    T vL[NV], vR[NV];
#pragma unroll
    for (int n = 0; n < NV; n++) {
      if (n == dd::BXn) continue;
      const T up = __shfl_up_sync(0xffffffffu, vrr[n], 1);
      vL[n] = lane == 0 ? cvr[n] : up;
      vR[n] = vl[n];
    }
    const bool face = (i >= beg && i <= end);
    const long long cc = row + i;
    T FA[NU];
    T cm = T(0);
#pragma unroll
    for (int n = 0; n < NU; n++) FA[n] = T(0);
    if (face) {
      const T bn = from_f64<T>(vs[frow + i]);
      vL[dd::BXn] = bn;
      vR[dd::BXn] = bn;
      RiemannOut<D, T> r;
      riemann<D, 0, SOLVER>(gam, (T)g.rgm1, vL, vR, r);
      store_emf<D, 0>(g, f, cc, r, vL, vR);
#pragma unroll
      for (int n = 0; n < NU; n++) FA[n] = r.F[n] * areaT;
      cm = r.cmax;
    }
    T FAp[NU];
#pragma unroll
    for (int n = 0; n < NU; n++) {
      const T up = __shfl_up_sync(0xffffffffu, FA[n], 1);
      FAp[n] = lane == 0 ? cFA[n] : up;
    }
    const T cpu = __shfl_up_sync(0xffffffffu, cm, 1);
    const T cp = lane == 0 ? ccp : cpu;
    if (active_col && face && i - 1 >= beg) {
      const long long cu = cc - 1;
#pragma unroll
      for (int n = 0; n < NU; n++) {
        const T rhs = -dtdVT * (FA[n] - FAp[n]);
        f.Uc[n * g.ncell + cu] = U(n, i - 1) + to_f64(rhs);
      }
      if (invdt) {
        const double prev = (invdt == 1) ? 0.0 : f.InvDt[cu];
        const double inv = prev + to_f64(T(0.5) * (cm + cp) * invdxT);
        f.InvDt[cu] = inv;
        if (inv > run_max) run_max = inv;
      }
    }
#pragma unroll
    for (int n = 0; n < NV; n++) cvr[n] = __shfl_sync(0xffffffffu, vrr[n], 31);
#pragma unroll
    for (int n = 0; n < NU; n++) cFA[n] = __shfl_sync(0xffffffffu, FA[n], 31);
    ccp = __shfl_sync(0xffffffffu, cm, 31);
    // chunk k-1 is no longer read: its slot takes chunk k-1+kXB
    __syncwarp();
    if (k >= 1 && k - 1 + kXB <= last) {
      if (lane == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fetch(k - 1 + kXB);
      }
      fetched = k - 1 + kXB;
    }
  }
  if (!ok) {  // a copy did not land: stop the cycle, drain what is in flight
    if (lane == 0) report_wait_timeout(ctl);
  }
  // every issued copy lands before the warp's shared memory is released
  for (int q = waited + 1; q <= fetched; q++) mbar_wait(bar + (q % kXB), (uint32_t)((q / kXB) & 1));
  __syncwarp();
  if (ok && last_dir && invdt && active_col)
    atomic_max_pos((unsigned long long*)&((Ctl*)ctl)->invdt_max_bits, run_max);
}

template <int D, int ORDER, int SOLVER, typename T>
__global__ void __launch_bounds__(32 * kXW) k_sweep_xbulk(Geo g, Fields f, const Ctl* ctl, int invdt, int last_dir) {
  extern __shared__ __align__(16) unsigned char xb_smem[];
  d_sweep_xbulk<D, ORDER, SOLVER, T>(g, f, ctl, invdt, last_dir, blockIdx, xb_smem);
}

template <int D, int DIR, int ORDER, int SOLVER, typename T>
__global__ void __launch_bounds__(kTM) k_sweep_march(Geo g, Fields f, const Ctl* ctl, int invdt, int last_dir, int seg) {
  d_sweep_march<D, DIR, ORDER, SOLVER, T>(g, f, ctl, invdt, last_dir, seg, blockIdx);
}

// ---------------------------------------------------------------------------
// Corner EMFs (ConstrainedTransport::CalcCornerEMF, calcCornerEmf.hpp;
// uct_hll / uct_hlld: calcRiemannEmf.hpp).  One thread per edge position
// (k,j,i) in [beg, end]^D; writes ez (and ex, ey in 3-D).
// ---------------------------------------------------------------------------
// E: type of the EMF buffers and of the averaging (the face field q is
// FP64 and is read in E)
template <typename E>
__device__ __forceinline__ E riemann_edge(int order, const double* q, long long fq, long long fs,
                                          const E* e, long long c, long long s,
                                          const E* AL, const E* AR, const E* DL,
                                          const E* DR, long long sp, E& phi) {
  const E h = E(0.5);
  const E aL = h * (AL[c - sp] + AL[c]);
  const E aR = h * (AR[c - sp] + AR[c]);
  const E dL = h * (DL[c - sp] + DL[c]);
  const E dR = h * (DR[c - sp] + DR[c]);
  E bL, bR, vLv, vRv, db, dv;
  const long long fm = fq - fs, m = c - s;
  auto Q = [&](long long x) { return from_f64<E>(q[x]); };
  if (order == 4) {
    ppm_states(Q(fm - 2 * fs), Q(fm - fs), Q(fm), Q(fm + fs), Q(fm + 2 * fs), db, bL);
    ppm_states(Q(fq - 2 * fs), Q(fq - fs), Q(fq), Q(fq + fs), Q(fq + 2 * fs), bR, db);
    ppm_states(e[m - 2 * s], e[m - s], e[m], e[m + s], e[m + 2 * s], dv, vLv);
    ppm_states(e[c - 2 * s], e[c - s], e[c], e[c + s], e[c + 2 * s], vRv, dv);
  } else {
    db = lim_mc(Q(fm + fs) - Q(fm), Q(fm) - Q(fm - fs));
    bL = Q(fm) + h * db;
    db = lim_mc(Q(fq + fs) - Q(fq), Q(fq) - Q(fq - fs));
    bR = Q(fq) - h * db;
    dv = lim_mc(e[m + s] - e[m], e[m] - e[m - s]);
    vLv = e[m] + h * dv;
    dv = lim_mc(e[c + s] - e[c], e[c] - e[c - s]);
    vRv = e[c] - h * dv;
  }
  phi = dR * bR - dL * bL;
  return aL * vLv * bL + aR * vRv * bR;
}

// corner EMF components (corner_emfs MASK)
enum { kCx = 1, kCy = 2, kCz = 4, kCxyz = 7 };

// The corner EMFs of the edges at cell index c (face index fc): the
// components in MASK (ez alone in 2-D).  Each component is computed
// independently of the others.
// the EMF inputs of the averages, in the order of their arrays in a block's
// pool (the tensor map of the staged fused CT pass relies on it)
enum { kEaZi = 0, kEaZj, kEaXj, kEaXk, kEaYi, kEaYk, kEaSx, kEaSy, kEaSz, kEaC1, kEaC2, kEaC3, kEaN };

// corner EMF averages that read face and cell EMFs only (arithmetic, uct0,
// uct_contact; calcCornerEmf.hpp:14-282): get(array, di, dj, dk) is the
// input of that array at the edge's cell shifted by (di, dj, dk) (each -1
// or 0), from global memory or from a staged tile - the arithmetic is one
template <int D, typename E, int MASK, typename Get>
__device__ __forceinline__ void corner_emfs_avg(int emf_mode, Get get, E& exv, E& eyv, E& ezv) {
  constexpr bool CX = (D == 3) && (MASK & kCx) != 0;
  constexpr bool CY = (D == 3) && (MASK & kCy) != 0;
  constexpr bool CZ = (MASK & kCz) != 0;
  auto ezi = [&](int di, int dj, int dk) { return get(kEaZi, di, dj, dk); };
  auto ezj = [&](int di, int dj, int dk) { return get(kEaZj, di, dj, dk); };
  auto exj = [&](int di, int dj, int dk) { return get(kEaXj, di, dj, dk); };
  auto exk = [&](int di, int dj, int dk) { return get(kEaXk, di, dj, dk); };
  auto eyi = [&](int di, int dj, int dk) { return get(kEaYi, di, dj, dk); };
  auto eyk = [&](int di, int dj, int dk) { return get(kEaYk, di, dj, dk); };
  auto Ex1 = [&](int di, int dj, int dk) { return get(kEaC1, di, dj, dk); };
  auto Ex2 = [&](int di, int dj, int dk) { return get(kEaC2, di, dj, dk); };
  auto Ex3 = [&](int di, int dj, int dk) { return get(kEaC3, di, dj, dk); };
  if (emf_mode == kEmfArithmetic || emf_mode == kEmfUct0) {
    const E w = E(0.25);
    if (emf_mode == kEmfArithmetic) {
      if constexpr (CX) exv = w * (exj(0, 0, 0) + exj(0, 0, -1) + exk(0, 0, 0) + exk(0, -1, 0));
      if constexpr (CY) eyv = w * (eyi(0, 0, 0) + eyi(0, 0, -1) + eyk(0, 0, 0) + eyk(-1, 0, 0));
      if constexpr (CZ) ezv = w * (ezi(0, 0, 0) + ezi(0, -1, 0) + ezj(0, 0, 0) + ezj(-1, 0, 0));
    } else {
      // CalcUCT0Average: face EMFs become 2 e - (cell EMF average), computed
      // here for the four faces around the edge (calcCornerEmf.hpp:150-190)
      const E two = E(2), h = E(0.5);
      auto mz_i = [&](int dj) { E a = ezi(0, dj, 0) * two; return a - h * (Ex3(-1, dj, 0) + Ex3(0, dj, 0)); };
      auto mz_j = [&](int di) { E a = ezj(di, 0, 0) * two; return a - h * (Ex3(di, -1, 0) + Ex3(di, 0, 0)); };
      auto mx_j = [&](int dj, int dk) { E a = exj(0, dj, dk) * two; return a - h * (Ex1(0, dj - 1, dk) + Ex1(0, dj, dk)); };
      auto mx_k = [&](int dj, int dk) { E a = exk(0, dj, dk) * two; return a - h * (Ex1(0, dj, dk - 1) + Ex1(0, dj, dk)); };
      auto my_i = [&](int di, int dk) { E a = eyi(di, 0, dk) * two; return a - h * (Ex2(di - 1, 0, dk) + Ex2(di, 0, dk)); };
      auto my_k = [&](int di, int dk) { E a = eyk(di, 0, dk) * two; return a - h * (Ex2(di, 0, dk - 1) + Ex2(di, 0, dk)); };
      if constexpr (CX) exv = w * (mx_j(0, 0) + mx_j(0, -1) + mx_k(0, 0) + mx_k(-1, 0));
      if constexpr (CY) eyv = w * (my_i(0, 0) + my_i(0, -1) + my_k(0, 0) + my_k(-1, 0));
      if constexpr (CZ) ezv = w * (mz_i(0) + mz_i(-1) + mz_j(0) + mz_j(-1));
    }
    return;
  }
  // uct_contact (calcCornerEmf.hpp:224-282)
  auto wsx = [&](int di, int dj, int dk) { return get(kEaSx, di, dj, dk); };
  auto wsy = [&](int di, int dj, int dk) { return get(kEaSy, di, dj, dk); };
  const E q4 = E(0.25);
  if constexpr (CZ) {
    const E ez_l2 = upwind_term(wsx(0, -1, 0), ezj(0, 0, 0) - Ex3(0, -1, 0), ezj(-1, 0, 0) - Ex3(-1, -1, 0));
    const E ez_r2 = upwind_term(wsx(0, 0, 0), ezj(0, 0, 0) - Ex3(0, 0, 0), ezj(-1, 0, 0) - Ex3(-1, 0, 0));
    const E ez_l1 = upwind_term(wsy(-1, 0, 0), ezi(0, 0, 0) - Ex3(-1, 0, 0), ezi(0, -1, 0) - Ex3(-1, -1, 0));
    const E ez_r1 = upwind_term(wsy(0, 0, 0), ezi(0, 0, 0) - Ex3(0, 0, 0), ezi(0, -1, 0) - Ex3(0, -1, 0));
    ezv = q4 * (ez_l2 + ez_r2 + ez_l1 + ez_r1 + ezi(0, 0, 0) + ezi(0, -1, 0) + ezj(0, 0, 0) + ezj(-1, 0, 0));
  }
  if constexpr (D == 3) {
    auto wsz = [&](int di, int dj, int dk) { return get(kEaSz, di, dj, dk); };
    if constexpr (CX) {
      const E ex_l3 = upwind_term(wsy(0, 0, -1), exk(0, 0, 0) - Ex1(0, 0, -1), exk(0, -1, 0) - Ex1(0, -1, -1));
      const E ex_r3 = upwind_term(wsy(0, 0, 0), exk(0, 0, 0) - Ex1(0, 0, 0), exk(0, -1, 0) - Ex1(0, -1, 0));
      const E ex_l2 = upwind_term(wsz(0, -1, 0), exj(0, 0, 0) - Ex1(0, -1, 0), exj(0, 0, -1) - Ex1(0, -1, -1));
      const E ex_r2 = upwind_term(wsz(0, 0, 0), exj(0, 0, 0) - Ex1(0, 0, 0), exj(0, 0, -1) - Ex1(0, 0, -1));
      exv = q4 * (ex_l3 + ex_r3 + ex_l2 + ex_r2 + exj(0, 0, 0) + exj(0, 0, -1) + exk(0, 0, 0) + exk(0, -1, 0));
    }
    if constexpr (CY) {
      const E ey_l3 = upwind_term(wsx(0, 0, -1), eyk(0, 0, 0) - Ex2(0, 0, -1), eyk(-1, 0, 0) - Ex2(-1, 0, -1));
      const E ey_r3 = upwind_term(wsx(0, 0, 0), eyk(0, 0, 0) - Ex2(0, 0, 0), eyk(-1, 0, 0) - Ex2(-1, 0, 0));
      const E ey_l1 = upwind_term(wsz(-1, 0, 0), eyi(0, 0, 0) - Ex2(-1, 0, 0), eyi(0, 0, -1) - Ex2(-1, 0, -1));
      const E ey_r1 = upwind_term(wsz(0, 0, 0), eyi(0, 0, 0) - Ex2(0, 0, 0), eyi(0, 0, -1) - Ex2(0, 0, -1));
      eyv = q4 * (ey_l3 + ey_r3 + ey_l1 + ey_r1 + eyi(0, 0, 0) + eyi(0, 0, -1) + eyk(0, 0, 0) + eyk(-1, 0, 0));
    }
  }
}

template <int D, typename E, int MASK>
__device__ __forceinline__ void corner_emfs(const Geo& g, const Fields& f, long long c, long long fc, E& exv, E& eyv,
                                            E& ezv) {
  constexpr bool CX = (D == 3) && (MASK & kCx) != 0;
  constexpr bool CY = (D == 3) && (MASK & kCy) != 0;
  constexpr bool CZ = (MASK & kCz) != 0;
  const long long si = 1, sj = g.s[1], sk = g.s[2];
  const E* ezi = emf<E>(f.ezi);
  const E* ezj = emf<E>(f.ezj);
  const E *exj = emf<E>(f.exj), *exk = emf<E>(f.exk), *eyi = emf<E>(f.eyi), *eyk = emf<E>(f.eyk);
  if (g.emf == kEmfUctHll || g.emf == kEmfUctHlld) {
    const double* Vs1 = f.Vs;
    const double* Vs2 = f.Vs + g.nface;
    const E *aL0 = emf<E>(f.aL[0]), *aR0 = emf<E>(f.aR[0]), *dL0 = emf<E>(f.dL[0]), *dR0 = emf<E>(f.dR[0]);
    const E *aL1 = emf<E>(f.aL[1]), *aR1 = emf<E>(f.aR[1]), *dL1 = emf<E>(f.dL[1]), *dR1 = emf<E>(f.dR[1]);
    E phi, X;
    if constexpr (CZ) {
      X = riemann_edge<E>(g.order, Vs2, fc, 1, ezj, c, si, aL0, aR0, dL0, dR0, sj, phi);
      ezv = X + phi;
    }
    if constexpr (D == 3) {
      const double* Vs3 = f.Vs + 2 * g.nface;
      const E *aL2 = emf<E>(f.aL[2]), *aR2 = emf<E>(f.aR[2]), *dL2 = emf<E>(f.dL[2]), *dR2 = emf<E>(f.dR[2]);
      if constexpr (CY) {
        X = riemann_edge<E>(g.order, Vs3, fc, 1, eyk, c, si, aL0, aR0, dL0, dR0, sk, phi);
        eyv = X - phi;
      }
      if constexpr (CX) {
        X = riemann_edge<E>(g.order, Vs3, fc, g.fs[1], exk, c, sj, aL1, aR1, dL1, dR1, sk, phi);
        exv = X + phi;
      }
      if constexpr (CZ) {
        X = riemann_edge<E>(g.order, Vs1, fc, g.fs[1], ezi, c, sj, aL1, aR1, dL1, dR1, si, phi);
        ezv += X - phi;
      }
      if constexpr (CY) {
        X = riemann_edge<E>(g.order, Vs1, fc, g.fs[2], eyi, c, sk, aL2, aR2, dL2, dR2, si, phi);
        eyv += X + phi;
      }
      if constexpr (CX) {
        X = riemann_edge<E>(g.order, Vs2, fc, g.fs[2], exj, c, sk, aL2, aR2, dL2, dR2, sj, phi);
        exv += X - phi;
      }
    } else if constexpr (CZ) {
      X = riemann_edge<E>(g.order, Vs1, fc, g.fs[1], ezi, c, sj, aL1, aR1, dL1, dR1, si, phi);
      ezv += X - phi;
    }
    return;
  }
  // arithmetic, uct0, uct_contact: the inputs at this cell and its -i, -j,
  // -k neighbours, by array (kEa*) and offset
  const E* a[12] = {ezi, ezj, exj, exk, eyi, eyk, emf<E>(f.svx), emf<E>(f.svy), emf<E>(f.svz),
                    emf<E>(f.Ex1), emf<E>(f.Ex2), emf<E>(f.Ex3)};
  corner_emfs_avg<D, E, MASK>(g.emf, [&](int q, int di, int dj, int dk) -> E {
    return a[q][c + di * si + dj * sj + dk * sk];
  }, exv, eyv, ezv);
}

template <int D, typename E = double>
__device__ __forceinline__ void d_ct_corner(const Geo& g, const Fields& f, const Ctl* ctl, dim3 bid) {
  if (ctl->done) return;
  const int nx = g.n[0] + 1, ny = g.n[1] + 1;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)nx * ny * (D == 3 ? g.n[2] + 1 : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % nx);
  const long long r = tid / nx;
  const int j = g.beg[1] + (int)(r % ny);
  const int k = (D == 3) ? g.beg[2] + (int)(r / ny) : 0;
  const long long c = cidx(g, k, j, i);
  E exv, eyv, ezv;
  corner_emfs<D, E, kCxyz>(g, f, c, fidx(g, k, j, i), exv, eyv, ezv);
  if constexpr (D == 3) {
    emf<E>(f.ex)[c] = exv;
    emf<E>(f.ey)[c] = eyv;
  }
  emf<E>(f.ez)[c] = ezv;
}

template <int D, typename E = double>
__global__ void k_ct_corner(Geo g, Fields f, const Ctl* ctl) {
  d_ct_corner<D, E>(g, f, ctl, blockIdx);
}

// ---------------------------------------------------------------------------
// Face-field update Vs += dt curl E (evolveMagField.hpp:53-132, Cartesian),
// then the Runge-Kutta combination of the faces (AddAndStore).  Only faces
// that the next boundary pass does not overwrite are touched.
// ---------------------------------------------------------------------------
// Runge-Kutta combination wc u + w0 u0 (stateContainer AddAndStore).  The
// FP64 path keeps the reference's expression; the mixed path (FP32 EMF
// type) writes equal weights (RK2: 1/2, 1/2) as one product of the sum.
// combine argument of the face update: kCtCombine = the Runge-Kutta
// combination with Vs0; kCtSaveBegin = also write the updated face as the
// next cycle's Runge-Kutta begin copy (last stage of a cycle, periodic
// blocks: the next cycle's face fill then passes over the ghosts alone)
enum { kCtCombine = 1, kCtSaveBegin = 2 };

template <typename E>
__device__ __forceinline__ double rk_combine(double u, double u0, double wc, double w0) {
  if constexpr (sizeof(E) == 4) {
    // RK2's 1/2 (u + u0): the halving exact on the integer pipe
    if (wc == w0) return wc == 0.5 ? half_of(u + u0) : wc * (u + u0);
  }
  return wc * u + w0 * u0;
}

// Face-field update of the faces at face index fc from the corner EMFs
// around them: get(comp, off) gives corner EMF component comp (0: x, 1: y,
// 2: z) of the edge position off (0: this one, 1: +i, 2: +j, 3: +k).
// E: type of the corner EMFs; they are widened exactly to FP64 and the curl
// and the face update are FP64 on both paths (div B stays at FP64 round-off)
template <int D, typename E, typename Get>
__device__ __forceinline__ void faces_from_corners(const Geo& g, const Fields& f, const Ctl* ctl, long long fc,
                                                   bool in_i, bool in_j, bool in_k, int combine, double wc, double w0,
                                                   Get get) {
  auto Ex1 = [&](int o) { return to_f64(get(0, o)); };
  auto Ex2 = [&](int o) { return to_f64(get(1, o)); };
  auto Ex3 = [&](int o) { return to_f64(get(2, o)); };
  const double dtdx1 = ctl->dtdx[0], dtdx2 = ctl->dtdx[1], dtdx3 = ctl->dtdx[2];
  if constexpr (sizeof(E) == 4) {
    // mixed path: the same FP64 curl, each term fused into the face value
    // (Vs + c1 dE1 + c2 dE2 as two FMAs: 4 FP64 operations per face
    // instead of 7; the FP64 pipe bounds this pass)
    auto put = [&](int comp, double b) {
      const long long q = comp * g.nface + fc;
      if (combine & kCtCombine) b = rk_combine<E>(b, f.Vs0[q], wc, w0);
      f.Vs[q] = b;
      if (combine & kCtSaveBegin) f.Vs0[q] = b;
    };
    if (in_j && in_k) {
      double b = fma(-dtdx2, Ex3(2) - Ex3(0), f.Vs[fc]);
      if constexpr (D == 3) b = fma(dtdx3, Ex2(3) - Ex2(0), b);
      put(0, b);
    }
    if (in_i && in_k) {
      double b = fma(dtdx1, Ex3(1) - Ex3(0), f.Vs[g.nface + fc]);
      if constexpr (D == 3) b = fma(-dtdx3, Ex1(3) - Ex1(0), b);
      put(1, b);
    }
    if constexpr (D == 3) {
      if (in_i && in_j) {
        double b = fma(-dtdx1, Ex2(1) - Ex2(0), f.Vs[2 * g.nface + fc]);
        b = fma(dtdx2, Ex1(2) - Ex1(0), b);
        put(2, b);
      }
    }
    return;
  }
  // BX1s: faces i in [beg, end], j, k active
  if (in_j && in_k) {
    double rhs;
    const double z = 0.0;  // 0.0 - x: the reference's expression
    if constexpr (D == 2) {
      rhs = z - dtdx2 * (Ex3(2) - Ex3(0));
    } else {
      rhs = z - dtdx2 * (Ex3(2) - Ex3(0)) + dtdx3 * (Ex2(3) - Ex2(0));
    }
    double* vs = f.Vs;
    double b = vs[fc] + rhs;
    if (combine & kCtCombine) b = rk_combine<E>(b, f.Vs0[fc], wc, w0);
    vs[fc] = b;
    if (combine & kCtSaveBegin) f.Vs0[fc] = b;
  }
  if (in_i && in_k) {
    double rhs;
    if constexpr (D == 2) {
      rhs = dtdx1 * (Ex3(1) - Ex3(0));
    } else {
      rhs = dtdx1 * (Ex3(1) - Ex3(0)) - dtdx3 * (Ex1(3) - Ex1(0));
    }
    double* vs = f.Vs + g.nface;
    double b = vs[fc] + rhs;
    if (combine & kCtCombine) b = rk_combine<E>(b, f.Vs0[g.nface + fc], wc, w0);
    vs[fc] = b;
    if (combine & kCtSaveBegin) f.Vs0[g.nface + fc] = b;
  }
  if constexpr (D == 3) {
    if (in_i && in_j) {
      const double rhs = -dtdx1 * (Ex2(1) - Ex2(0)) + dtdx2 * (Ex1(2) - Ex1(0));
      double* vs = f.Vs + 2 * g.nface;
      double b = vs[fc] + rhs;
      if (combine & kCtCombine) b = rk_combine<E>(b, f.Vs0[2 * g.nface + fc], wc, w0);
      vs[fc] = b;
      if (combine & kCtSaveBegin) f.Vs0[2 * g.nface + fc] = b;
    }
  }
}

template <int D, typename E = double>
__device__ __forceinline__ void d_ct_faces(const Geo& g, const Fields& f, const Ctl* ctl, int combine, double wc, double w0, dim3 bid) {
  if (ctl->done) return;
  const int nx = g.n[0] + 1, ny = g.n[1] + 1;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)nx * ny * (D == 3 ? g.n[2] + 1 : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % nx);
  const long long r = tid / nx;
  const int j = g.beg[1] + (int)(r % ny);
  const int k = (D == 3) ? g.beg[2] + (int)(r / ny) : 0;
  const long long c = cidx(g, k, j, i);
  const long long off[4] = {0, 1, g.s[1], g.s[2]};
  const E* e[3] = {emf<E>(f.ex), emf<E>(f.ey), emf<E>(f.ez)};
  const bool in_i = i < g.end[0], in_j = j < g.end[1], in_k = (D == 2) || k < g.end[2];
  faces_from_corners<D, E>(g, f, ctl, fidx(g, k, j, i), in_i, in_j, in_k, combine, wc, w0,
                           [&](int comp, int o) { return e[comp][c + off[o]]; });
}

template <int D, typename E = double>
__global__ void k_ct_faces(Geo g, Fields f, const Ctl* ctl, int combine, double wc, double w0) {
  d_ct_faces<D, E>(g, f, ctl, combine, wc, w0, blockIdx);
}

// ---------------------------------------------------------------------------
// Corner EMFs fused with the face update (mixed path).  A CTA owns a tile of
// kCtTI x kCtTJ edge columns (i, j) and marches a segment of k layers: per
// layer it computes the corner EMFs of its edges - and of the +i column and
// +j row beyond the tile, which its faces also need (warp 0 the row, the
// first kCtTJ lanes of warp 1 the column) - into a shared-memory plane, and
// updates the faces of the layer below from that plane and the k+1 values
// kept in registers.  Two planes alternate, one barrier per layer.  The
// arithmetic is corner_emfs and faces_from_corners, as in k_ct_corner +
// k_ct_faces; the corner EMFs never reach global memory.  Only for the EMF
// averages that do not read the face field (uct_contact, arithmetic, uct0):
// the faces of a layer change while the corner EMFs of later layers and of
// other tiles are still being computed.
// ---------------------------------------------------------------------------
constexpr int kCtTI = 32, kCtTJ = 8, kCtKSeg = 32;

// the two alternating planes of corner EMFs (tile plus the +j row and the
// +i column)
template <typename E>
struct CtPlanes {
  E z[2][kCtTJ + 1][kCtTI + 1];
  E y[2][kCtTJ][kCtTI + 1];
  E x[2][kCtTJ + 1][kCtTI];
};
// where a thread of the fused CT kernel works
struct CtPos {
  int i, j, ti, tj;  // own edge column and its place in the tile
  bool own;          // the own edge column exists
  int hkind;         // halo edge: 1 = row beyond the tile (ez, ex), 2 = column (ez, ey), 0 = none
  int hi, hj;
  bool halo;         // the halo edge exists
};

// corner EMFs of layer k: the own edge into (ox, oy, oz) and plane b, the
// halo edge into plane b
template <int D, typename E>
__device__ __forceinline__ void ct_layer(const Geo& g, const Fields& f, CtPlanes<E>& P, const CtPos& p, int k, int b,
                                         E& ox, E& oy, E& oz) {
  if (p.own) {
    corner_emfs<D, E, kCxyz>(g, f, cidx(g, k, p.j, p.i), fidx(g, k, p.j, p.i), ox, oy, oz);
    P.z[b][p.tj][p.ti] = oz;
    if constexpr (D == 3) {
      P.y[b][p.tj][p.ti] = oy;
      P.x[b][p.tj][p.ti] = ox;
    }
  }
  if (p.halo) {
    E hx = E(0), hy = E(0), hz = E(0);
    if (p.hkind == 1) {
      corner_emfs<D, E, kCz | kCx>(g, f, cidx(g, k, p.hj, p.hi), fidx(g, k, p.hj, p.hi), hx, hy, hz);
      P.z[b][kCtTJ][p.ti] = hz;
      if constexpr (D == 3) P.x[b][kCtTJ][p.ti] = hx;
    } else {
      corner_emfs<D, E, kCz | kCy>(g, f, cidx(g, k, p.hj, p.hi), fidx(g, k, p.hj, p.hi), hx, hy, hz);
      P.z[b][p.ti][kCtTI] = hz;
      if constexpr (D == 3) P.y[b][p.ti][kCtTI] = hy;
    }
  }
}

// L2 prefetch of what the corner EMFs (uct_contact, arithmetic, uct0) and
// the face update of cell c / face fc read at that cell: the fused pass
// marches layers, so two layers ahead the lines reach L2 before the loads
// (its warps otherwise wait on DRAM latency at 3 CTAs per SM; measured:
// 1.99 -> 1.87 ms per 256^3 mixed cycle, the same with an L1 prefetch)
template <typename E>
__device__ __forceinline__ void ct_prefetch(const Geo& g, const Fields& f, long long c, long long fc, bool faces0) {
  // one lane in eight: the lanes of a warp hold consecutive cells, so eight
  // FP32 values (or four FP64) share a 32-byte sector
  if (threadIdx.x & 7) return;
  prefetch_l2(emf<E>(f.ezi) + c);
  prefetch_l2(emf<E>(f.ezj) + c);
  prefetch_l2(emf<E>(f.exj) + c);
  prefetch_l2(emf<E>(f.exk) + c);
  prefetch_l2(emf<E>(f.eyi) + c);
  prefetch_l2(emf<E>(f.eyk) + c);
  prefetch_l2(emf<E>(f.Ex1) + c);
  prefetch_l2(emf<E>(f.Ex2) + c);
  prefetch_l2(emf<E>(f.Ex3) + c);
  prefetch_l2(emf<E>(f.svx) + c);
  prefetch_l2(emf<E>(f.svy) + c);
  prefetch_l2(emf<E>(f.svz) + c);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    prefetch_l2(f.Vs + d * g.nface + fc);
    prefetch_l2(f.Vs + d * g.nface + fc + 4);
    if (faces0) {
      prefetch_l2(f.Vs0 + d * g.nface + fc);
      prefetch_l2(f.Vs0 + d * g.nface + fc + 4);
    }
  }
}

template <int D, typename E>
__global__ void __launch_bounds__(kCtTI * kCtTJ, 3) k_ct_fused(Geo g, Fields f, const Ctl* ctl, int combine, double wc,
                                                           double w0) {
  if (ctl->done) return;
  __shared__ CtPlanes<E> P;
  CtPos p;
  p.ti = threadIdx.x;
  p.tj = threadIdx.y;
  const int i0 = g.beg[0] + (int)blockIdx.x * kCtTI, j0 = g.beg[1] + (int)blockIdx.y * kCtTJ;
  p.i = i0 + p.ti;
  p.j = j0 + p.tj;
  const int ie = g.end[0], je = g.end[1];  // edge positions run over [beg, end]
  p.own = p.i <= ie && p.j <= je;
  // warp 0 takes the row j0 + kCtTJ, the first kCtTJ lanes of warp 1 the column i0 + kCtTI
  p.hkind = (p.tj == 0) ? 1 : (p.tj == 1 && p.ti < kCtTJ) ? 2 : 0;
  p.hi = (p.hkind == 1) ? p.i : i0 + kCtTI;
  p.hj = (p.hkind == 1) ? j0 + kCtTJ : j0 + p.ti;
  p.halo = p.hkind != 0 && p.hi <= ie && p.hj <= je;
  const int i = p.i, j = p.j, ti = p.ti, tj = p.tj;
  int k0 = 0, k1 = 1, ke = 0;
  if constexpr (D == 3) {
    ke = g.end[2];
    k0 = g.beg[2] + (int)blockIdx.z * kCtKSeg;
    k1 = min(k0 + kCtKSeg, ke + 1);  // face layers k0 .. k1-1
  }
  E cx = E(0), cy = E(0), cz = E(0);  // own corner EMFs of layer k
  ct_layer<D, E>(g, f, P, p, k0, 0, cx, cy, cz);
  __syncthreads();
  for (int k = k0; k < k1; k++) {
    const int b = (k - k0) & 1;
    E nx = E(0), ny = E(0), nz = E(0);  // own corner EMFs of layer k + 1
    if (D == 3 && k + 2 <= ke) {
      const bool f0 = (combine & (kCtCombine | kCtSaveBegin)) != 0;
      if (p.own) ct_prefetch<E>(g, f, cidx(g, k + 2, j, i), fidx(g, k + 2, j, i), f0);
      if (p.halo) ct_prefetch<E>(g, f, cidx(g, k + 2, p.hj, p.hi), fidx(g, k + 2, p.hj, p.hi), false);
    }
    if (D == 3 && k + 1 <= ke) ct_layer<D, E>(g, f, P, p, k + 1, b ^ 1, nx, ny, nz);
    if (p.own) {
      const bool in_i = i < ie, in_j = j < je, in_k = (D == 2) || k < ke;
      faces_from_corners<D, E>(g, f, ctl, fidx(g, k, j, i), in_i, in_j, in_k, combine, wc, w0,
                               [&](int comp, int o) -> E {
                                 if (comp == 2) return o == 0 ? cz : (o == 1 ? P.z[b][tj][ti + 1] : P.z[b][tj + 1][ti]);
                                 if (comp == 1) return o == 0 ? cy : (o == 1 ? P.y[b][tj][ti + 1] : ny);
                                 return o == 0 ? cx : (o == 2 ? P.x[b][tj + 1][ti] : nx);
                               });
    }
    cx = nx;
    cy = ny;
    cz = nz;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Stage end over the active cells: RK combination of Uc (AddAndStore),
// cell-centred field from the faces (ReconstructVcField on Uc), and
// ConvertConsToPrim.  Writes Uc and Vc.
// ---------------------------------------------------------------------------
// E: EMF type of the path (FP32: mixed path, see rk_combine).  out (mixed
// path, periodic blocks): kSeOutputs also writes what the next stage begin
// derives for the active cells - the FP32 primitives and (kSbCellEmf) the
// cell EMF - and kSeSaveBegin the Runge-Kutta begin copy of the next cycle
// (Uc0 = Uc), so that the next stage begin only fills the ghost cells.
// kSeNoUcField: the cell-centred field is not stored into Uc (the mixed
// path's sweeps and stage begins read the hydro variables of Uc alone; the
// host rebuilds the field part from the faces before it hands Uc out).
enum { kSeOutputs = 16, kSeSaveBegin = 32, kSeNoUcField = 64 };
template <int D, typename E = double>
__device__ __forceinline__ void d_stage_end(const Geo& g, const Fields& f, const Ctl* ctl, int combine, double wc,
                                            double w0, dim3 bid, int out = 0) {
  if (ctl->done) return;
  using v = Var<D>;
  constexpr int NV = v::NV;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)g.n[0] * g.n[1] * (D == 3 ? g.n[2] : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % g.n[0]);
  const long long r = tid / g.n[0];
  const int j = g.beg[1] + (int)(r % g.n[1]);
  const int k = (D == 3) ? g.beg[2] + (int)(r / g.n[1]) : 0;
  const long long c = cidx(g, k, j, i);
  const long long fc = fidx(g, k, j, i);
  if (tid == 0) ((Ctl*)ctl)->uc_fresh = 1;  // read by the next stage begin
  double U[NV], V[NV];
#pragma unroll
  for (int n = 0; n < v::BX1; n++) {
    double u = f.Uc[n * g.ncell + c];
    if (combine) u = rk_combine<E>(u, f.Uc0[n * g.ncell + c], wc, w0);
    U[n] = u;
  }
#pragma unroll
  for (int d = 0; d < D; d++) {
    const double* vs = f.Vs + d * g.nface;
    U[v::BX1 + d] = 0.5 * (vs[fc] + vs[fc + g.fs[d]]);
  }
  // mixed path (E = float): the fused FP64 pressure recovery
  cons_to_prim<D, true, double, sizeof(E) == 4>(g.gm1, V, U);
#pragma unroll
  for (int n = 0; n < NV; n++) {
    if (n < v::BX1 || !(out & kSeNoUcField)) f.Uc[n * g.ncell + c] = U[n];
    f.Vc[n * g.ncell + c] = V[n];
  }
  if (out & kSeOutputs) cell_outputs<D, E>(f, g, c, V, (out & kSbCellEmf) != 0);
  if (out & kSeSaveBegin) {
#pragma unroll
    for (int n = 0; n < v::BX1; n++) f.Uc0[n * g.ncell + c] = U[n];
  }
}

template <int D, typename E = double>
__global__ void k_stage_end(Geo g, Fields f, const Ctl* ctl, int combine, double wc, double w0, int out) {
  d_stage_end<D, E>(g, f, ctl, combine, wc, w0, blockIdx, out);
}

// ---------------------------------------------------------------------------
// Diagnostics: divB estimator (checkDivB.hpp:14-68) and NaN count
// (checkNan.hpp:17-45), as device reductions.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void d_divb(const Geo& g, const Fields& f, Ctl* ctl, dim3 bid) {
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)g.n[0] * g.n[1] * (D == 3 ? g.n[2] : 1);
  // every lane reaches the warp reduction below; lanes past the end give 0
  const bool in = tid < tot;
  const long long t = in ? tid : 0;
  const int i = g.beg[0] + (int)(t % g.n[0]);
  const long long r = t / g.n[0];
  const int j = g.beg[1] + (int)(r % g.n[1]);
  const int k = (D == 3) ? g.beg[2] + (int)(r / g.n[1]) : 0;
  const long long fc = fidx(g, k, j, i);
  const double* B1s = f.Vs;
  const double* B2s = f.Vs + g.nface;
  const double A1 = g.A[0], A2 = g.A[1], A3 = g.A[2];
  const double dB1 = (A1 * B1s[fc + 1] - A1 * B1s[fc]);
  const double dB2 = (A2 * B2s[fc + g.fs[1]] - A2 * B2s[fc]);
  const double d1 = 0.5 * (A1 + A1), d2 = 0.5 * (A2 + A2);
  const double b1 = 0.5 * (B1s[fc + 1] + B1s[fc]);
  const double b2 = 0.5 * (B2s[fc + g.fs[1]] + B2s[fc]);
  double amplitude = 1e-40;
  double val;
  if constexpr (D == 2) {
    amplitude += fabs(b1) * d1 + fabs(b2) * d2;
    val = fabs(dB1 + dB2) / amplitude;
  } else {
    const double* B3s = f.Vs + 2 * g.nface;
    const double dB3 = (A3 * B3s[fc + g.fs[2]] - A3 * B3s[fc]);
    const double d3 = 0.5 * (A3 + A3);
    const double b3 = 0.5 * (B3s[fc + g.fs[2]] + B3s[fc]);
    amplitude += fabs(b1) * d1 + fabs(b2) * d2 + fabs(b3) * d3;
    val = fabs(dB1 + dB2 + dB3) / amplitude;
  }
  // max over the warp, then one atomic per warp (NaN ignored, as before)
  if (!in || !(val >= 0.0)) val = 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, val, o);
    if (w > val) val = w;
  }
  if ((threadIdx.x & 31) == 0) atomic_max_pos(&ctl->divb_bits, val);
}

template <int D>
__global__ void k_divb(Geo g, Fields f, Ctl* ctl) {
  d_divb<D>(g, f, ctl, blockIdx);
}

template <int D>
__device__ __forceinline__ void d_nan_count(const Geo& g, const Fields& f, Ctl* ctl, dim3 bid) {
  using v = Var<D>;
  const long long tid = (long long)bid.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0] + 1, ny = g.n[1] + 1;
  const long long tot = (long long)nx * ny * (D == 3 ? g.n[2] + 1 : 1);
  if (tid >= tot) return;
  const int i = g.beg[0] + (int)(tid % nx);
  const long long r = tid / nx;
  const int j = g.beg[1] + (int)(r % ny);
  const int k = (D == 3) ? g.beg[2] + (int)(r / ny) : 0;
  unsigned long long n = 0;
  const bool cell = i < g.end[0] && j < g.end[1] && (D == 2 || k < g.end[2]);
  if (cell) {
    const long long c = cidx(g, k, j, i);
    for (int q = 0; q < v::NV; q++) n += isnan(f.Vc[q * g.ncell + c]) ? 1 : 0;
  }
  const long long fc = fidx(g, k, j, i);
  for (int q = 0; q < D; q++) n += isnan(f.Vs[q * g.nface + fc]) ? 1 : 0;
  if (n) atomicAdd(&ctl->nan_count, n);
}

template <int D>
__global__ void k_nan_count(Geo g, Fields f, Ctl* ctl) {
  d_nan_count<D>(g, f, ctl, blockIdx);
}

// ---------------------------------------------------------------------------
// Time-integrator control (timeIntegrator.cpp:246-414, main.cpp:190-225),
// single thread.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void d_cycle_begin(const Geo& g, Ctl* ctl, int use_tstop) {
  if (ctl->done) return;
  if (use_tstop) {
    if (!(ctl->t < ctl->tstop)) {
      ctl->done = 1;
      return;
    }
    if (ctl->tstop - ctl->t < ctl->dt) ctl->dt = ctl->tstop - ctl->t;
  }
  const double dt = ctl->dt;
  double dV = g.dx[0] * g.dx[1];
  if (g.D == 3) dV = dV * g.dx[2];
  ctl->dtdV = dt / dV;
  for (int d = 0; d < 3; d++) ctl->dtdx[d] = dt / g.dx[d];
  ctl->t0 = ctl->t;
  ctl->invdt_max_bits = 0ull;
}

__device__ __forceinline__ void d_cycle_end(Ctl* ctl) {
  if (ctl->done) return;
  const double invmax = __longlong_as_double((long long)ctl->invdt_max_bits);
  const double dtmin = 1.0 / invmax;  // = min over cells of 1/InvDt (division is monotone)
  const double newdt = ctl->cfl * dtmin;
  ctl->t = ctl->t0 + ctl->dt;
  if (newdt > ctl->cflmax * ctl->dt) {
    ctl->dt = ctl->cflmax * ctl->dt;
  } else {
    if (ctl->ncycles == 0 && newdt < 0.5 * ctl->dt) {
      ctl->status = kErrFirstDt;
      ctl->done = 1;
      return;
    }
    ctl->dt = newdt;
  }
  if (ctl->dt < 1e-15) {
    ctl->status = kErrDtSmall;
    ctl->done = 1;
    return;
  }
  ctl->ncycles++;
}

__device__ __forceinline__ void d_check_divb(Ctl* ctl) {
  if (ctl->done) return;
  const double v = __longlong_as_double((long long)ctl->divb_bits);
  if (v > ctl->maxdivb) {
    ctl->status = kErrDivB;
    ctl->done = 1;
  }
}

__device__ __forceinline__ void d_check_nan(Ctl* ctl) {
  if (ctl->done) return;
  if (ctl->nan_count > 0) {
    ctl->status = kErrNan;
    ctl->done = 1;
  }
}

static __global__ void k_cycle_begin(Geo g, Ctl* ctl, int use_tstop) { d_cycle_begin(g, ctl, use_tstop); }
static __global__ void k_cycle_end(Ctl* ctl) { d_cycle_end(ctl); }
static __global__ void k_check_divb(Ctl* ctl) { d_check_divb(ctl); }
static __global__ void k_check_nan(Ctl* ctl) { d_check_nan(ctl); }

}  // namespace idfx
