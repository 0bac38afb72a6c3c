// Device arithmetic of the ideal-MHD stage: cons/prim, physical flux, slope
// limiters, face reconstruction and the HLLD / HLL / Roe / TVDLF Riemann
// solvers, templated on the arithmetic type T.
//
// T = double is the parity path: compiled with --fmad=false, every
// expression keeps the operation order of the reference so that results are
// bit-identical to it (the reference's GPU CI also disables contraction,
// pytools/idfx_test.py:121).  Literals are written T(x), which is the same
// double for T = double.  T = float is the mixed-precision path (FP32
// reconstruction and Riemann solve; the callers keep the conserved state,
// cons->prim and the CT face update in FP64).
//
// D is the number of dimensions (= components, 2 or 3).  Variable order
// follows src/idefix.hpp:74-108: RHO, MX1..MXD, ENG(=PRS), BX1..BXD.
#pragma once
#include <cstdint>

#include "exact_ops.cuh"
#include "intdiv.cuh"
#include "rdiv.cuh"

namespace idfx {

template <int D>
struct Var {
  static constexpr int NV = 2 * D + 2;
  static constexpr int RHO = 0, MX1 = 1, MX2 = 2, MX3 = 3;
  static constexpr int ENG = D + 1, PRS = D + 1;
  static constexpr int BX1 = D + 2, BX2 = D + 3, BX3 = D + 4;
};

// normal / tangent / bi-tangent indices for a sweep (hlldMHD.hpp:158-165)
template <int D, int DIR>
struct Dir {
  using V = Var<D>;
  static constexpr int Xn = V::MX1 + DIR;
  static constexpr int Xt = (DIR == 0 ? V::MX2 : V::MX1);
  static constexpr int Xb = (DIR == 2 ? V::MX2 : V::MX3);
  static constexpr int BXn = V::BX1 + DIR;
  static constexpr int BXt = (DIR == 0 ? V::BX2 : V::BX1);
  static constexpr int BXb = (DIR == 2 ? V::BX2 : V::BX3);
};

constexpr double kSmallPressureFix = 1.0e-5;  // fluid_defs.hpp:23
constexpr double kEpsUctContact = 1.0e-6;     // fluid_defs.hpp:24

// FP32 quotient for the mixed path: the approximate reciprocal (MUFU) and
// one FMA correction of the quotient, q' = q + (a - q b) r with q = a r
// (the correction step of Markstein's FMA division, P. W. Markstein, IBM J.
// Res. Dev. 34 (1990)): within about an ulp, at the cost of the bare
// reciprocal-multiply plus two FMAs; no special-case path (the mixed path
// divides by nonzero finite values; subnormals flush to zero).  Against IEEE
// division it leaves the mixed path's errors against FP64 unchanged while
// the bare reciprocal-multiply (2 ulp) had doubled them.
__device__ __forceinline__ float rcp_approx(float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return r;
}
__device__ __forceinline__ float fdiv_corrected(float a, float b) {
  const float r = rcp_approx(b);
  const float q = a * r;
  const float e = __fmaf_rn(-q, b, a);
  return __fmaf_rn(e, r, q);
}

// division: FP64 IEEE correctly rounded (the bit-identical path); FP32 (the
// mixed path, FP32-accurate rather than bit-matched) fdiv_corrected
template <typename T>
__device__ __forceinline__ T dv(T a, T b) {
  if constexpr (sizeof(T) == 4) {
    return fdiv_corrected(a, b);
  } else {
    return a / b;
  }
}

// square root: FP64 IEEE (the bit-identical path); FP32 x * rsqrt(x), within
// 2 ulp (the tiny offset keeps sqrt(0) = 0; negative arguments stay NaN) -
// measured not to change the mixed path's errors against FP64
template <typename T>
__device__ __forceinline__ T sqr(T x) {
  if constexpr (sizeof(T) == 4) {
    return x * rsqrtf(x + 1.2e-38f);
  } else {
    return sqrt(x);
  }
}

// 1 / b: FP64 the correctly rounded reciprocal (__drcp_rn, one instruction
// sequence shorter than a general division, equal to 1 / b); FP32 as dv
template <typename T>
__device__ __forceinline__ T rcp(T b) {
  if constexpr (sizeof(T) == 8) {
    return rcp_rn(b);
  } else {
    return fdiv_corrected(T(1), b);
  }
}

// the same quotient computed on the integer pipe for FP64 (intdiv.cuh): used
// by the memory-bound whole-array kernels (cons <-> prim), where it takes the
// division off the FP64 pipe; the sweeps keep the hardware sequence, whose
// shorter dependency chain suits their low occupancy
template <typename T>
__device__ __forceinline__ T dvi(T a, T b) {
  if constexpr (sizeof(T) == 8) {
    return div_rn(a, b);
  } else {
    return a / b;
  }
}

// a b + c: one fused multiply-add on the FP32 (mixed) path; on the FP64
// path the product and the sum, rounded separately as the reference
// evaluates them (the library is built without FMA contraction), so that
// every FP64 expression written with it keeps the reference's bits
template <typename T>
__device__ __forceinline__ T mad(T a, T b, T c) {
  if constexpr (sizeof(T) == 4) {
    return fmaf(a, b, c);
  } else {
    return a * b + c;
  }
}

// sum of squares of the first D entries, in reference order
template <int D, typename T>
__device__ __forceinline__ T sumsq(T a, T b, T c) {
  T s = mad(b, b, a * a);
  if constexpr (D == 3) s = mad(c, c, s);
  return s;
}

// ---------------------------------------------------------------------------
// cons <-> prim (convertConsToPrim.hpp:15-100; eos_adiabatic.hpp:38-45)
// gm1 = gamma - 1.0, evaluated once on the host
// ---------------------------------------------------------------------------
// QUOT: how p / gm1 is formed - 0 the hardware division, 1 on the integer
// pipe (whole-array kernels), 2 from rgm1 = RN(1 / gm1) formed once on the
// host (Riemann solvers, FP64: Markstein's correction, rdiv.cuh); all three
// give the correctly rounded quotient
template <int D, int QUOT = 0, typename T>
__device__ __forceinline__ void prim_to_cons(T gm1, T* U, const T* V, T rgm1 = T(0)) {
  using v = Var<D>;
  U[v::RHO] = V[v::RHO];
  U[v::MX1] = V[v::MX1] * V[v::RHO];
  U[v::MX2] = V[v::MX2] * V[v::RHO];
  if constexpr (D == 3) U[v::MX3] = V[v::MX3] * V[v::RHO];
  U[v::BX1] = V[v::BX1];
  U[v::BX2] = V[v::BX2];
  if constexpr (D == 3) U[v::BX3] = V[v::BX3];
  const T z = T(0);
  T kin, mag;
  if constexpr (D == 3) {
    kin = sumsq<3>(V[v::MX1], V[v::MX2], V[v::MX3]);
    mag = sumsq<3>(U[v::BX1], U[v::BX2], U[v::BX3]);
  } else {
    kin = sumsq<2>(V[v::MX1], V[v::MX2], z);
    mag = sumsq<2>(U[v::BX1], U[v::BX2], z);
  }
  T pq;
  if constexpr (QUOT == 1) {
    pq = dvi(V[v::PRS], gm1);
  } else if constexpr (QUOT == 2 && sizeof(T) == 8) {
    pq = div_r(V[v::PRS], Recip{gm1, rgm1});
  } else {
    (void)rgm1;
    pq = dv(V[v::PRS], gm1);
  }
  U[v::ENG] = mad(T(0.5), mag, mad(T(0.5) * V[v::RHO], kin, pq));
}

// FUSED (mixed path, FP64 state): the same FP64 pressure recovery with the
// sums of squares and the two subtractions as fused multiply-adds
// (p = (E - k m^2 - b^2 / 2) gm1 in 8 FP64 operations instead of 15, each
// fused step rounding once); the bit-exact path keeps the reference's
// operations
template <int D, bool INTDIV = false, typename T, bool FUSED = false>
__device__ __forceinline__ void cons_to_prim(T gm1, T* V, const T* U) {
  using v = Var<D>;
  auto q = [](T a, T b) { return INTDIV ? dvi(a, b) : dv(a, b); };
  if constexpr (FUSED) {
    V[v::RHO] = U[v::RHO];
    V[v::MX1] = q(U[v::MX1], U[v::RHO]);
    V[v::MX2] = q(U[v::MX2], U[v::RHO]);
    if constexpr (D == 3) V[v::MX3] = q(U[v::MX3], U[v::RHO]);
    V[v::BX1] = U[v::BX1];
    V[v::BX2] = U[v::BX2];
    if constexpr (D == 3) V[v::BX3] = U[v::BX3];
    T m2 = fma(U[v::MX2], U[v::MX2], U[v::MX1] * U[v::MX1]);
    T b2 = fma(U[v::BX2], U[v::BX2], U[v::BX1] * U[v::BX1]);
    if constexpr (D == 3) {
      m2 = fma(U[v::MX3], U[v::MX3], m2);
      b2 = fma(U[v::BX3], U[v::BX3], b2);
    }
    const T e = fma(-q(T(0.5), U[v::RHO]), m2, U[v::ENG]);
    V[v::PRS] = fma(T(-0.5), b2, e) * gm1;
    if (V[v::PRS] <= T(0)) V[v::PRS] = T(kSmallPressureFix);
    return;
  }
  V[v::RHO] = U[v::RHO];
  V[v::MX1] = q(U[v::MX1], U[v::RHO]);
  V[v::MX2] = q(U[v::MX2], U[v::RHO]);
  if constexpr (D == 3) V[v::MX3] = q(U[v::MX3], U[v::RHO]);
  V[v::BX1] = U[v::BX1];
  V[v::BX2] = U[v::BX2];
  if constexpr (D == 3) V[v::BX3] = U[v::BX3];
  const T z = T(0);
  T m2, b2;
  if constexpr (D == 3) {
    m2 = sumsq<3>(U[v::MX1], U[v::MX2], U[v::MX3]);
    b2 = sumsq<3>(U[v::BX1], U[v::BX2], U[v::BX3]);
  } else {
    m2 = sumsq<2>(U[v::MX1], U[v::MX2], z);
    b2 = sumsq<2>(U[v::BX1], U[v::BX2], z);
  }
  const T kin = q(T(0.5), U[v::RHO]) * m2;
  const T mag = T(0.5) * b2;
  V[v::PRS] = (U[v::ENG] - kin - mag) * gm1;
  // floor; the reference's energy repair only touches a discarded local copy
  if (V[v::PRS] <= T(0)) V[v::PRS] = T(kSmallPressureFix);
}

// induction flux of the transverse and bi-transverse field components
// (flux.hpp:28-95)
template <int D, int DIR, typename T>
__device__ __forceinline__ T flux_bt(const T* V) {
  using d = Dir<D, DIR>;
  return mad(V[d::Xn], V[d::BXt], -(V[d::BXn] * V[d::Xt]));
}
template <int D, int DIR, typename T>
__device__ __forceinline__ T flux_bb(const T* V) {
  using d = Dir<D, DIR>;
  return mad(V[d::Xn], V[d::BXb], -(V[d::BXn] * V[d::Xb]));
}

// physical MHD flux along DIR (flux.hpp:28-95); U is read before F is written
template <int D, int DIR, typename T>
__device__ __forceinline__ void phys_flux(T* F, const T* V, const T* U) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  const T uXn = U[d::Xn], uE = U[v::ENG];
  const T u1 = U[v::MX1], u2 = U[v::MX2];
  T u3 = T(0);
  if constexpr (D == 3) u3 = U[v::MX3];
  F[v::RHO] = uXn;
  F[v::MX1] = mad(u1, V[d::Xn], -(V[d::BXn] * V[v::BX1]));
  F[v::MX2] = mad(u2, V[d::Xn], -(V[d::BXn] * V[v::BX2]));
  if constexpr (D == 3) F[v::MX3] = mad(u3, V[d::Xn], -(V[d::BXn] * V[v::BX3]));
  F[d::BXn] = T(0);
  F[d::BXt] = flux_bt<D, DIR>(V);
  if constexpr (D == 3) F[d::BXb] = flux_bb<D, DIR>(V);
  T Bmag2, vB;
  if constexpr (D == 3) {
    Bmag2 = sumsq<3>(V[v::BX1], V[v::BX2], V[v::BX3]);
    vB = mad(V[v::MX3], V[v::BX3], mad(V[v::MX2], V[v::BX2], V[v::MX1] * V[v::BX1]));
  } else {
    Bmag2 = sumsq<2>(V[v::BX1], V[v::BX2], T(0));
    vB = mad(V[v::MX2], V[v::BX2], V[v::MX1] * V[v::BX1]);
  }
  const T ptot = mad(T(0.5), Bmag2, V[v::PRS]);
  F[v::ENG] = mad(uE + ptot, V[d::Xn], -(V[d::BXn] * (vB)));
  F[d::Xn] += ptot;
}

// ---------------------------------------------------------------------------
// slope limiters (slopeLimiter.hpp)
// ---------------------------------------------------------------------------
// The reference MinModLim shadows its result variable and always returns 0
// (slopeLimiter.hpp:16-23); every "revert to minmod" path therefore adds 0.
template <typename T>
__device__ __forceinline__ T lim_minmod(T, T) {
  return T(0);
}

template <typename T>
// ipipe: the quotient on the integer pipe (dvi, the same correctly rounded
// value).  The FP64 sweeps are bound by the narrow FP64 pipe while the
// integer pipe idles: half of the limiter quotients go there (the FP64 cycle
// 140.1 -> 137.7 ms at 256^3; all of them, or the right-state twins of the
// HLLD quotients as well, gave nothing - the integer division's latency)
__device__ __forceinline__ T lim_vanleer(T dvp, T dvm, bool ipipe = false) {  // :54-57
  if (dvp * dvm > T(0)) return ipipe ? dvi(T(2) * dvp * dvm, dvp + dvm) : dv(T(2) * dvp * dvm, dvp + dvm);
  return T(0);
}

template <typename T>
__device__ __forceinline__ T lim_mc(T dvp, T dvm) {  // :68-76
  T dq = T(0);
  if (dvp * dvm > T(0)) {
    T dqc = T(0.5) * (dvp + dvm);
    T d2q = T(2) * (fabs(dvp) < fabs(dvm) ? dvp : dvm);
    dq = fabs(d2q) < fabs(dqc) ? d2q : dqc;
  }
  return dq;
}

// e2: (r dx)^2 and its correctly rounded reciprocal, formed on the host; the
// FP64 path divides by it and by 3 with Markstein's correction (rdiv.cuh),
// bit-identical to the divisions
template <typename T>
__device__ __forceinline__ T lim_limo3(T dvp, T dvm, T dx, const Recip& e2) {  // :25-52
  const T r = T(0.1), eps = T(1.e-12);
  T th = dv(dvm, dvp + T(1.e-16));
  T q;
  if constexpr (sizeof(T) == 8) {
    q = div_r(T(2) + th, Recip{3.0, 1.0 / 3.0});
  } else {
    q = dv(T(2) + th, T(3));
  }
  T a = fmin(T(1.5), T(2) * th);
  a = fmin(q, a);
  T b = fmax(T(-0.5) * th, a);
  T c = fmin(q, b);
  T psi = fmax(T(0), c);
  T eta = r * dx;
  if constexpr (sizeof(T) == 8) {
    eta = div_r(dvm * dvm + dvp * dvp, e2);
  } else {
    (void)e2;
    eta = dv(dvm * dvm + dvp * dvp, eta * eta);
  }
  T lim;
  if (eta <= T(1) - eps) {
    lim = q;
  } else if (eta >= T(1) + eps) {
    lim = psi;
  } else {
    psi = (T(1) - dv(eta - T(1), eps)) * q + (T(1) + dv(eta - T(1), eps)) * psi;
    lim = T(0.5) * psi;
  }
  return lim;
}

template <typename T>
__device__ __forceinline__ int sgn(T v) {
  return (T(0) < v) - (v < T(0));
}

template <typename T>
__device__ __forceinline__ void ppm_limit_face(T vm1, T v0, T vp1, T vp2, T& vph) {  // :121-140
  if ((vp1 - vph) * (vph - v0) < T(0)) {
    const T deltaL = (vm1 - 2 * v0 + vp1);
    const T deltaC = 3 * (v0 - 2 * vph + vp1);
    const T deltaR = (v0 - 2 * vp1 + vp2);
    T delta = T(0);
    if (sgn(deltaL) == sgn(deltaC) && sgn(deltaR) == sgn(deltaC)) {
      const T C = T(1.25);
      delta = C * fmin(fabs(deltaL), fabs(deltaR));
      delta = sgn(deltaC) * fmin(delta, fabs(deltaC));
    }
    T d6;
    if constexpr (sizeof(T) == 8) {
      d6 = div_r(delta, Recip{6.0, 1.0 / 6.0});
    } else {
      d6 = dv(delta, T(6));
    }
    vph = T(0.5) * (v0 + vp1) - d6;
  }
}

template <typename T>
__device__ __forceinline__ void ppm_states(T vm2, T vm1, T v0, T vp1, T vp2, T& vl,
                                           T& vr) {  // :142-191
  const int n = 2;
  const T c7 = T(7.0 / 12.0), c1 = T(1.0 / 12.0);
  vr = c7 * (v0 + vp1) - c1 * (vm1 + vp2);
  vl = c7 * (vm1 + v0) - c1 * (vm2 + vp1);
  ppm_limit_face(vm2, vm1, v0, vp1, vl);
  ppm_limit_face(vm1, v0, vp1, vp2, vr);
  T d2qf = T(6) * (vl + vr - T(2) * v0);
  T d2qc0 = vm1 + vp1 - T(2) * v0;
  T d2qcp1 = v0 + vp2 - T(2) * vp1;
  T d2qcm1 = vm2 + v0 - T(2) * vm1;
  T d2q = T(0);
  if (sgn(d2qf) == sgn(d2qc0) && sgn(d2qf) == sgn(d2qcp1) && sgn(d2qf) == sgn(d2qcm1)) {
    const T C = T(1.25);
    d2q = fmin(fabs(d2qc0), fabs(d2qcp1));
    d2q = C * fmin(fabs(d2qcm1), d2q);
    d2q = sgn(d2qf) * fmin(fabs(d2qf), d2q);
  }
  T qmax = fmax(fmax(fabs(vm1), fabs(v0)), fabs(vp1));
  T rho = T(0);
  if (fabs(d2qf) > T(1e-12) * qmax) rho = dv(d2q, d2qf);
  if (((vr - v0) * (v0 - vl) <= T(0)) || (vm1 - v0) * (v0 - vp1) <= T(0)) {
    if (rho <= (T(1) - T(1e-12))) {
      vl = v0 - rho * (v0 - vl);
      vr = v0 + rho * (vr - v0);
    }
  } else {
    if (fabs(vr - v0) >= n * fabs(v0 - vl)) vr = v0 + n * (v0 - vl);
    if (fabs(vl - v0) >= n * fabs(v0 - vr)) vl = v0 + n * (v0 - vr);
  }
}

// Cell-interface states of one cell from its stencil w[0..2*H] (centre w[H]):
// vl = value at its left face (the "vR" of that face), vr = value at its
// right face (the "vL" of the next face).  This is the per-cell form of
// ExtrapolateToFaces::ExtrapolatePrimVar (extrapolateToFaces.hpp:75-309):
// the reference evaluates the same limiter twice per cell (once for each
// face); here it is evaluated once and shared, with identical arithmetic.
// pos = true for RHO and PRS (positivity fallbacks of ORDER 3 and 4).
// ORDER 5 (learned) is the learned sweep's own (learned.cu); its stencil
// half-width is PLM's.
template <int ORDER>
struct Recon {
  static constexpr int H = (ORDER == 1 ? 0 : (ORDER == 4 ? 2 : 1));  // ORDER 5: 1
  // shock: the cell is flagged by shock flattening (minmod slope, PLM and
  // LimO3 only, extrapolateToFaces.hpp:96-218)
  template <typename T>
  // e2: (0.1 dx)^2 and its reciprocal (LimO3, FP64 path; Geo::l3b, l3y)
  __device__ __forceinline__ static void cell(const T* w, T dx, bool pos, T& vl, T& vr, bool shock = false,
                                              const Recip& e2 = Recip{0.0, 0.0}, bool ipipe = false) {
    if constexpr (ORDER == 1) {
      vl = w[0];
      vr = w[0];
    } else if constexpr (ORDER == 2) {
      const T dvm = w[1] - w[0];
      const T dvp = w[2] - w[1];
      const T d = shock ? lim_minmod(dvp, dvm) : lim_vanleer(dvp, dvm, ipipe);
      vr = mad(T(0.5), d, w[1]);
      vl = mad(T(-0.5), d, w[1]);
    } else if constexpr (ORDER == 3) {
      const T dm = w[1] - w[0];
      const T dp = w[2] - w[1];
      T d = shock ? lim_minmod(dp, dm) : dp * lim_limo3(dp, dm, dx, e2);
      vr = w[1] + T(0.5) * d;
      if (pos && vr <= T(0)) {
        d = lim_minmod(dp, dm);
        vr = w[1] + T(0.5) * d;
      }
      d = shock ? lim_minmod(dp, dm) : dm * lim_limo3(dm, dp, dx, e2);
      vl = w[1] - T(0.5) * d;
      if (pos && vl <= T(0)) {
        d = lim_minmod(dp, dm);
        vl = w[1] - T(0.5) * d;
      }
    } else {
      ppm_states(w[0], w[1], w[2], w[3], w[4], vl, vr);
      if (pos && vr <= T(0)) {
        T d = lim_vanleer(w[3] - w[2], w[2] - w[1]);
        vr = w[2] + T(0.5) * d;
      }
      if (pos && vl <= T(0)) {
        T d = lim_vanleer(w[3] - w[2], w[2] - w[1]);
        vl = w[2] - T(0.5) * d;
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Riemann solvers.  In: face states vL, vR (BXn already set from Vs).
// Out: F, cmax, sl/sr (for uct_hll(d)), uL/uR (for uct_hlld).
// ---------------------------------------------------------------------------
enum Solver { kHLLD = 0, kHLL = 1, kROE = 2, kTVDLF = 3 };

template <int D, typename T>
struct RiemannOut {
  T F[Var<D>::NV];
  T uL[Var<D>::NV], uR[Var<D>::NV];
  T cmax, sl, sr;
};

// a / b where several quotients share b: on the FP64 path with the
// reciprocal R = recip(b) formed once (Markstein, rdiv.cuh), bit-identical to
// a / b; the FP32 path divides
template <typename T>
__device__ __forceinline__ T shared_div(T a, T b, const Recip& R) {
  if constexpr (sizeof(T) == 8) {
    return div_r(a, R);
  } else {
    return dv(a, b);
  }
}
template <typename T>
__device__ __forceinline__ Recip shared_recip(T b) {
  if constexpr (sizeof(T) == 8) {
    return recip(b);
  } else {
    return Recip{0.0, 0.0};
  }
}

// fast magnetosonic speed of one face state (hlldMHD.hpp:205-238)
template <int D, int DIR, typename T>
__device__ __forceinline__ T fast_speed(T gamma, const T* v) {
  using vv = Var<D>;
  using d = Dir<D, DIR>;
  const T gpr = gamma * v[vv::PRS];
  const T b1 = v[d::BXn];
  const T b2 = v[d::BXt];
  T b3 = T(0);
  if constexpr (D == 3) b3 = v[d::BXb];
  const T Btmag2 = mad(b3, b3, b2 * b2);
  const T Bmag2 = mad(b1, b1, Btmag2);
  T c = gpr - Bmag2;
  c = gpr + Bmag2 + sqr(mad(T(4) * gpr, Btmag2, c * c));
  c = sqr(dv(T(0.5) * c, v[vv::RHO]));
  return c;
}

template <int D, typename T>
__device__ __forceinline__ T half_b2(const T* v) {
  using vv = Var<D>;
  if constexpr (D == 3) return T(0.5) * (sumsq<3>(v[vv::BX1], v[vv::BX2], v[vv::BX3]));
  return T(0.5) * (sumsq<2>(v[vv::BX1], v[vv::BX2], T(0)));
}

// HLLD (Miyoshi & Kusano 2005) with the reference's HLLC fall-back near
// degeneracy (hlldMHD.hpp:147-457, energy equation branch).
//
// The reference computes both sides' physical fluxes and star states and
// then picks one of five flux expressions (supersonic left / right, single
// star left / right, double star left / right).  Every one of them is the
// physical flux of ONE side plus corrections from that side's star states,
// so here the side is chosen first - from the same sign tests - and its
// operands are selected (integer selects of the bit patterns); the physical
// flux, the star momentum / energy and the double-star state are then
// evaluated for that side only, each with the reference's expression and
// operation order, so every face flux is bit-identical to the reference's.
// Only the HLLC fall-back reads the transverse-field fluxes of both sides.
// On the FP64 path this removes one physical flux, one side's star energy
// and momenta and one side's double-star state per face, and the divergent
// selection of the end (lanes of a warp on both sides issued both branches).
template <int D, int DIR, typename T>
__device__ __forceinline__ void riemann_hlld(T gamma, T rgm1, const T* vL, const T* vR, RiemannOut<D, T>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int RHO = v::RHO, ENG = v::ENG, Xn = d::Xn, Xt = d::Xt, Xb = d::Xb;
  constexpr int BXn = d::BXn, BXt = d::BXt, BXb = d::BXb;
  T* uL = r.uL;
  T* uR = r.uR;
  const T cL = fast_speed<D, DIR>(gamma, vL);
  const T cR = fast_speed<D, DIR>(gamma, vR);
  const T cminL = vL[Xn] - cL, cmaxL = vL[Xn] + cL;
  const T cminR = vR[Xn] - cR, cmaxR = vR[Xn] + cR;
  const T sl = fmin(cminL, cminR);
  const T sr = fmax(cmaxL, cmaxR);
  r.sl = sl;
  r.sr = sr;
  r.cmax = fmax(fabs(sl), fabs(sr));
  const T gm1 = gamma - T(1);
  prim_to_cons<D, 2>(gm1, uL, vL, rgm1);
  prim_to_cons<D, 2>(gm1, uR, vR, rgm1);
  const T ptL = vL[v::PRS] + half_b2<D>(vL);
  const T ptR = vR[v::PRS] + half_b2<D>(vR);
  // supersonic faces: the left physical flux if sl > 0, else the right one
  // if sr < 0; every other face is subsonic and takes star states
  bool sideL = gt0(sl);
  const bool sub = !(sideL || lt0(sr));
  bool dbl = false;
  T Bx = T(0), sBx = T(1), SM = T(0), pts = T(0), duL = T(0), duR = T(0);
  uint64_t sBxb = 0ull;
  Recip RsL{}, RsR{};
  T rhoL = T(0), rhoR = T(0), sqrL = T(0), sqrR = T(0), S1L = T(0), S1R = T(0);
  T bn = T(0), bLt = T(0), bLb = T(0), bRt = T(0), bRb = T(0);  // star field components
  T vsL = T(0), vsR = T(0), wsL = T(0), wsR = T(0);
  if (sub) {
    T scrh = rcp(sr - sl);
    Bx = (sr * vR[BXn] - sl * vL[BXn]) * scrh;
    const bool bpos = gt0(Bx);
    sBx = (bpos ? T(1) : T(-1));
    sBxb = bpos ? 0ull : (1ull << 63);  // its sign bit
    duL = sl - vL[Xn];
    duR = sr - vR[Xn];
    scrh = rcp(duR * uR[RHO] - duL * uL[RHO]);
    SM = (duR * uR[Xn] - duL * uL[Xn] - ptR + ptL) * scrh;
    pts = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR + vL[RHO] * vR[RHO] * duR * duL * (vR[Xn] - vL[Xn]);
    pts *= scrh;
    // (sl - SM) and (sr - SM) divide the star density and the star energy
    RsL = shared_recip(sl - SM);
    RsR = shared_recip(sr - SM);
    rhoL = shared_div(uL[RHO] * duL, sl - SM, RsL);
    rhoR = shared_div(uR[RHO] * duR, sr - SM, RsR);
    sqrL = sqr(rhoL);
    sqrR = sqr(rhoR);
    S1L = SM - dv(fabs(Bx), sqrL);
    S1R = SM + dv(fabs(Bx), sqrR);
    int revert_to_hllc = 0;
    if ((S1L - sl) < T(1.e-4) * (SM - sl)) revert_to_hllc = 1;
    if ((S1R - sr) > T(-1.e-4) * (sr - SM)) revert_to_hllc = 1;
    if (revert_to_hllc) {
      // field components of the HLL state (sr uR - sl uL + FL - FR) / (sr - sl);
      // the normal component's fluxes are zero
      scrh = rcp(sr - sl);
      auto uhll = [&](T ul, T ur, T fl, T fr) {
        T u = sr * ur - sl * ul + fl - fr;
        u *= scrh;
        return u;
      };
      bn = uhll(uL[BXn], uR[BXn], T(0), T(0));
      bLt = bRt = uhll(uL[BXt], uR[BXt], flux_bt<D, DIR>(vL), flux_bt<D, DIR>(vR));
      if constexpr (D == 3) bLb = bRb = uhll(uL[BXb], uR[BXb], flux_bb<D, DIR>(vL), flux_bb<D, DIR>(vR));
      S1L = S1R = SM;
    } else {
      const T scrhL = dv(uL[RHO] * duL * duL - Bx * Bx, uL[RHO] * duL * (sl - SM) - Bx * Bx);
      const T scrhR = dv(uR[RHO] * duR * duR - Bx * Bx, uR[RHO] * duR * (sr - SM) - Bx * Bx);
      bn = Bx;
      bLt = uL[BXt] * scrhL;
      bRt = uR[BXt] * scrhR;
      if constexpr (D == 3) {
        bLb = uL[BXb] * scrhL;
        bRb = uR[BXb] * scrhR;
      }
    }
    const T scrhL = dv(Bx, uL[RHO] * duL);
    const T scrhR = dv(Bx, uR[RHO] * duR);
    vsL = vL[Xt] - scrhL * (bLt - uL[BXt]);
    vsR = vR[Xt] - scrhR * (bRt - uR[BXt]);
    if constexpr (D == 3) {
      wsL = vL[Xb] - scrhL * (bLb - uL[BXb]);
      wsR = vR[Xb] - scrhR * (bRb - uR[BXb]);
    }
    // single star left if S1L >= 0, else single star right if S1R <= 0,
    // else double star on the side of the contact (SM >= 0: left)
    sideL = ge0(S1L) || (!le0(S1R) && ge0(SM));
    dbl = !ge0(S1L) && !le0(S1R);
  }
  // the chosen side's primitive and conserved state and its physical flux
  T vS[NV], uS[NV];
#pragma unroll
  for (int n = 0; n < NV; n++) {
    vS[n] = sideL ? vL[n] : vR[n];
    uS[n] = sideL ? uL[n] : uR[n];
  }
  T* F = r.F;
  phys_flux<D, DIR>(F, vS, uS);
  if (!sub) return;
  // star state of the chosen side (us)
  const T s = sideL ? sl : sr;
  const T du = sideL ? duL : duR;
  const T pt = sideL ? ptL : ptR;
  const Recip Rs = sideL ? RsL : RsR;
  const T vs = sideL ? vsL : vsR;
  const T ws = sideL ? wsL : wsR;
  T us[NV];
  us[RHO] = sideL ? rhoL : rhoR;
  us[BXn] = bn;
  us[BXt] = sideL ? bLt : bRt;
  if constexpr (D == 3) us[BXb] = sideL ? bLb : bRb;
  us[Xn] = us[RHO] * SM;
  us[Xt] = us[RHO] * vs;
  if constexpr (D == 3) us[Xb] = us[RHO] * ws;
  {
    T a = vS[Xn] * Bx + vS[Xt] * uS[BXt];
    if constexpr (D == 3) a = a + vS[Xb] * uS[BXb];
    T b = SM * Bx + vs * us[BXt];
    if constexpr (D == 3) b = b + ws * us[BXb];
    T scrh = a;
    scrh -= b;
    us[ENG] = du * uS[ENG] - pt * vS[Xn] + pts * SM + Bx * scrh;
    us[ENG] = shared_div(us[ENG], s - SM, Rs);
  }
  if (dbl) {
    // double-star state of the chosen side (uss); F += S1 (uss - us)
    const Recip Rq = shared_recip(sqrL + sqrR);  // divides the four double-star values
    T vss = sqrL * vsL + sqrR * vsR + times_sign(bRt - bLt, sBx, sBxb);
    vss = shared_div(vss, sqrL + sqrR, Rq);
    T wss = T(0);
    if constexpr (D == 3) {
      wss = sqrL * wsL + sqrR * wsR + times_sign(bRb - bLb, sBx, sBxb);
      wss = shared_div(wss, sqrL + sqrR, Rq);
    }
    T uss[NV];
    uss[RHO] = us[RHO];
    uss[Xn] = uss[RHO] * SM;
    uss[Xt] = uss[RHO] * vss;
    if constexpr (D == 3) uss[Xb] = uss[RHO] * wss;
    uss[BXn] = Bx;
    uss[BXt] = sqrL * bRt + sqrR * bLt + times_sign(sqrL * sqrR * (vsR - vsL), sBx, sBxb);
    uss[BXt] = shared_div(uss[BXt], sqrL + sqrR, Rq);
    if constexpr (D == 3) {
      uss[BXb] = sqrL * bRb + sqrR * bLb + times_sign(sqrL * sqrR * (wsR - wsL), sBx, sBxb);
      uss[BXb] = shared_div(uss[BXb], sqrL + sqrR, Rq);
    }
    T a = SM * Bx + vs * us[BXt];
    if constexpr (D == 3) a = a + ws * us[BXb];
    T b = SM * Bx + vss * uss[BXt];
    if constexpr (D == 3) b = b + wss * uss[BXb];
    T scrh = a;
    scrh -= b;
    // left: usL - sign(Bx) sqrL scrh, right: usR + sign(Bx) sqrR scrh; the
    // left difference is the sum with the sign-flipped term (IEEE defines
    // x - y as x + (-y), so the bits are the same)
    const T sq = sideL ? sqrL : sqrR;
    const T sgn = sideL ? -sBx : sBx;
    const uint64_t sgnb = sideL ? (sBxb ^ (1ull << 63)) : sBxb;
    uss[ENG] = us[ENG] + times_sign(sq * scrh, sgn, sgnb);
    const T S1 = sideL ? S1L : S1R;
#pragma unroll
    for (int n = 0; n < NV; n++) F[n] = mad(S1, uss[n] - us[n], F[n]);
  }
  // F += s (us - u) of the chosen side: single star F = Fs + s (us - u),
  // double star F = (Fs + S1 (uss - us)) + s (us - u), the reference's order
#pragma unroll
  for (int n = 0; n < NV; n++) F[n] = mad(s, us[n] - uS[n], F[n]);
}

// HLL (hllMHD.hpp:154-453; the Hall whistler term is not part of ideal MHD)
template <int D, int DIR, typename T>
__device__ __forceinline__ void riemann_hll(T gamma, T rgm1, const T* vL, const T* vR, RiemannOut<D, T>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  T* uL = r.uL;
  T* uR = r.uR;
  T fluxL[NV], fluxR[NV];
  const T cL = fast_speed<D, DIR>(gamma, vL);
  const T cR = fast_speed<D, DIR>(gamma, vR);
  const T cminL = vL[d::Xn] - cL, cmaxL = vL[d::Xn] + cL;
  const T cminR = vR[d::Xn] - cR, cmaxR = vR[d::Xn] + cR;
  const T sl = fmin(cminL, cminR);
  const T sr = fmax(cmaxL, cmaxR);
  r.sl = sl;
  r.sr = sr;
  r.cmax = fmax(fabs(sl), fabs(sr));
  const T gm1 = gamma - T(1);
  prim_to_cons<D, 2>(gm1, uL, vL, rgm1);
  prim_to_cons<D, 2>(gm1, uR, vR, rgm1);
  phys_flux<D, DIR>(fluxL, vL, uL);
  phys_flux<D, DIR>(fluxR, vR, uR);
  T* F = r.F;
  if (sl > T(0)) {
#pragma unroll
    for (int n = 0; n <= D; n++) F[n] = fluxL[n];
  } else if (sr < T(0)) {
#pragma unroll
    for (int n = 0; n <= D; n++) F[n] = fluxR[n];
  } else {
#pragma unroll
    for (int n = 0; n <= D; n++)
      F[n] = dv(sl * sr * uR[n] - sl * sr * uL[n] + sr * fluxL[n] - sl * fluxR[n], sr - sl);
  }
  if (sl > T(0)) {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) F[n] = fluxL[n];
    F[v::ENG] = fluxL[v::ENG];
  } else if (sr < T(0)) {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) F[n] = fluxR[n];
    F[v::ENG] = fluxR[v::ENG];
  } else {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) {
      F[n] = sl * sr * uR[n] - sl * sr * uL[n] + sr * fluxL[n] - sl * fluxR[n];
      F[n] *= rcp(sr - sl);
    }
    F[v::ENG] = sl * sr * uR[v::ENG] - sl * sr * uL[v::ENG] + sr * fluxL[v::ENG] - sl * fluxR[v::ENG];
    F[v::ENG] *= rcp(sr - sl);
  }
}

// TVDLF / Rusanov (tvdlfMHD.hpp:140-232)
template <int D, int DIR, typename T>
__device__ __forceinline__ void riemann_tvdlf(T gamma, T rgm1, const T* vL, const T* vR, RiemannOut<D, T>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  T vv[NV];
#pragma unroll
  for (int n = 0; n < NV; n++) vv[n] = T(0.5) * (vL[n] + vR[n]);
  const T gpr = gamma * vv[v::PRS];
  T Bt2 = T(0) + vv[d::BXt] * vv[d::BXt];
  if constexpr (D == 3) Bt2 = Bt2 + vv[d::BXb] * vv[d::BXb];
  const T B2 = Bt2 + vv[d::BXn] * vv[d::BXn];
  T cRL = gpr - B2;
  cRL = cRL + B2 + sqr(cRL * cRL + T(4) * gpr * Bt2);
  cRL = sqr(dv(T(0.5) * cRL, vv[v::RHO]));
  const T cmax = fmax(fabs(vv[d::Xn] + cRL), fabs(vv[d::Xn] - cRL));
  r.sl = -cmax;
  r.sr = cmax;
  r.cmax = cmax;
  T fluxL[NV], fluxR[NV];
  const T gm1 = gamma - T(1);
  prim_to_cons<D, 2>(gm1, r.uL, vL, rgm1);
  prim_to_cons<D, 2>(gm1, r.uR, vR, rgm1);
  phys_flux<D, DIR>(fluxL, vL, r.uL);
  phys_flux<D, DIR>(fluxR, vR, r.uR);
#pragma unroll
  for (int n = 0; n < NV; n++) r.F[n] = T(0.5) * (fluxL[n] + fluxR[n] + cmax * (r.uL[n] - r.uR[n]));
}

// Roe with the entropy fix (roeMHD.hpp:175-650, energy equation branch)
template <int D, int DIR, typename T>
__device__ __forceinline__ void riemann_roe(T gamma, T rgm1, const T* vL, const T* vR, RiemannOut<D, T>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int RHO = v::RHO, ENG = v::ENG, PRS = v::PRS, Xn = d::Xn, Xt = d::Xt, Xb = d::Xb;
  constexpr int BXn = d::BXn, BXt = d::BXt, BXb = d::BXb;
  constexpr int KFASTM = 0, KFASTP = 1, KDIVB = 2, KENTRP = 3, KSLOWM = 4, KSLOWP = 5, KALFVM = 6,
                KALFVP = 7;
  const T delta = T(1.e-6);
  T dV[NV], dU[NV], fluxL[NV], fluxR[NV];
  T Rc[NV][NV];
  T* uL = r.uL;
  T* uR = r.uR;
#pragma unroll
  for (int n = 0; n < NV; n++) dV[n] = vR[n] - vL[n];
  const T gm1 = gamma - T(1);
  prim_to_cons<D, 2>(gm1, uL, vL, rgm1);
  prim_to_cons<D, 2>(gm1, uR, vR, rgm1);
#pragma unroll
  for (int n = 0; n < NV; n++) dU[n] = uR[n] - uL[n];
  phys_flux<D, DIR>(fluxL, vL, uL);
  phys_flux<D, DIR>(fluxR, vR, uR);
#pragma unroll
  for (int a = 0; a < NV; a++)
#pragma unroll
    for (int b = 0; b < NV; b++) Rc[a][b] = T(0);
  const T sqr_rho_L = sqr(vL[RHO]);
  const T sqr_rho_R = sqr(vR[RHO]);
  const T sl = dv(sqr_rho_L, sqr_rho_L + sqr_rho_R);
  const T sr = dv(sqr_rho_R, sqr_rho_L + sqr_rho_R);
  const T rho = sr * vL[RHO] + sl * vR[RHO];
  const T sqrt_rho = sqr(rho);
  T w = T(0), Bz = T(0), bz = T(0);
  const T u = sl * vL[Xn] + sr * vR[Xn];
  const T vv = sl * vL[Xt] + sr * vR[Xt];
  if constexpr (D == 3) w = sl * vL[Xb] + sr * vR[Xb];
  const T Bx = sr * vL[BXn] + sl * vR[BXn];
  const T By = sr * vL[BXt] + sl * vR[BXt];
  if constexpr (D == 3) Bz = sr * vL[BXb] + sl * vR[BXb];
  const T sBx = (Bx >= T(0) ? T(1) : T(-1));
  const T bx = dv(Bx, sqrt_rho);
  const T by = dv(By, sqrt_rho);
  if constexpr (D == 3) bz = dv(Bz, sqrt_rho);
  T bt2 = T(0) + by * by;
  if constexpr (D == 3) bt2 = bt2 + bz * bz;
  const T b2 = bx * bx + bt2;
  const T Btmag = sqr(bt2 * rho);
  T X = dV[BXn] * dV[BXn] + dV[BXt] * dV[BXt];
  if constexpr (D == 3) X = X + dV[BXb] * dV[BXb];
  X = dv(X, (sqr_rho_L + sqr_rho_R) * (sqr_rho_L + sqr_rho_R) * T(2));
  T Bmag2L, Bmag2R, vdm, BdB, vel2;
  if constexpr (D == 3) {
    Bmag2L = sumsq<3>(vL[v::BX1], vL[v::BX2], vL[v::BX3]);
    Bmag2R = sumsq<3>(vR[v::BX1], vR[v::BX2], vR[v::BX3]);
    vdm = u * dU[Xn] + vv * dU[Xt] + w * dU[Xb];
    BdB = Bx * dU[BXn] + By * dU[BXt] + Bz * dU[BXb];
    vel2 = u * u + vv * vv + w * w;
  } else {
    Bmag2L = sumsq<2>(vL[v::BX1], vL[v::BX2], T(0));
    Bmag2R = sumsq<2>(vR[v::BX1], vR[v::BX2], T(0));
    vdm = u * dU[Xn] + vv * dU[Xt];
    BdB = Bx * dU[BXn] + By * dU[BXt];
    vel2 = u * u + vv * vv;
  }
  const T pL = vL[PRS] + T(0.5) * Bmag2L;
  const T pR = vR[PRS] + T(0.5) * Bmag2R;
  dV[PRS] = (gamma - T(1)) * ((T(0.5) * vel2 - X) * dV[RHO] - vdm + dU[ENG] - BdB);
  const T HL = dv(uL[ENG] + pL, vL[RHO]);
  const T HR = dv(uR[ENG] + pR, vR[RHO]);
  const T H = sl * HL + sr * HR;
  const T Hgas = H - b2;
  const T a2 = (T(2) - gamma) * X + (gamma - T(1)) * (Hgas - T(0.5) * vel2);
  T scrh = a2 - b2;
  const T ca2 = bx * bx;
  scrh = scrh * scrh + T(4) * bt2 * a2;
  scrh = sqr(scrh);
  const T cf2 = T(0.5) * (a2 + b2 + scrh);
  const T cs2 = dv(a2 * ca2, cf2);
  const T cf = sqr(cf2);
  const T cs = sqr(cs2);
  const T ca = sqr(ca2);
  const T a = sqr(a2);
  T alpha_f, alpha_s;
  if (cf == cs) {
    alpha_f = T(1);
    alpha_s = T(0);
  } else if (a <= cs) {
    alpha_f = T(0);
    alpha_s = T(1);
  } else if (cf <= a) {
    alpha_f = T(1);
    alpha_s = T(0);
  } else {
    scrh = rcp(cf2 - cs2);
    alpha_f = (a2 - cs2) * scrh;
    alpha_s = (cf2 - a2) * scrh;
    alpha_f = fmax(T(0), alpha_f);
    alpha_s = fmax(T(0), alpha_s);
    alpha_f = sqr(alpha_f);
    alpha_s = sqr(alpha_s);
  }
  T beta_y, beta_z = T(0);
  if constexpr (D == 2) {
    beta_y = (Btmag > T(1.e-9)) ? ((By) >= T(0) ? T(1) : T(-1)) : T(1);
  } else {
    if (Btmag > T(1.e-9)) {
      beta_y = dv(By, Btmag);
      beta_z = dv(Bz, Btmag);
    } else {
      beta_z = beta_y = T(1);
    }
  }
  T lambda[NV], alambda[NV], eta[NV];
  T beta_dv = T(0) + beta_y * dV[Xt];
  T beta_dB = T(0) + beta_y * dV[BXt];
  T beta_v = T(0) + beta_y * vv;
  if constexpr (D == 3) {
    beta_dv = beta_dv + beta_z * dV[Xb];
    beta_dB = beta_dB + beta_z * dV[BXb];
    beta_v = beta_v + beta_z * w;
  }
  const T half_a2 = dv(T(0.5), a2);
  int kk = KFASTM;
  lambda[kk] = u - cf;
  scrh = alpha_s * cs * sBx;
  Rc[RHO][kk] = alpha_f;
  Rc[Xn][kk] = alpha_f * lambda[kk];
  Rc[Xt][kk] = alpha_f * vv + scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_f * w + scrh * beta_z;
  Rc[BXt][kk] = dv(alpha_s * a * beta_y, sqrt_rho);
  if constexpr (D == 3) Rc[BXb][kk] = dv(alpha_s * a * beta_z, sqrt_rho);
  Rc[ENG][kk] = alpha_f * (Hgas - u * cf) + scrh * beta_v + dv(alpha_s * a * Btmag, sqrt_rho);
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]);
  eta[kk] += rho * scrh * beta_dv - rho * alpha_f * cf * dV[Xn] + sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= half_a2;

  kk = KFASTP;
  lambda[kk] = u + cf;
  Rc[RHO][kk] = alpha_f;
  Rc[Xn][kk] = alpha_f * lambda[kk];
  Rc[Xt][kk] = alpha_f * vv - scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_f * w - scrh * beta_z;
  Rc[BXt][kk] = Rc[BXt][KFASTM];
  if constexpr (D == 3) Rc[BXb][kk] = Rc[BXb][KFASTM];
  Rc[ENG][kk] = alpha_f * (Hgas + u * cf) - scrh * beta_v + dv(alpha_s * a * Btmag, sqrt_rho);
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv + rho * alpha_f * cf * dV[Xn] +
            sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= half_a2;

  kk = KENTRP;
  lambda[kk] = u;
  Rc[RHO][kk] = T(1);
  Rc[Xn][kk] = u;
  Rc[Xt][kk] = vv;
  if constexpr (D == 3) Rc[Xb][kk] = w;
  Rc[ENG][kk] = T(0.5) * vel2 + dv(gamma - T(2), gamma - T(1)) * X;
  eta[kk] = dv((a2 - X) * dV[RHO] - dV[PRS], a2);

  kk = KDIVB;
  lambda[kk] = u;
  eta[kk] = T(0);

  scrh = alpha_f * cf * sBx;
  kk = KSLOWM;
  lambda[kk] = u - cs;
  Rc[RHO][kk] = alpha_s;
  Rc[Xn][kk] = alpha_s * lambda[kk];
  Rc[Xt][kk] = alpha_s * vv - scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_s * w - scrh * beta_z;
  Rc[BXt][kk] = dv(-alpha_f * a * beta_y, sqrt_rho);
  if constexpr (D == 3) Rc[BXb][kk] = dv(-alpha_f * a * beta_z, sqrt_rho);
  Rc[ENG][kk] = alpha_s * (Hgas - u * cs) - scrh * beta_v - dv(alpha_f * a * Btmag, sqrt_rho);
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv - rho * alpha_s * cs * dV[Xn] -
            sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= half_a2;

  kk = KSLOWP;
  lambda[kk] = u + cs;
  Rc[RHO][kk] = alpha_s;
  Rc[Xn][kk] = alpha_s * lambda[kk];
  Rc[Xt][kk] = alpha_s * vv + scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_s * w + scrh * beta_z;
  Rc[BXt][kk] = Rc[BXt][KSLOWM];
  if constexpr (D == 3) Rc[BXb][kk] = Rc[BXb][KSLOWM];
  Rc[ENG][kk] = alpha_s * (Hgas + u * cs) + scrh * beta_v - dv(alpha_f * a * Btmag, sqrt_rho);
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv + rho * alpha_s * cs * dV[Xn] -
            sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= half_a2;

  if constexpr (D == 3) {
    kk = KALFVM;
    lambda[kk] = u - ca;
    Rc[Xt][kk] = -rho * beta_z;
    Rc[Xb][kk] = +rho * beta_y;
    Rc[BXt][kk] = -sBx * sqrt_rho * beta_z;
    Rc[BXb][kk] = sBx * sqrt_rho * beta_y;
    Rc[ENG][kk] = -rho * (vv * beta_z - w * beta_y);
    eta[kk] = +beta_y * dV[Xb] - beta_z * dV[Xt] + dv(sBx, sqrt_rho) * (beta_y * dV[BXb] - beta_z * dV[BXt]);
    eta[kk] *= T(0.5);
    kk = KALFVP;
    lambda[kk] = u + ca;
    Rc[Xt][kk] = -Rc[Xt][KALFVM];
    Rc[Xb][kk] = -Rc[Xb][KALFVM];
    Rc[BXt][kk] = Rc[BXt][KALFVM];
    Rc[BXb][kk] = Rc[BXb][KALFVM];
    Rc[ENG][kk] = -Rc[ENG][KALFVM];
    eta[kk] = -beta_y * dV[Xb] + beta_z * dV[Xt] + dv(sBx, sqrt_rho) * (beta_y * dV[BXb] - beta_z * dV[BXt]);
    eta[kk] *= T(0.5);
  }
  r.cmax = fabs(u) + cf;
  r.sl = lambda[KFASTM];
  r.sr = lambda[KFASTP];
#pragma unroll
  for (int n = 0; n < NV; n++) alambda[n] = fabs(lambda[n]);
  const T hd = T(0.5) * delta, qd = T(0.25) * delta;
  if (alambda[KFASTM] < hd) alambda[KFASTM] = dv(lambda[KFASTM] * lambda[KFASTM], delta) + qd;
  if (alambda[KFASTP] < hd) alambda[KFASTP] = dv(lambda[KFASTP] * lambda[KFASTP], delta) + qd;
  if (alambda[KSLOWM] < hd) alambda[KSLOWM] = dv(lambda[KSLOWM] * lambda[KSLOWM], delta) + qd;
  if (alambda[KSLOWP] < hd) alambda[KSLOWP] = dv(lambda[KSLOWP] * lambda[KSLOWP], delta) + qd;
#pragma unroll
  for (int n1 = 0; n1 < NV; n1++) {
    T s = T(0);
#pragma unroll
    for (int n2 = 0; n2 < NV; n2++) s += alambda[n2] * eta[n2] * Rc[n1][n2];
    r.F[n1] = T(0.5) * (fluxL[n1] + fluxR[n1] - s);
  }
}

// rgm1 = RN(1 / (gamma - 1)), used by the FP64 path
template <int D, int DIR, int SOLVER, typename T>
__device__ __forceinline__ void riemann(T gamma, T rgm1, const T* vL, const T* vR, RiemannOut<D, T>& r) {
  if constexpr (SOLVER == kHLLD) riemann_hlld<D, DIR>(gamma, rgm1, vL, vR, r);
  if constexpr (SOLVER == kHLL) riemann_hll<D, DIR>(gamma, rgm1, vL, vR, r);
  if constexpr (SOLVER == kROE) riemann_roe<D, DIR>(gamma, rgm1, vL, vR, r);
  if constexpr (SOLVER == kTVDLF) riemann_tvdlf<D, DIR>(gamma, rgm1, vL, vR, r);
}

}  // namespace idfx
