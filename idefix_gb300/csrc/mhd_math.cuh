// Device arithmetic of the ideal-MHD stage: cons/prim, physical flux, slope
// limiters, face reconstruction and the HLLD / HLL / Roe / TVDLF Riemann
// solvers.  FP64, compiled with --fmad=false: every expression keeps the
// operation order of the reference so that results are bit-identical to it
// (the reference's GPU CI also disables contraction, pytools/idfx_test.py:121).
//
// D is the number of dimensions (= components, 2 or 3).  Variable order
// follows src/idefix.hpp:74-108: RHO, MX1..MXD, ENG(=PRS), BX1..BXD.
#pragma once
#include <cstdint>

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

// sum of squares of the first D entries starting at a, in reference order
template <int D>
__device__ __forceinline__ double sumsq(double a, double b, double c) {
  double s = a * a + b * b;
  if constexpr (D == 3) s = s + c * c;
  return s;
}

// ---------------------------------------------------------------------------
// cons <-> prim (convertConsToPrim.hpp:15-100; eos_adiabatic.hpp:38-45)
// gm1 = gamma - 1.0, evaluated once on the host
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void prim_to_cons(double gm1, double* U, const double* V) {
  using v = Var<D>;
  U[v::RHO] = V[v::RHO];
  U[v::MX1] = V[v::MX1] * V[v::RHO];
  U[v::MX2] = V[v::MX2] * V[v::RHO];
  if constexpr (D == 3) U[v::MX3] = V[v::MX3] * V[v::RHO];
  U[v::BX1] = V[v::BX1];
  U[v::BX2] = V[v::BX2];
  if constexpr (D == 3) U[v::BX3] = V[v::BX3];
  double kin, mag;
  if constexpr (D == 3) {
    kin = sumsq<3>(V[v::MX1], V[v::MX2], V[v::MX3]);
    mag = sumsq<3>(U[v::BX1], U[v::BX2], U[v::BX3]);
  } else {
    kin = sumsq<2>(V[v::MX1], V[v::MX2], 0.0);
    mag = sumsq<2>(U[v::BX1], U[v::BX2], 0.0);
  }
  U[v::ENG] = V[v::PRS] / gm1 + 0.5 * V[v::RHO] * kin + 0.5 * mag;
}

template <int D>
__device__ __forceinline__ void cons_to_prim(double gm1, double* V, const double* U) {
  using v = Var<D>;
  V[v::RHO] = U[v::RHO];
  V[v::MX1] = U[v::MX1] / U[v::RHO];
  V[v::MX2] = U[v::MX2] / U[v::RHO];
  if constexpr (D == 3) V[v::MX3] = U[v::MX3] / U[v::RHO];
  V[v::BX1] = U[v::BX1];
  V[v::BX2] = U[v::BX2];
  if constexpr (D == 3) V[v::BX3] = U[v::BX3];
  double m2, b2;
  if constexpr (D == 3) {
    m2 = sumsq<3>(U[v::MX1], U[v::MX2], U[v::MX3]);
    b2 = sumsq<3>(U[v::BX1], U[v::BX2], U[v::BX3]);
  } else {
    m2 = sumsq<2>(U[v::MX1], U[v::MX2], 0.0);
    b2 = sumsq<2>(U[v::BX1], U[v::BX2], 0.0);
  }
  double kin = 0.5 / U[v::RHO] * m2;
  double mag = 0.5 * b2;
  V[v::PRS] = (U[v::ENG] - kin - mag) * gm1;
  // floor; the reference's energy repair only touches a discarded local copy
  if (V[v::PRS] <= 0.0) V[v::PRS] = kSmallPressureFix;
}

// physical MHD flux along DIR (flux.hpp:28-95); U is read before F is written
template <int D, int DIR>
__device__ __forceinline__ void phys_flux(double* F, const double* V, const double* U) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  const double uXn = U[d::Xn], uE = U[v::ENG];
  const double u1 = U[v::MX1], u2 = U[v::MX2];
  double u3 = 0.0;
  if constexpr (D == 3) u3 = U[v::MX3];
  F[v::RHO] = uXn;
  F[v::MX1] = u1 * V[d::Xn] - V[d::BXn] * V[v::BX1];
  F[v::MX2] = u2 * V[d::Xn] - V[d::BXn] * V[v::BX2];
  if constexpr (D == 3) F[v::MX3] = u3 * V[d::Xn] - V[d::BXn] * V[v::BX3];
  F[d::BXn] = 0.0;
  F[d::BXt] = V[d::Xn] * V[d::BXt] - V[d::BXn] * V[d::Xt];
  if constexpr (D == 3) F[d::BXb] = V[d::Xn] * V[d::BXb] - V[d::BXn] * V[d::Xb];
  double Bmag2, vB;
  if constexpr (D == 3) {
    Bmag2 = sumsq<3>(V[v::BX1], V[v::BX2], V[v::BX3]);
    vB = V[v::MX1] * V[v::BX1] + V[v::MX2] * V[v::BX2] + V[v::MX3] * V[v::BX3];
  } else {
    Bmag2 = sumsq<2>(V[v::BX1], V[v::BX2], 0.0);
    vB = V[v::MX1] * V[v::BX1] + V[v::MX2] * V[v::BX2];
  }
  const double ptot = V[v::PRS] + 0.5 * Bmag2;
  F[v::ENG] = (uE + ptot) * V[d::Xn] - V[d::BXn] * (vB);
  F[d::Xn] += ptot;
}

// ---------------------------------------------------------------------------
// slope limiters (slopeLimiter.hpp)
// ---------------------------------------------------------------------------
// The reference MinModLim shadows its result variable and always returns 0
// (slopeLimiter.hpp:16-23); every "revert to minmod" path therefore adds 0.
__device__ __forceinline__ double lim_minmod(double, double) { return 0.0; }

__device__ __forceinline__ double lim_vanleer(double dvp, double dvm) {  // :54-57
  return (dvp * dvm > 0.0 ? 2.0 * dvp * dvm / (dvp + dvm) : 0.0);
}

__device__ __forceinline__ double lim_mc(double dvp, double dvm) {  // :68-76
  double dq = 0;
  if (dvp * dvm > 0.0) {
    double dqc = 0.5 * (dvp + dvm);
    double d2q = 2.0 * (fabs(dvp) < fabs(dvm) ? dvp : dvm);
    dq = fabs(d2q) < fabs(dqc) ? d2q : dqc;
  }
  return dq;
}

__device__ __forceinline__ double lim_limo3(double dvp, double dvm, double dx) {  // :25-52
  const double r = 0.1, eps = 1.e-12;
  double th = dvm / (dvp + 1.e-16);
  double q = (2.0 + th) / 3.0;
  double a = fmin(1.5, 2.0 * th);
  a = fmin(q, a);
  double b = fmax(-0.5 * th, a);
  double c = fmin(q, b);
  double psi = fmax(0.0, c);
  double eta = r * dx;
  eta = (dvm * dvm + dvp * dvp) / (eta * eta);
  double lim;
  if (eta <= 1.0 - eps) {
    lim = q;
  } else if (eta >= 1.0 + eps) {
    lim = psi;
  } else {
    psi = (1.0 - (eta - 1.0) / eps) * q + (1.0 + (eta - 1.0) / eps) * psi;
    lim = 0.5 * psi;
  }
  return lim;
}

__device__ __forceinline__ int sgn(double v) { return (0.0 < v) - (v < 0.0); }

__device__ __forceinline__ void ppm_limit_face(double vm1, double v0, double vp1, double vp2,
                                               double& vph) {  // :121-140
  if ((vp1 - vph) * (vph - v0) < 0.0) {
    const double deltaL = (vm1 - 2 * v0 + vp1);
    const double deltaC = 3 * (v0 - 2 * vph + vp1);
    const double deltaR = (v0 - 2 * vp1 + vp2);
    double delta = 0.0;
    if (sgn(deltaL) == sgn(deltaC) && sgn(deltaR) == sgn(deltaC)) {
      const double C = 1.25;
      delta = C * fmin(fabs(deltaL), fabs(deltaR));
      delta = sgn(deltaC) * fmin(delta, fabs(deltaC));
    }
    vph = 0.5 * (v0 + vp1) - delta / 6.0;
  }
}

__device__ __forceinline__ void ppm_states(double vm2, double vm1, double v0, double vp1, double vp2,
                                           double& vl, double& vr) {  // :142-191
  const int n = 2;
  vr = 7.0 / 12.0 * (v0 + vp1) - 1.0 / 12.0 * (vm1 + vp2);
  vl = 7.0 / 12.0 * (vm1 + v0) - 1.0 / 12.0 * (vm2 + vp1);
  ppm_limit_face(vm2, vm1, v0, vp1, vl);
  ppm_limit_face(vm1, v0, vp1, vp2, vr);
  double d2qf = 6.0 * (vl + vr - 2.0 * v0);
  double d2qc0 = vm1 + vp1 - 2.0 * v0;
  double d2qcp1 = v0 + vp2 - 2.0 * vp1;
  double d2qcm1 = vm2 + v0 - 2.0 * vm1;
  double d2q = 0.0;
  if (sgn(d2qf) == sgn(d2qc0) && sgn(d2qf) == sgn(d2qcp1) && sgn(d2qf) == sgn(d2qcm1)) {
    const double C = 1.25;
    d2q = fmin(fabs(d2qc0), fabs(d2qcp1));
    d2q = C * fmin(fabs(d2qcm1), d2q);
    d2q = sgn(d2qf) * fmin(fabs(d2qf), d2q);
  }
  double qmax = fmax(fmax(fabs(vm1), fabs(v0)), fabs(vp1));
  double rho = 0.0;
  if (fabs(d2qf) > 1e-12 * qmax) rho = d2q / d2qf;
  if (((vr - v0) * (v0 - vl) <= 0) || (vm1 - v0) * (v0 - vp1) <= 0) {
    if (rho <= (1.0 - 1e-12)) {
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
template <int ORDER>
struct Recon {
  static constexpr int H = (ORDER == 1 ? 0 : (ORDER == 4 ? 2 : 1));
  __device__ __forceinline__ static void cell(const double* w, double dx, bool pos, double& vl,
                                              double& vr) {
    if constexpr (ORDER == 1) {
      vl = w[0];
      vr = w[0];
    } else if constexpr (ORDER == 2) {
      const double dvm = w[1] - w[0];
      const double dvp = w[2] - w[1];
      const double dv = lim_vanleer(dvp, dvm);
      vr = w[1] + 0.5 * dv;
      vl = w[1] - 0.5 * dv;
    } else if constexpr (ORDER == 3) {
      const double dm = w[1] - w[0];
      const double dp = w[2] - w[1];
      double dv = dp * lim_limo3(dp, dm, dx);
      vr = w[1] + 0.5 * dv;
      if (pos && vr <= 0.0) {
        dv = lim_minmod(dp, dm);
        vr = w[1] + 0.5 * dv;
      }
      dv = dm * lim_limo3(dm, dp, dx);
      vl = w[1] - 0.5 * dv;
      if (pos && vl <= 0.0) {
        dv = lim_minmod(dp, dm);
        vl = w[1] - 0.5 * dv;
      }
    } else {
      ppm_states(w[0], w[1], w[2], w[3], w[4], vl, vr);
      if (pos && vr <= 0.0) {
        double dv = lim_vanleer(w[3] - w[2], w[2] - w[1]);
        vr = w[2] + 0.5 * dv;
      }
      if (pos && vl <= 0.0) {
        double dv = lim_vanleer(w[3] - w[2], w[2] - w[1]);
        vl = w[2] - 0.5 * dv;
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Riemann solvers.  In: face states vL, vR (BXn already set from Vs).
// Out: F, cmax, sl/sr (for uct_hll(d)), uL/uR (for uct_hlld).
// ---------------------------------------------------------------------------
enum Solver { kHLLD = 0, kHLL = 1, kROE = 2, kTVDLF = 3 };

template <int D>
struct RiemannOut {
  double F[Var<D>::NV];
  double uL[Var<D>::NV], uR[Var<D>::NV];
  double cmax, sl, sr;
};

// fast magnetosonic speed of one face state (hlldMHD.hpp:205-238)
template <int D, int DIR>
__device__ __forceinline__ double fast_speed(double gamma, const double* v) {
  using vv = Var<D>;
  using d = Dir<D, DIR>;
  const double gpr = gamma * v[vv::PRS];
  const double b1 = v[d::BXn];
  const double b2 = v[d::BXt];
  double b3 = 0.0;
  if constexpr (D == 3) b3 = v[d::BXb];
  const double Btmag2 = b2 * b2 + b3 * b3;
  const double Bmag2 = b1 * b1 + Btmag2;
  double c = gpr - Bmag2;
  c = gpr + Bmag2 + sqrt(c * c + 4.0 * gpr * Btmag2);
  c = sqrt(0.5 * c / v[vv::RHO]);
  return c;
}

template <int D>
__device__ __forceinline__ double half_b2(const double* v) {
  using vv = Var<D>;
  if constexpr (D == 3) return 0.5 * (sumsq<3>(v[vv::BX1], v[vv::BX2], v[vv::BX3]));
  return 0.5 * (sumsq<2>(v[vv::BX1], v[vv::BX2], 0.0));
}

// HLLD (Miyoshi & Kusano 2005) with the reference's HLLC fall-back near
// degeneracy (hlldMHD.hpp:147-457, energy equation branch)
template <int D, int DIR>
__device__ __forceinline__ void riemann_hlld(double gamma, const double* vL, const double* vR,
                                             RiemannOut<D>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int RHO = v::RHO, ENG = v::ENG, Xn = d::Xn, Xt = d::Xt, Xb = d::Xb;
  constexpr int BXn = d::BXn, BXt = d::BXt, BXb = d::BXb;
  double* uL = r.uL;
  double* uR = r.uR;
  double fluxL[NV], fluxR[NV];
  const double cL = fast_speed<D, DIR>(gamma, vL);
  const double cR = fast_speed<D, DIR>(gamma, vR);
  const double cminL = vL[Xn] - cL, cmaxL = vL[Xn] + cL;
  const double cminR = vR[Xn] - cR, cmaxR = vR[Xn] + cR;
  const double sl = fmin(cminL, cminR);
  const double sr = fmax(cmaxL, cmaxR);
  r.sl = sl;
  r.sr = sr;
  r.cmax = fmax(fabs(sl), fabs(sr));
  const double gm1 = gamma - 1.0;
  prim_to_cons<D>(gm1, uL, vL);
  prim_to_cons<D>(gm1, uR, vR);
  phys_flux<D, DIR>(fluxL, vL, uL);
  phys_flux<D, DIR>(fluxR, vR, uR);
  const double ptL = vL[v::PRS] + half_b2<D>(vL);
  const double ptR = vR[v::PRS] + half_b2<D>(vR);
  double* F = r.F;
  if (sl > 0) {
#pragma unroll
    for (int n = 0; n < NV; n++) F[n] = fluxL[n];
    return;
  }
  if (sr < 0) {
#pragma unroll
    for (int n = 0; n < NV; n++) F[n] = fluxR[n];
    return;
  }
  double usL[NV], usR[NV];
  double scrh, scrhL, scrhR;
  double vsL = 0, vsR = 0, wsL = 0, wsR = 0;
  int revert_to_hllc = 0;
  scrh = 1.0 / (sr - sl);
  const double Bx = (sr * vR[BXn] - sl * vL[BXn]) * scrh;
  const double sBx = (Bx > 0.0 ? 1.0 : -1.0);
  const double duL = sl - vL[Xn];
  const double duR = sr - vR[Xn];
  scrh = 1.0 / (duR * uR[RHO] - duL * uL[RHO]);
  const double SM = (duR * uR[Xn] - duL * uL[Xn] - ptR + ptL) * scrh;
  double pts = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR + vL[RHO] * vR[RHO] * duR * duL * (vR[Xn] - vL[Xn]);
  pts *= scrh;
  usL[RHO] = uL[RHO] * duL / (sl - SM);
  usR[RHO] = uR[RHO] * duR / (sr - SM);
  const double sqrL = sqrt(usL[RHO]);
  const double sqrR = sqrt(usR[RHO]);
  double S1L = SM - fabs(Bx) / sqrL;
  double S1R = SM + fabs(Bx) / sqrR;
  if ((S1L - sl) < 1.e-4 * (SM - sl)) revert_to_hllc = 1;
  if ((S1R - sr) > -1.e-4 * (sr - SM)) revert_to_hllc = 1;
  if (revert_to_hllc) {
    scrh = 1.0 / (sr - sl);
    double Uhll[NV];
#pragma unroll
    for (int n = 0; n < NV; n++) {
      Uhll[n] = sr * uR[n] - sl * uL[n] + fluxL[n] - fluxR[n];
      Uhll[n] *= scrh;
    }
    usL[BXn] = usR[BXn] = Uhll[BXn];
    usL[BXt] = usR[BXt] = Uhll[BXt];
    if constexpr (D == 3) usL[BXb] = usR[BXb] = Uhll[BXb];
    S1L = S1R = SM;
  } else {
    scrhL = (uL[RHO] * duL * duL - Bx * Bx) / (uL[RHO] * duL * (sl - SM) - Bx * Bx);
    scrhR = (uR[RHO] * duR * duR - Bx * Bx) / (uR[RHO] * duR * (sr - SM) - Bx * Bx);
    usL[BXn] = Bx;
    usL[BXt] = uL[BXt] * scrhL;
    if constexpr (D == 3) usL[BXb] = uL[BXb] * scrhL;
    usR[BXn] = Bx;
    usR[BXt] = uR[BXt] * scrhR;
    if constexpr (D == 3) usR[BXb] = uR[BXb] * scrhR;
  }
  scrhL = Bx / (uL[RHO] * duL);
  scrhR = Bx / (uR[RHO] * duR);
  vsL = vL[Xt] - scrhL * (usL[BXt] - uL[BXt]);
  vsR = vR[Xt] - scrhR * (usR[BXt] - uR[BXt]);
  if constexpr (D == 3) {
    wsL = vL[Xb] - scrhL * (usL[BXb] - uL[BXb]);
    wsR = vR[Xb] - scrhR * (usR[BXb] - uR[BXb]);
  }
  usL[Xn] = usL[RHO] * SM;
  usR[Xn] = usR[RHO] * SM;
  usL[Xt] = usL[RHO] * vsL;
  usR[Xt] = usR[RHO] * vsR;
  if constexpr (D == 3) {
    usL[Xb] = usL[RHO] * wsL;
    usR[Xb] = usR[RHO] * wsR;
  }
  {
    double a = vL[Xn] * Bx + vL[Xt] * uL[BXt];
    if constexpr (D == 3) a = a + vL[Xb] * uL[BXb];
    double b = SM * Bx + vsL * usL[BXt];
    if constexpr (D == 3) b = b + wsL * usL[BXb];
    scrhL = a;
    scrhL -= b;
  }
  usL[ENG] = duL * uL[ENG] - ptL * vL[Xn] + pts * SM + Bx * scrhL;
  usL[ENG] /= sl - SM;
  {
    double a = vR[Xn] * Bx + vR[Xt] * uR[BXt];
    if constexpr (D == 3) a = a + vR[Xb] * uR[BXb];
    double b = SM * Bx + vsR * usR[BXt];
    if constexpr (D == 3) b = b + wsR * usR[BXb];
    scrhR = a;
    scrhR -= b;
  }
  usR[ENG] = duR * uR[ENG] - ptR * vR[Xn] + pts * SM + Bx * scrhR;
  usR[ENG] /= sr - SM;

  if (S1L >= 0.0) {
#pragma unroll
    for (int n = 0; n < NV; n++) F[n] = fluxL[n] + sl * (usL[n] - uL[n]);
  } else if (S1R <= 0.0) {
#pragma unroll
    for (int n = 0; n < NV; n++) F[n] = fluxR[n] + sr * (usR[n] - uR[n]);
  } else {
    double vss = 0, wss = 0;
    double ussl[NV], ussr[NV];
    ussl[RHO] = usL[RHO];
    ussr[RHO] = usR[RHO];
    vss = sqrL * vsL + sqrR * vsR + (usR[BXt] - usL[BXt]) * sBx;
    vss /= sqrL + sqrR;
    if constexpr (D == 3) {
      wss = sqrL * wsL + sqrR * wsR + (usR[BXb] - usL[BXb]) * sBx;
      wss /= sqrL + sqrR;
    }
    ussl[Xn] = ussl[RHO] * SM;
    ussr[Xn] = ussr[RHO] * SM;
    ussl[Xt] = ussl[RHO] * vss;
    ussr[Xt] = ussr[RHO] * vss;
    if constexpr (D == 3) {
      ussl[Xb] = ussl[RHO] * wss;
      ussr[Xb] = ussr[RHO] * wss;
    }
    ussl[BXn] = ussr[BXn] = Bx;
    ussl[BXt] = sqrL * usR[BXt] + sqrR * usL[BXt] + sqrL * sqrR * (vsR - vsL) * sBx;
    ussl[BXt] /= sqrL + sqrR;
    ussr[BXt] = ussl[BXt];
    if constexpr (D == 3) {
      ussl[BXb] = sqrL * usR[BXb] + sqrR * usL[BXb] + sqrL * sqrR * (wsR - wsL) * sBx;
      ussl[BXb] /= sqrL + sqrR;
      ussr[BXb] = ussl[BXb];
    }
    {
      double a = SM * Bx + vsL * usL[BXt];
      if constexpr (D == 3) a = a + wsL * usL[BXb];
      double b = SM * Bx + vss * ussl[BXt];
      if constexpr (D == 3) b = b + wss * ussl[BXb];
      scrhL = a;
      scrhL -= b;
      a = SM * Bx + vsR * usR[BXt];
      if constexpr (D == 3) a = a + wsR * usR[BXb];
      b = SM * Bx + vss * ussr[BXt];
      if constexpr (D == 3) b = b + wss * ussr[BXb];
      scrhR = a;
      scrhR -= b;
    }
    ussl[ENG] = usL[ENG] - sqrL * scrhL * sBx;
    ussr[ENG] = usR[ENG] + sqrR * scrhR * sBx;
    if (SM >= 0.0) {
#pragma unroll
      for (int n = 0; n < NV; n++) F[n] = fluxL[n] + S1L * (ussl[n] - usL[n]) + sl * (usL[n] - uL[n]);
    } else {
#pragma unroll
      for (int n = 0; n < NV; n++) F[n] = fluxR[n] + S1R * (ussr[n] - usR[n]) + sr * (usR[n] - uR[n]);
    }
  }
}

// HLL (hllMHD.hpp:154-453; the Hall whistler term is not part of ideal MHD)
template <int D, int DIR>
__device__ __forceinline__ void riemann_hll(double gamma, const double* vL, const double* vR,
                                            RiemannOut<D>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  double* uL = r.uL;
  double* uR = r.uR;
  double fluxL[NV], fluxR[NV];
  const double cL = fast_speed<D, DIR>(gamma, vL);
  const double cR = fast_speed<D, DIR>(gamma, vR);
  const double cminL = vL[d::Xn] - cL, cmaxL = vL[d::Xn] + cL;
  const double cminR = vR[d::Xn] - cR, cmaxR = vR[d::Xn] + cR;
  const double sl = fmin(cminL, cminR);
  const double sr = fmax(cmaxL, cmaxR);
  r.sl = sl;
  r.sr = sr;
  r.cmax = fmax(fabs(sl), fabs(sr));
  const double gm1 = gamma - 1.0;
  prim_to_cons<D>(gm1, uL, vL);
  prim_to_cons<D>(gm1, uR, vR);
  phys_flux<D, DIR>(fluxL, vL, uL);
  phys_flux<D, DIR>(fluxR, vR, uR);
  double* F = r.F;
  if (sl > 0) {
#pragma unroll
    for (int n = 0; n <= D; n++) F[n] = fluxL[n];
  } else if (sr < 0) {
#pragma unroll
    for (int n = 0; n <= D; n++) F[n] = fluxR[n];
  } else {
#pragma unroll
    for (int n = 0; n <= D; n++)
      F[n] = (sl * sr * uR[n] - sl * sr * uL[n] + sr * fluxL[n] - sl * fluxR[n]) / (sr - sl);
  }
  if (sl > 0) {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) F[n] = fluxL[n];
    F[v::ENG] = fluxL[v::ENG];
  } else if (sr < 0) {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) F[n] = fluxR[n];
    F[v::ENG] = fluxR[v::ENG];
  } else {
#pragma unroll
    for (int n = v::BX1; n < v::BX1 + D; n++) {
      F[n] = sl * sr * uR[n] - sl * sr * uL[n] + sr * fluxL[n] - sl * fluxR[n];
      F[n] *= (1.0 / (sr - sl));
    }
    F[v::ENG] = sl * sr * uR[v::ENG] - sl * sr * uL[v::ENG] + sr * fluxL[v::ENG] - sl * fluxR[v::ENG];
    F[v::ENG] *= (1.0 / (sr - sl));
  }
}

// TVDLF / Rusanov (tvdlfMHD.hpp:140-232)
template <int D, int DIR>
__device__ __forceinline__ void riemann_tvdlf(double gamma, const double* vL, const double* vR,
                                              RiemannOut<D>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  double vv[NV];
#pragma unroll
  for (int n = 0; n < NV; n++) vv[n] = 0.5 * (vL[n] + vR[n]);
  const double gpr = gamma * vv[v::PRS];
  double Bt2 = 0.0 + vv[d::BXt] * vv[d::BXt];
  if constexpr (D == 3) Bt2 = Bt2 + vv[d::BXb] * vv[d::BXb];
  const double B2 = Bt2 + vv[d::BXn] * vv[d::BXn];
  double cRL = gpr - B2;
  cRL = cRL + B2 + sqrt(cRL * cRL + 4.0 * gpr * Bt2);
  cRL = sqrt(0.5 * cRL / vv[v::RHO]);
  const double cmax = fmax(fabs(vv[d::Xn] + cRL), fabs(vv[d::Xn] - cRL));
  r.sl = -cmax;
  r.sr = cmax;
  r.cmax = cmax;
  double fluxL[NV], fluxR[NV];
  const double gm1 = gamma - 1.0;
  prim_to_cons<D>(gm1, r.uL, vL);
  prim_to_cons<D>(gm1, r.uR, vR);
  phys_flux<D, DIR>(fluxL, vL, r.uL);
  phys_flux<D, DIR>(fluxR, vR, r.uR);
#pragma unroll
  for (int n = 0; n < NV; n++) r.F[n] = 0.5 * (fluxL[n] + fluxR[n] + cmax * (r.uL[n] - r.uR[n]));
}

// Roe with the entropy fix (roeMHD.hpp:175-650, energy equation branch)
template <int D, int DIR>
__device__ __forceinline__ void riemann_roe(double gamma, const double* vL, const double* vR,
                                            RiemannOut<D>& r) {
  using v = Var<D>;
  using d = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int RHO = v::RHO, ENG = v::ENG, PRS = v::PRS, Xn = d::Xn, Xt = d::Xt, Xb = d::Xb;
  constexpr int BXn = d::BXn, BXt = d::BXt, BXb = d::BXb;
  constexpr int KFASTM = 0, KFASTP = 1, KDIVB = 2, KENTRP = 3, KSLOWM = 4, KSLOWP = 5, KALFVM = 6,
                KALFVP = 7;
  const double delta = 1.e-6;
  double dV[NV], dU[NV], fluxL[NV], fluxR[NV];
  double Rc[NV][NV];
  double* uL = r.uL;
  double* uR = r.uR;
#pragma unroll
  for (int n = 0; n < NV; n++) dV[n] = vR[n] - vL[n];
  const double gm1 = gamma - 1.0;
  prim_to_cons<D>(gm1, uL, vL);
  prim_to_cons<D>(gm1, uR, vR);
#pragma unroll
  for (int n = 0; n < NV; n++) dU[n] = uR[n] - uL[n];
  phys_flux<D, DIR>(fluxL, vL, uL);
  phys_flux<D, DIR>(fluxR, vR, uR);
#pragma unroll
  for (int a = 0; a < NV; a++)
#pragma unroll
    for (int b = 0; b < NV; b++) Rc[a][b] = 0;
  const double sqr_rho_L = sqrt(vL[RHO]);
  const double sqr_rho_R = sqrt(vR[RHO]);
  const double sl = sqr_rho_L / (sqr_rho_L + sqr_rho_R);
  const double sr = sqr_rho_R / (sqr_rho_L + sqr_rho_R);
  const double rho = sr * vL[RHO] + sl * vR[RHO];
  const double sqrt_rho = sqrt(rho);
  double w = 0, Bz = 0, bz = 0;
  const double u = sl * vL[Xn] + sr * vR[Xn];
  const double vv = sl * vL[Xt] + sr * vR[Xt];
  if constexpr (D == 3) w = sl * vL[Xb] + sr * vR[Xb];
  const double Bx = sr * vL[BXn] + sl * vR[BXn];
  const double By = sr * vL[BXt] + sl * vR[BXt];
  if constexpr (D == 3) Bz = sr * vL[BXb] + sl * vR[BXb];
  const double sBx = (Bx >= 0.0 ? 1.0 : -1.0);
  const double bx = Bx / sqrt_rho;
  const double by = By / sqrt_rho;
  if constexpr (D == 3) bz = Bz / sqrt_rho;
  double bt2 = 0.0 + by * by;
  if constexpr (D == 3) bt2 = bt2 + bz * bz;
  const double b2 = bx * bx + bt2;
  const double Btmag = sqrt(bt2 * rho);
  double X = dV[BXn] * dV[BXn] + dV[BXt] * dV[BXt];
  if constexpr (D == 3) X = X + dV[BXb] * dV[BXb];
  X /= (sqr_rho_L + sqr_rho_R) * (sqr_rho_L + sqr_rho_R) * 2.0;
  double Bmag2L, Bmag2R, vdm, BdB, vel2;
  if constexpr (D == 3) {
    Bmag2L = sumsq<3>(vL[v::BX1], vL[v::BX2], vL[v::BX3]);
    Bmag2R = sumsq<3>(vR[v::BX1], vR[v::BX2], vR[v::BX3]);
    vdm = u * dU[Xn] + vv * dU[Xt] + w * dU[Xb];
    BdB = Bx * dU[BXn] + By * dU[BXt] + Bz * dU[BXb];
    vel2 = u * u + vv * vv + w * w;
  } else {
    Bmag2L = sumsq<2>(vL[v::BX1], vL[v::BX2], 0.0);
    Bmag2R = sumsq<2>(vR[v::BX1], vR[v::BX2], 0.0);
    vdm = u * dU[Xn] + vv * dU[Xt];
    BdB = Bx * dU[BXn] + By * dU[BXt];
    vel2 = u * u + vv * vv;
  }
  const double pL = vL[PRS] + 0.5 * Bmag2L;
  const double pR = vR[PRS] + 0.5 * Bmag2R;
  dV[PRS] = (gamma - 1.0) * ((0.5 * vel2 - X) * dV[RHO] - vdm + dU[ENG] - BdB);
  const double HL = (uL[ENG] + pL) / vL[RHO];
  const double HR = (uR[ENG] + pR) / vR[RHO];
  const double H = sl * HL + sr * HR;
  const double Hgas = H - b2;
  const double a2 = (2.0 - gamma) * X + (gamma - 1.0) * (Hgas - 0.5 * vel2);
  double scrh = a2 - b2;
  const double ca2 = bx * bx;
  scrh = scrh * scrh + 4.0 * bt2 * a2;
  scrh = sqrt(scrh);
  const double cf2 = 0.5 * (a2 + b2 + scrh);
  const double cs2 = a2 * ca2 / cf2;
  const double cf = sqrt(cf2);
  const double cs = sqrt(cs2);
  const double ca = sqrt(ca2);
  const double a = sqrt(a2);
  double alpha_f, alpha_s;
  if (cf == cs) {
    alpha_f = 1.0;
    alpha_s = 0.0;
  } else if (a <= cs) {
    alpha_f = 0.0;
    alpha_s = 1.0;
  } else if (cf <= a) {
    alpha_f = 1.0;
    alpha_s = 0.0;
  } else {
    scrh = 1.0 / (cf2 - cs2);
    alpha_f = (a2 - cs2) * scrh;
    alpha_s = (cf2 - a2) * scrh;
    alpha_f = fmax(0.0, alpha_f);
    alpha_s = fmax(0.0, alpha_s);
    alpha_f = sqrt(alpha_f);
    alpha_s = sqrt(alpha_s);
  }
  double beta_y, beta_z = 0;
  if constexpr (D == 2) {
    beta_y = (Btmag > 1.e-9) ? ((By) >= 0.0 ? (1.0) : (-1.0)) : 1.0;
  } else {
    if (Btmag > 1.e-9) {
      beta_y = By / Btmag;
      beta_z = Bz / Btmag;
    } else {
      beta_z = beta_y = 1.0;
    }
  }
  double lambda[NV], alambda[NV], eta[NV];
  double beta_dv = 0.0 + beta_y * dV[Xt];
  double beta_dB = 0.0 + beta_y * dV[BXt];
  double beta_v = 0.0 + beta_y * vv;
  if constexpr (D == 3) {
    beta_dv = beta_dv + beta_z * dV[Xb];
    beta_dB = beta_dB + beta_z * dV[BXb];
    beta_v = beta_v + beta_z * w;
  }
  int kk = KFASTM;
  lambda[kk] = u - cf;
  scrh = alpha_s * cs * sBx;
  Rc[RHO][kk] = alpha_f;
  Rc[Xn][kk] = alpha_f * lambda[kk];
  Rc[Xt][kk] = alpha_f * vv + scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_f * w + scrh * beta_z;
  Rc[BXt][kk] = alpha_s * a * beta_y / sqrt_rho;
  if constexpr (D == 3) Rc[BXb][kk] = alpha_s * a * beta_z / sqrt_rho;
  Rc[ENG][kk] = alpha_f * (Hgas - u * cf) + scrh * beta_v + alpha_s * a * Btmag / sqrt_rho;
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]);
  eta[kk] += rho * scrh * beta_dv - rho * alpha_f * cf * dV[Xn] + sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KFASTP;
  lambda[kk] = u + cf;
  Rc[RHO][kk] = alpha_f;
  Rc[Xn][kk] = alpha_f * lambda[kk];
  Rc[Xt][kk] = alpha_f * vv - scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_f * w - scrh * beta_z;
  Rc[BXt][kk] = Rc[BXt][KFASTM];
  if constexpr (D == 3) Rc[BXb][kk] = Rc[BXb][KFASTM];
  Rc[ENG][kk] = alpha_f * (Hgas + u * cf) - scrh * beta_v + alpha_s * a * Btmag / sqrt_rho;
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv + rho * alpha_f * cf * dV[Xn] +
            sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KENTRP;
  lambda[kk] = u;
  Rc[RHO][kk] = 1.0;
  Rc[Xn][kk] = u;
  Rc[Xt][kk] = vv;
  if constexpr (D == 3) Rc[Xb][kk] = w;
  Rc[ENG][kk] = 0.5 * vel2 + (gamma - 2.0) / (gamma - 1.0) * X;
  eta[kk] = ((a2 - X) * dV[RHO] - dV[PRS]) / a2;

  kk = KDIVB;
  lambda[kk] = u;
  eta[kk] = 0.0;

  scrh = alpha_f * cf * sBx;
  kk = KSLOWM;
  lambda[kk] = u - cs;
  Rc[RHO][kk] = alpha_s;
  Rc[Xn][kk] = alpha_s * lambda[kk];
  Rc[Xt][kk] = alpha_s * vv - scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_s * w - scrh * beta_z;
  Rc[BXt][kk] = -alpha_f * a * beta_y / sqrt_rho;
  if constexpr (D == 3) Rc[BXb][kk] = -alpha_f * a * beta_z / sqrt_rho;
  Rc[ENG][kk] = alpha_s * (Hgas - u * cs) - scrh * beta_v - alpha_f * a * Btmag / sqrt_rho;
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv - rho * alpha_s * cs * dV[Xn] -
            sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KSLOWP;
  lambda[kk] = u + cs;
  Rc[RHO][kk] = alpha_s;
  Rc[Xn][kk] = alpha_s * lambda[kk];
  Rc[Xt][kk] = alpha_s * vv + scrh * beta_y;
  if constexpr (D == 3) Rc[Xb][kk] = alpha_s * w + scrh * beta_z;
  Rc[BXt][kk] = Rc[BXt][KSLOWM];
  if constexpr (D == 3) Rc[BXb][kk] = Rc[BXb][KSLOWM];
  Rc[ENG][kk] = alpha_s * (Hgas + u * cs) + scrh * beta_v - alpha_f * a * Btmag / sqrt_rho;
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv + rho * alpha_s * cs * dV[Xn] -
            sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  if constexpr (D == 3) {
    kk = KALFVM;
    lambda[kk] = u - ca;
    Rc[Xt][kk] = -rho * beta_z;
    Rc[Xb][kk] = +rho * beta_y;
    Rc[BXt][kk] = -sBx * sqrt_rho * beta_z;
    Rc[BXb][kk] = sBx * sqrt_rho * beta_y;
    Rc[ENG][kk] = -rho * (vv * beta_z - w * beta_y);
    eta[kk] = +beta_y * dV[Xb] - beta_z * dV[Xt] + sBx / sqrt_rho * (beta_y * dV[BXb] - beta_z * dV[BXt]);
    eta[kk] *= 0.5;
    kk = KALFVP;
    lambda[kk] = u + ca;
    Rc[Xt][kk] = -Rc[Xt][KALFVM];
    Rc[Xb][kk] = -Rc[Xb][KALFVM];
    Rc[BXt][kk] = Rc[BXt][KALFVM];
    Rc[BXb][kk] = Rc[BXb][KALFVM];
    Rc[ENG][kk] = -Rc[ENG][KALFVM];
    eta[kk] = -beta_y * dV[Xb] + beta_z * dV[Xt] + sBx / sqrt_rho * (beta_y * dV[BXb] - beta_z * dV[BXt]);
    eta[kk] *= 0.5;
  }
  r.cmax = fabs(u) + cf;
  r.sl = lambda[KFASTM];
  r.sr = lambda[KFASTP];
#pragma unroll
  for (int n = 0; n < NV; n++) alambda[n] = fabs(lambda[n]);
  if (alambda[KFASTM] < 0.5 * delta) alambda[KFASTM] = lambda[KFASTM] * lambda[KFASTM] / delta + 0.25 * delta;
  if (alambda[KFASTP] < 0.5 * delta) alambda[KFASTP] = lambda[KFASTP] * lambda[KFASTP] / delta + 0.25 * delta;
  if (alambda[KSLOWM] < 0.5 * delta) alambda[KSLOWM] = lambda[KSLOWM] * lambda[KSLOWM] / delta + 0.25 * delta;
  if (alambda[KSLOWP] < 0.5 * delta) alambda[KSLOWP] = lambda[KSLOWP] * lambda[KSLOWP] / delta + 0.25 * delta;
#pragma unroll
  for (int n1 = 0; n1 < NV; n1++) {
    double s = 0.0;
#pragma unroll
    for (int n2 = 0; n2 < NV; n2++) s += alambda[n2] * eta[n2] * Rc[n1][n2];
    r.F[n1] = 0.5 * (fluxL[n1] + fluxR[n1] - s);
  }
}

template <int D, int DIR, int SOLVER>
__device__ __forceinline__ void riemann(double gamma, const double* vL, const double* vR,
                                        RiemannOut<D>& r) {
  if constexpr (SOLVER == kHLLD) riemann_hlld<D, DIR>(gamma, vL, vR, r);
  if constexpr (SOLVER == kHLL) riemann_hll<D, DIR>(gamma, vL, vR, r);
  if constexpr (SOLVER == kROE) riemann_roe<D, DIR>(gamma, vL, vR, r);
  if constexpr (SOLVER == kTVDLF) riemann_tvdlf<D, DIR>(gamma, vL, vR, r);
}

}  // namespace idfx
