/*
 * Dimension-specialised body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * Included twice by ofx.c, with OFX_D = 2 and OFX_D = 3.  COMPONENTS equals
 * DIMENSIONS in both cases, so the reference's EXPAND and D_EXPAND macros
 * (src/macros.hpp:15-53) coincide; CX() below plays that role.  Where the
 * reference omits a term for fewer components, CX omits it too, so every
 * floating-point expression tree matches the reference's operation for
 * operation (this is what makes bit-for-bit comparison possible).
 */
#ifndef OFX_D
#error "define OFX_D before including ofx_core.h"
#endif

#undef CX
#undef NV
#undef MX3
#undef BX1
#undef BX2
#undef BX3
#undef ENG
#undef PRS
#undef SFX
#undef CX
#undef NV
#undef MX3
#undef BX1
#undef BX2
#undef BX3
#undef ENG
#undef PRS
#if OFX_D == 2
#define CX(a, b, c) a b
#define NV 6
#define MX3 254 /* absent: never indexed when OFX_D == 2 */
#define ENG 3
#define BX1 4
#define BX2 5
#define BX3 251
#define SFX(name) name##_d2
#else
#define CX(a, b, c) a b c
#define NV 8
#define MX3 3
#define ENG 4
#define BX1 5
#define BX2 6
#define BX3 7
#define SFX(name) name##_d3
#endif
#define PRS ENG

/* ---------------------------------------------------------------------- */
/* Equation of state and cons/prim (eos_adiabatic.hpp:38-45,            */
/* convertConsToPrim.hpp:15-100)                                         */
/* ---------------------------------------------------------------------- */
static void SFX(p2c)(double gamma, double* U, const double* V) {
  U[RHO] = V[RHO];
  CX(U[MX1] = V[MX1] * V[RHO];, U[MX2] = V[MX2] * V[RHO];, U[MX3] = V[MX3] * V[RHO];)
  CX(U[BX1] = V[BX1];, U[BX2] = V[BX2];, U[BX3] = V[BX3];)
  U[ENG] = V[PRS] / (gamma - 1.0)
         + 0.5 * V[RHO] * (CX(V[MX1] * V[MX1], + V[MX2] * V[MX2], + V[MX3] * V[MX3]))
         + 0.5 * (CX(U[BX1] * U[BX1], + U[BX2] * U[BX2], + U[BX3] * U[BX3]));
}

static void SFX(c2p)(double gamma, double* V, const double* U) {
  V[RHO] = U[RHO];
  CX(V[MX1] = U[MX1] / U[RHO];, V[MX2] = U[MX2] / U[RHO];, V[MX3] = U[MX3] / U[RHO];)
  CX(V[BX1] = U[BX1];, V[BX2] = U[BX2];, V[BX3] = U[BX3];)
  double kin = 0.5 / U[RHO] * (CX(U[MX1] * U[MX1], + U[MX2] * U[MX2], + U[MX3] * U[MX3]));
  double mag = 0.5 * (CX(U[BX1] * U[BX1], + U[BX2] * U[BX2], + U[BX3] * U[BX3]));
  V[PRS] = (U[ENG] - kin - mag) * (gamma - 1.0);
  /* pressure floor; the reference repairs only its local copy of the energy,
     which is then discarded (convertConsToPrim.hpp:43-51,131-141) */
  if (V[PRS] <= 0.0) V[PRS] = OFX_SMALL_PRESSURE_FIX;
}

/* physical flux along dir (flux.hpp:28-95); U is read before F is written */
static void SFX(kflux)(int dir, double* F, const double* V, const double* Uin) {
  double U[NV];
  for (int n = 0; n < NV; n++) U[n] = Uin[n];
  const int Xn = MX1 + dir;
  const int BXn = BX1 + dir;
  const int Xt = (dir == 0 ? MX2 : MX1);
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int Xb = (dir == 2 ? MX2 : MX3);
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  F[RHO] = U[Xn];
  CX(F[MX1] = U[MX1] * V[Xn] - V[BXn] * V[BX1];,
     F[MX2] = U[MX2] * V[Xn] - V[BXn] * V[BX2];,
     F[MX3] = U[MX3] * V[Xn] - V[BXn] * V[BX3];)
  CX(F[BXn] = 0.0;, F[BXt] = V[Xn] * V[BXt] - V[BXn] * V[Xt];,
     F[BXb] = V[Xn] * V[BXb] - V[BXn] * V[Xb];)
  double Bmag2 = CX(V[BX1] * V[BX1], + V[BX2] * V[BX2], + V[BX3] * V[BX3]);
  double ptot = V[PRS] + 0.5 * Bmag2;
  F[ENG] = (U[ENG] + ptot) * V[Xn] - V[BXn] * (CX(V[MX1] * V[BX1], + V[MX2] * V[BX2], + V[MX3] * V[BX3]));
  F[Xn] += ptot;
}

/* ---------------------------------------------------------------------- */
/* Riemann solvers.  Output: F[NV], cmax, sl, sr (+uL,uR for uct_hlld)   */
/* ---------------------------------------------------------------------- */
typedef struct {
  double F[NV];
  double uL[NV], uR[NV];
  double cmax, sl, sr;
} SFX(rsout);

/* fast magnetosonic speed of one state (hlldMHD.hpp:205-238) */
static double SFX(fastspeed)(int dir, double gamma, const double* v) {
  const int BXn = BX1 + dir;
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  double gpr = gamma * v[PRS];
  double b1, b2, b3;
  b1 = b2 = b3 = 0.0;
  CX(b1 = v[BXn];, b2 = v[BXt];, b3 = v[BXb];)
  double Btmag2 = b2 * b2 + b3 * b3;
  double Bmag2 = b1 * b1 + Btmag2;
  double c = gpr - Bmag2;
  c = gpr + Bmag2 + sqrt(c * c + 4.0 * gpr * Btmag2);
  c = sqrt(0.5 * c / v[RHO]);
  return c;
}

/* HLLD, Miyoshi & Kusano with the HLLC degeneracy fallback (hlldMHD.hpp:147-589) */
static void SFX(hlld)(int dir, double gamma, const double* vL, const double* vR, SFX(rsout) * r) {
  const int Xn = MX1 + dir;
  const int BXn = BX1 + dir;
  const int Xt = (dir == 0 ? MX2 : MX1);
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int Xb = (dir == 2 ? MX2 : MX3);
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  double* uL = r->uL;
  double* uR = r->uR;
  double fluxL[NV], fluxR[NV];
  double* F = r->F;
  double cL = SFX(fastspeed)(dir, gamma, vL);
  double cR = SFX(fastspeed)(dir, gamma, vR);
  double cminL = vL[Xn] - cL, cmaxL = vL[Xn] + cL;
  double cminR = vR[Xn] - cR, cmaxR = vR[Xn] + cR;
  double sl = fmin(cminL, cminR);
  double sr = fmax(cmaxL, cmaxR);
  r->sl = sl;
  r->sr = sr;
  r->cmax = fmax(fabs(sl), fabs(sr));
  SFX(p2c)(gamma, uL, vL);
  SFX(p2c)(gamma, uR, vR);
  SFX(kflux)(dir, fluxL, vL, uL);
  SFX(kflux)(dir, fluxR, vR, uR);
  double ptL = vL[PRS] + 0.5 * (CX(vL[BX1] * vL[BX1], + vL[BX2] * vL[BX2], + vL[BX3] * vL[BX3]));
  double ptR = vR[PRS] + 0.5 * (CX(vR[BX1] * vR[BX1], + vR[BX2] * vR[BX2], + vR[BX3] * vR[BX3]));

  if (sl > 0) {
    for (int nv = 0; nv < NV; nv++) F[nv] = fluxL[nv];
    return;
  }
  if (sr < 0) {
    for (int nv = 0; nv < NV; nv++) F[nv] = fluxR[nv];
    return;
  }
  double usL[NV], usR[NV], Uhll[NV];
  double scrh, scrhL, scrhR, duL, duR, sBx, Bx, SM, S1L, S1R, pts, sqrL, sqrR;
  double vsL = 0, vsR = 0, wsL = 0, wsR = 0;
  int revert_to_hllc = 0;
  (void)wsL; (void)wsR;

  scrh = 1.0 / (sr - sl);
  Bx = (sr * vR[BXn] - sl * vL[BXn]) * scrh;
  sBx = (Bx > 0.0 ? 1.0 : -1.0);
  duL = sl - vL[Xn];
  duR = sr - vR[Xn];
  scrh = 1.0 / (duR * uR[RHO] - duL * uL[RHO]);
  SM = (duR * uR[Xn] - duL * uL[Xn] - ptR + ptL) * scrh;
  pts = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR + vL[RHO] * vR[RHO] * duR * duL * (vR[Xn] - vL[Xn]);
  pts *= scrh;
  usL[RHO] = uL[RHO] * duL / (sl - SM);
  usR[RHO] = uR[RHO] * duR / (sr - SM);
  sqrL = sqrt(usL[RHO]);
  sqrR = sqrt(usR[RHO]);
  S1L = SM - fabs(Bx) / sqrL;
  S1R = SM + fabs(Bx) / sqrR;
  if ((S1L - sl) < 1.e-4 * (SM - sl)) revert_to_hllc = 1;
  if ((S1R - sr) > -1.e-4 * (sr - SM)) revert_to_hllc = 1;
  if (revert_to_hllc) {
    scrh = 1.0 / (sr - sl);
    for (int nv = 0; nv < NV; nv++) {
      Uhll[nv] = sr * uR[nv] - sl * uL[nv] + fluxL[nv] - fluxR[nv];
      Uhll[nv] *= scrh;
    }
    CX(usL[BXn] = usR[BXn] = Uhll[BXn];, usL[BXt] = usR[BXt] = Uhll[BXt];,
       usL[BXb] = usR[BXb] = Uhll[BXb];)
    S1L = S1R = SM;
  } else {
    scrhL = (uL[RHO] * duL * duL - Bx * Bx) / (uL[RHO] * duL * (sl - SM) - Bx * Bx);
    scrhR = (uR[RHO] * duR * duR - Bx * Bx) / (uR[RHO] * duR * (sr - SM) - Bx * Bx);
    CX(usL[BXn] = Bx;, usL[BXt] = uL[BXt] * scrhL;, usL[BXb] = uL[BXb] * scrhL;)
    CX(usR[BXn] = Bx;, usR[BXt] = uR[BXt] * scrhR;, usR[BXb] = uR[BXb] * scrhR;)
  }
  scrhL = Bx / (uL[RHO] * duL);
  scrhR = Bx / (uR[RHO] * duR);
  CX(;, vsL = vL[Xt] - scrhL * (usL[BXt] - uL[BXt]); vsR = vR[Xt] - scrhR * (usR[BXt] - uR[BXt]);,
     wsL = vL[Xb] - scrhL * (usL[BXb] - uL[BXb]); wsR = vR[Xb] - scrhR * (usR[BXb] - uR[BXb]);)
  CX(usL[Xn] = usL[RHO] * SM; usR[Xn] = usR[RHO] * SM;, usL[Xt] = usL[RHO] * vsL;
     usR[Xt] = usR[RHO] * vsR;, usL[Xb] = usL[RHO] * wsL; usR[Xb] = usR[RHO] * wsR;)
  scrhL = CX(vL[Xn] * Bx, + vL[Xt] * uL[BXt], + vL[Xb] * uL[BXb]);
  scrhL -= CX(SM * Bx, + vsL * usL[BXt], + wsL * usL[BXb]);
  usL[ENG] = duL * uL[ENG] - ptL * vL[Xn] + pts * SM + Bx * scrhL;
  usL[ENG] /= sl - SM;
  scrhR = CX(vR[Xn] * Bx, + vR[Xt] * uR[BXt], + vR[Xb] * uR[BXb]);
  scrhR -= CX(SM * Bx, + vsR * usR[BXt], + wsR * usR[BXb]);
  usR[ENG] = duR * uR[ENG] - ptR * vR[Xn] + pts * SM + Bx * scrhR;
  usR[ENG] /= sr - SM;

  if (S1L >= 0.0) {
    for (int nv = 0; nv < NV; nv++) F[nv] = fluxL[nv] + sl * (usL[nv] - uL[nv]);
  } else if (S1R <= 0.0) {
    for (int nv = 0; nv < NV; nv++) F[nv] = fluxR[nv] + sr * (usR[nv] - uR[nv]);
  } else {
    double vss = 0, wss = 0;
    double ussl[NV], ussr[NV];
    (void)wss;
    ussl[RHO] = usL[RHO];
    ussr[RHO] = usR[RHO];
    CX(;, vss = sqrL * vsL + sqrR * vsR + (usR[BXt] - usL[BXt]) * sBx; vss /= sqrL + sqrR;,
       wss = sqrL * wsL + sqrR * wsR + (usR[BXb] - usL[BXb]) * sBx; wss /= sqrL + sqrR;)
    CX(ussl[Xn] = ussl[RHO] * SM; ussr[Xn] = ussr[RHO] * SM;, ussl[Xt] = ussl[RHO] * vss;
       ussr[Xt] = ussr[RHO] * vss;, ussl[Xb] = ussl[RHO] * wss; ussr[Xb] = ussr[RHO] * wss;)
    CX(ussl[BXn] = ussr[BXn] = Bx;,
       ussl[BXt] = sqrL * usR[BXt] + sqrR * usL[BXt] + sqrL * sqrR * (vsR - vsL) * sBx;
       ussl[BXt] /= sqrL + sqrR; ussr[BXt] = ussl[BXt];,
       ussl[BXb] = sqrL * usR[BXb] + sqrR * usL[BXb] + sqrL * sqrR * (wsR - wsL) * sBx;
       ussl[BXb] /= sqrL + sqrR; ussr[BXb] = ussl[BXb];)
    scrhL = CX(SM * Bx, + vsL * usL[BXt], + wsL * usL[BXb]);
    scrhL -= CX(SM * Bx, + vss * ussl[BXt], + wss * ussl[BXb]);
    scrhR = CX(SM * Bx, + vsR * usR[BXt], + wsR * usR[BXb]);
    scrhR -= CX(SM * Bx, + vss * ussr[BXt], + wss * ussr[BXb]);
    ussl[ENG] = usL[ENG] - sqrL * scrhL * sBx;
    ussr[ENG] = usR[ENG] + sqrR * scrhR * sBx;
    if (SM >= 0.0) {
      for (int nv = 0; nv < NV; nv++)
        F[nv] = fluxL[nv] + S1L * (ussl[nv] - usL[nv]) + sl * (usL[nv] - uL[nv]);
    } else {
      for (int nv = 0; nv < NV; nv++)
        F[nv] = fluxR[nv] + S1R * (ussr[nv] - usR[nv]) + sr * (usR[nv] - uR[nv]);
    }
  }
}

/* HLL (hllMHD.hpp:154-453, Hall term disabled) */
static void SFX(hll)(int dir, double gamma, const double* vL, const double* vR, SFX(rsout) * r) {
  const int Xn = MX1 + dir;
  double* uL = r->uL;
  double* uR = r->uR;
  double fluxL[NV], fluxR[NV];
  double* F = r->F;
  double cL = SFX(fastspeed)(dir, gamma, vL);
  double cR = SFX(fastspeed)(dir, gamma, vR);
  double cminL = vL[Xn] - cL, cmaxL = vL[Xn] + cL;
  double cminR = vR[Xn] - cR, cmaxR = vR[Xn] + cR;
  double sl = fmin(cminL, cminR);
  double sr = fmax(cmaxL, cmaxR);
  double SLb = sl, SRb = sr;
  r->sl = sl;
  r->sr = sr;
  r->cmax = fmax(fabs(SLb), fabs(SRb));
  SFX(p2c)(gamma, uL, vL);
  SFX(p2c)(gamma, uR, vR);
  SFX(kflux)(dir, fluxL, vL, uL);
  SFX(kflux)(dir, fluxR, vR, uR);
  if (sl > 0) {
    F[RHO] = fluxL[RHO];
    CX(F[MX1] = fluxL[MX1];, F[MX2] = fluxL[MX2];, F[MX3] = fluxL[MX3];)
  } else if (sr < 0) {
    F[RHO] = fluxR[RHO];
    CX(F[MX1] = fluxR[MX1];, F[MX2] = fluxR[MX2];, F[MX3] = fluxR[MX3];)
  } else {
    F[RHO] = (sl * sr * uR[RHO] - sl * sr * uL[RHO] + sr * fluxL[RHO] - sl * fluxR[RHO]) / (sr - sl);
    CX(F[MX1] = (sl * sr * uR[MX1] - sl * sr * uL[MX1] + sr * fluxL[MX1] - sl * fluxR[MX1]) / (sr - sl);,
       F[MX2] = (sl * sr * uR[MX2] - sl * sr * uL[MX2] + sr * fluxL[MX2] - sl * fluxR[MX2]) / (sr - sl);,
       F[MX3] = (sl * sr * uR[MX3] - sl * sr * uL[MX3] + sr * fluxL[MX3] - sl * fluxR[MX3]) / (sr - sl);)
  }
  if (SLb > 0) {
    for (int nv = BX1; nv < BX1 + OFX_D; nv++) F[nv] = fluxL[nv];
    F[ENG] = fluxL[ENG];
  } else if (SRb < 0) {
    for (int nv = BX1; nv < BX1 + OFX_D; nv++) F[nv] = fluxR[nv];
    F[ENG] = fluxR[ENG];
  } else {
    for (int nv = BX1; nv < BX1 + OFX_D; nv++) {
      F[nv] = SLb * SRb * uR[nv] - SLb * SRb * uL[nv] + SRb * fluxL[nv] - SLb * fluxR[nv];
      F[nv] *= (1.0 / (SRb - SLb));
    }
    F[ENG] = SLb * SRb * uR[ENG] - SLb * SRb * uL[ENG] + SRb * fluxL[ENG] - SLb * fluxR[ENG];
    F[ENG] *= (1.0 / (SRb - SLb));
  }
}

/* TVDLF / Rusanov (tvdlfMHD.hpp:140-232) */
static void SFX(tvdlf)(int dir, double gamma, const double* vL, const double* vR, SFX(rsout) * r) {
  const int Xn = MX1 + dir;
  const int BXn = BX1 + dir;
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  double v[NV];
  double* uL = r->uL;
  double* uR = r->uR;
  double fluxL[NV], fluxR[NV];
  for (int nv = 0; nv < NV; nv++) v[nv] = 0.5 * (vL[nv] + vR[nv]);
  double gpr = gamma * v[PRS];
  double Bt2 = CX(0.0, + v[BXt] * v[BXt], + v[BXb] * v[BXb]);
  double B2 = Bt2 + v[BXn] * v[BXn];
  double cRL = gpr - B2;
  cRL = cRL + B2 + sqrt(cRL * cRL + 4.0 * gpr * Bt2);
  cRL = sqrt(0.5 * cRL / v[RHO]);
  double cmax = fmax(fabs(v[Xn] + cRL), fabs(v[Xn] - cRL));
  r->sl = -cmax;
  r->sr = cmax;
  r->cmax = cmax;
  SFX(p2c)(gamma, uL, vL);
  SFX(p2c)(gamma, uR, vR);
  SFX(kflux)(dir, fluxL, vL, uL);
  SFX(kflux)(dir, fluxR, vR, uR);
  for (int nv = 0; nv < NV; nv++) r->F[nv] = 0.5 * (fluxL[nv] + fluxR[nv] + cmax * (uL[nv] - uR[nv]));
}

/* Roe linearised solver with entropy fix (roeMHD.hpp:175-650) */
static void SFX(roe)(int dir, double gamma, const double* vL, const double* vR, SFX(rsout) * r) {
  enum { KFASTM = 0, KFASTP = 1, KDIVB = 2, KENTRP = 3, KSLOWM = 4, KSLOWP = 5, KALFVM = 6, KALFVP = 7 };
  const int Xn = MX1 + dir;
  const int BXn = BX1 + dir;
  const int Xt = (dir == 0 ? MX2 : MX1);
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int Xb = (dir == 2 ? MX2 : MX3);
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  double dV[NV], dU[NV], fluxL[NV], fluxR[NV], Rc[NV][NV];
  double* uL = r->uL;
  double* uR = r->uR;
  const double delta = 1.e-6;
  for (int nv = 0; nv < NV; nv++) dV[nv] = vR[nv] - vL[nv];
  SFX(p2c)(gamma, uL, vL);
  SFX(p2c)(gamma, uR, vR);
  for (int nv = 0; nv < NV; nv++) dU[nv] = uR[nv] - uL[nv];
  SFX(kflux)(dir, fluxL, vL, uL);
  SFX(kflux)(dir, fluxR, vR, uR);
  for (int a = 0; a < NV; a++)
    for (int b = 0; b < NV; b++) Rc[a][b] = 0;

  double sqr_rho_L = sqrt(vL[RHO]);
  double sqr_rho_R = sqrt(vR[RHO]);
  double sl = sqr_rho_L / (sqr_rho_L + sqr_rho_R);
  double sr = sqr_rho_R / (sqr_rho_L + sqr_rho_R);
  double rho = sr * vL[RHO] + sl * vR[RHO];
  double sqrt_rho = sqrt(rho);
  double u = 0, v = 0, w = 0, Bx = 0, By = 0, Bz = 0, bx = 0, by = 0, bz = 0;
  (void)w; (void)Bz; (void)bz;
  CX(u = sl * vL[Xn] + sr * vR[Xn];, v = sl * vL[Xt] + sr * vR[Xt];, w = sl * vL[Xb] + sr * vR[Xb];)
  CX(Bx = sr * vL[BXn] + sl * vR[BXn];, By = sr * vL[BXt] + sl * vR[BXt];, Bz = sr * vL[BXb] + sl * vR[BXb];)
  double sBx = (Bx >= 0.0 ? 1.0 : -1.0);
  CX(bx = Bx / sqrt_rho;, by = By / sqrt_rho;, bz = Bz / sqrt_rho;)
  double bt2 = CX(0.0, + by * by, + bz * bz);
  double b2 = bx * bx + bt2;
  double Btmag = sqrt(bt2 * rho);
  double X = CX(dV[BXn] * dV[BXn], + dV[BXt] * dV[BXt], + dV[BXb] * dV[BXb]);
  X /= (sqr_rho_L + sqr_rho_R) * (sqr_rho_L + sqr_rho_R) * 2.0;
  double Bmag2L = CX(vL[BX1] * vL[BX1], + vL[BX2] * vL[BX2], + vL[BX3] * vL[BX3]);
  double Bmag2R = CX(vR[BX1] * vR[BX1], + vR[BX2] * vR[BX2], + vR[BX3] * vR[BX3]);
  double pL = vL[PRS] + 0.5 * Bmag2L;
  double pR = vR[PRS] + 0.5 * Bmag2R;
  double vdm = CX(u * dU[Xn], + v * dU[Xt], + w * dU[Xb]);
  double BdB = CX(Bx * dU[BXn], + By * dU[BXt], + Bz * dU[BXb]);
  double vel2 = CX(u * u, + v * v, + w * w);
  dV[PRS] = (gamma - 1.0) * ((0.5 * vel2 - X) * dV[RHO] - vdm + dU[ENG] - BdB);
  double HL = (uL[ENG] + pL) / vL[RHO];
  double HR = (uR[ENG] + pR) / vR[RHO];
  double H = sl * HL + sr * HR;
  double Hgas = H - b2;
  double a2 = (2.0 - gamma) * X + (gamma - 1.0) * (Hgas - 0.5 * vel2);

  double scrh, ca, cf, cs, ca2, cf2, cs2, alpha_f, alpha_s, beta_y = 0, beta_z = 0, a;
  (void)beta_z;
  scrh = a2 - b2;
  ca2 = bx * bx;
  scrh = scrh * scrh + 4.0 * bt2 * a2;
  scrh = sqrt(scrh);
  cf2 = 0.5 * (a2 + b2 + scrh);
  cs2 = a2 * ca2 / cf2;
  cf = sqrt(cf2);
  cs = sqrt(cs2);
  ca = sqrt(ca2);
  a = sqrt(a2);
  (void)ca;
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
#if OFX_D == 2
  if (Btmag > 1.e-9) {
    beta_y = ((By) >= 0.0 ? (1.0) : (-1.0));
  } else {
    beta_y = 1.0;
  }
#else
  if (Btmag > 1.e-9) {
    beta_y = By / Btmag;
    beta_z = Bz / Btmag;
  } else {
    beta_z = beta_y = 1.0;
  }
#endif
  double lambda[8], alambda[8], eta[8];
  double beta_dv, beta_dB, beta_v;
  int kk = KFASTM;
  lambda[kk] = u - cf;
  scrh = alpha_s * cs * sBx;
  beta_dv = CX(0.0, + beta_y * dV[Xt], + beta_z * dV[Xb]);
  beta_dB = CX(0.0, + beta_y * dV[BXt], + beta_z * dV[BXb]);
  Rc[RHO][kk] = alpha_f;
  CX(Rc[Xn][kk] = alpha_f * lambda[kk];, Rc[Xt][kk] = alpha_f * v + scrh * beta_y;,
     Rc[Xb][kk] = alpha_f * w + scrh * beta_z;)
  CX(;, Rc[BXt][kk] = alpha_s * a * beta_y / sqrt_rho;, Rc[BXb][kk] = alpha_s * a * beta_z / sqrt_rho;)
  beta_v = CX(0.0, + beta_y * v, + beta_z * w);
  Rc[ENG][kk] = alpha_f * (Hgas - u * cf) + scrh * beta_v + alpha_s * a * Btmag / sqrt_rho;
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]);
  eta[kk] += rho * scrh * beta_dv - rho * alpha_f * cf * dV[Xn] + sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KFASTP;
  lambda[kk] = u + cf;
  Rc[RHO][kk] = alpha_f;
  CX(Rc[Xn][kk] = alpha_f * lambda[kk];, Rc[Xt][kk] = alpha_f * v - scrh * beta_y;,
     Rc[Xb][kk] = alpha_f * w - scrh * beta_z;)
  CX(;, Rc[BXt][kk] = Rc[BXt][KFASTM];, Rc[BXb][kk] = Rc[BXb][KFASTM];)
  Rc[ENG][kk] = alpha_f * (Hgas + u * cf) - scrh * beta_v + alpha_s * a * Btmag / sqrt_rho;
  eta[kk] = alpha_f * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv + rho * alpha_f * cf * dV[Xn]
          + sqrt_rho * alpha_s * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KENTRP;
  lambda[kk] = u;
  Rc[RHO][kk] = 1.0;
  CX(Rc[Xn][kk] = u;, Rc[Xt][kk] = v;, Rc[Xb][kk] = w;)
  Rc[ENG][kk] = 0.5 * vel2 + (gamma - 2.0) / (gamma - 1.0) * X;
  eta[kk] = ((a2 - X) * dV[RHO] - dV[PRS]) / a2;

  kk = KDIVB;
  lambda[kk] = u;
  eta[kk] = 0.0;

  scrh = alpha_f * cf * sBx;
  kk = KSLOWM;
  lambda[kk] = u - cs;
  Rc[RHO][kk] = alpha_s;
  CX(Rc[Xn][kk] = alpha_s * lambda[kk];, Rc[Xt][kk] = alpha_s * v - scrh * beta_y;,
     Rc[Xb][kk] = alpha_s * w - scrh * beta_z;)
  CX(;, Rc[BXt][kk] = -alpha_f * a * beta_y / sqrt_rho;, Rc[BXb][kk] = -alpha_f * a * beta_z / sqrt_rho;)
  Rc[ENG][kk] = alpha_s * (Hgas - u * cs) - scrh * beta_v - alpha_f * a * Btmag / sqrt_rho;
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv - rho * alpha_s * cs * dV[Xn]
          - sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= 0.5 / a2;

  kk = KSLOWP;
  lambda[kk] = u + cs;
  Rc[RHO][kk] = alpha_s;
  CX(Rc[Xn][kk] = alpha_s * lambda[kk];, Rc[Xt][kk] = alpha_s * v + scrh * beta_y;,
     Rc[Xb][kk] = alpha_s * w + scrh * beta_z;)
  CX(;, Rc[BXt][kk] = Rc[BXt][KSLOWM];, Rc[BXb][kk] = Rc[BXb][KSLOWM];)
  Rc[ENG][kk] = alpha_s * (Hgas + u * cs) + scrh * beta_v - alpha_f * a * Btmag / sqrt_rho;
  eta[kk] = alpha_s * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv + rho * alpha_s * cs * dV[Xn]
          - sqrt_rho * alpha_f * a * beta_dB;
  eta[kk] *= 0.5 / a2;

#if OFX_D == 3
  kk = KALFVM;
  lambda[kk] = u - ca;
  Rc[Xt][kk] = -rho * beta_z;
  Rc[Xb][kk] = +rho * beta_y;
  Rc[BXt][kk] = -sBx * sqrt_rho * beta_z;
  Rc[BXb][kk] = sBx * sqrt_rho * beta_y;
  Rc[ENG][kk] = -rho * (v * beta_z - w * beta_y);
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
#endif

  double cmax = fabs(u) + cf;
  r->sl = lambda[KFASTM];
  r->sr = lambda[KFASTP];
  for (int nv = 0; nv < NV; nv++) alambda[nv] = fabs(lambda[nv]);
  if (alambda[KFASTM] < 0.5 * delta) alambda[KFASTM] = lambda[KFASTM] * lambda[KFASTM] / delta + 0.25 * delta;
  if (alambda[KFASTP] < 0.5 * delta) alambda[KFASTP] = lambda[KFASTP] * lambda[KFASTP] / delta + 0.25 * delta;
  if (alambda[KSLOWM] < 0.5 * delta) alambda[KSLOWM] = lambda[KSLOWM] * lambda[KSLOWM] / delta + 0.25 * delta;
  if (alambda[KSLOWP] < 0.5 * delta) alambda[KSLOWP] = lambda[KSLOWP] * lambda[KSLOWP] / delta + 0.25 * delta;
  for (int nv1 = 0; nv1 < NV; nv1++) {
    scrh = 0.0;
    for (int nv2 = 0; nv2 < NV; nv2++) scrh += alambda[nv2] * eta[nv2] * Rc[nv1][nv2];
    r->F[nv1] = 0.5 * (fluxL[nv1] + fluxR[nv1] - scrh);
  }
  r->cmax = cmax;
}

/* ---------------------------------------------------------------------- */
/* Reconstruction (extrapolateToFaces.hpp:75-309, slopeLimiter.hpp)      */
/* ---------------------------------------------------------------------- */
static void SFX(recon)(const ofx* o, int dir, size_t base, double* vL, double* vR) {
  const size_t s = o->stride[dir];
  const double dxv = o->dx[dir];
  /* shock flags of the two cells (extrapolateToFaces.hpp:96-121, 139-218) */
  const int shL = o->shock && o->flag[base - s];
  const int shR = o->shock && o->flag[base];
  for (int nv = 0; nv < NV; nv++) {
    const double* q = o->Vc + (size_t)nv * o->ncell + base;
    if (o->order == 1) {
      vL[nv] = q[-(ptrdiff_t)s];
      vR[nv] = q[0];
    } else if (o->order == 2) {
      double dvm = q[-(ptrdiff_t)s] - q[-2 * (ptrdiff_t)s];
      double dvp = q[0] - q[-(ptrdiff_t)s];
      double dv = shL ? ofx_minmod(dvp, dvm) : ofx_vanleer(dvp, dvm);
      vL[nv] = q[-(ptrdiff_t)s] + 0.5 * dv;
      dvm = dvp;
      dvp = q[s] - q[0];
      dv = shR ? ofx_minmod(dvp, dvm) : ofx_vanleer(dvp, dvm);
      vR[nv] = q[0] - 0.5 * dv;
    } else if (o->order == 3) {
      double dvm = q[-(ptrdiff_t)s] - q[-2 * (ptrdiff_t)s];
      double dvp = q[0] - q[-(ptrdiff_t)s];
      double dv = shL ? ofx_minmod(dvp, dvm) : dvp * ofx_limo3(dvp, dvm, dxv);
      vL[nv] = q[-(ptrdiff_t)s] + 0.5 * dv;
      if (nv == RHO || nv == PRS) {
        if (vL[nv] <= 0.0) {
          dv = ofx_minmod(dvp, dvm);
          vL[nv] = q[-(ptrdiff_t)s] + 0.5 * dv;
        }
      }
      dvm = dvp;
      dvp = q[s] - q[0];
      dv = shR ? ofx_minmod(dvp, dvm) : dvm * ofx_limo3(dvm, dvp, dxv);
      vR[nv] = q[0] - 0.5 * dv;
      if (nv == RHO || nv == PRS) {
        if (vR[nv] <= 0.0) {
          dv = ofx_minmod(dvp, dvm);
          vR[nv] = q[0] - 0.5 * dv;
        }
      }
    } else { /* PPM */
      double vm2 = q[-3 * (ptrdiff_t)s];
      double vm1 = q[-2 * (ptrdiff_t)s];
      double v0 = q[-(ptrdiff_t)s];
      double vp1 = q[0];
      double vp2 = q[s];
      double vr, vl;
      ofx_ppm_states(vm2, vm1, v0, vp1, vp2, &vl, &vr);
      if (nv == RHO || nv == PRS) {
        if (vr <= 0.0) {
          double dv = ofx_vanleer(vp1 - v0, v0 - vm1);
          vr = v0 + 0.5 * dv;
        }
      }
      vL[nv] = vr;
      vm2 = vm1;
      vm1 = v0;
      v0 = vp1;
      vp1 = vp2;
      vp2 = q[2 * s];
      ofx_ppm_states(vm2, vm1, v0, vp1, vp2, &vl, &vr);
      if (nv == RHO || nv == PRS) {
        if (vl <= 0.0) {
          double dv = ofx_vanleer(vp1 - v0, v0 - vm1);
          vl = v0 - 0.5 * dv;
        }
      }
      vR[nv] = vl;
    }
  }
}

/* ---------------------------------------------------------------------- */
/* HLL-type EMF side outputs (storeFlux.hpp:46-208)                       */
/* ---------------------------------------------------------------------- */
static void SFX(store_hll)(ofx* o, int dir, size_t c, double st, double sb, const SFX(rsout) * r,
                           const double* vL, const double* vR, double* Et, double* Eb) {
  const int Xn = MX1 + dir;
  const int BXn = BX1 + dir;
  const int Xt = (dir == 0 ? MX2 : MX1);
#if OFX_D == 3
  const int Xb = (dir == 2 ? MX2 : MX3);
#endif
  (void)sb; (void)Eb; (void)Xn; (void)BXn;
  double* aL = o->aL[dir];
  double* aR = o->aR[dir];
  double* dL = o->dL[dir];
  double* dR = o->dR[dir];
  const double sl = r->sl, sr = r->sr;
  if (o->emf == OFX_UCT_HLL) {
    double ar = fmax(0.0, sr);
    double al = fmin(0.0, sl);
    double scrh = 1.0 / (ar - al);
    CX(Et[c] = -st * (ar * vL[Xt] - al * vR[Xt]) * scrh;, , Eb[c] = -sb * (ar * vL[Xb] - al * vR[Xb]) * scrh;)
    aL[c] = ar * scrh;
    aR[c] = -al * scrh;
    dR[c] = -al * ar * scrh;
    dL[c] = dR[c];
    return;
  }
  /* uct_hlld */
  const double* uL = r->uL;
  const double* uR = r->uR;
  double ptL = vL[PRS] + 0.5 * (CX(vL[BX1] * vL[BX1], + vL[BX2] * vL[BX2], + vL[BX3] * vL[BX3]));
  double ptR = vR[PRS] + 0.5 * (CX(vR[BX1] * vR[BX1], + vR[BX2] * vR[BX2], + vR[BX3] * vR[BX3]));
  int revert_to_hll = 0;
  double Bn = (sr * vR[BXn] - sl * vL[BXn]) / (sr - sl);
  double duL = sl - vL[Xn];
  double duR = sr - vR[Xn];
  double scrh = 1.0 / (duR * uR[RHO] - duL * uL[RHO]);
  double Sc = (duR * uR[Xn] - duL * uL[Xn] - ptR + ptL) * scrh;
  double usLRHO = uL[RHO] * duL / (sl - Sc);
  double usRRHO = uR[RHO] * duR / (sr - Sc);
  double sqrL = sqrt(usLRHO);
  double sqrR = sqrt(usRRHO);
  double SaL = Sc - fabs(Bn) / sqrL;
  double SaR = Sc + fabs(Bn) / sqrR;
  if ((SaL - sl) < 1e-4 * (Sc - sl)) revert_to_hll = 1;
  if ((SaR - sr) > -1e-4 * (sr - Sc)) revert_to_hll = 1;
  double chiL = (vL[Xn] - Sc) * (sl - Sc) / (SaL + sl - 2.0 * Sc);
  double chiR = (vR[Xn] - Sc) * (sr - Sc) / (SaR + sr - 2.0 * Sc);
  double nuL = (SaL + sl) / (fabs(SaL) + fabs(sl));
  double nuR = (SaR + sr) / (fabs(SaR) + fabs(sr));
  double nuLR = (SaL + SaR) / (fabs(SaL) + fabs(SaR));
  if (fabs(SaR - SaL) > 1.e-9 * fabs(sr - sl)) {
    dL[c] = 0.5 * (chiL * nuL - chiL * nuLR) + 0.5 * (fabs(SaL) - nuLR * SaL);
    dR[c] = 0.5 * (chiR * nuR - chiR * nuLR) + 0.5 * (fabs(SaR) - nuLR * SaR);
    aL[c] = 0.5 * (1.0 + nuLR);
    aR[c] = 0.5 * (1.0 - nuLR);
  } else {
    dL[c] = 0.5 * chiL * nuL + 0.5 * fabs(SaL);
    dR[c] = 0.5 * chiR * nuR + 0.5 * fabs(SaR);
    aL[c] = 0.5;
    aR[c] = 0.5;
  }
  double ar = fmax(0.0, sr);
  double al = fmin(0.0, sl);
  scrh = 1.0 / (ar - al);
  if (revert_to_hll) {
    aL[c] = ar * scrh;
    aR[c] = -al * scrh;
    dR[c] = -al * ar * scrh;
    dL[c] = dR[c];
  }
  CX(Et[c] = -st * (ar * vL[Xt] - al * vR[Xt]) * scrh;, , Eb[c] = -sb * (ar * vL[Xb] - al * vR[Xb]) * scrh;)
}

/* one upwinded edge contribution of CalcRiemannAverage
   (calcRiemannEmf.hpp:62-420).  q is a face-field component indexed on the
   Vs grid (index fq, stride fs along the upwinding direction); e is a face
   EMF on the cell grid (index c, stride s); the a/d weights are averaged
   over the two faces c-sp and c.  Returns aL*vL*bL + aR*vR*bR, sets phi. */
static double SFX(riemann_edge_f)(const ofx* o, const double* q, size_t fq, size_t fs, const double* e,
                                  size_t c, size_t s, const double* AL, const double* AR,
                                  const double* DL, const double* DR, size_t sp, double* phi) {
  const ptrdiff_t S = (ptrdiff_t)s, FS = (ptrdiff_t)fs;
  double aL = 0.5 * (AL[c - sp] + AL[c]);
  double aR = 0.5 * (AR[c - sp] + AR[c]);
  double dL = 0.5 * (DL[c - sp] + DL[c]);
  double dR = 0.5 * (DR[c - sp] + DR[c]);
  double bL, bR, vLv, vRv, db, dv;
  const size_t fm = fq - FS, m = c - S;
  if (o->order == 4) {
    ofx_ppm_states(q[fm - 2 * FS], q[fm - FS], q[fm], q[fm + FS], q[fm + 2 * FS], &db, &bL);
    ofx_ppm_states(q[fq - 2 * FS], q[fq - FS], q[fq], q[fq + FS], q[fq + 2 * FS], &bR, &db);
    ofx_ppm_states(e[m - 2 * S], e[m - S], e[m], e[m + S], e[m + 2 * S], &dv, &vLv);
    ofx_ppm_states(e[c - 2 * S], e[c - S], e[c], e[c + S], e[c + 2 * S], &vRv, &dv);
  } else {
    db = ofx_mclim(q[fm + FS] - q[fm], q[fm] - q[fm - FS]);
    bL = q[fm] + 0.5 * db;
    db = ofx_mclim(q[fq + FS] - q[fq], q[fq] - q[fq - FS]);
    bR = q[fq] - 0.5 * db;
    dv = ofx_mclim(e[m + S] - e[m], e[m] - e[m - S]);
    vLv = e[m] + 0.5 * dv;
    dv = ofx_mclim(e[c + S] - e[c], e[c] - e[c - S]);
    vRv = e[c] - 0.5 * dv;
  }
  *phi = dR * bR - dL * bL;
  return aL * vLv * bL + aR * vRv * bR;
}

static void SFX(riemann_emf)(ofx* o) {
  const size_t si = 1, sj = o->stride[1], sk = o->stride[2];
  (void)sk;
  const double* Vs1 = o->Vs;
  const double* Vs2 = o->Vs + o->nface;
#if OFX_D == 3
  const double* Vs3 = o->Vs + 2 * o->nface;
#endif
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = o->beg[2]; k < o->end[2] + (OFX_D == 3); k++)
    for (int j = o->beg[1]; j < o->end[1] + 1; j++)
      for (int i = o->beg[0]; i < o->end[0] + 1; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        const size_t f = OFX_FIDX(o, k, j, i);
        double phi, X;
        /* IDIR part: z-edge from ezj/BX2s upwinded in x */
        X = SFX(riemann_edge_f)(o, Vs2, f, 1, o->ezj, c, 1, o->aL[0], o->aR[0], o->dL[0], o->dR[0], sj, &phi);
        o->ez[c] = X + phi;
#if OFX_D == 3
        X = SFX(riemann_edge_f)(o, Vs3, f, 1, o->eyk, c, 1, o->aL[0], o->aR[0], o->dL[0], o->dR[0], sk, &phi);
        o->ey[c] = X - phi;
        X = SFX(riemann_edge_f)(o, Vs3, f, o->fstride[1], o->exk, c, sj, o->aL[1], o->aR[1], o->dL[1], o->dR[1], sk, &phi);
        o->ex[c] = X + phi;
#endif
        X = SFX(riemann_edge_f)(o, Vs1, f, o->fstride[1], o->ezi, c, sj, o->aL[1], o->aR[1], o->dL[1], o->dR[1], si, &phi);
        o->ez[c] += X - phi;
#if OFX_D == 3
        X = SFX(riemann_edge_f)(o, Vs1, f, o->fstride[2], o->eyi, c, sk, o->aL[2], o->aR[2], o->dL[2], o->dR[2], si, &phi);
        o->ey[c] += X + phi;
        X = SFX(riemann_edge_f)(o, Vs2, f, o->fstride[2], o->exj, c, sk, o->aL[2], o->aR[2], o->dL[2], o->dR[2], sj, &phi);
        o->ex[c] += X - phi;
#endif
      }
}

/* ---------------------------------------------------------------------- */
/* Flux sweep along dir: RiemannSolver::CalcFlux<dir> + K_Store*         */
/* ---------------------------------------------------------------------- */
/* ---------------------------------------------------------------------- */
/* ShockFlattening::FindShock (shockFlattening.hpp:82-168, 185-201):       */
/* flag cells with div v < 0 and a pressure jump above smoothing x pmin    */
/* ---------------------------------------------------------------------- */
static void SFX(find_shock)(ofx* o) {
  const int kb = o->beg[2] - (OFX_D == 3), ke = o->end[2] + (OFX_D == 3);
  const size_t si = o->stride[0], sj = o->stride[1], sk = o->stride[2];
  const double* vx = o->Vc + (size_t)1 * o->ncell;
  const double* vy = o->Vc + (size_t)2 * o->ncell;
  const double* p = o->Vc + (size_t)PRS * o->ncell;
#if OFX_D == 3
  const double* vz = o->Vc + (size_t)MX3 * o->ncell;
#endif
  (void)sk;
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = kb; k < ke; k++)
    for (int j = o->beg[1] - 1; j < o->end[1] + 1; j++)
      for (int i = o->beg[0] - 1; i < o->end[0] + 1; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        o->flag[c] = 0;
        double divV = CX((vx[c + si] - vx[c - si]) / (2 * o->dx[0]), + (vy[c + sj] - vy[c - sj]) / (2 * o->dx[1]),
                         + (vz[c + sk] - vz[c - sk]) / (2 * o->dx[2]));
        if (divV < 0.0) {
          double pmin = p[c];
          pmin = fmin(pmin, p[c + si]);
          pmin = fmin(pmin, p[c - si]);
          double gradP = fabs(p[c + si] - p[c - si]);
          pmin = fmin(pmin, p[c + sj]);
          pmin = fmin(pmin, p[c - sj]);
          gradP += fabs(p[c + sj] - p[c - sj]);
#if OFX_D == 3
          pmin = fmin(pmin, p[c + sk]);
          pmin = fmin(pmin, p[c - sk]);
          gradP += fabs(p[c + sk] - p[c - sk]);
#endif
          if (gradP > o->smoothing * pmin) o->flag[c] = 1;
        }
      }
}

static void SFX(calc_flux)(ofx* o, int dir) {
  const int io = dir == 0, jo = dir == 1, ko = dir == 2;
  if (o->shock) SFX(find_shock)(o);  /* RiemannSolver::CalcFlux (calcFlux.hpp:33) */
  int ext = 1;
  if ((o->emf == OFX_UCT_HLL || o->emf == OFX_UCT_HLLD) && (o->solver == OFX_HLLD || o->solver == OFX_HLL))
    ext = o->ng;
  const int iext = io ? 0 : ext;
  const int jext = jo ? 0 : ext;
  const int kext = (OFX_D > 2 && !ko) ? ext : 0;
  const int BXt = (dir == 0 ? BX2 : BX1);
#if OFX_D == 3
  const int BXb = (dir == 2 ? BX2 : BX3);
#endif
  double st = 1.0, sb = 1.0;
  double *Et = 0, *Eb = 0, *SV = 0;
  (void)sb; (void)Eb;
  if (dir == 0) { st = -1.0; sb = +1.0; Et = o->ezi; Eb = o->eyi; SV = o->svx; }
  if (dir == 1) { st = +1.0; sb = -1.0; Et = o->ezj; Eb = o->exj; SV = o->svy; }
  if (dir == 2) { st = -1.0; sb = +1.0; Et = o->eyk; Eb = o->exk; SV = o->svz; }
  const int kb = o->beg[2] - kext, ke = o->end[2] + ko + kext;
  const int jb = o->beg[1] - jext, je = o->end[1] + jo + jext;
  const int ib = o->beg[0] - iext, ie = o->end[0] + io + iext;
  const double gamma = o->gamma;
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = kb; k < ke; k++)
    for (int j = jb; j < je; j++)
      for (int i = ib; i < ie; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        double vL[NV], vR[NV];
        SFX(rsout) r;
        SFX(recon)(o, dir, c, vL, vR);
        vL[BX1 + dir] = o->Vs[(size_t)dir * o->nface + OFX_FIDX(o, k, j, i)];
        vR[BX1 + dir] = vL[BX1 + dir];
        switch (o->solver) {
          case OFX_HLLD: SFX(hlld)(dir, gamma, vL, vR, &r); break;
          case OFX_HLL: SFX(hll)(dir, gamma, vL, vR, &r); break;
          case OFX_ROE: SFX(roe)(dir, gamma, vL, vR, &r); break;
          default: SFX(tvdlf)(dir, gamma, vL, vR, &r); break;
        }
        for (int nv = 0; nv < NV; nv++) o->Flux[(size_t)nv * o->ncell + c] = r.F[nv];
        o->cMax[c] = r.cmax;
        if (o->emf == OFX_ARITHMETIC || o->emf == OFX_UCT0 || o->emf == OFX_UCT_CONTACT) {
          /* K_StoreEMF (storeFlux.hpp:14-29) */
          CX(Et[c] = st * r.F[BXt];, , Eb[c] = sb * r.F[BXb];)
          if (o->emf == OFX_UCT_CONTACT) {
            /* K_StoreContact (storeFlux.hpp:31-44) */
            double sv = 0.5;
            if (r.F[RHO] > OFX_EPS_UCT_CONTACT) sv = 1.0;
            if (r.F[RHO] < -OFX_EPS_UCT_CONTACT) sv = 0.0;
            SV[c] = sv;
          }
        } else {
          SFX(store_hll)(o, dir, c, st, sb, &r, vL, vR, Et, Eb);
        }
      }
}

/* ---------------------------------------------------------------------- */
/* Flux correction (xA) and conservative update (calcRightHandSide.hpp)  */
/* ---------------------------------------------------------------------- */
static void SFX(calc_rhs)(ofx* o, int dir, double dt) {
  const int io = dir == 0, jo = dir == 1, ko = dir == 2;
  const double A = o->A[dir];
  const size_t sd = o->stride[dir];
  /* Fluid_CorrectFluxFunctor: Cartesian => Flux *= A  (:84-195) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = o->beg[2]; k < o->end[2] + ko; k++)
    for (int j = o->beg[1]; j < o->end[1] + jo; j++)
      for (int i = o->beg[0]; i < o->end[0] + io; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        for (int nv = 0; nv < NV; nv++) o->Flux[(size_t)nv * o->ncell + c] = o->Flux[(size_t)nv * o->ncell + c] * A;
      }
  /* Fluid_CalcRHSFunctor (:333-550) */
  const double dV = o->dV;
  const double dl = o->dx[dir];
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = o->beg[2]; k < o->end[2]; k++)
    for (int j = o->beg[1]; j < o->end[1]; j++)
      for (int i = o->beg[0]; i < o->end[0]; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        double dtdV = dt / dV;
        double rhs[NV];
        for (int nv = 0; nv < NV; nv++)
          rhs[nv] = -dtdV * (o->Flux[(size_t)nv * o->ncell + c + sd] - o->Flux[(size_t)nv * o->ncell + c]);
        o->InvDt[c] = o->InvDt[c] + 0.5 * (o->cMax[c + sd] + o->cMax[c]) / (dl);
        for (int nv = 0; nv < NV; nv++) {
          if (nv >= BX1) continue; /* field evolved by CT */
          o->Uc[(size_t)nv * o->ncell + c] = o->Uc[(size_t)nv * o->ncell + c] + rhs[nv];
        }
      }
}

/* ---------------------------------------------------------------------- */
/* Cons <-> prim over the whole block (incl. ghosts)                      */
/* ---------------------------------------------------------------------- */
static void SFX(prim_to_cons)(ofx* o) {
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
  for (long c = 0; c < (long)o->ncell; c++) {
    double U[NV], V[NV];
    for (int nv = 0; nv < NV; nv++) V[nv] = o->Vc[(size_t)nv * o->ncell + c];
    SFX(p2c)(o->gamma, U, V);
    for (int nv = 0; nv < NV; nv++) o->Uc[(size_t)nv * o->ncell + c] = U[nv];
  }
}

static void SFX(cons_to_prim)(ofx* o) {
  ofx_reconstruct_vc_field(o, o->Uc);
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
  for (long c = 0; c < (long)o->ncell; c++) {
    double U[NV], V[NV];
    for (int nv = 0; nv < NV; nv++) U[nv] = o->Uc[(size_t)nv * o->ncell + c];
    SFX(c2p)(o->gamma, V, U);
    for (int nv = 0; nv < NV; nv++) o->Vc[(size_t)nv * o->ncell + c] = V[nv];
  }
}

/* ---------------------------------------------------------------------- */
/* Constrained transport (calcCornerEmf.hpp, evolveMagField.hpp)         */
/* ---------------------------------------------------------------------- */
static void SFX(cell_emf)(ofx* o) {
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
  for (long c = 0; c < (long)o->ncell; c++) {
    double vx1 = 0, vx2 = 0, vx3 = 0, Bx1 = 0, Bx2 = 0, Bx3 = 0;
    (void)vx3; (void)Bx3;
    CX(vx1 = o->Vc[(size_t)MX1 * o->ncell + c];, vx2 = o->Vc[(size_t)MX2 * o->ncell + c];,
       vx3 = o->Vc[(size_t)MX3 * o->ncell + c];)
    CX(Bx1 = o->Vc[(size_t)BX1 * o->ncell + c];, Bx2 = o->Vc[(size_t)BX2 * o->ncell + c];,
       Bx3 = o->Vc[(size_t)BX3 * o->ncell + c];)
#if OFX_D == 3
    o->Ex1[c] = (vx3 * Bx2 - vx2 * Bx3);
    o->Ex2[c] = (vx1 * Bx3 - vx3 * Bx1);
#endif
    o->Ex3[c] = (vx2 * Bx1 - vx1 * Bx2);
  }
}

static void SFX(corner_emf)(ofx* o) {
  const size_t si = 1, sj = o->stride[1], sk = o->stride[2];
  (void)sk;
  const int emf = o->emf;
  if (emf == OFX_UCT0) {
    /* CalcUCT0Average face-centred part (calcCornerEmf.hpp:150-172) */
    SFX(cell_emf)(o);
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
    for (int k = o->beg[2] - (OFX_D == 3); k < o->end[2] + (OFX_D == 3); k++)
      for (int j = o->beg[1] - 1; j < o->end[1] + 1; j++)
        for (int i = o->beg[0] - 1; i < o->end[0] + 1; i++) {
          const size_t c = OFX_IDX(o, k, j, i);
#if OFX_D == 3
          o->exj[c] *= 2.0;
          o->exk[c] *= 2.0;
          o->eyi[c] *= 2.0;
          o->eyk[c] *= 2.0;
          o->exj[c] -= 0.5 * (o->Ex1[c - sj] + o->Ex1[c]);
          o->exk[c] -= 0.5 * (o->Ex1[c - sk] + o->Ex1[c]);
          o->eyi[c] -= 0.5 * (o->Ex2[c - si] + o->Ex2[c]);
          o->eyk[c] -= 0.5 * (o->Ex2[c - sk] + o->Ex2[c]);
#endif
          o->ezi[c] *= 2.0;
          o->ezj[c] *= 2.0;
          o->ezi[c] -= 0.5 * (o->Ex3[c - si] + o->Ex3[c]);
          o->ezj[c] -= 0.5 * (o->Ex3[c - sj] + o->Ex3[c]);
        }
  }
  if (emf == OFX_UCT_CONTACT) SFX(cell_emf)(o);
  if (emf == OFX_UCT_HLL || emf == OFX_UCT_HLLD) {
    SFX(riemann_emf)(o);
    return;
  }
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
  for (int k = o->beg[2]; k < o->end[2] + (OFX_D == 3); k++)
    for (int j = o->beg[1]; j < o->end[1] + 1; j++)
      for (int i = o->beg[0]; i < o->end[0] + 1; i++) {
        const size_t c = OFX_IDX(o, k, j, i);
        const double* ezi = o->ezi;
        const double* ezj = o->ezj;
        if (emf == OFX_ARITHMETIC || emf == OFX_UCT0) {
          /* CalcArithmeticAverage / CalcUCT0CornerEMF (calcCornerEmf.hpp:62-78,174-190) */
          const double w = 0.25;
#if OFX_D == 3
          o->ex[c] = w * (o->exj[c] + o->exj[c - sk] + o->exk[c] + o->exk[c - sj]);
          o->ey[c] = w * (o->eyi[c] + o->eyi[c - sk] + o->eyk[c] + o->eyk[c - si]);
#endif
          o->ez[c] = w * (ezi[c] + ezi[c - sj] + ezj[c] + ezj[c - si]);
        } else {
          /* CalcContactAverage (calcCornerEmf.hpp:224-282) */
          const double* wsx = o->svx;
          const double* wsy = o->svy;
          const double* Ex3 = o->Ex3;
          double ez_l2 = (1 - wsx[c - sj]) * (ezj[c] - Ex3[c - sj]) + (wsx[c - sj]) * (ezj[c - si] - Ex3[c - sj - si]);
          double ez_r2 = (1 - wsx[c]) * (ezj[c] - Ex3[c]) + (wsx[c]) * (ezj[c - si] - Ex3[c - si]);
          double ez_l1 = (1 - wsy[c - si]) * (ezi[c] - Ex3[c - si]) + (wsy[c - si]) * (ezi[c - sj] - Ex3[c - sj - si]);
          double ez_r1 = (1 - wsy[c]) * (ezi[c] - Ex3[c]) + (wsy[c]) * (ezi[c - sj] - Ex3[c - sj]);
          o->ez[c] = 0.25 * (ez_l2 + ez_r2 + ez_l1 + ez_r1 + ezi[c] + ezi[c - sj] + ezj[c] + ezj[c - si]);
#if OFX_D == 3
          const double* wsz = o->svz;
          const double* Ex1 = o->Ex1;
          const double* Ex2 = o->Ex2;
          const double *exj = o->exj, *exk = o->exk, *eyi = o->eyi, *eyk = o->eyk;
          double ex_l3 = (1 - wsy[c - sk]) * (exk[c] - Ex1[c - sk]) + (wsy[c - sk]) * (exk[c - sj] - Ex1[c - sk - sj]);
          double ex_r3 = (1 - wsy[c]) * (exk[c] - Ex1[c]) + (wsy[c]) * (exk[c - sj] - Ex1[c - sj]);
          double ex_l2 = (1 - wsz[c - sj]) * (exj[c] - Ex1[c - sj]) + (wsz[c - sj]) * (exj[c - sk] - Ex1[c - sk - sj]);
          double ex_r2 = (1 - wsz[c]) * (exj[c] - Ex1[c]) + (wsz[c]) * (exj[c - sk] - Ex1[c - sk]);
          o->ex[c] = 0.25 * (ex_l3 + ex_r3 + ex_l2 + ex_r2 + exj[c] + exj[c - sk] + exk[c] + exk[c - sj]);
          double ey_l3 = (1 - wsx[c - sk]) * (eyk[c] - Ex2[c - sk]) + (wsx[c - sk]) * (eyk[c - si] - Ex2[c - sk - si]);
          double ey_r3 = (1 - wsx[c]) * (eyk[c] - Ex2[c]) + (wsx[c]) * (eyk[c - si] - Ex2[c - si]);
          double ey_l1 = (1 - wsz[c - si]) * (eyi[c] - Ex2[c - si]) + (wsz[c - si]) * (eyi[c - sk] - Ex2[c - sk - si]);
          double ey_r1 = (1 - wsz[c]) * (eyi[c] - Ex2[c]) + (wsz[c]) * (eyi[c - sk] - Ex2[c - sk]);
          o->ey[c] = 0.25 * (ey_l3 + ey_r3 + ey_l1 + ey_r1 + eyi[c] + eyi[c - sk] + eyk[c] + eyk[c - si]);
#endif
        }
      }
}

/* Vs += curl(E) dt  (evolveMagField.hpp:53-132, Cartesian).  Only the
   faces that are not refilled by the next boundary pass are updated. */
static void SFX(evolve_mag_field)(ofx* o, double dt) {
  const size_t si = 1, sj = o->stride[1], sk = o->stride[2];
  (void)sk;
  const double dx1 = o->dx[0], dx2 = o->dx[1], dx3 = o->dx[2];
  (void)dx3;
  const double *Ex1 = o->ex, *Ex2 = o->ey, *Ex3 = o->ez;
  (void)Ex1; (void)Ex2;
  for (int comp = 0; comp < OFX_D; comp++) {
    const int io = comp == 0, jo = comp == 1, ko = comp == 2;
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
    for (int k = o->beg[2]; k < o->end[2] + ko; k++)
      for (int j = o->beg[1]; j < o->end[1] + jo; j++)
        for (int i = o->beg[0]; i < o->end[0] + io; i++) {
          const size_t c = OFX_IDX(o, k, j, i);
          double* vs = &o->Vs[(size_t)comp * o->nface + OFX_FIDX(o, k, j, i)];
          double rhs;
          if (comp == 0) {
#if OFX_D == 2
            rhs = 0.0 - dt / dx2 * (Ex3[c + sj] - Ex3[c]);
#else
            rhs = 0.0 - dt / dx2 * (Ex3[c + sj] - Ex3[c]) + dt / dx3 * (Ex2[c + sk] - Ex2[c]);
#endif
          } else if (comp == 1) {
#if OFX_D == 2
            rhs = dt / dx1 * (Ex3[c + si] - Ex3[c]);
#else
            rhs = dt / dx1 * (Ex3[c + si] - Ex3[c]) - dt / dx3 * (Ex1[c + sk] - Ex1[c]);
#endif
          } else {
#if OFX_D == 3
            rhs = -dt / dx1 * (Ex2[c + si] - Ex2[c]) + dt / dx2 * (Ex1[c + sj] - Ex1[c]);
#else
            rhs = 0.0;
#endif
          }
          *vs = *vs + rhs;
        }
  }
}

static void SFX(evolve_stage)(ofx* o, double t, double dt) {
  (void)t;
  for (int dir = 0; dir < OFX_D; dir++) {
    OFX_PHASE(OFX_PH_SWEEP_X + dir);
    SFX(calc_flux)(o, dir);
    SFX(calc_rhs)(o, dir, dt);
  }
  OFX_PHASE(OFX_PH_CT_CORNER);
  SFX(corner_emf)(o);
  OFX_PHASE(OFX_PH_CT_FACES);
  SFX(evolve_mag_field)(o, dt);
  ofx_reconstruct_vc_field(o, o->Uc);
  OFX_PHASE(OFX_PH_OTHER);
}

#undef SFX
#undef CX
#undef NV
#undef MX3
#undef BX1
#undef BX2
#undef BX3
#undef ENG
#undef PRS
