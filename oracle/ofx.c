/*
 * CPU oracle for the ideal-MHD Godunov stage — TEST INFRASTRUCTURE ONLY.
 * See ofx.h.  Compile with -O2 -ffp-contract=off (no -ffast-math); OpenMP
 * optional (all reductions are min/max, so results do not depend on the
 * thread count).
 */
#include "ofx.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#define RHO 0
#define MX1 1
#define MX2 2

/* Phases of a cycle for the operation-counting build (opcount.cpp defines
   OFX_PHASE to switch its counters); no-ops in the plain oracle. */
enum { OFX_PH_OTHER = 0, OFX_PH_SWEEP_X, OFX_PH_SWEEP_Y, OFX_PH_SWEEP_Z, OFX_PH_CT_CORNER,
       OFX_PH_CT_FACES, OFX_PH_BOUNDARIES, OFX_PH_PRIM2CONS, OFX_PH_RK, OFX_PH_CONS2PRIM,
       OFX_PH_TIMESTEP, OFX_PH_CHECKS, OFX_NPH };
#ifndef OFX_PHASE
#define OFX_PHASE(p) ((void)0)
#endif

#define OFX_SMALL_PRESSURE_FIX (1.0e-5) /* fluid_defs.hpp:23 */
#define OFX_EPS_UCT_CONTACT (1.0e-6)    /* fluid_defs.hpp:24 */

struct ofx {
  int D, nvar, ng, order, solver, emf, nstages;
  int n[3], nt[3], ntv[3], beg[3], end[3];
  size_t stride[3], fstride[3];
  size_t ncell, nface;
  double dx[3], xb[3], xe[3];
  double A[3], dV;
  double gamma, cfl, cflmax, maxdivb;
  double t, dt;
  long ncycles;
  int log_period, check_nan_period;
  int nthreads;
  double *Vc, *Uc, *Vs, *Uc0, *Vs0, *Flux, *cMax, *InvDt;
  double *ezi, *ezj, *exj, *exk, *eyi, *eyk, *svx, *svy, *svz;
  double *Ex1, *Ex2, *Ex3, *ex, *ey, *ez;
  double *aL[3], *aR[3], *dL[3], *dR[3];
  int lbound[3], rbound[3]; /* 0 periodic, 1 reflective, 2 outflow    */
  int shock;            /* [Hydro] shockFlattening present              */
  double smoothing;     /* its value                                    */
  unsigned char* flag;  /* FlagShock per cell (1 = Shock), zero outside */
};

#define OFX_IDX(o, k, j, i) (((size_t)(k) * (o)->nt[1] + (size_t)(j)) * (o)->nt[0] + (size_t)(i))
#define OFX_FIDX(o, k, j, i) (((size_t)(k) * (o)->ntv[1] + (size_t)(j)) * (o)->ntv[0] + (size_t)(i))

/* ---------------------------------------------------------------------- */
/* Slope limiters (slopeLimiter.hpp)                                       */
/* ---------------------------------------------------------------------- */
/* SlopeLimiter::MinModLim declares an inner `dq` that shadows the returned
   one, so the reference limiter always yields 0 (slopeLimiter.hpp:16-23). */
static double ofx_minmod(double dvp, double dvm) {
  (void)dvp;
  (void)dvm;
  return 0.0;
}

static double ofx_vanleer(double dvp, double dvm) { /* :54-57 */
  return (dvp * dvm > 0.0 ? 2.0 * dvp * dvm / (dvp + dvm) : 0.0);
}

static double ofx_mclim(double dvp, double dvm) { /* :68-76 */
  double dq = 0;
  if (dvp * dvm > 0.0) {
    double dqc = 0.5 * (dvp + dvm);
    double d2q = 2.0 * (fabs(dvp) < fabs(dvm) ? dvp : dvm);
    dq = fabs(d2q) < fabs(dqc) ? d2q : dqc;
  }
  return dq;
}

static double ofx_limo3(double dvp, double dvm, double dx) { /* :25-52 */
  double r = 0.1;
  double a, b, c, q, th, lim;
  double eta, psi, eps = 1.e-12;
  th = dvm / (dvp + 1.e-16);
  q = (2.0 + th) / 3.0;
  a = fmin(1.5, 2.0 * th);
  a = fmin(q, a);
  b = fmax(-0.5 * th, a);
  c = fmin(q, b);
  psi = fmax(0.0, c);
  eta = r * dx;
  eta = (dvm * dvm + dvp * dvp) / (eta * eta);
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

static int ofx_sign(double v) { return (0.0 < v) - (v < 0.0); }

static void ofx_limit_ppm_face(double vm1, double v0, double vp1, double vp2, double* vph) { /* :121-140 */
  if ((vp1 - *vph) * (*vph - v0) < 0.0) {
    const double deltaL = (vm1 - 2 * v0 + vp1);
    const double deltaC = 3 * (v0 - 2 * (*vph) + vp1);
    const double deltaR = (v0 - 2 * vp1 + vp2);
    double delta = 0.0;
    if (ofx_sign(deltaL) == ofx_sign(deltaC) && ofx_sign(deltaR) == ofx_sign(deltaC)) {
      const double C = 1.25;
      delta = C * fmin(fabs(deltaL), fabs(deltaR));
      delta = ofx_sign(deltaC) * fmin(delta, fabs(deltaC));
    }
    *vph = 0.5 * (v0 + vp1) - delta / 6.0;
  }
}

static void ofx_ppm_states(double vm2, double vm1, double v0, double vp1, double vp2, double* vl,
                           double* vr) { /* :142-191 */
  const int n = 2;
  *vr = 7.0 / 12.0 * (v0 + vp1) - 1.0 / 12.0 * (vm1 + vp2);
  *vl = 7.0 / 12.0 * (vm1 + v0) - 1.0 / 12.0 * (vm2 + vp1);
  ofx_limit_ppm_face(vm2, vm1, v0, vp1, vl);
  ofx_limit_ppm_face(vm1, v0, vp1, vp2, vr);
  double d2qf = 6.0 * (*vl + *vr - 2.0 * v0);
  double d2qc0 = vm1 + vp1 - 2.0 * v0;
  double d2qcp1 = v0 + vp2 - 2.0 * vp1;
  double d2qcm1 = vm2 + v0 - 2.0 * vm1;
  double d2q = 0.0;
  if (ofx_sign(d2qf) == ofx_sign(d2qc0) && ofx_sign(d2qf) == ofx_sign(d2qcp1) &&
      ofx_sign(d2qf) == ofx_sign(d2qcm1)) {
    const double C = 1.25;
    d2q = fmin(fabs(d2qc0), fabs(d2qcp1));
    d2q = C * fmin(fabs(d2qcm1), d2q);
    d2q = ofx_sign(d2qf) * fmin(fabs(d2qf), d2q);
  }
  double qmax = fmax(fmax(fabs(vm1), fabs(v0)), fabs(vp1));
  double rho = 0.0;
  if (fabs(d2qf) > 1e-12 * qmax) rho = d2q / d2qf;
  if (((*vr - v0) * (v0 - *vl) <= 0) || (vm1 - v0) * (v0 - vp1) <= 0) {
    if (rho <= (1.0 - 1e-12)) {
      *vl = v0 - rho * (v0 - *vl);
      *vr = v0 + rho * (*vr - v0);
    }
  } else {
    if (fabs(*vr - v0) >= n * fabs(v0 - *vl)) *vr = v0 + n * (v0 - *vl);
    if (fabs(*vl - v0) >= n * fabs(v0 - *vr)) *vl = v0 + n * (v0 - *vr);
  }
}

/* Vc(BXd) = 0.5 (Vs(d,i) + Vs(d,i+1)) over the whole block
   (boundary.hpp:388-404) */
static void ofx_reconstruct_vc_field(ofx* o, double* arr) {
  const int BX1 = o->D + 2;
  for (int d = 0; d < o->D; d++) {
    const size_t fs = o->fstride[d];
    const double* vs = o->Vs + (size_t)d * o->nface;
    double* out = arr + (size_t)(BX1 + d) * o->ncell;
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads)
    for (int k = 0; k < o->nt[2]; k++)
      for (int j = 0; j < o->nt[1]; j++)
        for (int i = 0; i < o->nt[0]; i++) {
          const size_t f = OFX_FIDX(o, k, j, i);
          out[OFX_IDX(o, k, j, i)] = 0.5 * (vs[f] + vs[f + fs]);
        }
  }
}

#define OFX_D 2
#include "ofx_core.h"
#undef OFX_D
#define OFX_D 3
#include "ofx_core.h"
#undef OFX_D

/* ---------------------------------------------------------------------- */
/* Periodic ghost fill (boundary.hpp:576-673 with BoundaryFor* ranges)    */
/* ---------------------------------------------------------------------- */
static int ofx_wrap(int i, int g, int n) { return g + (i + g * (n - 1)) % n; }

/* reference index of a ghost point along dir for one boundary type
   (boundary.hpp:582-600 periodic, 687-689 reflective, 750-752 outflow);
   n: active cells along dir, side 0 left / 1 right */
static int ofx_bc_ref(int type, int idx, int g, int n, int side) {
  if (type == 0) return ofx_wrap(idx, g, n);
  if (type == 1) return 2 * (g + side * n) - idx - 1;
  return g + side * (n - 1);
}

/* ReconstructNormalField (boundary.hpp:408-532): the normal field in the
   ghost faces of dir from div B = 0, outwards from the boundary face */
static void ofx_normal_field(ofx* o, int dir) {
  const int left = o->lbound[dir] != 0, right = o->rbound[dir] != 0;
  if (!left && !right) return;
  double* V1 = o->Vs;
  double* V2 = o->Vs + o->nface;
  double* V3 = o->D == 3 ? o->Vs + 2 * o->nface : 0;
  const double A1 = o->A[0], A2 = o->A[1], A3 = o->A[2];
  const int nb = o->beg[dir] - 1, ne = o->end[dir];
#define F1(k, j, i) V1[OFX_FIDX(o, k, j, i)]
#define F2(k, j, i) V2[OFX_FIDX(o, k, j, i)]
#define F3(k, j, i) V3[OFX_FIDX(o, k, j, i)]
  if (dir == 0) {
    for (int k = 0; k < o->nt[2]; k++)
      for (int j = 0; j < o->nt[1]; j++) {
        if (left)
          for (int i = nb; i >= 0; i--) {
            double t = 0.0 + A2 * F2(k, j + 1, i) - A2 * F2(k, j, i);
            if (o->D == 3) t = t + A3 * F3(k + 1, j, i) - A3 * F3(k, j, i);
            F1(k, j, i) = 1.0 / A1 * (A1 * F1(k, j, i + 1) + (t));
          }
        if (right)
          for (int i = ne; i < o->nt[0]; i++) {
            double t = 0.0 + A2 * F2(k, j + 1, i) - A2 * F2(k, j, i);
            if (o->D == 3) t = t + A3 * F3(k + 1, j, i) - A3 * F3(k, j, i);
            F1(k, j, i + 1) = 1.0 / A1 * (A1 * F1(k, j, i) - (t));
          }
      }
  } else if (dir == 1) {
    for (int k = 0; k < o->nt[2]; k++)
      for (int i = 0; i < o->nt[0]; i++) {
        if (left)
          for (int j = nb; j >= 0; j--) {
            double t = A1 * F1(k, j, i + 1) - A1 * F1(k, j, i);
            if (o->D == 3) t = t + 1 * (A3 * F3(k + 1, j, i) - A3 * F3(k, j, i));
            F2(k, j, i) = 1.0 / A2 * (A2 * F2(k, j + 1, i) + (t));
          }
        if (right)
          for (int j = ne; j < o->nt[1]; j++) {
            double t = A1 * F1(k, j, i + 1) - A1 * F1(k, j, i);
            if (o->D == 3) t = t + 1 * (A3 * F3(k + 1, j, i) - A3 * F3(k, j, i));
            F2(k, j + 1, i) = 1.0 / A2 * (A2 * F2(k, j, i) - (t));
          }
      }
  } else {
    for (int j = 0; j < o->nt[1]; j++)
      for (int i = 0; i < o->nt[0]; i++) {
        if (left)
          for (int k = nb; k >= 0; k--) {
            F3(k, j, i) = 1.0 / A3 * (A3 * F3(k + 1, j, i) + (A1 * F1(k, j, i + 1) - A1 * F1(k, j, i) +
                                                              A2 * F2(k, j + 1, i) - A2 * F2(k, j, i)));
          }
        if (right)
          for (int k = ne; k < o->nt[2]; k++) {
            F3(k + 1, j, i) = 1.0 / A3 * (A3 * F3(k, j, i) - (A1 * F1(k, j, i + 1) - A1 * F1(k, j, i) +
                                                              A2 * F2(k, j + 1, i) - A2 * F2(k, j, i)));
          }
      }
  }
#undef F1
#undef F2
#undef F3
}

/* Boundary::SetBoundaries (boundary.hpp:240-280): per direction, both sides
   of the cell-centred variables and of the face field (BoundaryFor* ranges,
   boundary.hpp:971-1100), then the normal field; finally the cell field. */
void ofx_set_boundaries(ofx* o) {
  const int g = o->ng;
  const int BX1v = o->D + 2;
  for (int dir = 0; dir < o->D; dir++) {
    for (int side = 0; side < 2; side++) {
      const int type = side ? o->rbound[dir] : o->lbound[dir];
      /* cell-centred: BoundaryForAll */
      int lo[3], hi[3];
      for (int d = 0; d < 3; d++) {
        lo[d] = 0;
        hi[d] = o->nt[d];
      }
      lo[dir] = side * (g + o->n[dir]);
      hi[dir] = g + side * (g + o->n[dir]);
      for (int nv = 0; nv < o->nvar; nv++) {
        double* a = o->Vc + (size_t)nv * o->ncell;
        /* reflective: normal velocity and tangential field change sign */
        const int sign = (nv == 1 + dir || (nv >= BX1v && nv != BX1v + dir)) ? -1 : 1;
        for (int k = lo[2]; k < hi[2]; k++)
          for (int j = lo[1]; j < hi[1]; j++)
            for (int i = lo[0]; i < hi[0]; i++) {
              const int ir = dir == 0 ? ofx_bc_ref(type, i, g, o->n[0], side) : i;
              const int jr = dir == 1 ? ofx_bc_ref(type, j, g, o->n[1], side) : j;
              const int kr = dir == 2 ? ofx_bc_ref(type, k, g, o->n[2], side) : k;
              const double src = a[OFX_IDX(o, kr, jr, ir)];
              double* dst = &a[OFX_IDX(o, k, j, i)];
              if (type == 0) {
                *dst = src;
              } else if (type == 1) {
                *dst = sign * src;
              } else {
                /* outflow: no inflow through the boundary (boundary.hpp:757-762) */
                const int sg = 1 - 2 * side;
                if (nv == 1 + dir && sg * src >= 0.0) *dst = 0.0;
                else *dst = src;
              }
            }
      }
      /* face-centred: BoundaryForX{1,2,3}s; periodic copies every component,
         the others only the tangential ones (the normal one is rebuilt) */
      for (int comp = 0; comp < o->D; comp++) {
        if (type != 0 && comp == dir) continue;
        int flo[3], fhi[3];
        for (int d = 0; d < 3; d++) {
          int nn = o->n[d] + (d == comp);
          int gd = (d < o->D) ? g : 0;
          flo[d] = 0;
          fhi[d] = o->nt[d] + (d == comp);
          if (d == dir) {
            flo[d] = side * (gd + nn);
            fhi[d] = gd + side * (gd + nn);
          }
        }
        double* a = o->Vs + (size_t)comp * o->nface;
        for (int k = flo[2]; k < fhi[2]; k++)
          for (int j = flo[1]; j < fhi[1]; j++)
            for (int i = flo[0]; i < fhi[0]; i++) {
              const int ir = dir == 0 ? ofx_bc_ref(type, i, g, o->n[0], side) : i;
              const int jr = dir == 1 ? ofx_bc_ref(type, j, g, o->n[1], side) : j;
              const int kr = dir == 2 ? ofx_bc_ref(type, k, g, o->n[2], side) : k;
              const double src = a[OFX_FIDX(o, kr, jr, ir)];
              a[OFX_FIDX(o, k, j, i)] = (type == 1) ? -src : src;
            }
      }
    }
    ofx_normal_field(o, dir);
  }
  ofx_reconstruct_vc_field(o, o->Vc);
}

int ofx_set_bc(ofx* o, int dir, int left, int right) {
  if (dir < 0 || dir >= o->D || left < 0 || left > 2 || right < 0 || right > 2) return OFX_ERR_CONFIG;
  if ((left == 0) != (right == 0)) return OFX_ERR_CONFIG;
  o->lbound[dir] = left;
  o->rbound[dir] = right;
  return OFX_OK;
}

/* ---------------------------------------------------------------------- */
static double* ofx_zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

ofx* ofx_create(int dims, int nx, int ny, int nz, double xb0, double xe0, double xb1, double xe1,
                double xb2, double xe2, int order, int solver, int emf, int nstages, double gamma,
                double cfl, double cfl_max_var, double first_dt) {
  if (dims != 2 && dims != 3) return NULL;
  if (order < 1 || order > 4 || solver < 0 || solver > 3 || emf < 0 || emf > 4) return NULL;
  if (nstages < 1 || nstages > 3) return NULL;
  if (emf == OFX_UCT_HLLD && (solver == OFX_HLL || solver == OFX_TVDLF)) return NULL;
  ofx* o = (ofx*)calloc(1, sizeof(ofx));
  o->D = dims;
  o->nvar = 2 * dims + 2;
  o->ng = (order == 4) ? 3 : 2; /* grid.cpp:60-65 */
  o->order = order;
  o->solver = solver;
  o->emf = emf;
  o->nstages = nstages;
  int n[3] = {nx, ny, dims == 3 ? nz : 1};
  double xb[3] = {xb0, xb1, xb2}, xe[3] = {xe0, xe1, xe2};
  for (int d = 0; d < 3; d++) {
    int active = d < dims;
    int g = active ? o->ng : 0;
    o->n[d] = n[d];
    o->nt[d] = n[d] + 2 * g;
    o->ntv[d] = o->nt[d] + active;
    o->beg[d] = g;
    o->end[d] = g + n[d];
    o->xb[d] = active ? xb[d] : 0.0;
    o->xe[d] = active ? xe[d] : 1.0;
    o->dx[d] = (o->xe[d] - o->xb[d]) / (n[d]); /* gridHost.cpp:80-86 */
  }
  o->stride[0] = 1;
  o->stride[1] = (size_t)o->nt[0];
  o->stride[2] = (size_t)o->nt[0] * o->nt[1];
  o->fstride[0] = 1;
  o->fstride[1] = (size_t)o->ntv[0];
  o->fstride[2] = (size_t)o->ntv[0] * o->ntv[1];
  o->ncell = (size_t)o->nt[0] * o->nt[1] * o->nt[2];
  o->nface = (size_t)o->ntv[0] * o->ntv[1] * o->ntv[2];
  /* Cartesian areas and volume (makeGeometry.cpp:67-70,146-147,178-179,201-202) */
  if (dims == 2) {
    o->dV = o->dx[0] * o->dx[1];
    o->A[0] = 1.0 * o->dx[1];
    o->A[1] = o->dx[0] * 1.0;
    o->A[2] = 1.0;
  } else {
    o->dV = o->dx[0] * o->dx[1] * o->dx[2];
    o->A[0] = 1.0 * o->dx[1] * o->dx[2];
    o->A[1] = o->dx[0] * 1.0 * o->dx[2];
    o->A[2] = o->dx[0] * o->dx[1] * 1.0;
  }
  o->gamma = gamma;
  o->cfl = cfl;
  o->cflmax = cfl_max_var;
  o->maxdivb = 1e-6;
  o->t = 0.0;
  o->dt = first_dt;
  o->ncycles = 0;
  o->log_period = 0;
  o->check_nan_period = 0;
  o->nthreads = 1;
  size_t nc = o->ncell, NVv = (size_t)o->nvar;
  o->Vc = ofx_zalloc(NVv * nc);
  o->Uc = ofx_zalloc(NVv * nc);
  o->Uc0 = ofx_zalloc(NVv * nc);
  o->Flux = ofx_zalloc(NVv * nc);
  o->Vs = ofx_zalloc((size_t)dims * o->nface);
  o->Vs0 = ofx_zalloc((size_t)dims * o->nface);
  o->cMax = ofx_zalloc(nc);
  o->InvDt = ofx_zalloc(nc);
  o->ezi = ofx_zalloc(nc);
  o->ezj = ofx_zalloc(nc);
  o->exj = ofx_zalloc(nc);
  o->exk = ofx_zalloc(nc);
  o->eyi = ofx_zalloc(nc);
  o->eyk = ofx_zalloc(nc);
  o->svx = ofx_zalloc(nc);
  o->svy = ofx_zalloc(nc);
  o->svz = ofx_zalloc(nc);
  o->Ex1 = ofx_zalloc(nc);
  o->Ex2 = ofx_zalloc(nc);
  o->Ex3 = ofx_zalloc(nc);
  o->ex = ofx_zalloc(nc);
  o->ey = ofx_zalloc(nc);
  o->ez = ofx_zalloc(nc);
  for (int d = 0; d < 3; d++) {
    o->aL[d] = ofx_zalloc(nc);
    o->aR[d] = ofx_zalloc(nc);
    o->dL[d] = ofx_zalloc(nc);
    o->dR[d] = ofx_zalloc(nc);
  }
  o->flag = (unsigned char*)calloc(nc ? nc : 1, 1);
  return o;
}

void ofx_destroy(ofx* o) {
  if (!o) return;
  double* arrs[] = {o->Vc, o->Uc, o->Uc0, o->Flux, o->Vs, o->Vs0, o->cMax, o->InvDt, o->ezi, o->ezj,
                    o->exj, o->exk, o->eyi, o->eyk, o->svx, o->svy, o->svz, o->Ex1, o->Ex2, o->Ex3,
                    o->ex, o->ey, o->ez};
  for (size_t a = 0; a < sizeof(arrs) / sizeof(arrs[0]); a++) free(arrs[a]);
  for (int d = 0; d < 3; d++) {
    free(o->aL[d]);
    free(o->aR[d]);
    free(o->dL[d]);
    free(o->dR[d]);
  }
  free(o->flag);
  free(o);
}

int ofx_nvar(const ofx* o) { return o->nvar; }
int ofx_nghost(const ofx* o) { return o->ng; }
long ofx_ncell(const ofx* o) { return (long)o->ncell; }
long ofx_nface(const ofx* o) { return (long)o->nface; }
void ofx_set_threads(ofx* o, int n) { o->nthreads = n > 0 ? n : 1; }

void ofx_set_prim(ofx* o, const double* Vc, const double* Vs) {
  memcpy(o->Vc, Vc, sizeof(double) * o->nvar * o->ncell);
  memcpy(o->Vs, Vs, sizeof(double) * o->D * o->nface);
}
void ofx_get_prim(const ofx* o, double* Vc, double* Vs) {
  if (Vc) memcpy(Vc, o->Vc, sizeof(double) * o->nvar * o->ncell);
  if (Vs) memcpy(Vs, o->Vs, sizeof(double) * o->D * o->nface);
}
void ofx_get_cons(const ofx* o, double* Uc) { memcpy(Uc, o->Uc, sizeof(double) * o->nvar * o->ncell); }
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
  o->shock = enabled != 0;
  o->smoothing = smoothing;
}

void ofx_set_checks(ofx* o, int log_period, int check_nan_period, double maxdivb) {
  o->log_period = log_period;
  o->check_nan_period = check_nan_period;
  o->maxdivb = maxdivb;
}

void ofx_prim_to_cons(ofx* o) {
  if (o->D == 2) prim_to_cons_d2(o);
  else prim_to_cons_d3(o);
}
void ofx_cons_to_prim(ofx* o) {
  if (o->D == 2) cons_to_prim_d2(o);
  else cons_to_prim_d3(o);
}
void ofx_reset_stage(ofx* o) { memset(o->InvDt, 0, sizeof(double) * o->ncell); }
void ofx_evolve_stage(ofx* o, double t, double dt) {
  if (o->D == 2) evolve_stage_d2(o, t, dt);
  else evolve_stage_d3(o, t, dt);
}

double ofx_compute_timestep(ofx* o) { /* dataBlock.cpp:333-364 */
  double dt = HUGE_VAL;
  for (int k = o->beg[2]; k < o->end[2]; k++)
    for (int j = o->beg[1]; j < o->end[1]; j++)
      for (int i = o->beg[0]; i < o->end[0]; i++) dt = fmin(1.0 / o->InvDt[OFX_IDX(o, k, j, i)], dt);
  return dt;
}

double ofx_check_divb(ofx* o) { /* checkDivB.hpp:14-68 (Cartesian) */
  double divB = 0.0; /* Kokkos::Max identity is the lowest double; every term is >= 0 */
  const double A1 = o->A[0], A2 = o->A[1], A3 = o->A[2];
  (void)A3;
  for (int k = o->beg[2]; k < o->end[2]; k++)
    for (int j = o->beg[1]; j < o->end[1]; j++)
      for (int i = o->beg[0]; i < o->end[0]; i++) {
        const double* B1s = o->Vs;
        const double* B2s = o->Vs + o->nface;
        const size_t f = OFX_FIDX(o, k, j, i);
        double dB1 = (A1 * B1s[f + 1] - A1 * B1s[f]);
        double dB2 = (A2 * B2s[f + o->fstride[1]] - A2 * B2s[f]);
        double d1 = 0.5 * (A1 + A1);
        double d2 = 0.5 * (A2 + A2);
        double B1 = 0.5 * (B1s[f + 1] + B1s[f]);
        double B2 = 0.5 * (B2s[f + o->fstride[1]] + B2s[f]);
        double amplitude = 1e-40;
        double v;
        if (o->D == 2) {
          amplitude += fabs(B1) * d1 + fabs(B2) * d2;
          v = fabs(dB1 + dB2) / amplitude;
        } else {
          const double* B3s = o->Vs + 2 * o->nface;
          double dB3 = (A3 * B3s[f + o->fstride[2]] - A3 * B3s[f]);
          double d3 = 0.5 * (A3 + A3);
          double B3 = 0.5 * (B3s[f + o->fstride[2]] + B3s[f]);
          amplitude += fabs(B1) * d1 + fabs(B2) * d2 + fabs(B3) * d3;
          v = fabs(dB1 + dB2 + dB3) / amplitude;
        }
        divB = fmax(v, divB);
      }
  return divB;
}

long ofx_check_nan(ofx* o) { /* checkNan.hpp:17-45 */
  long n = 0;
  for (int nv = 0; nv < o->nvar; nv++)
    for (int k = o->beg[2]; k < o->end[2]; k++)
      for (int j = o->beg[1]; j < o->end[1]; j++)
        for (int i = o->beg[0]; i < o->end[0]; i++)
          if (isnan(o->Vc[(size_t)nv * o->ncell + OFX_IDX(o, k, j, i)])) n++;
  /* every component over the union face range, as the reference does */
  for (int comp = 0; comp < o->D; comp++)
    for (int k = o->beg[2]; k < o->end[2] + (o->D == 3); k++)
      for (int j = o->beg[1]; j < o->end[1] + 1; j++)
        for (int i = o->beg[0]; i < o->end[0] + 1; i++)
          if (isnan(o->Vs[(size_t)comp * o->nface + OFX_FIDX(o, k, j, i)])) n++;
  return n;
}

/* TimeIntegrator::Cycle (timeIntegrator.cpp:246-414) */
int ofx_cycle(ofx* o) {
  double wc[2] = {0, 0}, w0[2] = {0, 0};
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
  OFX_PHASE(OFX_PH_CHECKS);
  if (o->log_period > 0 && o->ncycles % o->log_period == 0) {
    if (ofx_check_divb(o) > o->maxdivb) return OFX_ERR_DIVB;
  }
  OFX_PHASE(OFX_PH_OTHER);
  const double t0 = o->t;
  double newdt = 0.0;
  ofx_reset_stage(o);
  for (int stage = 0; stage < o->nstages; stage++) {
    OFX_PHASE(OFX_PH_BOUNDARIES);
    ofx_set_boundaries(o);
    OFX_PHASE(OFX_PH_PRIM2CONS);
    ofx_prim_to_cons(o);
    OFX_PHASE(OFX_PH_OTHER);
    if (o->nstages > 1 && stage == 0) {
      memcpy(o->Uc0, o->Uc, sizeof(double) * o->nvar * o->ncell);
      memcpy(o->Vs0, o->Vs, sizeof(double) * o->D * o->nface);
    }
    ofx_evolve_stage(o, o->t, o->dt);
    o->t += o->dt;
    OFX_PHASE(OFX_PH_CHECKS);
    if (o->check_nan_period > 0 && o->ncycles % o->check_nan_period == 0) {
      if (ofx_check_nan(o) > 0) return OFX_ERR_NAN;
    }
    OFX_PHASE(OFX_PH_TIMESTEP);
    if (stage == 0) newdt = o->cfl * ofx_compute_timestep(o);
    OFX_PHASE(OFX_PH_RK);
    if (stage > 0) {
      const double wcs = wc[stage - 1], w0s = w0[stage - 1];
      const size_t nu = (size_t)o->nvar * o->ncell, ns = (size_t)o->D * o->nface;
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
      for (long a = 0; a < (long)nu; a++) o->Uc[a] = wcs * o->Uc[a] + w0s * o->Uc0[a];
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
      for (long a = 0; a < (long)ns; a++) o->Vs[a] = wcs * o->Vs[a] + w0s * o->Vs0[a];
      o->t = wcs * o->t + w0s * t0;
    }
    OFX_PHASE(OFX_PH_CONS2PRIM);
    ofx_cons_to_prim(o);
    OFX_PHASE(OFX_PH_OTHER);
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
  return OFX_OK;
}

/* main loop (main.cpp:190-225) */
int ofx_run(ofx* o, double tstop, long max_cycles) {
  long done = 0;
  while (1) {
    if (tstop >= 0 && !(o->t < tstop)) break;
    if (max_cycles >= 0 && done >= max_cycles) break;
    if (tstop >= 0 && tstop - o->t < o->dt) o->dt = tstop - o->t;
    int st = ofx_cycle(o);
    if (st) return st;
    done++;
  }
  return OFX_OK;
}
