/*
 * CPU oracle for the ideal-MHD Godunov stage — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm (Idefix v2.2.02,
 * Cartesian, uniform grid, periodic, reflective or outflow boundaries,
 * COMPONENTS == DIMENSIONS in {2,3}).
 * It is the oracle of the CUDA path: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  Nothing in the product library
 * links or calls it.
 *
 * Parity pin: the same entry points are also built from the reference's own
 * hot-path headers (see ref_harness.cpp in this folder); the tests compare the
 * two bit for bit on seeded inputs, and the golden fixtures under
 * tests/golden/ were produced by that reference build.
 *
 * Arrays use the reference layout (LayoutRight):
 *   Vc[nvar][nt2][nt1][nt0]            nt = n + 2*nghost (1 in unused dims)
 *   Vs[dims][nt2+ko][nt1+jo][nt0+io]   face-centred field, +1 in active dims
 * Variable order: RHO, MX1..MXd, ENG(=PRS), BX1..BXd   (src/idefix.hpp:74-108)
 *
 * Build with -ffp-contract=off: the reference CI compares CPU and GPU results
 * with FMA contraction disabled (pytools/idfx_test.py:121-123).
 */
#ifndef OFX_H_
#define OFX_H_
#ifdef __cplusplus
extern "C" {
#endif

/* reconstruction order (CMakeLists.txt:198-209 ORDER) */
enum { OFX_ORDER1 = 1, OFX_PLM = 2, OFX_LIMO3 = 3, OFX_PPM = 4 };
/* Riemann solvers (riemannSolver.hpp:27) */
enum { OFX_HLLD = 0, OFX_HLL = 1, OFX_ROE = 2, OFX_TVDLF = 3 };
/* EMF averaging (constrainedTransport.hpp:155-179) */
enum { OFX_UCT_CONTACT = 0, OFX_ARITHMETIC = 1, OFX_UCT0 = 2, OFX_UCT_HLL = 3, OFX_UCT_HLLD = 4 };

/* status codes: same meaning as the product C-ABI */
enum { OFX_OK = 0, OFX_ERR_CONFIG = 1, OFX_ERR_NAN = 2, OFX_ERR_DIVB = 3,
       OFX_ERR_DT_SMALL = 4, OFX_ERR_FIRST_DT = 5 };

typedef struct ofx ofx;

ofx*   ofx_create(int dims, int nx, int ny, int nz,
                  double xb0, double xe0, double xb1, double xe1, double xb2, double xe2,
                  int order, int solver, int emf, int nstages,
                  double gamma, double cfl, double cfl_max_var, double first_dt);
void   ofx_destroy(ofx* o);
int    ofx_nvar(const ofx* o);
int    ofx_nghost(const ofx* o);
long   ofx_ncell(const ofx* o);     /* nt0*nt1*nt2          */
long   ofx_nface(const ofx* o);     /* (nt0+io)*(nt1+jo)*.. */
void   ofx_set_threads(ofx* o, int n);

/* state transfer in the reference layout */
void   ofx_set_prim(ofx* o, const double* Vc, const double* Vs);
void   ofx_get_prim(const ofx* o, double* Vc, double* Vs);
void   ofx_get_cons(const ofx* o, double* Uc);
void   ofx_set_time(ofx* o, double t, double dt, long ncycles);
void   ofx_get_time(const ofx* o, double* t, double* dt, long* ncycles);
/* diagnostic periods: 0 disables (TimeIntegrator "log" and "check_nan") */
void   ofx_set_checks(ofx* o, int log_period, int check_nan_period, double maxdivb);

/* [Hydro] shockFlattening <smoothing> (riemannSolver.hpp:153-159): cells
 * flagged by ShockFlattening::FindShock use the minmod slope */
void   ofx_set_shock(ofx* o, int enabled, double smoothing);

/* [Boundary] X?-beg / X?-end of direction dir: 0 periodic, 1 reflective,
 * 2 outflow (periodic on both sides or on neither); returns a status */
int    ofx_set_bc(ofx* o, int dir, int left, int right);

/* building blocks (one call = one reference method) */
void   ofx_set_boundaries(ofx* o);                 /* Boundary::SetBoundaries       */
void   ofx_prim_to_cons(ofx* o);                   /* Fluid::ConvertPrimToCons      */
void   ofx_cons_to_prim(ofx* o);                   /* Fluid::ConvertConsToPrim      */
void   ofx_reset_stage(ofx* o);                    /* Fluid::ResetStage             */
void   ofx_evolve_stage(ofx* o, double t, double dt); /* Fluid::EvolveStage         */
double ofx_compute_timestep(ofx* o);               /* DataBlock::ComputeTimestep    */
double ofx_check_divb(ofx* o);                     /* Fluid::CheckDivB              */
long   ofx_check_nan(ofx* o);                      /* Fluid::CheckNan               */

/* one TimeIntegrator::Cycle; returns a status code */
int    ofx_cycle(ofx* o);
/* main-loop driver: cycle until t >= tstop or ncycles reached (either <0 = off) */
int    ofx_run(ofx* o, double tstop, long max_cycles);

#ifdef __cplusplus
}
#endif
#endif
