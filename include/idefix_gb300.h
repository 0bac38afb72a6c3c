/*
 * idefix_gb300 — C ABI of the GB300 (sm_103a) ideal-MHD Godunov stage.
 *
 * Drop-in for the hot path of Idefix v2.2.02: one Cartesian block with
 * periodic, reflective or outflow boundaries (COMPONENTS == DIMENSIONS in
 * {2, 3}), advanced by the reference's
 * TimeIntegrator::Cycle semantics with PLM / LimO3 / PPM reconstruction,
 * HLLD / HLL / Roe / TVDLF fluxes and constrained transport.  In FP64 mode
 * the results are bit-identical to the reference built without FMA
 * contraction (its GPU CI setting).
 *
 * Conventions
 *  - Host arrays use the reference layout (LayoutRight, ghosts included):
 *      Vc[nvar][nt2][nt1][nt0]        nt = n + 2*nghost (1 in unused dims)
 *      Vs[dims][nt2+ko][nt1+jo][nt0+io]  (+1 in every active dimension)
 *    variable order RHO, VX1..VXd, PRS, BX1..BXd   (src/idefix.hpp:74-108)
 *  - Every function returns an idfx_status; idfx_gpu_last_error() returns
 *    the message of the last failure.  Nothing traps on the device.
 *  - A handle is used by one host thread at a time; work is ordered on the
 *    handle's CUDA stream.  No device pointer crosses the ABI except in the
 *    *_device entry points, which take pointers into this process's GPU
 *    memory.
 */
#ifndef IDEFIX_GB300_H_
#define IDEFIX_GB300_H_
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  IDFX_OK = 0,
  IDFX_ERR_CONFIG = 1,      /* IDEFIX_ERROR on an invalid setup            */
  IDFX_ERR_NAN = 2,         /* "Nan found after integration cycle"         */
  IDFX_ERR_DIVB = 3,        /* "divB too large, check your calculation"    */
  IDFX_ERR_DT_SMALL = 4,    /* "dt = ... is too small."                    */
  IDFX_ERR_FIRST_DT = 5,    /* "Your guessed first_dt is too large."       */
  IDFX_ERR_CUDA = 6,        /* CUDA runtime failure                         */
  IDFX_ERR_STATE = 7        /* call out of order / null handle             */
} idfx_status;

/* reconstruction order: Idefix_RECONSTRUCTION (CMakeLists.txt:198-209);
 * IDFX_LEARNED (no counterpart in the reference) is PLM corrected by the
 * learned interface-state network, 3-D HLLD FP64 only (idfx_gpu_set_learned) */
enum { IDFX_ORDER1 = 1, IDFX_PLM = 2, IDFX_LIMO3 = 3, IDFX_PPM = 4, IDFX_LEARNED = 5 };
/* [Hydro] solver (riemannSolver.hpp:27) */
enum { IDFX_HLLD = 0, IDFX_HLL = 1, IDFX_ROE = 2, IDFX_TVDLF = 3 };
/* [Hydro] emf (constrainedTransport.hpp:155-179) */
enum {
  IDFX_EMF_UCT_CONTACT = 0,
  IDFX_EMF_ARITHMETIC = 1,
  IDFX_EMF_UCT0 = 2,
  IDFX_EMF_UCT_HLL = 3,
  IDFX_EMF_UCT_HLLD = 4
};
/* arithmetic of the reconstruction and Riemann solve: IDFX_FP64 is the
 * bit-exact path; IDFX_MIXED runs reconstruction and Riemann solver in FP32
 * while the conserved-state accumulation across stages, ConsToPrim and the
 * CT face-field update stay FP64 */
enum { IDFX_FP64 = 0, IDFX_MIXED = 1 };

typedef struct {
  int dims;                 /* 2 or 3 (DIMENSIONS, with COMPONENTS == DIMENSIONS) */
  int n[3];                 /* active cells per direction, n[2] = 1 in 2-D        */
  double xbeg[3], xend[3];  /* [Grid] X?-grid uniform patch bounds                */
  int order;                /* IDFX_ORDER1 .. IDFX_PPM                            */
  int solver;               /* IDFX_HLLD ..                                       */
  int emf;                  /* IDFX_EMF_* (default uct_contact)                   */
  int nstages;              /* [TimeIntegrator] nstages: 1, 2 or 3                */
  double gamma;             /* [Hydro] gamma (default 5/3)                        */
  double cfl;               /* [TimeIntegrator] CFL                               */
  double cfl_max_var;       /* [TimeIntegrator] CFL_max_var (default 1.1)         */
  double first_dt;          /* [TimeIntegrator] first_dt                          */
  double maxdivb;           /* [TimeIntegrator] maxdivB (default 1e-6)            */
  int log_period;           /* [Output] log: divB check period, 0 = off           */
  int check_nan_period;     /* [TimeIntegrator] check_nan, 0 = off                */
  int precision;            /* IDFX_FP64 or IDFX_MIXED                            */
  int shock_flattening;     /* [Hydro] shockFlattening present (0 = off)          */
  double shock_smoothing;   /* its value (shockFlattening.hpp:164)                */
  int lbound[3], rbound[3]; /* [Boundary] X?-beg / X?-end: IDFX_BC_* per direction
                               (DataBlock::lbound/rbound, boundary.hpp:287-386);
                               periodic on both sides or on neither               */
} idfx_gpu_config;

/* boundary types (BoundaryType, idefix.hpp:220), ghosts filled as
 * Boundary::EnforcePeriodic / EnforceReflective / EnforceOutflow
 * (boundary.hpp:575-809) with the normal field rebuilt from div B = 0
 * (ReconstructNormalField, boundary.hpp:408-532) */
enum { IDFX_BC_PERIODIC = 0, IDFX_BC_REFLECTIVE = 1, IDFX_BC_OUTFLOW = 2 };

typedef struct idfx_gpu idfx_gpu;

/* Fills a config with the reference's defaults for the given grid. */
void idfx_gpu_default_config(idfx_gpu_config* cfg, int dims, int nx, int ny, int nz);

/* Replaces: Fluid<Phys>::Fluid + RiemannSolver + ConstrainedTransport +
 * TimeIntegrator construction (fluid.hpp:263-755, timeIntegrator.cpp:22-86).
 * stream: a cudaStream_t, or NULL for a stream owned by the handle. */
int idfx_gpu_create(const idfx_gpu_config* cfg, void* stream, idfx_gpu** out);
int idfx_gpu_destroy(idfx_gpu* h);
int idfx_gpu_last_error(const idfx_gpu* h, char* buf, size_t len);

/* sizes of the host arrays (in doubles) */
int idfx_gpu_sizes(const idfx_gpu* h, int* nvar, int* nghost, long long* vc_len, long long* vs_len);

/* Replaces: DataBlockHost::SyncToDevice / SyncFromDevice of Vc, Vs, Uc
 * (dataBlockHost.hpp:94-95).  Host pointers, reference layout. */
int idfx_gpu_upload_prim(idfx_gpu* h, const double* Vc, const double* Vs);
int idfx_gpu_download_prim(idfx_gpu* h, double* Vc, double* Vs);
int idfx_gpu_download_cons(idfx_gpu* h, double* Uc);
/* same, with device pointers of this process */
int idfx_gpu_upload_prim_device(idfx_gpu* h, const double* Vc, const double* Vs);
int idfx_gpu_download_prim_device(idfx_gpu* h, double* Vc, double* Vs);

/* DataBlock::t, DataBlock::dt, TimeIntegrator::ncycles */
int idfx_gpu_set_time(idfx_gpu* h, double t, double dt, long long ncycles);
int idfx_gpu_get_time(idfx_gpu* h, double* t, double* dt, long long* ncycles);

/* Replaces: TimeIntegrator::Cycle (timeIntegrator.cpp:246-414). Synchronous. */
int idfx_gpu_cycle(idfx_gpu* h);
/* Replaces: the main loop of main.cpp:190-225: cycles while t < tstop
 * (tstop < 0: no time limit) and at most max_cycles cycles (< 0: no limit).
 * Cycles are queued without host synchronisation between them. */
int idfx_gpu_run(idfx_gpu* h, double tstop, long long max_cycles);

/* Building blocks (each synchronous), same meaning as the reference methods */
int idfx_gpu_set_boundaries(idfx_gpu* h);                   /* Boundary::SetBoundaries     */
int idfx_gpu_prim_to_cons(idfx_gpu* h);                     /* Fluid::ConvertPrimToCons    */
int idfx_gpu_cons_to_prim(idfx_gpu* h);                     /* Fluid::ConvertConsToPrim    */
int idfx_gpu_reset_stage(idfx_gpu* h);                     /* Fluid::ResetStage (InvDt=0) */
int idfx_gpu_evolve_stage(idfx_gpu* h, double t, double dt);/* Fluid::EvolveStage          */
int idfx_gpu_compute_timestep(idfx_gpu* h, double* dt);     /* DataBlock::ComputeTimestep  */
int idfx_gpu_check_divb(idfx_gpu* h, double* divb);         /* Fluid::CheckDivB            */
int idfx_gpu_check_nan(idfx_gpu* h, long long* count);      /* Fluid::CheckNan             */

/* Per-kernel timing (no counterpart in the reference, which times regions
 * through Kokkos-Tools, profiler.cpp:55-130): when enabled, every launch of
 * the kernel classes below is bracketed by CUDA events on the handle's
 * stream.  Enabling clears the record; read returns total ms and launch
 * counts per class. */
enum {
  IDFX_K_FILL_FACES = 0,
  IDFX_K_STAGE_BEGIN,
  IDFX_K_SWEEP_X,
  IDFX_K_SWEEP_Y,
  IDFX_K_SWEEP_Z,
  IDFX_K_CT_CORNER,
  IDFX_K_CT_FACES,
  IDFX_K_STAGE_END,
  IDFX_K_CONTROL,
  IDFX_K_CHECKS,
  IDFX_K_LEARNED,
  IDFX_K_NUM
};
int idfx_gpu_profile(idfx_gpu* h, int enable);
int idfx_gpu_profile_read(idfx_gpu* h, double* ms, long long* launches, int nclasses);
/* Autotuner (no counterpart in the reference): picks, per sweep direction,
 * the sweep kernel (below) and its segment length (cells per thread or per
 * tile along the sweep) of the fastest sweep, timed over reps launches; the
 * state is saved and restored, and the results do not depend on the choice.
 * get/set_segments read and set the segment lengths. */
int idfx_gpu_autotune(idfx_gpu* h, int reps);
int idfx_gpu_get_segments(const idfx_gpu* h, int* seg);
int idfx_gpu_set_segments(idfx_gpu* h, const int* seg);  /* 1..1024 cells per thread */
/* Sweep kernel per direction (no counterpart in the reference): the
 * per-thread march, or for the y and z sweeps of 3-D mixed-precision blocks
 * (PLM, LimO3, PPM; nt0 a multiple of 4) the tile sweep, whose operands
 * arrive in shared memory by tensor-map bulk copies.  Both give the same
 * bits; the autotuner picks the faster one with its segment length. */
enum { IDFX_SWEEP_MARCH = 0, IDFX_SWEEP_TILE = 1 };
int idfx_gpu_get_sweep_kernels(const idfx_gpu* h, int* kind);
int idfx_gpu_set_sweep_kernels(idfx_gpu* h, const int* kind);
/* measured FP64 FMA throughput of the current device (thread operations
 * per second / 1e9), the roof of the FP64-bound sweeps; stream may be NULL */
int idfx_measure_fp64_peak(double* gops, void* stream);
/* self-check of the library's two FP64 division forms - on the integer pipe
 * (whole-array cons <-> prim passes) and from a correctly rounded reciprocal
 * with Markstein's correction (flux sweeps): n random operand pairs compared
 * bit for bit with the hardware division */
int idfx_check_division(long long n, unsigned long long seed, long long* mismatches);
/* self-check of the FP32 <-> FP64 conversions computed on the integer pipe
 * (mixed-precision path): n random values each way, bit for bit against the
 * hardware conversions */
int idfx_check_conversions(long long n, unsigned long long seed, long long* mismatches);
/* self-check of the bounded device wait (no counterpart in the reference):
 * the mbarrier wait of the bulk-copy staged sweep, at most `limit` try_wait
 * attempts, on a barrier that never completes (mode 0, as when a copy never
 * lands) or completes at once (mode 1); reports whether the wait gave up and
 * the control block's status / done words that its give-up path leaves
 * (IDFX_ERR_CUDA and 1 after a timeout).  The context stays usable. */
int idfx_check_wait_timeout(int mode, long long limit, int* gave_up, int* status, int* done);
/* self-check of the 5th-generation tensor-core path of the learned
 * correction (no counterpart in the reference): D[128][N] = A[128][K] .
 * B[N][K]^T with A and B rounded to BF16, FP32 accumulation in tensor memory
 * (tcgen05.mma / tcgen05.ld); host arrays, row-major; N, K multiples of 16 in
 * 16..256 */
int idfx_check_umma(int N, int K, const float* A, const float* B, float* D);

/* Allocation-free Fluid::EvolveStage — no counterpart in the reference.
 * For callers that may not allocate GPU memory while they step (state held
 * in their own pools or arenas, regions where cudaMalloc is forbidden):
 * Vc (in), Uc and Vs (in/out) are device arrays of this process in the
 * reference layout, as after Boundary::SetBoundaries and ConvertPrimToCons;
 * the stage's other work arrays live in a static device array of
 * IDFX_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB, held by every GPU that
 * loads the library until exit).  Blocks that do not fit are refused with
 * IDFX_ERR_CONFIG and a message in err.  Asynchronous on `stream` (NULL =
 * legacy default stream).  All calls share the scratch: calls whose GPU
 * work overlaps race.  The first call on a device looks up the scratch
 * address; make it before any stream capture.  Results equal
 * idfx_gpu_reset_stage + idfx_gpu_evolve_stage on the same arrays. */
#define IDFX_NOALLOC_SCRATCH_DOUBLES (4u * 1024u * 1024u)
int idfx_evolve_stage_noalloc(const idfx_gpu_config* cfg, const double* Vc, double* Uc, double* Vs,
                              double t, double dt, void* stream, char* err, size_t errlen);

/* Restart dumps in the reference's format: Dump::Write / Dump::Read
 * (output/dump.cpp:30-985).  Host arrays of one block in the layout above;
 * the dump holds the active cells of RHO, VX1..VXd, PRS, the active faces of
 * the face field, time, dt and vtkFileNumber (read skips fields of other
 * modules, as the reference does).  Reading needs the same grid; ghost
 * values are left as they are (the next boundary pass fills them). */
int idfx_dump_write(const char* path, const idfx_gpu_config* cfg, const double* Vc, const double* Vs, double t,
                    double dt, int vtk_file_number);
int idfx_dump_read(const char* path, const idfx_gpu_config* cfg, double* Vc, double* Vs, double* t, double* dt);

/* Learned interface-state correction — no counterpart in the reference.
 * A network (216 -> 128 -> 128 -> 16, SiLU, BF16 tensor-core arithmetic
 * with FP32 accumulation) reads the 3x3x3 primitive stencil of a cell in
 * the frame rotated to the sweep direction, scaled by the centre cell, and
 * corrects the cell's two PLM face states; cells whose stencil leaves the
 * trained feature range, or whose corrected density or pressure is not
 * positive, keep the plain PLM states.  Parameters: packed FP32 host array
 * W1[216][128] b1[128] W2[128][128] b2[128] W3[128][16] b3[16]. */
#define IDFX_MLP_NPARAM 46352
#define IDFX_MLP_NIN 216
/* loads the network into a handle created with order IDFX_LEARNED; fmin /
 * fmax: trained feature range (IDFX_MLP_NIN each), or NULL for no range
 * check.  Resets the counters of idfx_gpu_learned_stats. */
int idfx_gpu_set_learned(idfx_gpu* h, const float* params, const float* fmin, const float* fmax);
/* Boundary::SetBoundaries, then the learned face states of the current Vc:
 * ls[3][16][ncell] doubles (direction, minus-face vars 0-7 / plus-face vars
 * 8-15 in the solver's variable order, cell of the ghosted layout); cells
 * without a full 3x3x3 stencil hold zeros */
int idfx_gpu_learned_states(idfx_gpu* h, double* ls);
/* cells evaluated (per direction and stage) and cells that fell back to PLM */
int idfx_gpu_learned_stats(idfx_gpu* h, long long* cells, long long* fallbacks);

/* Trainer of the network (Adam, masked squared error of the normalised
 * corrections).  The *_device entry points take pointers to this process's
 * GPU memory; the training snapshots stay owned by the caller. */
typedef struct idfx_mlp idfx_mlp;
int idfx_mlp_create(int max_batch, void* stream, idfx_mlp** out);
int idfx_mlp_destroy(idfx_mlp* h);
int idfx_mlp_set_params(idfx_mlp* h, const float* params); /* host; resets Adam */
int idfx_mlp_get_params(idfx_mlp* h, float* params);
/* snapshots: coarse primitives float[nsnap][8][nc^3] and raw face targets
 * float[nsnap][3][16][nc^3] (idfx_learn_coarsen_device, converted) */
int idfx_mlp_set_dataset_device(idfx_mlp* h, const float* prims, const float* targets, int nsnap, int nc,
                                double gamma);
/* steps of Adam on random batches (cosine learning rate lr -> lr_end);
 * losses: host float[steps] or NULL */
int idfx_mlp_train(idfx_mlp* h, int steps, int batch, float lr, float lr_end, unsigned long long seed,
                   float* losses);
/* loss of one random batch with the network and with no correction */
int idfx_mlp_eval(idfx_mlp* h, int batch, unsigned long long seed, double* loss, double* loss_zero);
/* range of every feature over the training batches so far (host arrays) */
int idfx_mlp_feature_range(idfx_mlp* h, float* fmin, float* fmax);
/* one batch: features X (bfloat16 [batch][224]) and targets T (float [batch][16]) */
int idfx_mlp_batch_device(idfx_mlp* h, int batch, unsigned long long seed, long long base, void* X, float* T);
/* loss and gradient (host float[IDFX_MLP_NPARAM]) of a given batch */
int idfx_mlp_grad_device(idfx_mlp* h, const void* X, const float* T, int batch, float* grad, double* loss);
/* network output Y (device float [batch][16]) of a given batch */
int idfx_mlp_forward_device(idfx_mlp* h, const void* X, int batch, float* Y);
/* coarsening of a 3-D periodic snapshot by r: Vc / Vs in the reference
 * layout (device); outputs compact double prim[8][nc^3], faces[3][nc^3]
 * (left faces) and targets[3][16][nc^3] (face-layer means, rotated order) */
int idfx_learn_coarsen_device(const double* Vc, const double* Vs, int nf, int nghost, int r, double gamma,
                              double* prim, double* faces, double* targets, void* stream);

/* Ensemble of independent periodic blocks of uneven sizes advanced together
 * — no counterpart in the reference, which runs one block per process
 * (main.cpp:190-225 loops TimeIntegrator::Cycle on one DataBlock).  Every
 * box has its own grid, gamma, CFL and first_dt and its own time step (per-box
 * CFL dt); the scheme (dims, order, solver, emf, nstages, precision, log and
 * NaN-check periods) is shared.  Each phase of a stage is one launch over the
 * blocks of every box and one cycle is replayed as a CUDA graph; each box
 * evolves exactly as an idfx_gpu handle with the same config would. */
typedef struct idfx_ens idfx_ens;
int idfx_ens_create(int nbox, const idfx_gpu_config* cfgs, void* stream, idfx_ens** out);
int idfx_ens_destroy(idfx_ens* h);
int idfx_ens_last_error(const idfx_ens* h, char* buf, size_t len);
int idfx_ens_sizes(const idfx_ens* h, int box, int* nvar, int* nghost, long long* vc_len, long long* vs_len);
/* host arrays of one box, same layout as idfx_gpu_upload_prim */
int idfx_ens_upload_prim(idfx_ens* h, int box, const double* Vc, const double* Vs);
int idfx_ens_download_prim(idfx_ens* h, int box, double* Vc, double* Vs);
/* same, into device arrays of this process */
int idfx_ens_download_prim_device(idfx_ens* h, int box, double* Vc, double* Vs);
/* t, dt, cycle count and status (idfx_status) of one box */
int idfx_ens_get_time(idfx_ens* h, int box, double* t, double* dt, long long* ncycles, int* status);
/* every box cycles until its t reaches tstop (< 0: no limit), at most
 * max_cycles cycles (< 0: no limit); a box that stops or fails leaves the
 * others running.  mode: IDFX_ENS_GRAPH (1) replays one CUDA graph of
 * batched launches (one per phase) per cycle; IDFX_ENS_LAUNCHES (0) queues
 * the same launches one by one; IDFX_ENS_PERSISTENT (2) runs each chunk of
 * 64 cycles as ONE persistent cooperative launch (replayed from a CUDA
 * graph where the capture of a cooperative launch is available), its phases
 * separated by a grid-wide barrier whose every wait is bounded (a wait that
 * gives up stops every box with IDFX_ERR_CUDA).  All modes give identical
 * results. */
enum { IDFX_ENS_LAUNCHES = 0, IDFX_ENS_GRAPH = 1, IDFX_ENS_PERSISTENT = 2 };
int idfx_ens_run(idfx_ens* h, double tstop, long long max_cycles, int mode);
/* co-resident blocks of the persistent launch, and whether it replays from
 * a CUDA graph (after a persistent run) */
int idfx_ens_persistent_info(idfx_ens* h, int* blocks, int* graph);
/* Autotuner: per box size and direction, the march segment length of the
 * fastest batched sweep (timed over reps launches); the state is restored. */
int idfx_ens_autotune(idfx_ens* h, int reps);
int idfx_ens_get_segments(const idfx_ens* h, int box, int* seg);
/* block order of the batched launches: 0 largest box first, 1 box order */
int idfx_ens_set_schedule(idfx_ens* h, int schedule);

#ifdef __cplusplus
}
#endif
#endif /* IDEFIX_GB300_H_ */
