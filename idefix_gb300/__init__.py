"""idefix_gb300: the ideal-MHD Godunov stage of Idefix on one GB300 GPU.

Host-side mirror of the reference interface for this path, over the C ABI
of ``libidefix_gb300.so`` (declared in include/idefix_gb300.h):

* :class:`GpuBlock` — one Cartesian block on the GPU (periodic, reflective
  or outflow boundaries): state
  upload/download in the reference layout, ``cycle`` / ``run`` with the
  semantics of ``TimeIntegrator::Cycle`` and the main loop, and the
  building blocks (``set_boundaries``, ``prim_to_cons``, ``evolve_stage``,
  ``compute_timestep``, ``cons_to_prim``, ``check_divb``, ``check_nan``).
* :class:`Fluid`, :class:`TimeIntegrator` — thin facades carrying the
  reference's class and method names (src/fluid/fluid.hpp:53-247,
  src/timeIntegrator.hpp:25).

Errors follow the reference: numerical failures (NaN, divB, dt too small)
raise ``RuntimeError`` like the ``std::runtime_error`` that main.cpp
catches; invalid setups and a too large first_dt raise :class:`IdefixError`
(the reference's ``IDEFIX_ERROR``).  The library must be built
(``__graft_entry__.build()``); there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

__all__ = ["GpuBlock", "Fluid", "TimeIntegrator", "IdefixError", "load_library", "LIB_PATH"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libidefix_gb300.so")

ORDER = {"order1": 1, "plm": 2, "limo3": 3, "ppm": 4, "learned": 5}
SOLVER = {"hlld": 0, "hll": 1, "roe": 2, "tvdlf": 3}
EMF = {"uct_contact": 0, "arithmetic": 1, "uct0": 2, "uct_hll": 3, "uct_hlld": 4}
PRECISION = {"fp64": 0, "mixed": 1}

OK, ERR_CONFIG, ERR_NAN, ERR_DIVB, ERR_DT_SMALL, ERR_FIRST_DT, ERR_CUDA, ERR_STATE = range(8)


class IdefixError(Exception):
    """Fatal error of the reference (IDEFIX_ERROR): invalid setup, first_dt."""


class Config(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("xbeg", ctypes.c_double * 3),
        ("xend", ctypes.c_double * 3),
        ("order", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("emf", ctypes.c_int),
        ("nstages", ctypes.c_int),
        ("gamma", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("cfl_max_var", ctypes.c_double),
        ("first_dt", ctypes.c_double),
        ("maxdivb", ctypes.c_double),
        ("log_period", ctypes.c_int),
        ("check_nan_period", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("shock_flattening", ctypes.c_int),
        ("shock_smoothing", ctypes.c_double),
        ("lbound", ctypes.c_int * 3),
        ("rbound", ctypes.c_int * 3),
    ]


# [Boundary] types (BoundaryType, idefix.hpp:220)
BOUNDARY = {"periodic": 0, "reflective": 1, "outflow": 2}


EXPORTS = [
    "idfx_gpu_default_config", "idfx_gpu_create", "idfx_gpu_destroy", "idfx_gpu_last_error",
    "idfx_gpu_sizes", "idfx_gpu_upload_prim", "idfx_gpu_download_prim", "idfx_gpu_download_cons",
    "idfx_gpu_upload_prim_device", "idfx_gpu_download_prim_device", "idfx_gpu_set_time",
    "idfx_gpu_get_time", "idfx_gpu_cycle", "idfx_gpu_run", "idfx_gpu_set_boundaries",
    "idfx_gpu_prim_to_cons", "idfx_gpu_cons_to_prim", "idfx_gpu_reset_stage",
    "idfx_gpu_evolve_stage", "idfx_gpu_compute_timestep", "idfx_gpu_check_divb",
    "idfx_gpu_check_nan", "idfx_gpu_profile", "idfx_gpu_profile_read",
    "idfx_evolve_stage_noalloc",
    "idfx_ens_create", "idfx_ens_destroy", "idfx_ens_last_error", "idfx_ens_sizes",
    "idfx_ens_upload_prim", "idfx_ens_download_prim", "idfx_ens_get_time", "idfx_ens_run",
    "idfx_ens_autotune", "idfx_ens_get_segments", "idfx_ens_set_schedule",
    "idfx_ens_download_prim_device", "idfx_ens_persistent_info",
    "idfx_gpu_set_learned", "idfx_gpu_learned_states", "idfx_gpu_learned_stats", "idfx_mlp_create", "idfx_mlp_destroy",
    "idfx_mlp_set_params", "idfx_mlp_get_params", "idfx_mlp_set_dataset_device", "idfx_mlp_train",
    "idfx_mlp_eval", "idfx_mlp_feature_range", "idfx_mlp_batch_device", "idfx_mlp_grad_device",
    "idfx_mlp_forward_device", "idfx_learn_coarsen_device", "idfx_measure_fp64_peak",
    "idfx_gpu_autotune", "idfx_gpu_get_segments", "idfx_gpu_set_segments", "idfx_gpu_get_sweep_kernels",
    "idfx_gpu_set_sweep_kernels", "idfx_check_division",
    "idfx_check_conversions", "idfx_check_wait_timeout", "idfx_check_umma",
    "idfx_dump_write", "idfx_dump_read",
]

KERNEL_CLASSES = ["fill_faces", "stage_begin", "sweep_x", "sweep_y", "sweep_z", "ct_corner",
                  "ct_faces", "stage_end", "control", "checks", "learned_recon"]

_lib = None


def load_library(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    P, D, I, LL = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_longlong
    dp = ctypes.POINTER(ctypes.c_double)
    lib.idfx_gpu_default_config.restype = None
    lib.idfx_gpu_default_config.argtypes = [ctypes.POINTER(Config), I, I, I, I]
    lib.idfx_gpu_create.argtypes = [ctypes.POINTER(Config), P, ctypes.POINTER(P)]
    lib.idfx_gpu_destroy.argtypes = [P]
    lib.idfx_gpu_last_error.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    lib.idfx_gpu_sizes.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(LL),
                                   ctypes.POINTER(LL)]
    for f in ("idfx_gpu_upload_prim", "idfx_gpu_download_prim", "idfx_gpu_upload_prim_device",
              "idfx_gpu_download_prim_device"):
        getattr(lib, f).argtypes = [P, P, P]
    lib.idfx_gpu_download_cons.argtypes = [P, P]
    lib.idfx_gpu_set_time.argtypes = [P, D, D, LL]
    lib.idfx_gpu_get_time.argtypes = [P, dp, dp, ctypes.POINTER(LL)]
    lib.idfx_gpu_cycle.argtypes = [P]
    lib.idfx_gpu_run.argtypes = [P, D, LL]
    for f in ("idfx_gpu_set_boundaries", "idfx_gpu_prim_to_cons", "idfx_gpu_cons_to_prim",
              "idfx_gpu_reset_stage"):
        getattr(lib, f).argtypes = [P]
    lib.idfx_gpu_evolve_stage.argtypes = [P, D, D]
    lib.idfx_gpu_compute_timestep.argtypes = [P, dp]
    lib.idfx_gpu_check_divb.argtypes = [P, dp]
    lib.idfx_gpu_check_nan.argtypes = [P, ctypes.POINTER(LL)]
    lib.idfx_gpu_profile.argtypes = [P, I]
    lib.idfx_gpu_profile_read.argtypes = [P, dp, ctypes.POINTER(LL), I]
    lib.idfx_evolve_stage_noalloc.argtypes = [ctypes.POINTER(Config), P, P, P, D, D, P,
                                              ctypes.c_char_p, ctypes.c_size_t]
    lib.idfx_ens_create.argtypes = [I, ctypes.POINTER(Config), P, ctypes.POINTER(P)]
    lib.idfx_ens_destroy.argtypes = [P]
    lib.idfx_ens_last_error.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    lib.idfx_ens_sizes.argtypes = [P, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(LL),
                                   ctypes.POINTER(LL)]
    lib.idfx_ens_upload_prim.argtypes = [P, I, P, P]
    lib.idfx_ens_download_prim.argtypes = [P, I, P, P]
    lib.idfx_ens_get_time.argtypes = [P, I, dp, dp, ctypes.POINTER(LL), ctypes.POINTER(I)]
    lib.idfx_ens_run.argtypes = [P, D, LL, I]
    lib.idfx_ens_persistent_info.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I)]
    lib.idfx_ens_autotune.argtypes = [P, I]
    lib.idfx_ens_get_segments.argtypes = [P, I, ctypes.POINTER(I)]
    lib.idfx_ens_set_schedule.argtypes = [P, I]
    lib.idfx_ens_download_prim_device.argtypes = [P, I, P, P]
    fp = ctypes.POINTER(ctypes.c_float)
    U64 = ctypes.c_ulonglong
    lib.idfx_measure_fp64_peak.argtypes = [dp, P]
    lib.idfx_gpu_autotune.argtypes = [P, I]
    lib.idfx_dump_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(Config), P, P, D, D, I]
    lib.idfx_dump_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(Config), P, P, dp, dp]
    lib.idfx_check_division.argtypes = [LL, ctypes.c_ulonglong, ctypes.POINTER(LL)]
    lib.idfx_check_conversions.argtypes = [LL, ctypes.c_ulonglong, ctypes.POINTER(LL)]
    ip = ctypes.POINTER(ctypes.c_int)
    lib.idfx_check_wait_timeout.argtypes = [ctypes.c_int, LL, ip, ip, ip]
    fp = ctypes.POINTER(ctypes.c_float)
    lib.idfx_check_umma.argtypes = [ctypes.c_int, ctypes.c_int, fp, fp, fp]
    lib.idfx_gpu_get_segments.argtypes = [P, ctypes.POINTER(I)]
    lib.idfx_gpu_set_segments.argtypes = [P, ctypes.POINTER(I)]
    lib.idfx_gpu_get_sweep_kernels.argtypes = [P, ctypes.POINTER(I)]
    lib.idfx_gpu_set_sweep_kernels.argtypes = [P, ctypes.POINTER(I)]
    lib.idfx_gpu_set_learned.argtypes = [P, fp, fp, fp]
    lib.idfx_gpu_learned_states.argtypes = [P, P]
    lib.idfx_gpu_learned_stats.argtypes = [P, ctypes.POINTER(LL), ctypes.POINTER(LL)]
    lib.idfx_mlp_create.argtypes = [I, P, ctypes.POINTER(P)]
    lib.idfx_mlp_destroy.argtypes = [P]
    lib.idfx_mlp_set_params.argtypes = [P, fp]
    lib.idfx_mlp_get_params.argtypes = [P, fp]
    lib.idfx_mlp_set_dataset_device.argtypes = [P, P, P, I, I, D]
    lib.idfx_mlp_train.argtypes = [P, I, I, ctypes.c_float, ctypes.c_float, U64, fp]
    lib.idfx_mlp_eval.argtypes = [P, I, U64, dp, dp]
    lib.idfx_mlp_feature_range.argtypes = [P, fp, fp]
    lib.idfx_mlp_batch_device.argtypes = [P, I, U64, LL, P, P]
    lib.idfx_mlp_grad_device.argtypes = [P, P, P, I, fp, dp]
    lib.idfx_mlp_forward_device.argtypes = [P, P, I, P]
    lib.idfx_learn_coarsen_device.argtypes = [P, P, I, I, I, D, P, P, P, P]
    for f in EXPORTS:
        if f != "idfx_gpu_default_config":
            getattr(lib, f).restype = I
    _lib = lib
    return lib


def measure_fp64_peak(stream=None):
    """measured FP64 FMA throughput of the current GPU, Gop/s"""
    lib = load_library()
    g = ctypes.c_double()
    rc = lib.idfx_measure_fp64_peak(ctypes.byref(g), ctypes.c_void_p(stream))
    if rc != OK:
        raise IdefixError(f"idfx_measure_fp64_peak failed with status {rc}")
    return g.value


def _shapes(cfg):
    dims = cfg.dims
    ng = 3 if cfg.order == ORDER["ppm"] else 2
    nt = [cfg.n[d] + 2 * ng if d < dims else 1 for d in range(3)]
    ntv = [nt[d] + (1 if d < dims else 0) for d in range(3)]
    return (2 * dims + 2, nt[2], nt[1], nt[0]), (dims, ntv[2], ntv[1], ntv[0])


def write_dump(path, cfg, Vc, Vs, t, dt, vtk_file_number=0):
    """idfx_dump_write: host arrays of one block -> reference-format dump."""
    lib = load_library()
    sc, ss = _shapes(cfg)
    Vc = np.ascontiguousarray(Vc, dtype=np.float64)
    Vs = np.ascontiguousarray(Vs, dtype=np.float64)
    if Vc.shape != sc or Vs.shape != ss:
        raise IdefixError(f"state shapes {Vc.shape}/{Vs.shape} != {sc}/{ss}")
    rc = lib.idfx_dump_write(os.fsencode(path), ctypes.byref(cfg), _as_ptr(Vc), _as_ptr(Vs), float(t), float(dt),
                             int(vtk_file_number))
    if rc != OK:
        raise IdefixError(f"idfx_dump_write failed with status {rc}")


def read_dump(path, cfg):
    """idfx_dump_read -> (Vc, Vs, t, dt), ghosts zero."""
    lib = load_library()
    sc, ss = _shapes(cfg)
    Vc = np.zeros(sc)
    Vs = np.zeros(ss)
    t, dt = ctypes.c_double(), ctypes.c_double()
    rc = lib.idfx_dump_read(os.fsencode(path), ctypes.byref(cfg), _as_ptr(Vc), _as_ptr(Vs), ctypes.byref(t),
                            ctypes.byref(dt))
    if rc != OK:
        raise IdefixError(f"idfx_dump_read failed with status {rc}")
    return Vc, Vs, t.value, dt.value


def make_config(dims, n, xbeg=(0.0, 0.0, 0.0), xend=(1.0, 1.0, 1.0), order="plm", solver="hlld",
                emf="uct_contact", nstages=2, gamma=5.0 / 3.0, cfl=0.9, cfl_max_var=1.1,
                first_dt=1.0e-10, maxdivb=1e-6, log_period=0, check_nan_period=0, precision="fp64",
                shock_flattening=None, bc=None):
    """idfx_gpu_config from the input-file style arguments of GpuBlock."""
    lib = load_library()
    n = list(n) + [1] * (3 - len(n))
    cfg = Config()
    lib.idfx_gpu_default_config(ctypes.byref(cfg), dims, n[0], n[1], n[2])
    for d in range(3):
        cfg.xbeg[d] = float(xbeg[d]) if d < len(xbeg) else 0.0
        cfg.xend[d] = float(xend[d]) if d < len(xend) else 1.0
    try:
        cfg.order, cfg.solver, cfg.emf = ORDER[order], SOLVER[solver], EMF[emf]
        cfg.precision = PRECISION[precision]
    except KeyError as exc:
        raise IdefixError(f"unknown scheme option {exc}") from None
    cfg.nstages = nstages
    cfg.gamma, cfg.cfl, cfg.cfl_max_var = gamma, cfl, cfl_max_var
    cfg.first_dt, cfg.maxdivb = first_dt, maxdivb
    cfg.log_period, cfg.check_nan_period = log_period, check_nan_period
    if shock_flattening is not None:  # [Hydro] shockFlattening <smoothing>
        cfg.shock_flattening, cfg.shock_smoothing = 1, float(shock_flattening)
    for d, sides in enumerate(bc or ()):  # [Boundary] X?-beg, X?-end
        try:
            cfg.lbound[d], cfg.rbound[d] = BOUNDARY[sides[0]], BOUNDARY[sides[1]]
        except KeyError as exc:
            raise IdefixError(f"unknown boundary type {exc}") from None
    return cfg


def _as_ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class GpuBlock:
    """One Cartesian block advanced on the GPU.

    Arguments mirror the reference's input file: [Grid] (dims, n, xbeg,
    xend), [Hydro] (solver, emf, gamma, shockFlattening), [Boundary] (bc:
    per direction the (beg, end) pair of "periodic", "reflective",
    "outflow"; default periodic), [TimeIntegrator] (nstages, CFL,
    CFL_max_var, first_dt, maxdivB, check_nan), [Output] log, and the
    build-time reconstruction order.  precision: "fp64" (bit-identical to
    the reference) or "mixed" (FP32 reconstruction and Riemann solve, FP64
    conserved state, ConsToPrim and CT face update).
    """

    def __init__(self, dims, n, xbeg=(0.0, 0.0, 0.0), xend=(1.0, 1.0, 1.0), order="plm",
                 solver="hlld", emf="uct_contact", nstages=2, gamma=5.0 / 3.0, cfl=0.9,
                 cfl_max_var=1.1, first_dt=1.0e-10, maxdivb=1e-6, log_period=0,
                 check_nan_period=0, precision="fp64", stream=None, shock_flattening=None, bc=None):
        self.lib = load_library()
        n = list(n) + [1] * (3 - len(n))
        cfg = make_config(dims, n, xbeg, xend, order, solver, emf, nstages, gamma, cfl, cfl_max_var,
                          first_dt, maxdivb, log_period, check_nan_period, precision, shock_flattening,
                          bc)
        h = ctypes.c_void_p()
        rc = self.lib.idfx_gpu_create(ctypes.byref(cfg), ctypes.c_void_p(stream), ctypes.byref(h))
        if rc != OK:
            raise IdefixError(f"idfx_gpu_create failed with status {rc}")
        self.h = h
        self.cfg = cfg
        self.dims, self.n = dims, n
        nvar, ng, vcl, vsl = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        self.lib.idfx_gpu_sizes(self.h, ctypes.byref(nvar), ctypes.byref(ng), ctypes.byref(vcl),
                                ctypes.byref(vsl))
        self.nvar, self.ng = nvar.value, ng.value
        g = self.ng
        self.nt = [n[d] + 2 * g if d < dims else 1 for d in range(3)]
        self.ntv = [self.nt[d] + (1 if d < dims else 0) for d in range(3)]
        self.vc_shape = (self.nvar, self.nt[2], self.nt[1], self.nt[0])
        self.vs_shape = (dims, self.ntv[2], self.ntv[1], self.ntv[0])

    def close(self):
        if getattr(self, "h", None):
            self.lib.idfx_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # -- errors ---------------------------------------------------------
    def _check(self, rc):
        if rc == OK:
            return
        buf = ctypes.create_string_buffer(512)
        self.lib.idfx_gpu_last_error(self.h, buf, 512)
        msg = buf.value.decode(errors="replace")
        if rc in (ERR_NAN, ERR_DIVB, ERR_DT_SMALL):
            raise RuntimeError(msg)
        raise IdefixError(f"status {rc}: {msg}")

    # -- state ------------------------------------------------------------
    def upload(self, Vc, Vs):
        Vc = np.ascontiguousarray(Vc, dtype=np.float64)
        Vs = np.ascontiguousarray(Vs, dtype=np.float64)
        if Vc.shape != self.vc_shape or Vs.shape != self.vs_shape:
            raise IdefixError(f"state shapes {Vc.shape}/{Vs.shape} != {self.vc_shape}/{self.vs_shape}")
        self._check(self.lib.idfx_gpu_upload_prim(self.h, _as_ptr(Vc), _as_ptr(Vs)))

    def download(self, out=None):
        Vc = np.empty(self.vc_shape) if out is None else out[0]
        Vs = np.empty(self.vs_shape) if out is None else out[1]
        self._check(self.lib.idfx_gpu_download_prim(self.h, _as_ptr(Vc), _as_ptr(Vs)))
        return Vc, Vs

    def download_cons(self):
        Uc = np.empty(self.vc_shape)
        self._check(self.lib.idfx_gpu_download_cons(self.h, _as_ptr(Uc)))
        return Uc

    def upload_device(self, vc_ptr, vs_ptr):
        """state from device pointers (e.g. torch tensors' data_ptr())"""
        self._check(self.lib.idfx_gpu_upload_prim_device(self.h, ctypes.c_void_p(vc_ptr),
                                                         ctypes.c_void_p(vs_ptr)))

    def download_device(self, vc_ptr, vs_ptr):
        self._check(self.lib.idfx_gpu_download_prim_device(self.h, ctypes.c_void_p(vc_ptr),
                                                           ctypes.c_void_p(vs_ptr)))

    def set_time(self, t, dt, ncycles=0):
        self._check(self.lib.idfx_gpu_set_time(self.h, t, dt, ncycles))

    def get_time(self):
        t, dt, nc = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        self._check(self.lib.idfx_gpu_get_time(self.h, ctypes.byref(t), ctypes.byref(dt),
                                               ctypes.byref(nc)))
        return t.value, dt.value, nc.value

    # -- time integration -------------------------------------------------
    def cycle(self):
        self._check(self.lib.idfx_gpu_cycle(self.h))

    def run(self, tstop=-1.0, max_cycles=-1):
        self._check(self.lib.idfx_gpu_run(self.h, tstop, max_cycles))

    # -- building blocks --------------------------------------------------
    def set_boundaries(self):
        self._check(self.lib.idfx_gpu_set_boundaries(self.h))

    def prim_to_cons(self):
        self._check(self.lib.idfx_gpu_prim_to_cons(self.h))

    def cons_to_prim(self):
        self._check(self.lib.idfx_gpu_cons_to_prim(self.h))

    def reset_stage(self):
        self._check(self.lib.idfx_gpu_reset_stage(self.h))

    def evolve_stage(self, t, dt):
        self._check(self.lib.idfx_gpu_evolve_stage(self.h, t, dt))

    def compute_timestep(self):
        v = ctypes.c_double()
        self._check(self.lib.idfx_gpu_compute_timestep(self.h, ctypes.byref(v)))
        return v.value

    def check_divb(self):
        v = ctypes.c_double()
        self._check(self.lib.idfx_gpu_check_divb(self.h, ctypes.byref(v)))
        return v.value

    def check_nan(self):
        v = ctypes.c_longlong()
        self._check(self.lib.idfx_gpu_check_nan(self.h, ctypes.byref(v)))
        return v.value


    # -- per-kernel timing --------------------------------------------------
    def write_dump(self, path, vtk_file_number=0):
        """Restart dump of the current state in the reference's format."""
        Vc, Vs = self.download()
        t, dt, _ = self.get_time()
        write_dump(path, self.cfg, Vc, Vs, t, dt, vtk_file_number)

    def read_dump(self, path, ncycles=0):
        """Load a restart dump (reference format) as the current state."""
        Vc, Vs, t, dt = read_dump(path, self.cfg)
        self.upload(Vc, Vs)
        self.set_time(t, dt, ncycles)

    def autotune(self, reps=3):
        """pick the sweep kernel (march or, for the FP32 y / z sweeps of a 3-D
        block, tile) and its segment length of every direction by timing"""
        self._check(self.lib.idfx_gpu_autotune(self.h, int(reps)))

    SWEEP_KERNELS = ("march", "tile")

    def sweep_kernels(self):
        """the sweep kernel of every direction, "march" or "tile" """
        k = (ctypes.c_int * 3)()
        self._check(self.lib.idfx_gpu_get_sweep_kernels(self.h, k))
        return [self.SWEEP_KERNELS[v] for v in k]

    def set_sweep_kernels(self, kinds):
        k = (ctypes.c_int * 3)(*[self.SWEEP_KERNELS.index(x) for x in (list(kinds) + ["march"] * (3 - len(kinds)))])
        self._check(self.lib.idfx_gpu_set_sweep_kernels(self.h, k))

    def segments(self):
        seg = (ctypes.c_int * 3)()
        self._check(self.lib.idfx_gpu_get_segments(self.h, seg))
        return list(seg)

    def set_segments(self, seg):
        s = (ctypes.c_int * 3)(*(list(seg) + [1] * (3 - len(seg))))
        self._check(self.lib.idfx_gpu_set_segments(self.h, s))

    def set_learned(self, params, fmin=None, fmax=None):
        """Load the learned-reconstruction network (order "learned")."""
        fp = ctypes.POINTER(ctypes.c_float)
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != 46352:
            raise IdefixError("the network has 46352 parameters")
        lo = hi = None
        if fmin is not None:
            lo = np.ascontiguousarray(fmin, dtype=np.float32)
            hi = np.ascontiguousarray(fmax, dtype=np.float32)
        self._check(self.lib.idfx_gpu_set_learned(
            self.h, p.ctypes.data_as(fp), None if lo is None else lo.ctypes.data_as(fp),
            None if hi is None else hi.ctypes.data_as(fp)))
        self._learned_keep = (p, lo, hi)

    def learned_states(self):
        """face states of the learned reconstruction on the current state:
        [3 directions, 16 (minus 0-7, plus 8-15), nz, ny, nx] (ghosted)"""
        ls = np.zeros((3, 16) + self.vc_shape[1:])
        self._check(self.lib.idfx_gpu_learned_states(self.h, _as_ptr(ls)))
        return ls

    def learned_stats(self):
        """(cells evaluated, cells that fell back to plain PLM)"""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(self.lib.idfx_gpu_learned_stats(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def profile(self, enable=True):
        self._check(self.lib.idfx_gpu_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        n = len(KERNEL_CLASSES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        self._check(self.lib.idfx_gpu_profile_read(self.h, ms, cnt, n))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}


class Fluid:
    """Reference-named facade (Fluid<DefaultPhysics>, src/fluid/fluid.hpp)."""

    def __init__(self, block):
        self.block = block

    def ConvertPrimToCons(self):
        self.block.prim_to_cons()

    def ConvertConsToPrim(self):
        self.block.cons_to_prim()

    def ResetStage(self):
        self.block.reset_stage()

    def EvolveStage(self, t, dt):
        self.block.evolve_stage(t, dt)

    def CheckDivB(self):
        return self.block.check_divb()

    def CheckNan(self):
        return self.block.check_nan()


class TimeIntegrator:
    """Reference-named facade (src/timeIntegrator.hpp)."""

    def __init__(self, block):
        self.block = block

    def Cycle(self):
        self.block.cycle()

    def GetNCycles(self):
        return self.block.get_time()[2]


class Ensemble:
    """Independent periodic blocks of uneven sizes advanced together.

    boxes: list of dicts of GpuBlock keyword arguments (dims, n, xbeg, xend,
    gamma, cfl, first_dt, ...); the scheme keywords (dims, order, solver, emf,
    nstages, precision, log_period, check_nan_period) must agree.  Each box
    evolves exactly as a GpuBlock with the same arguments, with its own
    CFL time step.
    """

    def __init__(self, boxes, stream=None):
        self.lib = load_library()
        nbox = len(boxes)
        if nbox < 1:
            raise IdefixError("an ensemble needs at least one box")
        cfgs = (Config * nbox)()
        for b, kw in enumerate(boxes):
            cfgs[b] = make_config(**kw)
        h = ctypes.c_void_p()
        rc = self.lib.idfx_ens_create(nbox, cfgs, ctypes.c_void_p(stream), ctypes.byref(h))
        if rc != OK:
            raise IdefixError(f"idfx_ens_create failed with status {rc}")
        self.h = h
        self.nbox = nbox
        self.shapes = []
        for b, kw in enumerate(boxes):
            dims = kw["dims"]
            n = list(kw["n"]) + [1] * (3 - len(kw["n"]))
            nvar, ng = ctypes.c_int(), ctypes.c_int()
            self.lib.idfx_ens_sizes(self.h, b, ctypes.byref(nvar), ctypes.byref(ng), None, None)
            nt = [n[d] + 2 * ng.value if d < dims else 1 for d in range(3)]
            ntv = [nt[d] + (1 if d < dims else 0) for d in range(3)]
            self.shapes.append(((nvar.value, nt[2], nt[1], nt[0]), (dims, ntv[2], ntv[1], ntv[0])))

    def close(self):
        if getattr(self, "h", None):
            self.lib.idfx_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc == OK:
            return
        buf = ctypes.create_string_buffer(512)
        self.lib.idfx_ens_last_error(self.h, buf, 512)
        msg = buf.value.decode(errors="replace")
        if rc in (ERR_NAN, ERR_DIVB, ERR_DT_SMALL):
            raise RuntimeError(msg)
        raise IdefixError(f"status {rc}: {msg}")

    def upload(self, box, Vc, Vs):
        Vc = np.ascontiguousarray(Vc, dtype=np.float64)
        Vs = np.ascontiguousarray(Vs, dtype=np.float64)
        if (Vc.shape, Vs.shape) != self.shapes[box]:
            raise IdefixError(f"box {box}: state shapes {Vc.shape}/{Vs.shape} != {self.shapes[box]}")
        self._check(self.lib.idfx_ens_upload_prim(self.h, box, _as_ptr(Vc), _as_ptr(Vs)))

    def download(self, box):
        Vc = np.empty(self.shapes[box][0])
        Vs = np.empty(self.shapes[box][1])
        self._check(self.lib.idfx_ens_download_prim(self.h, box, _as_ptr(Vc), _as_ptr(Vs)))
        return Vc, Vs

    def download_device(self, box, vc_ptr, vs_ptr):
        """copy one box's Vc / Vs into device arrays of this process"""
        self._check(self.lib.idfx_ens_download_prim_device(self.h, box, ctypes.c_void_p(vc_ptr),
                                                           ctypes.c_void_p(vs_ptr)))

    def get_time(self, box):
        """(t, dt, ncycles, status) of one box."""
        t, dt = ctypes.c_double(), ctypes.c_double()
        nc, st = ctypes.c_longlong(), ctypes.c_int()
        self._check(self.lib.idfx_ens_get_time(self.h, box, ctypes.byref(t), ctypes.byref(dt),
                                               ctypes.byref(nc), ctypes.byref(st)))
        return t.value, dt.value, nc.value, st.value

    def run(self, tstop=-1.0, max_cycles=-1, graph=True, persistent=False):
        """persistent: every chunk of cycles as one persistent launch (grid
        barrier between phases); else one CUDA graph of batched launches per
        cycle (graph=True) or the launches queued one by one"""
        mode = 2 if persistent else (1 if graph else 0)
        self._check(self.lib.idfx_ens_run(self.h, float(tstop), int(max_cycles), mode))

    def persistent_info(self):
        """(co-resident blocks of the persistent launch, replayed from a graph)"""
        b, g = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.idfx_ens_persistent_info(self.h, ctypes.byref(b), ctypes.byref(g)))
        return b.value, bool(g.value)

    def write_dump(self, path, vtk_file_number=0):
        """Restart dump of the current state in the reference's format."""
        Vc, Vs = self.download()
        t, dt, _ = self.get_time()
        write_dump(path, self.cfg, Vc, Vs, t, dt, vtk_file_number)

    def read_dump(self, path, ncycles=0):
        """Load a restart dump (reference format) as the current state."""
        Vc, Vs, t, dt = read_dump(path, self.cfg)
        self.upload(Vc, Vs)
        self.set_time(t, dt, ncycles)

    def autotune(self, reps=3):
        self._check(self.lib.idfx_ens_autotune(self.h, int(reps)))

    def segments(self, box):
        seg = (ctypes.c_int * 3)()
        self._check(self.lib.idfx_ens_get_segments(self.h, box, seg))
        return list(seg)

    def set_schedule(self, schedule):
        """Block order of the batched launches: "largest_first" or "box_order"."""
        code = {"largest_first": 0, "box_order": 1}[schedule]
        self._check(self.lib.idfx_ens_set_schedule(self.h, code))
