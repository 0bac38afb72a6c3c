"""ctypes binding of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the oracle; the product library never imports this module.
The same API is served by three shared objects built by oracle/Makefile:

* ``oracle/libofx.so``          - the plain-C restatement (ofx.c)
* ``oracle/_ref/libofx_ref.so`` - the reference's own hot-path headers
  compiled against a small harness (ref_harness.cpp); only buildable where
  the reference sources are present.
* ``oracle/libofx_count.so``    - ofx.c with a scalar type that counts its
  floating-point operations (opcount.cpp; kind="count"); same results.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PORT = os.path.join(HERE, "libofx.so")
LIB_REF = os.path.join(HERE, "_ref", "libofx_ref.so")
LIB_COUNT = os.path.join(HERE, "libofx_count.so")

ORDER = {"order1": 1, "plm": 2, "limo3": 3, "ppm": 4}
SOLVER = {"hlld": 0, "hll": 1, "roe": 2, "tvdlf": 3}
EMF = {"uct_contact": 0, "arithmetic": 1, "uct0": 2, "uct_hll": 3, "uct_hlld": 4}

_libs = {}


def load(kind="port"):
    path = {"port": LIB_PORT, "count": LIB_COUNT}.get(kind, LIB_REF)
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library not built: {path}")
    lib = ctypes.CDLL(path)
    P, D, I, L = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_long
    dp = ctypes.POINTER(ctypes.c_double)
    lib.ofx_create.restype = P
    lib.ofx_create.argtypes = [I, I, I, I, D, D, D, D, D, D, I, I, I, I, D, D, D, D]
    lib.ofx_destroy.argtypes = [P]
    for f in ("ofx_nvar", "ofx_nghost"):
        getattr(lib, f).restype = I
        getattr(lib, f).argtypes = [P]
    for f in ("ofx_ncell", "ofx_nface"):
        getattr(lib, f).restype = L
        getattr(lib, f).argtypes = [P]
    lib.ofx_set_threads.argtypes = [P, I]
    lib.ofx_set_prim.argtypes = [P, dp, dp]
    lib.ofx_get_prim.argtypes = [P, dp, dp]
    lib.ofx_get_cons.argtypes = [P, dp]
    lib.ofx_set_time.argtypes = [P, D, D, L]
    lib.ofx_get_time.argtypes = [P, dp, dp, ctypes.POINTER(L)]
    lib.ofx_set_checks.argtypes = [P, I, I, D]
    lib.ofx_set_shock.argtypes = [P, I, D]
    lib.ofx_set_bc.restype = I
    lib.ofx_set_bc.argtypes = [P, I, I, I]
    for f in ("ofx_set_boundaries", "ofx_prim_to_cons", "ofx_cons_to_prim", "ofx_reset_stage"):
        getattr(lib, f).argtypes = [P]
    lib.ofx_evolve_stage.argtypes = [P, D, D]
    lib.ofx_compute_timestep.restype = D
    lib.ofx_compute_timestep.argtypes = [P]
    lib.ofx_check_divb.restype = D
    lib.ofx_check_divb.argtypes = [P]
    lib.ofx_check_nan.restype = L
    lib.ofx_check_nan.argtypes = [P]
    lib.ofx_cycle.restype = I
    lib.ofx_cycle.argtypes = [P]
    lib.ofx_run.restype = I
    lib.ofx_run.argtypes = [P, D, L]
    if kind == "count":
        lib.ofx_opcount_read.restype = I
        lib.ofx_opcount_read.argtypes = [ctypes.POINTER(ctypes.c_longlong), I]
        lib.ofx_opcount_read_phase.restype = I
        lib.ofx_opcount_read_phase.argtypes = [I, ctypes.POINTER(ctypes.c_longlong), I]
    _libs[path] = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


BOUNDARY = {"periodic": 0, "reflective": 1, "outflow": 2}


class Oracle:
    """One Cartesian block driven by the CPU oracle.  ``bc`` gives, per
    direction, the (X?-beg, X?-end) boundary types of the reference's
    [Boundary] block ("periodic", "reflective", "outflow"); default periodic."""

    def __init__(self, dims, n, xbeg=(0.0, 0.0, 0.0), xend=(1.0, 1.0, 1.0), order="plm",
                 solver="hlld", emf="uct_contact", nstages=2, gamma=5.0 / 3.0, cfl=0.6,
                 cfl_max_var=1.1, first_dt=1e-4, kind="port", threads=1, log_period=0,
                 check_nan_period=0, maxdivb=1e-6, shock_flattening=None, bc=None):
        self.lib = load(kind)
        n = list(n) + [1] * (3 - len(n))
        xbeg = tuple(xbeg) + (0.0, 0.0, 0.0)[len(xbeg):]
        xend = tuple(xend) + (1.0, 1.0, 1.0)[len(xend):]
        self.dims, self.n = dims, n
        h = self.lib.ofx_create(dims, n[0], n[1], n[2], xbeg[0], xend[0], xbeg[1], xend[1],
                                xbeg[2], xend[2], ORDER[order], SOLVER[solver], EMF[emf],
                                nstages, gamma, cfl, cfl_max_var, first_dt)
        if not h:
            raise ValueError("invalid oracle configuration")
        self.h = ctypes.c_void_p(h)
        self.nvar = self.lib.ofx_nvar(self.h)
        self.ng = self.lib.ofx_nghost(self.h)
        g = self.ng
        self.nt = [n[d] + 2 * g if d < dims else 1 for d in range(3)]
        self.ntv = [self.nt[d] + (1 if d < dims else 0) for d in range(3)]
        self.lib.ofx_set_threads(self.h, threads)
        self.lib.ofx_set_checks(self.h, log_period, check_nan_period, maxdivb)
        if shock_flattening is not None:  # [Hydro] shockFlattening <smoothing>
            self.lib.ofx_set_shock(self.h, 1, float(shock_flattening))
        for d, sides in enumerate(bc or ()):
            if self.lib.ofx_set_bc(self.h, d, BOUNDARY[sides[0]], BOUNDARY[sides[1]]) != 0:
                raise ValueError(f"invalid boundary pair {sides} in direction {d}")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ofx_destroy(self.h)
            self.h = None

    def set_prim(self, Vc, Vs):
        Vc = np.ascontiguousarray(Vc, dtype=np.float64)
        Vs = np.ascontiguousarray(Vs, dtype=np.float64)
        assert Vc.shape == (self.nvar, self.nt[2], self.nt[1], self.nt[0])
        assert Vs.shape == (self.dims, self.ntv[2], self.ntv[1], self.ntv[0])
        self.lib.ofx_set_prim(self.h, _ptr(Vc), _ptr(Vs))

    def get_prim(self):
        Vc = np.empty((self.nvar, self.nt[2], self.nt[1], self.nt[0]))
        Vs = np.empty((self.dims, self.ntv[2], self.ntv[1], self.ntv[0]))
        self.lib.ofx_get_prim(self.h, _ptr(Vc), _ptr(Vs))
        return Vc, Vs

    def get_cons(self):
        Uc = np.empty((self.nvar, self.nt[2], self.nt[1], self.nt[0]))
        self.lib.ofx_get_cons(self.h, _ptr(Uc))
        return Uc

    def set_time(self, t, dt, ncycles=0):
        self.lib.ofx_set_time(self.h, t, dt, ncycles)

    def get_time(self):
        t, dt, nc = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        self.lib.ofx_get_time(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(nc))
        return t.value, dt.value, nc.value

    def set_checks(self, log_period=0, check_nan_period=0, maxdivb=1e-6):
        self.lib.ofx_set_checks(self.h, log_period, check_nan_period, maxdivb)

    def cycle(self):
        return self.lib.ofx_cycle(self.h)

    def run(self, tstop=-1.0, max_cycles=-1):
        return self.lib.ofx_run(self.h, tstop, max_cycles)

    def check_divb(self):
        return self.lib.ofx_check_divb(self.h)
