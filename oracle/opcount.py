"""Floating-point operations per zone-cycle of the reference algorithm -
TEST INFRASTRUCTURE ONLY.

Runs the counting build of the CPU oracle (``opcount.cpp``, built by
``make -C oracle count``; results bit-identical to ``libofx.so``) on the 3-D
decaying-turbulence workload (HLLD + PLM + uct_contact, RK2, periodic; or,
with ``--workload lowbeta``, the low-beta workload with LimO3; with
``--workload ot3d``, the 3-D Orszag-Tang problem) and prints
one JSON line of operation counts per active zone and cycle, by kind:
add/sub, mul, div, sqrt, min/max, abs, compare, negate.  ``cycle`` counts a
whole TimeIntegrator::Cycle (timeIntegrator.cpp:246-414: boundaries,
cons/prim conversions, the two stages, the RK combination, the dt
reduction), also split by phase (``cycle_by_phase``: each direction's
reconstruction + Riemann + flux difference, the corner EMFs, the face
update, ...); ``stage`` counts one Fluid::EvolveStage alone (evolveStage.hpp:
13-90: reconstruction, Riemann fluxes and flux-difference update in three
directions, the corner EMFs and the face update).  The counts depend on the
data (HLLD fallbacks, limiter branches), so they are taken on the workload
itself.

    python -m oracle.opcount --n 256 --cycles 1
    python -m oracle.opcount --n 256 --workload lowbeta
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KINDS = ("add", "mul", "div", "sqrt", "minmax", "abs", "cmp", "neg")
# the OFX_PH_* phases of ofx.c, in order
PHASES = ("other", "sweep_x", "sweep_y", "sweep_z", "ct_corner", "ct_faces", "boundaries",
          "prim_to_cons", "rk_combine", "cons_to_prim", "timestep", "checks")


def _read(lib):
    c = (ctypes.c_longlong * len(KINDS))()
    lib.ofx_opcount_read(c, len(KINDS))
    return np.array(list(c), dtype=np.float64)


def _read_phase(lib, phase):
    c = (ctypes.c_longlong * len(KINDS))()
    assert lib.ofx_opcount_read_phase(phase, c, len(KINDS)) == len(PHASES)
    return np.array(list(c), dtype=np.float64)


def _summary(counts, units):
    per = counts / units
    d = {k: round(float(v), 2) for k, v in zip(KINDS, per)}
    # FLOP: each add, mul, div and sqrt counts one
    d["flop"] = round(float(per[0] + per[1] + per[2] + per[3]), 2)
    return d


# initial condition (idefix_gb300.ic: name, arguments of (n, seed)),
# reconstruction, CFL, description
WORKLOADS = {
    "turbulence": ("turbulence_3d", lambda n, seed: dict(n=n, seed=seed), "plm", 0.6,
                   "turbulence 3-D {n}^3 FP64, HLLD + PLM + uct_contact, RK2"),
    "lowbeta": ("low_beta_3d", lambda n, seed: dict(n=n, seed=seed), "limo3", 0.6,
                "low-beta 3-D {n}^3 FP64, HLLD + LimO3 + uct_contact, RK2"),
    "ot3d": ("orszag_tang_3d", lambda n, seed: dict(nx=n, ny=n, nz=n), "plm", 0.9,
             "Orszag-Tang 3-D {n}^3 FP64, HLLD + PLM + uct_contact, RK2, CFL 0.9"),
    # one box of the ensemble workload (Mach 1, beta 10/3, the middle of its ranges)
    "ot2d": ("orszag_tang_like_2d", lambda n, seed: dict(n=n, mach=1.0, beta=10.0 / 3.0), "plm", 0.6,
             "Orszag-Tang-like 2-D {n}^2 FP64, HLLD + PLM + uct_contact, RK2, CFL 0.6"),
}
DIMS = {"ot2d": 2}


def count(n=64, cycles=1, seed=1, workload="turbulence"):
    sys.path.insert(0, os.path.dirname(HERE))
    from idefix_gb300 import ic
    from oracle.pyofx import Oracle

    subprocess.run(["make", "-s", "-C", HERE, "libofx_count.so"], check=True)
    make_ic, ic_args, order, cfl, desc = WORKLOADS[workload]
    Vc, Vs = getattr(ic, make_ic)(**ic_args(n, seed))
    dims = DIMS.get(workload, 3)
    o = Oracle(dims, (n,) * dims, order=order, cfl=cfl, kind="count")
    o.set_prim(Vc, Vs)
    lib = o.lib
    lib.ofx_opcount_reset()
    for _ in range(cycles):
        st = o.cycle()
        if st != 0:
            raise RuntimeError(f"oracle cycle failed with status {st}")
    cyc = _read(lib)
    cells = n**dims
    phases = {name: _summary(_read_phase(lib, p), cells * cycles) for p, name in enumerate(PHASES)}
    # one stage on the current state, its inputs prepared outside the count
    t, dt, _ = o.get_time()
    lib.ofx_set_boundaries(o.h)
    lib.ofx_prim_to_cons(o.h)
    lib.ofx_reset_stage(o.h)
    lib.ofx_opcount_reset()
    lib.ofx_evolve_stage(o.h, t, dt)
    stage = _read(lib)
    return {
        "workload": desc.format(n=n),
        "cells": cells,
        "cycles": cycles,
        "cycle": _summary(cyc, cells * cycles),
        "stage": _summary(stage, cells),
        "cycle_by_phase": phases,
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--cycles", type=int, default=1)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--workload", default="turbulence", choices=sorted(WORKLOADS))
    a = ap.parse_args()
    print(json.dumps(count(a.n, a.cycles, a.seed, a.workload)))


if __name__ == "__main__":
    main()
