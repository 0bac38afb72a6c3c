"""Generate the golden fixtures of tests/golden/ from the reference's own
hot-path code (the harness oracle/_ref/libofx_ref_*.so, built by
`make -C oracle ref` from the reference tree).

Each fixture holds the active-region input state, the scheme, and the
active-region state after a fixed number of TimeIntegrator cycles, plus
t, dt and the cycle count.  Optional scheme keys: "bc" ([Boundary] types per
direction) and "shock" ([Hydro] shockFlattening smoothing).  Fixtures that
exist already are kept (--force rewrites them).  Run from the repository
root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle.pyofx as P  # noqa: E402
from idefix_gb300 import ic  # noqa: E402
from mhd_state import embed, extract  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name, dims, n, order, solver, emf, nstages, cfl, cycles
CASES = [
    ("ot2d_hlld_plm_contact", 2, (32, 32), "plm", "hlld", "uct_contact", 2, 0.6, 20),
    ("ot2d_roe_plm_contact", 2, (32, 32), "plm", "roe", "uct_contact", 2, 0.6, 20),
    ("ot2d_hll_limo3_arith", 2, (32, 32), "limo3", "hll", "arithmetic", 2, 0.6, 20),
    ("ot2d_tvdlf_ppm_uct0", 2, (32, 32), "ppm", "tvdlf", "uct0", 3, 0.6, 20),
    ("ot2d_hlld_plm_ucthll", 2, (32, 32), "plm", "hlld", "uct_hll", 2, 0.6, 20),
    ("ot2d_hlld_ppm_ucthlld", 2, (32, 32), "ppm", "hlld", "uct_hlld", 2, 0.6, 20),
    ("ot2d_hlld_order1_contact_rk1", 2, (32, 32), "order1", "hlld", "uct_contact", 1, 0.4, 20),
    ("turb3d_hlld_plm_contact", 3, (12, 12, 12), "plm", "hlld", "uct_contact", 2, 0.6, 6),
    ("turb3d_roe_limo3_contact", 3, (12, 12, 12), "limo3", "roe", "uct_contact", 2, 0.6, 6),
    ("turb3d_hll_ppm_uct0", 3, (12, 12, 12), "ppm", "hll", "uct0", 3, 0.6, 6),
    ("turb3d_hlld_plm_ucthlld", 3, (12, 12, 12), "plm", "hlld", "uct_hlld", 2, 0.6, 6),
]

O, R, PER = ("outflow", "outflow"), ("reflective", "reflective"), ("periodic", "periodic")
# name, dims, n, order, solver, emf, nstages, cfl, cycles, extra scheme keys
EXTRA_CASES = [
    ("ot2d_hlld_plm_contact_walls", 2, (32, 32), "plm", "hlld", "uct_contact", 2, 0.6, 20,
     dict(bc=(R, O))),
    ("ot2d_roe_ppm_ucthlld_mixedbc", 2, (32, 32), "ppm", "roe", "uct_hlld", 2, 0.6, 20,
     dict(bc=(("reflective", "outflow"), PER))),
    ("turb3d_hlld_plm_contact_bc", 3, (12, 12, 12), "plm", "hlld", "uct_contact", 2, 0.6, 6,
     dict(bc=(O, R, PER))),
    ("ot2d_hlld_limo3_contact_shock", 2, (32, 32), "limo3", "hlld", "uct_contact", 2, 0.6, 20,
     dict(shock=0.5)),
    ("turb3d_hlld_plm_contact_shock", 3, (12, 12, 12), "plm", "hlld", "uct_contact", 2, 0.6, 6,
     dict(shock=0.0)),
]


def initial(dims, n):
    if dims == 2:
        Vc, Vs = ic.orszag_tang_2d(n[0], nghost=2)
    else:
        Vc, Vs = ic.turbulence_3d(n[0], seed=7, nghost=2, kmax=4)
    return extract(dims, n, 2, Vc, Vs)


def all_cases():
    return [c + (dict(),) for c in CASES] + EXTRA_CASES


def make_case(case, ref_dir=os.path.join(ROOT, "oracle", "_ref")):
    """run one case through the reference harness -> (arrays, meta)"""
    name, dims, n, order, solver, emf, nstages, cfl, cycles, extra = case
    vc0, vs0 = initial(dims, n)
    P.LIB_REF = os.path.join(ref_dir, f"libofx_ref_d{dims}_o{P.ORDER[order]}.so")
    o = P.Oracle(dims, n, order=order, solver=solver, emf=emf, nstages=nstages, cfl=cfl,
                 kind="ref", bc=extra.get("bc"), shock_flattening=extra.get("shock"))
    Vc, Vs = embed(dims, n, o.ng, vc0, vs0)
    o.set_prim(Vc, Vs)
    st = o.run(max_cycles=cycles)
    assert st == 0, (name, st)
    vc1, vs1 = extract(dims, n, o.ng, *o.get_prim())
    t, dt, nc = o.get_time()
    arrays = {"vc0": vc0, "vc1": vc1, "t": t, "dt": dt, "ncycles": nc}
    for c in range(dims):
        arrays[f"vs0_{c}"] = vs0[c]
        arrays[f"vs1_{c}"] = vs1[c]
    meta = dict(dims=dims, n=list(n), order=order, solver=solver, emf=emf, nstages=nstages,
                cfl=cfl, cycles=cycles, gamma=5.0 / 3.0, first_dt=1e-4, **extra)
    return arrays, meta


def main(force=False):
    for case in all_cases():
        name = case[0]
        if os.path.exists(os.path.join(OUT, name + ".npz")) and not force:
            continue
        arrays, meta = make_case(case)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), meta=np.array(repr(meta)), **arrays)
        print(name, arrays["t"], arrays["dt"], arrays["ncycles"])


if __name__ == "__main__":
    main(force="--force" in sys.argv)
