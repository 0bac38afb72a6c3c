"""Pin the CPU oracle (oracle/ofx.c) to the reference.

* against the reference's own hot-path code (oracle/_ref harness) on seeded
  inputs, bit for bit, over the scheme matrix the reference tests
  (test/MHD/OrszagTang/testme.py:16-21, OrszagTang3D, LinearWaveTest);
* against the golden fixtures that the harness produced (these run on any
  machine, the reference tree is not needed);
* against the reference's analytic known-answer test for linear waves
  (test/MHD/LinearWaveTest/python/testidefix.py:23-64).
"""
import glob
import os

import numpy as np
import pytest

import oracle.pyofx as P
from idefix_gb300 import ic
from mhd_state import embed, extract

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

MATRIX = []
for dims in (2, 3):
    for order in ("order1", "plm", "limo3", "ppm"):
        for solver in ("hlld", "hll", "roe", "tvdlf"):
            for emf in ("uct_contact", "arithmetic", "uct0", "uct_hll", "uct_hlld"):
                if emf == "uct_hlld" and solver in ("hll", "tvdlf"):
                    continue
                MATRIX.append((dims, order, solver, emf))


def _initial(dims, small=True):
    if dims == 2:
        n = (24, 24)
        Vc, Vs = ic.orszag_tang_2d(n[0], nghost=2)
    else:
        n = (10, 10, 10)
        Vc, Vs = ic.turbulence_3d(n[0], seed=5, nghost=2, kmax=4)
    return n, extract(dims, n, 2, Vc, Vs)


def _run(kind, dims, n, state, cycles, **scheme):
    o = P.Oracle(dims, n, kind=kind, **scheme)
    o.set_prim(*embed(dims, n, o.ng, *state))
    st = o.run(max_cycles=cycles)
    return st, extract(dims, n, o.ng, *o.get_prim()), o.get_time()


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip([a[0]] + a[1], [b[0]] + b[1]))


@pytest.mark.parametrize("dims,order,solver,emf", MATRIX)
def test_oracle_matches_reference_bit_for_bit(oracle_lib, reference_libs, dims, order, solver, emf):
    n, state = _initial(dims)
    P.LIB_REF = os.path.join(reference_libs, f"libofx_ref_d{dims}_o{P.ORDER[order]}.so")
    scheme = dict(order=order, solver=solver, emf=emf, cfl=0.6 if dims == 2 else 0.4)
    port = _run("port", dims, n, state, 5, **scheme)
    ref = _run("ref", dims, n, state, 5, **scheme)
    assert port[0] == ref[0] == 0
    assert port[2] == ref[2]
    assert _same(port[1], ref[1])


@pytest.mark.parametrize("nstages", [1, 3])
def test_oracle_matches_reference_rk_variants(oracle_lib, reference_libs, nstages):
    n, state = _initial(2)
    P.LIB_REF = os.path.join(reference_libs, "libofx_ref_d2_o2.so")
    scheme = dict(order="plm", solver="hlld", emf="uct_contact", nstages=nstages, cfl=0.4)
    port = _run("port", 2, n, state, 8, **scheme)
    ref = _run("ref", 2, n, state, 8, **scheme)
    assert port[2] == ref[2] and _same(port[1], ref[1])


def test_oracle_matches_reference_to_tstop_with_cfl_limited_dt(oracle_lib, reference_libs):
    """OT 2-D to t=0.1: the CFL reduction and the t_stop clamp are exercised"""
    dims, n = 2, (24, 24)
    Vc, Vs = ic.orszag_tang_2d(n[0])
    state = extract(dims, n, 2, Vc, Vs)
    P.LIB_REF = os.path.join(reference_libs, "libofx_ref_d2_o2.so")
    res = []
    for kind in ("port", "ref"):
        o = P.Oracle(dims, n, kind=kind)
        o.set_prim(*embed(dims, n, o.ng, *state))
        o.set_checks(log_period=10, check_nan_period=10)
        assert o.run(tstop=0.1) == 0
        res.append((extract(dims, n, o.ng, *o.get_prim()), o.get_time(), o.check_divb()))
    assert res[0][1] == res[1][1]
    assert res[0][1][0] == 0.1
    assert _same(res[0][0], res[1][0])
    assert res[0][2] == res[1][2]


def _golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.mark.parametrize("path", _golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_golden_fixture(oracle_lib, path):
    z = np.load(path)
    meta = eval(str(z["meta"]))  # fixture written by tests/golden/make_golden.py
    dims, n = meta["dims"], tuple(meta["n"])
    state = (z["vc0"], [z[f"vs0_{c}"] for c in range(dims)])
    st, out, tm = _run("port", dims, n, state, meta["cycles"], order=meta["order"],
                       solver=meta["solver"], emf=meta["emf"], nstages=meta["nstages"],
                       cfl=meta["cfl"], bc=meta.get("bc"), shock_flattening=meta.get("shock"))
    assert st == 0
    assert tm == (float(z["t"]), float(z["dt"]), int(z["ncycles"]))
    assert np.array_equal(out[0], z["vc1"])
    for c in range(dims):
        assert np.array_equal(out[1][c], z[f"vs1_{c}"])


def test_golden_fixtures_regenerate_bit_for_bit(oracle_lib, reference_libs):
    """every committed fixture is what tests/golden/make_golden.py makes now
    from the reference harness: same initial state (the initial conditions
    have not drifted), same scheme, same result"""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    saved = P.LIB_REF
    try:
        cases = mg.all_cases()
        assert sorted(c[0] + ".npz" for c in cases) == sorted(os.path.basename(p) for p in _golden_cases())
        for case in cases:
            z = np.load(os.path.join(GOLDEN, case[0] + ".npz"))
            arrays, meta = mg.make_case(case, reference_libs)
            assert eval(str(z["meta"])) == meta, case[0]
            for k, v in arrays.items():
                assert np.array_equal(np.asarray(v), z[k]), (case[0], k)
    finally:
        P.LIB_REF = saved


def test_golden_fixtures_present():
    assert len(_golden_cases()) >= 16


def test_oracle_linear_fast_wave_known_answer(oracle_lib):
    """LinearWaveTest (fast mode, Roe, PLM, CFL 0.9): after one period the
    mean-removed L1 error x 1e6 must stay below 3e-2
    (test/MHD/LinearWaveTest/python/testidefix.py:23-64, idefix-fast.ini)."""
    n = (64, 32, 32)
    Vc, Vs = ic.linear_wave_3d(mode=1, nx=n[0], ny=n[1], nz=n[2])
    o = P.Oracle(3, n, xbeg=(0, 0, 0), xend=(3.0, 1.5, 1.5), order="plm", solver="roe",
                 emf="uct_contact", cfl=0.9, first_dt=1e-4, threads=os.cpu_count() or 1)
    o.set_prim(Vc, Vs)
    vc0, vs0 = extract(3, n, 2, Vc, Vs)
    assert o.run(tstop=0.5) == 0
    vc1, vs1 = extract(3, n, 2, *o.get_prim())
    # fields as in the reference dump: Vc RHO,VX1..3,PRS and the face fields
    # on the active cells (the dump holds n faces per direction)
    pairs = [(vc0[q], vc1[q]) for q in (0, 1, 2, 3, 4)]
    for c in range(3):
        s = [slice(None)] * 3
        s[2 - c] = slice(0, n[c])
        pairs.append((vs0[c][tuple(s)], vs1[c][tuple(s)]))
    err = 0.0
    for q0, q1 in pairs:
        q0 = q0 - np.mean(q0)
        q1 = q1 - np.mean(q1)
        err += np.mean(np.abs(q0 - q1)) ** 2
    err = np.sqrt(err / len(pairs))
    assert err * 1e6 < 3e-2, err * 1e6


SHOCK_CASES = [(dims, order, smoothing) for dims in (2, 3) for order in ("plm", "limo3", "ppm")
               for smoothing in (0.0, 0.5, 5.0)]


@pytest.mark.parametrize("dims,order,smoothing", SHOCK_CASES)
def test_oracle_matches_reference_with_shock_flattening(oracle_lib, reference_libs, dims, order, smoothing):
    # [Hydro] shockFlattening (ShockFlattening::FindShock compiled from the
    # reference, shockFlattening.hpp): flagged cells take the minmod slope
    if dims == 2:
        n = (48, 48)
        Vc, Vs = ic.orszag_tang_2d(n[0], nghost=2)
    else:
        n = (12, 12, 12)
        Vc, Vs = ic.turbulence_3d(n[0], seed=7, nghost=2, kmax=4)
    ng = 3 if order == "ppm" else 2
    state = extract(dims, n, 2, Vc, Vs)
    P.LIB_REF = os.path.join(reference_libs, f"libofx_ref_d{dims}_o{P.ORDER[order]}.so")
    scheme = dict(order=order, cfl=0.6 if dims == 2 else 0.4, shock_flattening=smoothing)
    cycles = 30 if dims == 2 else 8
    port = _run("port", dims, n, state, cycles, **scheme)
    ref = _run("ref", dims, n, state, cycles, **scheme)
    assert port[0] == ref[0]
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]
    del ng
    if order != "ppm" and smoothing == 0.0:
        # the flags fire on this flow: the result differs from no flattening
        plain = _run("port", dims, n, state, cycles, order=order, cfl=scheme["cfl"])
        assert not _same(port[1], plain[1])


O, R, PER = ("outflow", "outflow"), ("reflective", "reflective"), ("periodic", "periodic")
RO = ("reflective", "outflow")
BC_CASES = [
    (2, "plm", "hlld", (O, R)),
    (2, "plm", "hlld", (RO, PER)),
    (2, "ppm", "roe", (PER, ("outflow", "reflective"))),
    (2, "limo3", "hll", (O, O)),
    (3, "plm", "hlld", (O, R, PER)),
    (3, "ppm", "hlld", (RO, RO, RO)),
    (3, "limo3", "roe", (PER, O, R)),
]


def _full_same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("dims,order,solver,bc", BC_CASES)
def test_oracle_matches_reference_with_boundaries(oracle_lib, reference_libs, dims, order, solver, bc):
    # [Boundary] reflective / outflow (Boundary::EnforceReflective,
    # EnforceOutflow and ReconstructNormalField compiled from the reference,
    # boundary.hpp): the active state bit for bit, and the whole arrays,
    # ghosts included, once the boundaries are applied to the final state
    # (the reference's face update also writes one ghost row of tangential
    # faces, evolveMagField.hpp, which the next boundary pass overwrites)
    if dims == 2:
        n = (32, 24)
        Vc, Vs = ic.orszag_tang_2d(32, nghost=2)
        state = extract(dims, (32, 32), 2, Vc, Vs)
        state = (state[0][:, :, :24, :], [s[:, :24 + (c == 1), :] for c, s in enumerate(state[1])])
    else:
        n = (10, 10, 10)
        Vc, Vs = ic.turbulence_3d(n[0], seed=9, nghost=2, kmax=4)
        state = extract(dims, n, 2, Vc, Vs)
    P.LIB_REF = os.path.join(reference_libs, f"libofx_ref_d{dims}_o{P.ORDER[order]}.so")
    scheme = dict(order=order, solver=solver, cfl=0.6 if dims == 2 else 0.4, bc=bc)
    cycles = 20 if dims == 2 else 6
    out = {}
    for kind in ("port", "ref"):
        o = P.Oracle(dims, n, kind=kind, **scheme)
        o.set_prim(*embed(dims, n, o.ng, *state))
        st = o.run(max_cycles=cycles)
        active = extract(dims, n, o.ng, *o.get_prim())
        o.lib.ofx_set_boundaries(o.h)
        out[kind] = (st, active, o.get_time(), o.get_prim())
    assert out["port"][0] == out["ref"][0]
    assert _same(out["port"][1], out["ref"][1])
    assert out["port"][2] == out["ref"][2]
    assert _full_same(out["port"][3], out["ref"][3])
    # the boundaries act: the result differs from the periodic run
    per = _run("port", dims, n, state, cycles, order=order, solver=solver, cfl=scheme["cfl"])
    assert not _same(out["port"][1], per[1])


def test_oracle_refuses_half_periodic_boundaries(oracle_lib):
    with pytest.raises(ValueError):
        P.Oracle(2, (8, 8), bc=(("periodic", "outflow"), PER))


@pytest.mark.parametrize("problem", ["rotor", "shock_tube"])
def test_oracle_matches_reference_on_boundary_problems(oracle_lib, reference_libs, problem):
    # the reference's own outflow test problems (test/MHD/RotorCartesian,
    # test/MHD/sod run as a y-uniform 2-D block), Roe, their ini settings
    if problem == "rotor":
        n = (48, 48)
        state = extract(2, n, 2, *ic.rotor_2d(48))
        scheme = dict(solver="roe", cfl=0.2, bc=(O, O), xbeg=ic.ROTOR_DOMAIN[0], xend=ic.ROTOR_DOMAIN[1])
    else:
        n = (200, 2)
        state = extract(2, n, 2, *ic.shock_tube_2d(200, 2))
        xb, xe = ic.shock_tube_domain(200, 2)
        scheme = dict(solver="roe", cfl=0.8, gamma=ic.SHOCK_TUBE_GAMMA, bc=(O, PER), xbeg=xb, xend=xe)
    P.LIB_REF = os.path.join(reference_libs, "libofx_ref_d2_o2.so")
    port = _run("port", 2, n, state, 30, **scheme)
    ref = _run("ref", 2, n, state, 30, **scheme)
    assert port[0] == ref[0] == 0
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]


def test_oracle_matches_reference_on_field_loop(oracle_lib, reference_libs):
    # test/MHD/FieldLoop (HLLD, CFL 0.2, periodic; face field from a vector
    # potential), y-uniform with two cells
    n = (24, 2, 24)
    state = extract(3, n, 2, *ic.field_loop_3d(*n))
    xb, xe = ic.FIELD_LOOP_DOMAIN
    P.LIB_REF = os.path.join(reference_libs, "libofx_ref_d3_o2.so")
    scheme = dict(cfl=0.2, xbeg=xb, xend=xe)
    port = _run("port", 3, n, state, 25, **scheme)
    ref = _run("ref", 3, n, state, 25, **scheme)
    assert port[0] == ref[0] == 0
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]


def test_oracle_matches_reference_on_orszag_tang_3d(oracle_lib, reference_libs):
    # test/MHD/OrszagTang3D (32 x 64 x 32, HLLD, CFL 0.9, face field from a
    # vector potential; without its two passive tracers)
    n = (32, 64, 32)
    state = extract(3, n, 2, *ic.orszag_tang_3d(*n))
    P.LIB_REF = os.path.join(reference_libs, "libofx_ref_d3_o2.so")
    port = _run("port", 3, n, state, 10, cfl=0.9)
    ref = _run("ref", 3, n, state, 10, cfl=0.9)
    assert port[0] == ref[0] == 0
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]


COMBO_CASES = [
    (2, dict(order="plm", solver="hlld", shock_flattening=0.5, bc=(R, O))),
    (3, dict(order="limo3", solver="hll", emf="uct_hll", bc=(O, O, O))),
    (2, dict(order="ppm", solver="roe", nstages=3, bc=(R, PER))),
    (3, dict(order="plm", solver="tvdlf", emf="arithmetic", bc=(R, O, PER))),
    (3, dict(order="ppm", solver="hlld", emf="uct_hlld", shock_flattening=0.0, bc=(O, PER, RO))),
]


@pytest.mark.parametrize("dims,scheme", COMBO_CASES)
def test_oracle_matches_reference_on_combined_options(oracle_lib, reference_libs, dims, scheme):
    # boundaries together with shock flattening, RK3 and the other solvers /
    # EMF averages, against the reference harness
    if dims == 2:
        n = (32, 24)
        Vc, Vs = ic.orszag_tang_2d(32, nghost=2)
        state = extract(dims, (32, 32), 2, Vc, Vs)
        state = (state[0][:, :, :24, :], [st[:, :24 + (c == 1), :] for c, st in enumerate(state[1])])
    else:
        n = (10, 10, 10)
        Vc, Vs = ic.turbulence_3d(n[0], seed=9, nghost=2, kmax=4)
        state = extract(dims, n, 2, Vc, Vs)
    P.LIB_REF = os.path.join(reference_libs, f"libofx_ref_d{dims}_o{P.ORDER[scheme['order']]}.so")
    kw = dict(scheme, cfl=0.6 if dims == 2 else 0.4)
    cycles = 20 if dims == 2 else 6
    port = _run("port", dims, n, state, cycles, **kw)
    ref = _run("ref", dims, n, state, cycles, **kw)
    assert port[0] == ref[0] == 0
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]


NON_CUBIC = [
    dict(order="plm", solver="hlld", emf="uct_contact"),
    dict(order="limo3", solver="roe", emf="uct0"),
    dict(order="ppm", solver="hll", emf="arithmetic"),
    dict(order="plm", solver="tvdlf", emf="uct_hll", nstages=3),
]


@pytest.mark.parametrize("scheme", NON_CUBIC, ids=lambda s: "_".join(str(v) for v in s.values()))
def test_oracle_matches_reference_on_a_non_cubic_block(oracle_lib, reference_libs, scheme):
    """a 12 x 8 x 6 block (every direction its own extent and stride), cut
    from a periodic 12^3 state, against the reference harness"""
    n = (12, 8, 6)
    Vc, Vs = ic.turbulence_3d(12, seed=4, nghost=2, kmax=4)
    vc, vs = extract(3, (12, 12, 12), 2, Vc, Vs)
    state = (vc[:, :n[2], :n[1], :n[0]],
             [st[:n[2] + (c == 2), :n[1] + (c == 1), :n[0] + (c == 0)] for c, st in enumerate(vs)])
    P.LIB_REF = os.path.join(reference_libs, f"libofx_ref_d3_o{P.ORDER[scheme['order']]}.so")
    kw = dict(scheme, cfl=0.4)
    port = _run("port", 3, n, state, 6, **kw)
    ref = _run("ref", 3, n, state, 6, **kw)
    assert port[0] == ref[0] == 0
    assert _same(port[1], ref[1])
    assert port[2] == ref[2]
