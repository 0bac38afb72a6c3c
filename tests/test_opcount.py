"""The operation-counting build of the CPU oracle (oracle/opcount.cpp).

Its counts stand for the reference algorithm only if it computes exactly what
the plain oracle computes: the tests run both on the same seeded inputs,
over several schemes, and compare the states bit for bit, then check the
counts' structure (a cycle is two stages plus the work around them; every
kind the hot path uses is counted)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle.pyofx as P
from idefix_gb300 import ic
from mhd_state import embed, extract

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def count_lib(oracle_lib):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "libofx_count.so"], check=True)
    return P.load("count")


def _state(dims):
    if dims == 2:
        n = (24, 24)
        return n, extract(2, n, 2, *ic.orszag_tang_2d(24, nghost=2))
    n = (12, 12, 12)
    return n, extract(3, n, 2, *ic.turbulence_3d(12, seed=3, nghost=2, kmax=4))


def _read(lib):
    c = (ctypes.c_longlong * 8)()
    assert lib.ofx_opcount_read(c, 8) == 8
    return np.array(list(c))


@pytest.mark.parametrize("dims,order,solver,emf", [
    (2, "plm", "hlld", "uct_contact"),
    (3, "plm", "hlld", "uct_contact"),
    (3, "limo3", "hlld", "uct_hlld"),
    (3, "ppm", "roe", "uct0"),
    (2, "plm", "tvdlf", "uct_hll"),
])
def test_counting_build_is_bit_identical_to_the_oracle(count_lib, dims, order, solver, emf):
    n, state = _state(dims)
    out = {}
    for kind in ("port", "count"):
        o = P.Oracle(dims, n, kind=kind, order=order, solver=solver, emf=emf,
                     cfl=0.6 if dims == 2 else 0.4)
        o.set_prim(*embed(dims, n, o.ng, *state))
        assert o.run(max_cycles=4) == 0
        out[kind] = (o.get_prim(), o.get_time())
    (pa, ta), (ca, tc) = out["port"], out["count"]
    assert ta == tc
    for a, b in zip(pa, ca):
        assert np.array_equal(a, b)


def test_counts_of_a_cycle(count_lib):
    from oracle.opcount import KINDS, count

    lib = count_lib
    res = count(n=16, cycles=2)
    cyc, stage = res["cycle"], res["stage"]
    assert set(KINDS) <= set(cyc)
    # every kind the MHD step uses occurs
    assert all(cyc[k] > 0 for k in KINDS)
    # a RK2 cycle is two stages plus conversions, boundaries, combination, dt
    assert 2.0 * stage["flop"] < cyc["flop"] < 2.3 * stage["flop"]
    # the order of magnitude of an HLLD + PLM + CT step: ~10^3 FP64 FLOP,
    # ~10^2 divisions and tens of square roots per zone-cycle
    assert 2500 < cyc["flop"] < 5000
    assert 100 < cyc["div"] < 400 and 10 < cyc["sqrt"] < 100
    lib.ofx_opcount_reset()
    assert not _read(lib).any()


def test_bench_flop_figure_follows_the_count(count_lib):
    """bench.py's FP64 FLOP per zone-cycle is the count at 256^3; smaller
    boxes add the ghost-zone work of the conversions and boundaries, so the
    count at 64^3 lies a few percent above it."""
    import bench
    from oracle.opcount import count

    small = count(n=64, cycles=1)["cycle"]["flop"]
    assert bench.FP64_FLOP_PER_ZONE_CYCLE < small < 1.1 * bench.FP64_FLOP_PER_ZONE_CYCLE
    roof = bench.fp64_flop_roof(1.2e8, 600.0)
    assert roof["frac"] == pytest.approx(1.2e8 / roof["ceiling_zone_cycles_per_gpu"])
    assert roof["achieved"] == pytest.approx(1.2e8 * bench.FP64_FLOP_PER_ZONE_CYCLE / 1e9)
    assert bench.fp64_flop_roof(1.2e8, 0.0) is None


def test_limo3_workload_counts_its_limiter(count_lib):
    """LimO3 (slopeLimiter.hpp:25-52) adds divisions and min/max to every
    reconstructed value: the low-beta workload counts more of both."""
    from oracle.opcount import count

    plm = count(n=16, workload="turbulence")["cycle"]
    limo3 = count(n=16, seed=0, workload="lowbeta")["cycle"]
    assert limo3["div"] > 1.5 * plm["div"]
    assert limo3["minmax"] > 10 * plm["minmax"]


def test_phases_add_up_to_the_cycle(count_lib):
    """the per-phase counters split the cycle without losing or adding work;
    the three sweeps carry most of it"""
    from oracle.opcount import PHASES, count

    res = count(n=16, cycles=2)
    ph = res["cycle_by_phase"]
    assert tuple(ph) == PHASES
    for k in ("add", "mul", "div", "sqrt", "flop"):
        # each figure is rounded to 0.01
        assert sum(v[k] for v in ph.values()) == pytest.approx(res["cycle"][k], abs=0.01 * len(ph))
    sweeps = sum(ph[s]["flop"] for s in ("sweep_x", "sweep_y", "sweep_z"))
    assert 0.8 * res["cycle"]["flop"] < sweeps < res["cycle"]["flop"]
    assert ph["ct_corner"]["flop"] > 0 and ph["ct_faces"]["flop"] > 0


def test_orszag_tang_3d_costs_as_much_as_the_turbulence_workload(count_lib):
    """the reference's benchmark problem (3-D Orszag-Tang) and the bench's
    turbulence workload cost the same FP64 work per zone-cycle to a few %"""
    from oracle.opcount import count

    ot = count(n=24, workload="ot3d")["cycle"]["flop"]
    turb = count(n=24, workload="turbulence")["cycle"]["flop"]
    assert abs(ot - turb) < 0.05 * turb
