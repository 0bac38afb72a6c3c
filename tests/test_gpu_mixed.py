"""Mixed-precision path (FP32 reconstruction + Riemann solve, FP64 conserved
state, ConsToPrim and CT face update) against the bit-exact FP64 path.

The low-beta precision workload (beta = 1e-3, HLLD + LimO3 + CT, 384^3 at
full size) at reduced size: per-variable L1-relative and Linf errors of the mixed
run against the FP64 run, and div B, which the FP64 face update keeps at
round-off whatever the precision of the EMFs.
"""
import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import extract

pytestmark = pytest.mark.gpu


def _run(precision, Vc, Vs, n, cycles, **kw):
    blk = ig.GpuBlock(3, n, precision=precision, **kw)
    blk.upload(Vc, Vs)
    blk.run(max_cycles=cycles)
    out = extract(3, n, blk.ng, *blk.download())
    divb = blk.check_divb()
    tm = blk.get_time()
    blk.close()
    return out, divb, tm


def _errors(a, b):
    vc_a, vc_b = a[0], b[0]
    rows = {}
    for q, name in enumerate(["RHO", "VX1", "VX2", "VX3", "PRS"]):
        d = np.abs(vc_a[q] - vc_b[q])
        rows[name] = (float(d.sum() / np.abs(vc_b[q]).sum()), float(d.max()))
    for c in range(3):
        d = np.abs(a[1][c] - b[1][c])
        rows[f"BX{c + 1}s"] = (float(d.sum() / max(np.abs(b[1][c]).sum(), 1e-300)), float(d.max()))
    return rows


def test_mixed_low_beta_limo3_against_fp64():
    n = (64, 64, 64)
    Vc, Vs = ic.low_beta_3d(64, seed=3)
    kw = dict(order="limo3", solver="hlld", emf="uct_contact", cfl=0.6, first_dt=1e-4)
    fp64, divb64, t64 = _run("fp64", Vc, Vs, n, 40, **kw)
    mixed, divbm, tm = _run("mixed", Vc, Vs, n, 40, **kw)
    err = _errors(mixed, fp64)
    # the FP32 arithmetic is really used ...
    assert not np.array_equal(mixed[0], fp64[0])
    # ... and stays close to FP64 on the state (relative L1 per variable)
    assert err["RHO"][0] < 1e-5, err
    assert err["PRS"][0] < 1e-3, err
    assert err["BX1s"][0] < 1e-3 and err["BX3s"][0] < 1e-6, err
    assert divbm < 1e-10 and divb64 < 1e-10, (divbm, divb64)
    assert abs(tm[0] - t64[0]) < 1e-6 * t64[0]


@pytest.mark.parametrize("solver,order", [("hlld", "plm"), ("roe", "ppm"), ("hll", "order1")])
def test_mixed_turbulence_matches_fp64_closely(solver, order):
    n = (48, 48, 48)
    Vc, Vs = ic.turbulence_3d(48, seed=9, nghost=3 if order == "ppm" else 2)
    kw = dict(order=order, solver=solver, emf="uct_contact", cfl=0.6, first_dt=1e-4)
    fp64, _, _ = _run("fp64", Vc, Vs, n, 20, **kw)
    mixed, divbm, _ = _run("mixed", Vc, Vs, n, 20, **kw)
    err = _errors(mixed, fp64)
    assert err["RHO"][0] < 1e-5 and err["PRS"][0] < 1e-5, err
    assert divbm < 1e-10


# The tile sweep (FP32 y and z sweeps of 3-D blocks, operands staged in
# shared memory by tensor-map bulk copies) against the per-thread march:
# the same arithmetic lane for lane, so the runs must be bit-identical - for
# the three reconstruction orders it serves, segments that end inside the
# block and cover it whole, and sizes whose columns end inside a 16-column
# and an 8-row tile (stage 0 accumulates InvDt in the y and z sweeps, stage 1
# does not).
@pytest.mark.parametrize("order,n,seg", [("plm", 44, 32), ("plm", 32, 16), ("limo3", 36, 256), ("ppm", 30, 32)])
def test_tile_sweep_matches_march(order, n, seg):
    ng = 3 if order == "ppm" else 2
    Vc, Vs = ic.turbulence_3d(n, seed=11, nghost=ng, kmax=4)
    out = []
    for kinds in (["march"] * 3, ["march", "tile", "tile"]):
        blk = ig.GpuBlock(3, (n, n, n), order=order, cfl=0.6, first_dt=1e-4, precision="mixed")
        blk.upload(Vc, Vs)
        blk.set_segments([seg, seg, seg])
        blk.set_sweep_kernels(kinds)
        assert blk.sweep_kernels() == kinds
        blk.run(max_cycles=3)
        out.append((blk.download(), blk.get_time()))
        blk.close()
    (a, ta), (b, tb) = out
    assert ta == tb
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_tile_sweep_refused_where_it_does_not_apply():
    # 2-D, FP64, and the x direction run the march only
    blk = ig.GpuBlock(2, (32, 32), precision="mixed")
    with pytest.raises(ig.IdefixError):
        blk.set_sweep_kernels(["march", "tile"])
    blk.close()
    blk = ig.GpuBlock(3, (16, 16, 16), precision="fp64")
    with pytest.raises(ig.IdefixError):
        blk.set_sweep_kernels(["march", "tile", "tile"])
    blk.close()
    blk = ig.GpuBlock(3, (16, 16, 16), precision="mixed")
    with pytest.raises(ig.IdefixError):
        blk.set_sweep_kernels(["tile", "march", "march"])
    blk.set_sweep_kernels(["march", "tile", "march"])
    assert blk.sweep_kernels() == ["march", "tile", "march"]
    blk.close()


def test_mixed_download_cons_holds_the_cell_field():
    # the mixed path's stage ends leave the field part of Uc unstored; the
    # conserved state handed out must still hold the cell-centred field of
    # the faces (ReconstructVcField) and the hydro state the primitives came
    # from
    n = (24, 24, 24)
    Vc, Vs = ic.turbulence_3d(24, seed=5, kmax=3)
    blk = ig.GpuBlock(3, n, precision="mixed", cfl=0.6, first_dt=1e-4)
    blk.upload(Vc, Vs)
    blk.run(max_cycles=3)
    U = blk.download_cons()
    gVc, gVs = blk.download()
    blk.close()
    g = blk.ng
    a = (slice(g, g + n[2]), slice(g, g + n[1]), slice(g, g + n[0]))
    bx = 0.5 * (gVs[0][a] + gVs[0][a[0], a[1], slice(g + 1, g + n[0] + 1)])
    by = 0.5 * (gVs[1][a] + gVs[1][a[0], slice(g + 1, g + n[1] + 1), a[2]])
    bz = 0.5 * (gVs[2][a] + gVs[2][slice(g + 1, g + n[2] + 1), a[1], a[2]])
    assert np.array_equal(U[5][a], bx) and np.array_equal(U[6][a], by) and np.array_equal(U[7][a], bz)
    assert np.array_equal(U[5][a], gVc[5][a]) and np.array_equal(U[7][a], gVc[7][a])
    assert np.array_equal(U[0][a], gVc[0][a])  # density: the same value in both
    # velocity: the correctly rounded quotient ConsToPrim takes
    assert np.array_equal(U[1][a] / U[0][a], gVc[1][a]) and np.array_equal(U[3][a] / U[0][a], gVc[3][a])


def test_mixed_runs_in_pieces_match_one_run():
    # within a run the mixed path carries its state through the stage ends
    # (the next stage's inputs, the faces' Runge-Kutta begin copy) and
    # rebuilds the field part of Uc only when Uc is handed out; a run cut
    # into pieces - each starting with the full stage begin and face fill -
    # with or without downloads between them, and the NaN check on, must
    # give the bits of one uninterrupted run
    n = (24, 24, 24)
    Vc, Vs = ic.turbulence_3d(24, seed=7, kmax=3)
    kw = dict(precision="mixed", cfl=0.6, first_dt=1e-4, check_nan_period=4, log_period=5)

    def run(pieces, peek):
        blk = ig.GpuBlock(3, n, **kw)
        blk.upload(Vc, Vs)
        for p in pieces:
            blk.run(max_cycles=p)
            if peek:
                blk.download()
                blk.download_cons()
        out = blk.download()
        tm = blk.get_time()
        blk.close()
        return out, tm

    (a, b), t0 = run([7], False)
    for pieces, peek in (([3, 4], False), ([2, 1, 4], True)):
        (c, d), t1 = run(pieces, peek)
        assert t1 == t0
        assert np.array_equal(a, c) and np.array_equal(b, d), (pieces, peek)
