"""Reflective and outflow boundaries on the GPU ([Boundary] block; ghosts as
Boundary::EnforceReflective / EnforceOutflow, the normal field rebuilt from
div B = 0 as Boundary::ReconstructNormalField, boundary.hpp:408-809).

The oracle's boundary pass is pinned bit for bit to the reference's own
Boundary class (compiled into the reference harness); the GPU is compared
with the oracle: the boundary pass alone on the whole arrays (ghosts
included), then whole runs (active state and time bit for bit, the whole
arrays after a final boundary pass), in FP64.  The mixed-precision path is
checked against the FP64 one with a stated tolerance.
"""
import os

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import embed, extract

O, R, PER = ("outflow", "outflow"), ("reflective", "reflective"), ("periodic", "periodic")
RO, OR = ("reflective", "outflow"), ("outflow", "reflective")


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    build.build_oracle()
    ig.load_library()


def _ot_strip(nx, ny):
    """Orszag-Tang state cut to nx x ny cells (whole cells with their faces,
    so div B stays at round-off)"""
    m = max(nx, ny)
    Vc, Vs = ic.orszag_tang_2d(m, nghost=2)
    vc, vs = extract(2, (m, m), 2, Vc, Vs)
    return vc[:, :, :ny, :nx], [vs[0][:, :ny, :nx + 1], vs[1][:, :ny + 1, :nx]]


def _state(dims):
    if dims == 2:
        return (40, 28), _ot_strip(40, 28)
    n = (12, 10, 14)
    Vc, Vs = ic.turbulence_3d(14, seed=11, kmax=4)
    vc, vs = extract(3, (14, 14, 14), 2, Vc, Vs)
    return n, (vc[:, :14, :10, :12], [vs[0][:14, :10, :13], vs[1][:14, :11, :12], vs[2][:15, :10, :12]])


@pytest.mark.gpu
@pytest.mark.parametrize("dims,order,bc", [
    (2, "plm", (O, R)), (2, "ppm", (RO, PER)), (2, "limo3", (PER, OR)),
    (3, "plm", (O, R, PER)), (3, "ppm", (RO, OR, RO)), (3, "plm", (PER, PER, O)),
])
def test_gpu_boundary_pass_matches_oracle(dims, order, bc):
    """one SetBoundaries on a random state (ghosts random too): every value
    of both whole arrays"""
    from oracle.pyofx import Oracle

    n = (9, 7) if dims == 2 else (6, 5, 7)
    blk = ig.GpuBlock(dims, n, order=order, bc=bc)
    o = Oracle(dims, n, order=order, bc=bc)
    rng = np.random.default_rng(5)
    Vc = rng.standard_normal(blk.vc_shape)
    Vs = rng.standard_normal(blk.vs_shape)
    blk.upload(Vc, Vs)
    o.set_prim(Vc, Vs)
    blk.set_boundaries()
    o.lib.ofx_set_boundaries(o.h)
    gVc, gVs = blk.download()
    oVc, oVs = o.get_prim()
    nvar = 2 * dims + 2
    assert np.array_equal(gVc[:dims + 2], oVc[:dims + 2])  # the non-field variables
    assert np.array_equal(gVs, oVs)                          # every face, ghosts included
    assert np.array_equal(gVc[dims + 2:nvar], oVc[dims + 2:nvar])  # field rebuilt from the faces
    blk.close()


RUNS = [
    (2, "plm", "hlld", "uct_contact", (O, R)),
    (2, "ppm", "roe", "uct_hlld", (RO, PER)),
    (2, "limo3", "hll", "uct_hll", (O, O)),
    (2, "order1", "tvdlf", "arithmetic", (R, R)),
    (3, "plm", "hlld", "uct_contact", (O, R, PER)),
    (3, "ppm", "hlld", "uct_hlld", (RO, RO, RO)),
    (3, "limo3", "roe", "uct0", (PER, O, R)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,order,solver,emf,bc", RUNS)
def test_gpu_runs_with_boundaries_match_oracle(dims, order, solver, emf, bc):
    from oracle.pyofx import Oracle

    n, state = _state(dims)
    cfl = 0.6 if dims == 2 else 0.4
    cycles = 25 if dims == 2 else 8
    kw = dict(order=order, solver=solver, emf=emf, cfl=cfl, first_dt=1e-4, bc=bc)
    o = Oracle(dims, n, threads=os.cpu_count() or 1, **kw)
    o.set_prim(*embed(dims, n, o.ng, *state))
    assert o.run(max_cycles=cycles) == 0
    ref = extract(dims, n, o.ng, *o.get_prim())
    blk = ig.GpuBlock(dims, n, **kw)
    blk.upload(*embed(dims, n, blk.ng, *state))
    blk.run(max_cycles=cycles)
    out = extract(dims, n, blk.ng, *blk.download())
    assert np.array_equal(out[0], ref[0]), np.nanmax(np.abs(out[0] - ref[0]))
    for c in range(dims):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time()[:2] == o.get_time()[:2]
    blk.set_boundaries()
    o.lib.ofx_set_boundaries(o.h)
    gVc, gVs = blk.download()
    oVc, oVs = o.get_prim()
    assert np.array_equal(gVc, oVc) and np.array_equal(gVs, oVs)
    blk.close()


@pytest.mark.gpu
def test_gpu_orszag_tang_128_walls_to_t02_bit_identical():
    """the 2-D Orszag-Tang flow in a box with reflective walls in x and
    outflow in y, 128^2 to t = 0.2"""
    from oracle.pyofx import Oracle

    n = (128, 128)
    state = extract(2, n, 2, *ic.orszag_tang_2d(128, nghost=2))
    kw = dict(cfl=0.6, first_dt=1e-4, bc=(R, O))
    o = Oracle(2, n, threads=os.cpu_count() or 1, **kw)
    o.set_prim(*embed(2, n, o.ng, *state))
    assert o.run(tstop=0.2) == 0
    ref = extract(2, n, o.ng, *o.get_prim())
    blk = ig.GpuBlock(2, n, **kw)
    blk.upload(*embed(2, n, blk.ng, *state))
    blk.run(tstop=0.2)
    out = extract(2, n, blk.ng, *blk.download())
    assert np.array_equal(out[0], ref[0])
    for c in range(2):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time() == o.get_time()
    assert blk.check_divb() < 1e-12
    blk.close()


@pytest.mark.gpu
def test_gpu_mixed_precision_with_boundaries_tracks_fp64():
    """mixed precision (FP32 reconstruction and Riemann solve) with outflow
    and reflective walls: relative L1 distance to FP64 below 1e-4 per
    variable after 40 cycles, div B at round-off"""
    dims = 3
    n = (32, 32, 32)
    Vc, Vs = ic.turbulence_3d(32, seed=4, kmax=4)
    state = extract(3, n, 2, Vc, Vs)
    out = {}
    for prec in ("fp64", "mixed"):
        blk = ig.GpuBlock(dims, n, cfl=0.4, first_dt=1e-4, precision=prec, bc=(O, R, RO))
        blk.upload(*embed(dims, n, blk.ng, *state))
        blk.run(max_cycles=40)
        out[prec] = extract(dims, n, blk.ng, *blk.download())
        assert blk.check_divb() < 1e-11
        blk.close()
    a, b = out["fp64"][0], out["mixed"][0]
    for v in range(a.shape[0]):
        scale = np.mean(np.abs(a[v])) + 1e-30
        assert np.mean(np.abs(a[v] - b[v])) / scale < 1e-4, v


def test_boundary_configs_refused():
    """refused before any device work (runs without a GPU)"""
    with pytest.raises(ig.IdefixError):  # periodic on one side only
        ig.GpuBlock(2, (16, 16), bc=(("periodic", "outflow"), PER))
    with pytest.raises(ig.IdefixError):  # a mirror needs as many cells as ghosts
        ig.GpuBlock(2, (2, 16), order="ppm", bc=(R, PER))
    with pytest.raises(ig.IdefixError):  # the ensemble's boxes are periodic
        ig.Ensemble([dict(dims=2, n=(16, 16), bc=(O, O))])


def _oracle_and_gpu(dims, n, state, tstop, **kw):
    from oracle.pyofx import Oracle

    o = Oracle(dims, n, threads=os.cpu_count() or 1, **kw)
    o.set_prim(*embed(dims, n, o.ng, *state))
    assert o.run(tstop=tstop) == 0
    ref = extract(dims, n, o.ng, *o.get_prim())
    blk = ig.GpuBlock(dims, n, **kw)
    blk.upload(*embed(dims, n, blk.ng, *state))
    blk.run(tstop=tstop)
    out = extract(dims, n, blk.ng, *blk.download())
    return o, ref, blk, out


@pytest.mark.gpu
def test_gpu_rotor_256_to_t015_bit_identical():
    """test/MHD/RotorCartesian (Roe, CFL 0.2, outflow on all sides) at 256^2
    to its t_stop = 0.15: bit-identical to the oracle"""
    n = (256, 256)
    state = extract(2, n, 2, *ic.rotor_2d(256))
    xb, xe = ic.ROTOR_DOMAIN
    o, ref, blk, out = _oracle_and_gpu(2, n, state, 0.15, solver="roe", cfl=0.2, first_dt=1e-4, bc=(O, O),
                                       xbeg=xb, xend=xe)
    assert np.array_equal(out[0], ref[0])
    for c in range(2):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time() == o.get_time()
    assert blk.check_divb() < 1e-10
    blk.close()


@pytest.mark.gpu
def test_gpu_shock_tube_to_t10_bit_identical_and_uniform():
    """test/MHD/sod (Roe, CFL 0.8, gamma 1.66666666666667, outflow) as a
    y-uniform 800 x 4 block to its t_stop = 10: bit-identical to the oracle,
    every row identical, the compound-wave structure inside the tube"""
    n = (800, 4)
    state = extract(2, n, 2, *ic.shock_tube_2d(800, 4))
    xb, xe = ic.shock_tube_domain(800, 4)
    o, ref, blk, out = _oracle_and_gpu(2, n, state, 10.0, solver="roe", cfl=0.8, first_dt=1e-4,
                                       gamma=ic.SHOCK_TUBE_GAMMA, bc=(O, PER), xbeg=xb, xend=xe)
    assert np.array_equal(out[0], ref[0])
    for c in range(2):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time() == o.get_time()
    vc = out[0][:, 0]
    assert all(np.array_equal(vc[:, j], vc[:, 0]) for j in range(1, 4))
    rho = vc[0, 0]
    # the waves have not reached the ends by t = 10: the end states are intact
    assert rho[0] == 1.0 and rho[-1] == 0.125
    assert 0.1 < rho.min() and rho.max() < 1.1
    blk.close()


COMBOS = [
    (2, dict(order="plm", solver="hlld", shock_flattening=0.5, bc=(R, O))),
    (3, dict(order="limo3", solver="hll", emf="uct_hll", bc=(O, O, O))),
    (2, dict(order="ppm", solver="roe", nstages=3, bc=(R, PER))),
    (3, dict(order="plm", solver="tvdlf", emf="arithmetic", bc=(R, O, PER))),
    (3, dict(order="ppm", solver="hlld", emf="uct_hlld", shock_flattening=0.0, bc=(O, PER, RO))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,scheme", COMBOS)
def test_gpu_combined_options_match_oracle(dims, scheme):
    """boundaries together with shock flattening, RK3 and the other solvers /
    EMF averages (each combination pinned to the reference harness on the
    CPU): bit-identical to the oracle"""
    from oracle.pyofx import Oracle

    n, state = _state(dims)
    kw = dict(scheme, cfl=0.6 if dims == 2 else 0.4, first_dt=1e-4)
    cycles = 25 if dims == 2 else 8
    o = Oracle(dims, n, threads=os.cpu_count() or 1, **kw)
    o.set_prim(*embed(dims, n, o.ng, *state))
    assert o.run(max_cycles=cycles) == 0
    ref = extract(dims, n, o.ng, *o.get_prim())
    blk = ig.GpuBlock(dims, n, **kw)
    blk.upload(*embed(dims, n, blk.ng, *state))
    blk.run(max_cycles=cycles)
    out = extract(dims, n, blk.ng, *blk.download())
    assert np.array_equal(out[0], ref[0]), np.nanmax(np.abs(out[0] - ref[0]))
    for c in range(dims):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time()[:2] == o.get_time()[:2]
    blk.close()
