"""Parity of the CUDA path (through the C ABI) with the reference.

* golden fixtures produced by the reference's own hot-path code: bit for bit
* the CPU oracle (itself pinned bit for bit to the reference) over the scheme
  matrix, the building blocks, and the full Orszag-Tang 2-D run to t = 0.5
* the reference's linear-wave known-answer test
* at the 256^3 throughput size: size-independent properties (div B at
  round-off, conservation in the periodic box, run-to-run determinism)
The FP64 path is compiled without FMA contraction, like the reference's GPU
CI, so the tolerance of every comparison below is exact equality.
"""
import glob
import os

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import embed, extract

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    build.build_oracle()
    ig.load_library()


def _gpu(dims, n, state, cycles=None, tstop=-1.0, **kw):
    blk = ig.GpuBlock(dims, n, **kw)
    blk.upload(*embed(dims, n, blk.ng, *state))
    blk.run(tstop=tstop, max_cycles=-1 if cycles is None else cycles)
    out = extract(dims, n, blk.ng, *blk.download())
    tm = blk.get_time()
    blk.close()
    return out, tm


def _oracle(dims, n, state, cycles=None, tstop=-1.0, threads=None, **kw):
    from oracle.pyofx import Oracle

    o = Oracle(dims, n, threads=threads or os.cpu_count() or 1, **kw)
    o.set_prim(*embed(dims, n, o.ng, *state))
    assert o.run(tstop=tstop, max_cycles=-1 if cycles is None else cycles) == 0
    t, dt, nc = o.get_time()
    return extract(dims, n, o.ng, *o.get_prim()), (t, dt, nc)


def _assert_same(a, b):
    assert np.array_equal(a[0], b[0]), np.nanmax(np.abs(a[0] - b[0]))
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y), np.nanmax(np.abs(x - y))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_reference_golden_fixture(path):
    z = np.load(path)
    meta = eval(str(z["meta"]))  # written by tests/golden/make_golden.py
    dims, n = meta["dims"], tuple(meta["n"])
    state = (z["vc0"], [z[f"vs0_{c}"] for c in range(dims)])
    out, tm = _gpu(dims, n, state, cycles=meta["cycles"], order=meta["order"], solver=meta["solver"],
                   emf=meta["emf"], nstages=meta["nstages"], cfl=meta["cfl"], first_dt=meta["first_dt"],
                   bc=meta.get("bc"), shock_flattening=meta.get("shock"))
    assert tm == (float(z["t"]), float(z["dt"]), int(z["ncycles"]))
    _assert_same(out, (z["vc1"], [z[f"vs1_{c}"] for c in range(dims)]))


MATRIX = [(d, o, s, e) for d in (2, 3) for o in ("order1", "plm", "limo3", "ppm")
          for s in ("hlld", "hll", "roe", "tvdlf")
          for e in ("uct_contact", "arithmetic", "uct0", "uct_hll", "uct_hlld")
          if not (e == "uct_hlld" and s in ("hll", "tvdlf"))]


def _small_state(dims, seed=3):
    if dims == 2:
        n = (40, 24)
        Vc, Vs = ic.orszag_tang_2d(40)
        vc, vs = extract(2, (40, 40), 2, Vc, Vs)
        # non-square box: keep the first 24 rows (periodicity is not needed
        # for parity, only identical inputs)
        return n, (vc[:, :, :24, :], [vs[0][:, :24, :], vs[1][:, :25, :]])
    n = (12, 10, 8)
    Vc, Vs = ic.turbulence_3d(12, seed=seed, kmax=4)
    vc, vs = extract(3, (12, 12, 12), 2, Vc, Vs)
    return n, (vc[:, :8, :10, :], [vs[0][:8, :10, :], vs[1][:8, :11, :], vs[2][:9, :10, :]])


@pytest.mark.parametrize("dims,order,solver,emf", MATRIX)
def test_gpu_matches_oracle_scheme_matrix(dims, order, solver, emf):
    n, state = _small_state(dims)
    kw = dict(order=order, solver=solver, emf=emf, cfl=0.5, first_dt=1e-4)
    g = _gpu(dims, n, state, cycles=4, **kw)
    o = _oracle(dims, n, state, cycles=4, **kw)
    assert g[1] == o[1]
    _assert_same(g[0], o[0])


@pytest.mark.parametrize("nstages", [1, 3])
def test_gpu_matches_oracle_rk_variants(nstages):
    n, state = _small_state(3)
    kw = dict(order="plm", solver="hlld", emf="uct_contact", nstages=nstages, cfl=0.4, first_dt=1e-4)
    g = _gpu(3, n, state, cycles=6, **kw)
    o = _oracle(3, n, state, cycles=6, **kw)
    assert g[1] == o[1]
    _assert_same(g[0], o[0])


def test_gpu_orszag_tang_256_to_t05_bit_identical():
    """the reference's 2-D Orszag-Tang configuration (256^2, HLLD, PLM,
    uct_contact, RK2, CFL 0.6, first_dt 1e-4) integrated to t = 0.5"""
    n = (256, 256)
    Vc, Vs = ic.orszag_tang_2d(256)
    state = extract(2, n, 2, Vc, Vs)
    kw = dict(order="plm", solver="hlld", emf="uct_contact", cfl=0.6, first_dt=1e-4,
              log_period=100, check_nan_period=100)
    g = _gpu(2, n, state, tstop=0.5, **kw)
    o = _oracle(2, n, state, tstop=0.5, **kw)
    assert g[1] == o[1] and g[1][0] == 0.5
    _assert_same(g[0], o[0])


def test_gpu_turbulence_3d_48_cube_bit_identical():
    n = (48, 48, 48)
    Vc, Vs = ic.turbulence_3d(48, seed=11)
    state = extract(3, n, 2, Vc, Vs)
    kw = dict(order="plm", solver="hlld", emf="uct_contact", cfl=0.6, first_dt=1e-4)
    g = _gpu(3, n, state, cycles=12, **kw)
    o = _oracle(3, n, state, cycles=12, **kw)
    assert g[1] == o[1]
    _assert_same(g[0], o[0])


def test_gpu_linear_fast_wave_known_answer():
    """LinearWaveTest fast mode (Roe, PLM, CFL 0.9, 64x32x32 on 3x1.5x1.5):
    mean-removed L1 error after one period, x1e6, below 3e-2
    (test/MHD/LinearWaveTest/python/testidefix.py:23-64); and identical to
    the oracle."""
    n = (64, 32, 32)
    Vc, Vs = ic.linear_wave_3d(mode=1, nx=64, ny=32, nz=32)
    state = extract(3, n, 2, Vc, Vs)
    kw = dict(xbeg=(0, 0, 0), xend=(3.0, 1.5, 1.5), order="plm", solver="roe", emf="uct_contact",
              cfl=0.9, first_dt=1e-4)
    (vc1, vs1), tm = _gpu(3, n, state, tstop=0.5, **kw)
    assert tm[0] == 0.5
    vc0, vs0 = state
    pairs = [(vc0[q], vc1[q]) for q in range(5)]
    for c in range(3):
        s = [slice(None)] * 3
        s[2 - c] = slice(0, n[c])
        pairs.append((vs0[c][tuple(s)], vs1[c][tuple(s)]))
    err = np.sqrt(np.mean([np.mean(np.abs((a - a.mean()) - (b - b.mean()))) ** 2 for a, b in pairs]))
    assert err * 1e6 < 3e-2, err * 1e6
    o = _oracle(3, n, state, tstop=0.5, **kw)
    _assert_same((vc1, vs1), o[0])


def test_gpu_building_blocks_match_oracle():
    """SetBoundaries, ConvertPrimToCons, EvolveStage, ComputeTimestep,
    ConvertConsToPrim, CheckDivB called one by one"""
    from oracle.pyofx import Oracle

    n = (16, 12, 10)
    Vc, Vs = ic.turbulence_3d(16, seed=2, kmax=4)
    vc, vs = extract(3, (16, 16, 16), 2, Vc, Vs)
    state = (vc[:, :10, :12, :], [vs[0][:10, :12, :], vs[1][:10, :13, :], vs[2][:11, :12, :]])
    Vc, Vs = embed(3, n, 2, *state)
    blk = ig.GpuBlock(3, n)
    o = Oracle(3, n)
    blk.upload(Vc, Vs)
    o.set_prim(Vc, Vs)
    blk.set_boundaries()
    o.lib.ofx_set_boundaries(o.h)
    gVc, gVs = blk.download()
    oVc, oVs = o.get_prim()
    assert np.array_equal(gVc, oVc)
    blk.prim_to_cons()
    o.lib.ofx_prim_to_cons(o.h)
    blk.reset_stage()
    o.lib.ofx_reset_stage(o.h)
    dt = 2e-4
    blk.evolve_stage(0.0, dt)
    o.lib.ofx_evolve_stage(o.h, 0.0, dt)
    assert blk.compute_timestep() == o.lib.ofx_compute_timestep(o.h)
    g = 2
    act = (slice(None), slice(g, g + n[2]), slice(g, g + n[1]), slice(g, g + n[0]))
    assert np.array_equal(blk.download_cons()[act], o.get_cons()[act])
    blk.cons_to_prim()
    o.lib.ofx_cons_to_prim(o.h)
    gVc, gVs = blk.download()
    oVc, oVs = o.get_prim()
    _assert_same(extract(3, n, 2, gVc, gVs), extract(3, n, 2, oVc, oVs))
    assert blk.check_divb() == o.check_divb()
    assert blk.check_nan() == 0
    blk.close()


def test_gpu_reference_errors():
    """first_dt too large is fatal (IDEFIX_ERROR, timeIntegrator.cpp:393-398);
    a NaN in the state raises RuntimeError after the cycle (:306-310); a
    divergent face field fails the divB check (:165-176)."""
    n = (32, 32)
    Vc, Vs = ic.orszag_tang_2d(32)
    blk = ig.GpuBlock(2, n, cfl=0.6, first_dt=0.5)
    blk.upload(Vc, Vs)
    with pytest.raises(ig.IdefixError):
        blk.cycle()
    blk.close()
    bad = Vc.copy()
    bad[3, 0, 10, 10] = np.nan
    blk = ig.GpuBlock(2, n, cfl=0.6, first_dt=1e-4, check_nan_period=1)
    blk.upload(bad, Vs)
    with pytest.raises(RuntimeError, match="Nan"):
        blk.cycle()
    blk.close()
    rng = np.random.default_rng(0)
    noisy = Vs + 0.1 * rng.standard_normal(Vs.shape)
    blk = ig.GpuBlock(2, n, cfl=0.6, first_dt=1e-4, log_period=1)
    blk.upload(Vc, noisy)
    with pytest.raises(RuntimeError, match="divB"):
        blk.cycle()
    blk.close()


def test_gpu_turbulence_256_cube_properties():
    """the 256^3 throughput configuration: div B stays at round-off, the
    periodic box conserves mass, momentum and energy to round-off, and two
    runs are bit-identical"""
    n = (256, 256, 256)
    Vc, Vs = ic.turbulence_3d(256, seed=1)
    kw = dict(order="plm", solver="hlld", emf="uct_contact", cfl=0.6, first_dt=1e-4)
    res = []
    for _ in range(2):
        blk = ig.GpuBlock(3, n, **kw)
        blk.upload(Vc, Vs)
        blk.set_boundaries()
        blk.prim_to_cons()
        U0 = blk.download_cons()
        blk.run(max_cycles=5)
        U1 = blk.download_cons()
        divb = blk.check_divb()
        res.append((blk.download(), U0, U1, divb))
        blk.close()
    (a, U0, U1, divb), (b, _, _, _) = res
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert divb < 1e-11, divb
    g = 2
    act = (slice(g, g + 256),) * 3
    for q in (0, 1, 2, 3, 4):  # RHO, MX1..3, ENG
        s0 = np.sum(U0[q][act])
        s1 = np.sum(U1[q][act])
        scale = np.sum(np.abs(U0[q][act]))
        assert abs(s1 - s0) <= 1e-12 * scale, (q, s0, s1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotuned_segments_keep_results(precision):
    """the march segment length changes the launch shape only"""
    n = (24, 20, 16)
    Vc, Vs = ic.turbulence_3d(24, seed=9, kmax=4)
    Vc = np.ascontiguousarray(Vc[:, : n[2] + 4, : n[1] + 4, :])
    Vs = np.ascontiguousarray(Vs[:, : n[2] + 5, : n[1] + 5, :])
    out = []
    for tune in (False, True):
        blk = ig.GpuBlock(3, n, cfl=0.6, first_dt=1e-4, precision=precision)
        blk.upload(Vc, Vs)
        if tune:
            blk.autotune(2)
            assert all(s in (4, 8, 16, 32, 64, 128, 256) for s in blk.segments())
        blk.run(max_cycles=3)
        out.append((blk.download(), blk.get_time()))
        blk.close()
    (a, ta), (b, tb) = out
    assert ta == tb
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


SHOCK_GPU = [(dims, order, smoothing) for dims in (2, 3) for order in ("plm", "limo3", "ppm")
             for smoothing in (0.0, 0.5)]


@pytest.mark.parametrize("dims,order,smoothing", SHOCK_GPU)
def test_gpu_shock_flattening_matches_oracle(dims, order, smoothing):
    """[Hydro] shockFlattening: flags and minmod slopes bit-identical to the
    oracle (itself pinned to the reference's FindShock)"""
    from oracle.pyofx import Oracle

    if dims == 2:
        n = (48, 48)
        Vc, Vs = ic.orszag_tang_2d(48, nghost=2)
    else:
        n = (12, 12, 12)
        Vc, Vs = ic.turbulence_3d(12, seed=7, nghost=2, kmax=4)
    state = extract(dims, n, 2, Vc, Vs)
    cfl = 0.6 if dims == 2 else 0.4
    cycles = 30 if dims == 2 else 8
    o = Oracle(dims, n, order=order, cfl=cfl, first_dt=1e-4, shock_flattening=smoothing)
    o.set_prim(*embed(dims, n, o.ng, *state))
    o.run(max_cycles=cycles)
    ref = extract(dims, n, o.ng, *o.get_prim())
    blk = ig.GpuBlock(dims, n, order=order, cfl=cfl, first_dt=1e-4, shock_flattening=smoothing)
    blk.upload(*embed(dims, n, blk.ng, *state))
    blk.run(max_cycles=cycles)
    out = extract(dims, n, blk.ng, *blk.download())
    assert np.array_equal(out[0], ref[0])
    for c in range(dims):
        assert np.array_equal(out[1][c], ref[1][c])
    assert blk.get_time()[:2] == o.get_time()[:2]


def test_gpu_field_loop_to_t2_bit_identical():
    """test/MHD/FieldLoop (v = (1, 0, 1) across the periodic [-1,1]^3 box,
    HLLD, CFL 0.2) at 64 x 2 x 64 to its t_stop = 2, one crossing:
    bit-identical to the oracle; the y rows stay identical, the discrete
    div B of the faces stays at round-off, and the loop comes back where it
    started (correlation of the field energy density with the initial one
    above 0.9, magnetic energy 40-100 % of the initial)."""
    n = (64, 2, 64)
    state = extract(3, n, 2, *ic.field_loop_3d(*n))
    xb, xe = ic.FIELD_LOOP_DOMAIN
    kw = dict(cfl=0.2, first_dt=1e-4, xbeg=xb, xend=xe)
    gpu, tm = _gpu(3, n, state, tstop=2.0, **kw)
    ref, tref = _oracle(3, n, state, tstop=2.0, **kw)
    _assert_same(gpu, ref)
    assert tm == tref
    vc, vs = gpu
    assert np.array_equal(vc[:, :, 0, :], vc[:, :, 1, :])
    dx, dy, dz = 2.0 / 64, 1.0, 2.0 / 64
    div = ((vs[0][:, :, 1:] - vs[0][:, :, :-1]) / dx + (vs[1][:, 1:, :] - vs[1][:, :-1, :]) / dy
           + (vs[2][1:] - vs[2][:-1]) / dz)
    bmax = max(np.abs(v).max() for v in vs)
    assert np.abs(div).max() * dx / bmax < 1e-12
    b0 = [0.5 * (state[1][0][:, :, 1:] + state[1][0][:, :, :-1]), 0.5 * (state[1][2][1:] + state[1][2][:-1])]
    e0 = b0[0] ** 2 + b0[1] ** 2
    e1 = vc[5] ** 2 + vc[6] ** 2 + vc[7] ** 2
    assert np.corrcoef(e0.ravel(), e1.ravel())[0, 1] > 0.9
    assert 0.4 < e1.sum() / e0.sum() < 1.0
