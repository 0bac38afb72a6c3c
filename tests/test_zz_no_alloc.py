"""The allocation-free stage entry point, idfx_evolve_stage_noalloc.

It serves callers that may not allocate GPU memory while they step (their
state lives in their own memory pools, or they run where cudaMalloc is not
allowed): they hand in their own device arrays and the stage's work arrays
come from a fixed static device array inside the library.  This file checks,
through the C ABI, that two calls in a row give exactly the results of the
allocating entry point (reset_stage + evolve_stage on a handle) - exact
equality, the tolerance of every FP64 parity test here - and that a block
larger than the static scratch is refused with a clear error.  It is
collected last so that a failure here leaves every other test already run,
and it needs nothing from the other tests.
"""
import ctypes

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from idefix_gb300 import build

    build.build_library()
    return ig.load_library()


def _config(lib, dims, n, **kw):
    cfg = ig.Config()
    lib.idfx_gpu_default_config(ctypes.byref(cfg), dims, n[0], n[1], n[2] if dims == 3 else 1)
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def _cut(Vc, Vs, n, g):
    """the leading n[1] x n[2] cells (and faces) of a cubic ghosted state"""
    Vc = np.ascontiguousarray(Vc[:, : n[2] + 2 * g, : n[1] + 2 * g, :])
    Vs = np.ascontiguousarray(Vs[:, : n[2] + 2 * g + 1, : n[1] + 2 * g + 1, :])
    return Vc, Vs


# (dims, n, order, solver, emf): the schemes of both ghost widths (PPM takes
# three), every Riemann solver, the five EMF averages, and a 48^3 block with
# uct_hll whose work arrays fill 94 % of the static scratch (the largest
# offsets into it)
CASES = [
    (3, (20, 18, 16), "plm", "hlld", "uct_contact"),
    (2, (48, 48, 1), "plm", "hlld", "uct_hll"),
    (3, (16, 14, 12), "ppm", "hlld", "uct_hlld"),
    (3, (16, 14, 12), "limo3", "roe", "uct_contact"),
    (2, (40, 36, 1), "ppm", "roe", "uct_hlld"),
    (2, (40, 36, 1), "plm", "tvdlf", "uct0"),
    (3, (12, 10, 8), "order1", "hll", "arithmetic"),
    (3, (48, 48, 48), "plm", "hlld", "uct_hll"),
]


@pytest.mark.parametrize("dims,n,order,solver,emf", CASES)
def test_noalloc_stage_matches_allocating_entry_point_twice(lib, dims, n, order, solver, emf):
    torch = pytest.importorskip("torch")
    g = 3 if order == "ppm" else 2
    if dims == 3:
        Vc, Vs = _cut(*ic.turbulence_3d(n[0], seed=4, nghost=g, kmax=4), n, g)
    else:
        Vc, Vs = ic.orszag_tang_2d(n[0], nghost=g)
        Vc = np.ascontiguousarray(Vc[:, :, : n[1] + 2 * g, :])
        Vs = np.ascontiguousarray(Vs[:, :, : n[1] + 2 * g + 1, :])
    blk = ig.GpuBlock(dims, n[:dims], order=order, emf=emf, solver=solver)
    blk.upload(Vc, Vs)
    blk.set_boundaries()
    blk.prim_to_cons()
    vc_in, vs0 = blk.download()
    uc0 = blk.download_cons()
    dt = 3e-4
    expect = []
    for call in range(2):
        blk.reset_stage()
        blk.evolve_stage(call * dt, dt)
        expect.append((blk.download_cons(), blk.download()[1]))
    blk.close()

    cfg = _config(lib, dims, n, order=ig.ORDER[order], emf=ig.EMF[emf], solver=ig.SOLVER[solver])
    dVc = torch.from_numpy(vc_in).cuda()
    dUc = torch.from_numpy(uc0).cuda()
    dVs = torch.from_numpy(vs0).cuda()
    err = ctypes.create_string_buffer(256)
    for call in range(2):
        torch.cuda.synchronize()
        rc = lib.idfx_evolve_stage_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dVc.data_ptr()),
                                           ctypes.c_void_p(dUc.data_ptr()),
                                           ctypes.c_void_p(dVs.data_ptr()), call * dt, dt, None,
                                           err, 256)
        assert rc == ig.OK, err.value
        torch.cuda.synchronize()
        uc, vs = dUc.cpu().numpy(), dVs.cpu().numpy()
        assert np.array_equal(uc, expect[call][0]), call
        assert np.array_equal(vs, expect[call][1]), call
    # the primitive input is left untouched
    assert np.array_equal(dVc.cpu().numpy(), vc_in)


def test_noalloc_scratch_need_of_the_largest_case():
    """the 48^3 uct_hll case sits just below the static scratch size"""
    n, ng = 48, 2
    nc = (n + 2 * ng) ** 3
    need = 28 * nc  # InvDt, 6 face EMFs, 3 flags, 3 cell EMFs, 3 corners, 12 weights
    assert 0.9 * 4 * 1024 * 1024 < need < 4 * 1024 * 1024


def test_noalloc_refuses_blocks_beyond_the_static_scratch(lib):
    n = (96, 96, 96)
    cfg = _config(lib, 3, n)
    err = ctypes.create_string_buffer(256)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.idfx_evolve_stage_noalloc(ctypes.byref(cfg), dummy, dummy, dummy, 0.0, 1e-3, None, err, 256)
    assert rc == ig.ERR_CONFIG
    assert b"scratch" in err.value
