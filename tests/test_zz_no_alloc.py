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


@pytest.mark.parametrize("dims,emf", [(3, 0), (2, 3)])
def test_noalloc_stage_matches_allocating_entry_point_twice(lib, dims, emf):
    torch = pytest.importorskip("torch")
    if dims == 3:
        n = (20, 18, 16)
        Vc, Vs = ic.turbulence_3d(20, seed=4, kmax=4)
        g = 2
        Vc = np.ascontiguousarray(Vc[:, : n[2] + 2 * g, : n[1] + 2 * g, :])
        Vs = np.ascontiguousarray(Vs[:, : n[2] + 2 * g + 1, : n[1] + 2 * g + 1, :])
    else:
        n = (48, 48, 1)
        Vc, Vs = ic.orszag_tang_2d(48)
    solver = 0
    blk = ig.GpuBlock(dims, n[:dims], emf=list(ig.EMF)[emf], solver=list(ig.SOLVER)[solver])
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

    cfg = _config(lib, dims, n, emf=emf, solver=solver)
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


def test_noalloc_refuses_blocks_beyond_the_static_scratch(lib):
    n = (96, 96, 96)
    cfg = _config(lib, 3, n)
    err = ctypes.create_string_buffer(256)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.idfx_evolve_stage_noalloc(ctypes.byref(cfg), dummy, dummy, dummy, 0.0, 1e-3, None, err, 256)
    assert rc == ig.ERR_CONFIG
    assert b"scratch" in err.value
