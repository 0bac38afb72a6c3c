"""The one device-side wait of the library - the mbarrier wait of the
bulk-copy staged x sweep - is bounded: on a barrier that never completes it
gives up after its limit of try_wait attempts, records a CUDA-side failure in
the control block (status IDFX_ERR_CUDA, cycle stopped) and returns, and the
context stays usable.  The failure is made on the device without a fault: a
barrier that nothing arrives on."""
import ctypes
import time

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    build.build_oracle()
    return ig.load_library()


def _probe(lib, mode, limit):
    gave_up, status, done = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_int(-1)
    t0 = time.perf_counter()
    rc = lib.idfx_check_wait_timeout(mode, limit, ctypes.byref(gave_up), ctypes.byref(status),
                                     ctypes.byref(done))
    return rc, gave_up.value, status.value, done.value, time.perf_counter() - t0


@pytest.mark.parametrize("limit", [1, 4096, 1 << 16])
def test_wait_gives_up_and_reports(built, limit):
    rc, gave_up, status, done, el = _probe(built, 0, limit)
    assert rc == ig.OK
    assert gave_up == 1
    assert status == ig.ERR_CUDA and done == 1
    assert el < 30.0


def test_completed_wait_returns_at_once(built):
    rc, gave_up, status, done, _ = _probe(built, 1, 4096)
    assert rc == ig.OK
    assert (gave_up, status, done) == (0, 0, 0)


def test_context_usable_after_timeout(built):
    """a bounded wait that ran out leaves the device usable: a run after it
    matches the oracle bit for bit"""
    from oracle.pyofx import Oracle

    assert _probe(built, 0, 4096)[1] == 1
    n = (32, 32)
    Vc, Vs = ic.orszag_tang_2d(32)
    blk = ig.GpuBlock(2, n, cfl=0.6, first_dt=1e-4)
    blk.upload(Vc, Vs)
    blk.run(max_cycles=3)
    gVc, _ = blk.download()
    blk.close()
    o = Oracle(2, n, cfl=0.6, first_dt=1e-4)
    o.set_prim(Vc, Vs)
    assert o.run(max_cycles=3) == 0
    oVc, _ = o.get_prim()
    a = (slice(None), slice(None), slice(2, 34), slice(2, 34))
    assert np.array_equal(gVc[a], oVc[a])
