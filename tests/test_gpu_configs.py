"""FP64 parity with the oracle at the full sizes of the stated workloads.

* 3-D decaying turbulence, 256^3 periodic, HLLD + PLM (van Leer) + CT
  (uct_contact), RK2, CFL 0.6, 100 cycles - the throughput workload;
* low-beta (beta = 1e-3) 3-D turbulence, 384^3 periodic, HLLD + LimO3 + CT
  (uct_contact), RK2, CFL 0.6, FP64 - the precision workload - over its first
  20 cycles (the oracle takes about two minutes per 1e9 zone-cycles on the
  16 host cores of a GB300 node; the 200-cycle run is compared with the mixed
  path by the workload driver).

The GPU runs through the C ABI; the oracle (OpenMP on every host core) is
pinned bit for bit to the reference's own kernels.  Tolerance: exact
equality of every active cell value, every evolved face value, t, dt and
the cycle count (stricter than an L1-relative bound of 1e-12).
"""
import os

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import extract

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from idefix_gb300 import build

    build.build_library()
    build.build_oracle()
    ig.load_library()


def _host_memory_gb():
    """MemAvailable of the host in GB (Linux), None where unknown"""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return None


def _need_host_memory(gb):
    """the oracle holds ~57 arrays of the ghosted cell count, the test the
    initial, GPU and oracle states: skip rather than drive the host out of
    memory"""
    avail = _host_memory_gb()
    if avail is not None and avail < gb:
        pytest.skip(f"{avail:.0f} GB of host memory available, {gb} GB needed")


def _run_both(n, Vc, Vs, cycles, **kw):
    from oracle.pyofx import Oracle

    blk = ig.GpuBlock(3, (n, n, n), log_period=100, check_nan_period=100, **kw)
    blk.upload(Vc, Vs)
    blk.run(max_cycles=cycles)
    g = blk.ng
    gpu = extract(3, (n, n, n), g, *blk.download())
    gtime = blk.get_time()
    blk.close()
    o = Oracle(3, (n, n, n), threads=os.cpu_count() or 1, log_period=100, check_nan_period=100, **kw)
    o.set_prim(Vc, Vs)
    assert o.run(max_cycles=cycles) == 0
    ref = extract(3, (n, n, n), o.ng, *o.get_prim())
    otime = o.get_time()
    del o
    return gpu, gtime, ref, otime


def _assert_identical(gpu, gtime, ref, otime, cycles):
    assert gtime == otime, (gtime, otime)
    assert gtime[2] == cycles
    for v in range(gpu[0].shape[0]):
        assert np.array_equal(gpu[0][v], ref[0][v]), (v, float(np.nanmax(np.abs(gpu[0][v] - ref[0][v]))))
    for c, (x, y) in enumerate(zip(gpu[1], ref[1])):
        assert np.array_equal(x, y), (c, float(np.nanmax(np.abs(x - y))))


def test_turbulence_256_cube_100_cycles_bit_identical():
    n, cycles = 256, 100
    _need_host_memory(24)
    Vc, Vs = ic.turbulence_3d(n, seed=1)
    kw = dict(order="plm", solver="hlld", emf="uct_contact", nstages=2, cfl=0.6, first_dt=1e-4)
    gpu, gtime, ref, otime = _run_both(n, Vc, Vs, cycles, **kw)
    _assert_identical(gpu, gtime, ref, otime, cycles)


def test_low_beta_384_cube_limo3_bit_identical():
    n, cycles = 384, 20
    _need_host_memory(72)
    Vc, Vs = ic.low_beta_3d(n, seed=0)
    kw = dict(order="limo3", solver="hlld", emf="uct_contact", nstages=2, cfl=0.6, first_dt=1e-4)
    gpu, gtime, ref, otime = _run_both(n, Vc, Vs, cycles, **kw)
    _assert_identical(gpu, gtime, ref, otime, cycles)
