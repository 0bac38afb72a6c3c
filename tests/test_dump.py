"""Restart dumps in the reference's format (output/dump.cpp, reader
pytools/dump_io.py): round trips, files with the reference writer's padding
and extra fields, the reference's own Python reader on our files (where
the reference tree is present), grid-mismatch errors, and - on the GPU - a
restart that continues bit for bit like the uninterrupted run."""
import os
import struct
import sys

import numpy as np
import pytest

import idefix_gb300 as ig
from idefix_gb300 import ic
from mhd_state import extract

from conftest import REFERENCE_SRC

REF_PYTOOLS = os.path.join(os.path.dirname(REFERENCE_SRC), "pytools")


@pytest.fixture(scope="module", autouse=True)
def lib():
    from idefix_gb300 import build

    build.build_library()
    return ig.load_library()


def _state(dims, n, seed=3):
    rng = np.random.default_rng(seed)
    cfg = ig.make_config(dims, n, xbeg=(-0.5, 0.0, 1.0), xend=(0.5, 2.0, 1.5))
    sc, ss = ig._shapes(cfg)
    return cfg, rng.standard_normal(sc), rng.standard_normal(ss)


def _active(cfg, Vc, Vs):
    n = [cfg.n[d] for d in range(cfg.dims)]
    return extract(cfg.dims, n, 2, Vc, Vs)


@pytest.mark.parametrize("dims,n", [(2, (12, 9)), (3, (6, 5, 4))])
def test_round_trip(tmp_path, dims, n):
    cfg, Vc, Vs = _state(dims, n)
    p = str(tmp_path / "dump.0000.dmp")
    ig.write_dump(p, cfg, Vc, Vs, 0.125, 3e-3, 7)
    Vc2, Vs2, t, dt = ig.read_dump(p, cfg)
    a, b = _active(cfg, Vc, Vs), _active(cfg, Vc2, Vs2)
    # the hydro variables and the face field travel; the cell-centred field
    # is rebuilt from the faces (not stored, as in the reference)
    assert np.array_equal(a[0][: dims + 2], b[0][: dims + 2])
    assert np.all(b[0][dims + 2:] == 0)
    for c in range(dims):
        assert np.array_equal(a[1][c], b[1][c])
    assert (t, dt) == (0.125, 3e-3)


@pytest.mark.skipif(not os.path.isdir(REF_PYTOOLS), reason="reference tree not present")
@pytest.mark.parametrize("dims,n", [(2, (12, 9)), (3, (6, 5, 4))])
def test_reference_reader_reads_our_dump(tmp_path, dims, n):
    sys.path.insert(0, REF_PYTOOLS)
    try:
        import dump_io
    finally:
        sys.path.remove(REF_PYTOOLS)
    cfg, Vc, Vs = _state(dims, n)
    p = str(tmp_path / "dump.0001.dmp")
    ig.write_dump(p, cfg, Vc, Vs, 0.5, 1e-4, 3)
    ds = dump_io.DumpDataset(p)
    vc, vs = _active(cfg, Vc, Vs)
    names = ["RHO", "VX1", "VX2"] + (["VX3"] if dims == 3 else []) + ["PRS"]
    for v, nm in enumerate(names):
        assert np.array_equal(ds.data["Vc-" + nm], vc[v].T)
    for c in range(dims):
        assert np.array_equal(ds.data[f"Vs-BX{c + 1}s"], vs[c].T)
    assert ds.data["time"][0] == 0.5 and ds.data["dt"][0] == 1e-4 and ds.data["vtkFileNumber"][0] == 3
    dx = (0.5 - -0.5) / n[0]
    assert np.array_equal(ds.x1, -0.5 + (np.arange(n[0]) + 0.5) * dx)
    # the header Dump::Write prints (dump.cpp:880-883)
    assert ds.header == "Idefix 2.2.02 Dump Data little endian"


def _raw_field(name, typ, dims, data, pad=b"\xab"):
    nm = name.encode() + b"\x00"
    nm = nm + pad * (16 - len(nm))
    fmt = {0: "d", 2: "i"}[typ]
    return nm + struct.pack("<ii", typ, len(dims)) + struct.pack(f"<{len(dims)}i", *dims) + \
        struct.pack(f"<{len(data)}{fmt}", *data)


def test_reads_reference_style_file_with_padding_and_extra_fields(tmp_path):
    # as Dump::Write lays it out: uninitialised bytes after the NULs of the
    # header and names, fields of other modules (here a tracer, a planet and
    # a central mass) among the fluid's, in std::map order
    dims, n = 2, (4, 3)
    cfg = ig.make_config(dims, n)
    rng = np.random.default_rng(0)
    head = b"Idefix 2.2.02 Dump Data little endian\x00"
    blob = head + b"\xcd" * (128 - len(head))
    for d in range(3):
        m = n[d] if d < dims else 1
        for nm in (f"x{d + 1}", f"xl{d + 1}", f"xr{d + 1}"):
            blob += _raw_field(nm, 0, [m], list(rng.standard_normal(m)))
    cells = {nm: rng.standard_normal(n[0] * n[1]) for nm in ("PRS", "RHO", "TR0", "VX1", "VX2")}
    faces = {1: rng.standard_normal((n[0] + 1) * n[1]), 2: rng.standard_normal(n[0] * (n[1] + 1))}
    for nm in ("PRS", "RHO", "TR0", "VX1", "VX2"):
        blob += _raw_field("Vc-" + nm, 0, [n[0], n[1], 1], list(cells[nm]))
    blob += _raw_field("Vs-BX1s", 0, [n[0] + 1, n[1], 1], list(faces[1]))
    blob += _raw_field("Vs-BX2s", 0, [n[0], n[1] + 1, 1], list(faces[2]))
    blob += _raw_field("centralMass", 0, [1], [1.0])
    blob += _raw_field("dt", 0, [1], [2.5e-3])
    blob += _raw_field("time", 0, [1], [0.75])
    blob += _raw_field("vtkFileNumber", 2, [1], [12])
    blob += _raw_field("x_p0", 0, [1], [0.1])
    blob += _raw_field("eof", 0, [1], [0.0])
    p = tmp_path / "dump.0002.dmp"
    p.write_bytes(blob)
    Vc, Vs, t, dt = ig.read_dump(str(p), cfg)
    assert (t, dt) == (0.75, 2.5e-3)
    vc, vs = _active(cfg, Vc, Vs)
    for v, nm in enumerate(("RHO", "VX1", "VX2", "PRS")):
        assert np.array_equal(vc[v][0], cells[nm].reshape(n[1], n[0]))
    assert np.array_equal(vs[0][0], faces[1].reshape(n[1], n[0] + 1))
    assert np.array_equal(vs[1][0], faces[2].reshape(n[1] + 1, n[0]))


def test_grid_mismatch_is_refused(tmp_path):
    cfg, Vc, Vs = _state(2, (12, 9))
    p = str(tmp_path / "dump.0003.dmp")
    ig.write_dump(p, cfg, Vc, Vs, 0.0, 1e-3)
    other = ig.make_config(2, (12, 10))
    with pytest.raises(ig.IdefixError):
        ig.read_dump(p, other)


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [2, 3])
def test_restart_continues_bit_for_bit(tmp_path, dims):
    if dims == 2:
        n = (64, 64)
        Vc, Vs = ic.orszag_tang_2d(64)
    else:
        n = (24, 24, 24)
        Vc, Vs = ic.turbulence_3d(24, seed=5, kmax=4)
    kw = dict(cfl=0.6, first_dt=1e-4, log_period=3, check_nan_period=2)
    whole = ig.GpuBlock(dims, n, **kw)
    whole.upload(Vc, Vs)
    whole.run(max_cycles=10)
    ref = whole.download()
    tref = whole.get_time()
    first = ig.GpuBlock(dims, n, **kw)
    first.upload(Vc, Vs)
    first.run(max_cycles=6)
    p = str(tmp_path / "dump.0000.dmp")
    first.write_dump(p)
    second = ig.GpuBlock(dims, n, **kw)
    second.read_dump(p, ncycles=6)
    second.run(max_cycles=4)
    out = second.download()
    t2 = second.get_time()
    assert t2 == tref
    a, b = extract(dims, n, 2, *ref), extract(dims, n, 2, *out)
    assert np.array_equal(a[0], b[0])
    for c in range(dims):
        assert np.array_equal(a[1][c], b[1][c])
