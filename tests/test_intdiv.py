"""The FP64 division computed on the integer pipe (csrc/intdiv.cuh), used by
the whole-array cons <-> prim passes, must equal IEEE-754 round-to-nearest
division bit for bit: checked on the host against the host's division (C++
build of the same header) and on the GPU against CUDA's."""
import os
import shutil
import subprocess

import pytest

import idefix_gb300 as ig

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_division_matches_host_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "intdiv_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe), os.path.join(HERE, "native", "intdiv_check.cpp")],
                   check=True)
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert r.stdout.strip().startswith("0 mismatches")


@pytest.mark.gpu
def test_integer_division_matches_cuda():
    import ctypes

    from idefix_gb300 import build

    build.build_library()
    lib = ig.load_library()
    bad = ctypes.c_longlong(-1)
    assert lib.idfx_check_division(1 << 26, 2024, ctypes.byref(bad)) == ig.OK
    assert bad.value == 0
