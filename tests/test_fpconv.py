"""Integer-pipe forms of floating-point operations must equal the IEEE-754
operations bit for bit: the FP32 <-> FP64 conversions of the mixed path
(csrc/fpconv.cuh; host: a stride of every binary32 pattern and random
binary64 values; GPU: against CUDA's) and the exact FP64 sign tests,
sign flips, halves and upwind products of the FP64 path (csrc/exact_ops.cuh;
host, over random patterns, zeros, subnormals, infinities, NaNs)."""
import os
import shutil
import subprocess

import pytest

import idefix_gb300 as ig

HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_host_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "fpconv_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe), os.path.join(HERE, "native", "fpconv_check.cpp")],
                   check=True)
    r = subprocess.run([str(exe), "13"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert r.stdout.strip().startswith("0 mismatches")


@pytest.mark.gpu
def test_conversions_match_cuda():
    import ctypes

    from idefix_gb300 import build

    build.build_library()
    lib = ig.load_library()
    bad = ctypes.c_longlong(-1)
    assert lib.idfx_check_conversions(1 << 26, 77, ctypes.byref(bad)) == ig.OK
    assert bad.value == 0


def test_exact_ops_match_host_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "exact_ops_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(HERE, "native", "exact_ops_check.cpp")], check=True)
    r = subprocess.run([str(exe), "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert r.stdout.strip().startswith("0 mismatches")
