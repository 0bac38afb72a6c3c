"""C ABI checks that need no GPU: the library exports every entry point that
include/*.h declares, host-only helpers behave, invalid setups are refused
before any CUDA call, and the package refuses to run without its library."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from idefix_gb300 import build

    build.build_library()
    import idefix_gb300

    return idefix_gb300.load_library()


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names |= set(re.findall(r"\b(idfx_\w+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    so = os.path.join(ROOT, "idefix_gb300", "libidefix_gb300.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (idfx_\w+)", out))
    declared = _declared()
    assert len(declared) >= 20
    missing = [d for d in declared if d not in exported]
    assert not missing, missing


def test_python_binding_covers_the_header(lib):
    import idefix_gb300

    assert sorted(idefix_gb300.EXPORTS) == _declared()


def test_default_config_is_the_reference_default(lib):
    import idefix_gb300 as ig

    cfg = ig.Config()
    lib.idfx_gpu_default_config(ctypes.byref(cfg), 3, 64, 32, 16)
    assert cfg.dims == 3 and list(cfg.n) == [64, 32, 16]
    assert cfg.nstages == 2 and cfg.order == 2 and cfg.solver == 0 and cfg.emf == 0
    assert cfg.cfl_max_var == 1.1 and cfg.first_dt == 1e-10 and cfg.maxdivb == 1e-6
    assert cfg.log_period == 100 and cfg.check_nan_period == 100
    assert abs(cfg.gamma - 5.0 / 3.0) < 1e-15


@pytest.mark.parametrize("field,value", [("dims", 4), ("order", 5), ("solver", 7), ("emf", 9),
                                         ("nstages", 4), ("precision", 3)])
def test_invalid_config_is_refused_without_gpu(lib, field, value):
    import idefix_gb300 as ig

    cfg = ig.Config()
    lib.idfx_gpu_default_config(ctypes.byref(cfg), 2, 16, 16, 1)
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    assert lib.idfx_gpu_create(ctypes.byref(cfg), None, ctypes.byref(h)) == ig.ERR_CONFIG
    assert not h.value


def test_uct_hlld_with_hll_is_refused(lib):
    """constrainedTransport.hpp:256-261: HLLD EMF needs HLLD or Roe fluxes"""
    import idefix_gb300 as ig

    cfg = ig.Config()
    lib.idfx_gpu_default_config(ctypes.byref(cfg), 2, 16, 16, 1)
    cfg.emf, cfg.solver = 4, 1
    h = ctypes.c_void_p()
    assert lib.idfx_gpu_create(ctypes.byref(cfg), None, ctypes.byref(h)) == ig.ERR_CONFIG


def test_null_handles_are_refused(lib):
    import idefix_gb300 as ig

    assert lib.idfx_gpu_cycle(None) == ig.ERR_STATE
    assert lib.idfx_gpu_destroy(None) == ig.ERR_STATE


def test_missing_library_fails_loudly(tmp_path):
    import idefix_gb300 as ig

    saved = ig._lib
    try:
        ig._lib = None
        with pytest.raises(ImportError):
            ig.load_library(str(tmp_path / "absent.so"))
    finally:
        ig._lib = saved


def _gxx():
    import shutil

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    return gxx


def test_cpp_facade_forwards_and_throws(tmp_path):
    """include/idefix_gb300.hpp against a scripted fake of the C ABI: the
    reference-named calls reach the right entry points in order, statuses
    become idefix_gb300::Error (a std::runtime_error), handles are freed once."""
    exe = tmp_path / "facade_check"
    subprocess.run([_gxx(), "-O1", "-std=c++17", "-Wall", "-Werror", "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "facade_check.cpp")], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "facade ok" in out.stdout


def test_cpp_facade_links_against_the_library(lib, tmp_path):
    """The facade compiles against include/idefix_gb300.h, links against the
    built library, and a refused setup arrives as Error(IDFX_ERR_CONFIG)
    before any CUDA call."""
    src = tmp_path / "facade_link.cpp"
    src.write_text(
        '#include "idefix_gb300.hpp"\n#include <cstdio>\n'
        "int main() {\n"
        "  idfx_gpu_config cfg;\n"
        "  idfx_gpu_default_config(&cfg, 2, 16, 16, 1);\n"
        "  cfg.nstages = 4;\n"
        "  try { idefix_gb300::DataBlock data(cfg); return 2; }\n"
        "  catch (const idefix_gb300::Error& e) {\n"
        '    std::printf("%d %s\\n", e.status(), e.what());\n'
        "    return e.status() == IDFX_ERR_CONFIG && !e.numerical() ? 0 : 1;\n"
        "  }\n}\n")
    libdir = os.path.join(ROOT, "idefix_gb300")
    exe = tmp_path / "facade_link"
    subprocess.run([_gxx(), "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir,
                    "-lidefix_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "invalid setup" in out.stdout
