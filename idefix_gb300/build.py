"""Build of the CUDA library libidefix_gb300.so (sm_103a) and of the CPU
oracle used by the tests.

The library is compiled in-tree with nvcc; every translation unit is built
in parallel.  --fmad=false keeps the FP64 arithmetic bit-identical to the
reference (its GPU CI compiles with FMA contraction disabled).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libidefix_gb300.so")

SOURCES = ["sweep_hlld.cu", "sweep_hll.cu", "sweep_roe.cu", "sweep_tvdlf.cu", "persist_hlld.cu", "persist_hll.cu",
           "persist_roe.cu", "persist_tvdlf.cu", "engine.cu", "noalloc.cu", "ensemble.cu", "learned.cu", "peak.cu",
           "dump.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _needs(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose=False, jobs=None, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp"))]
    headers.append(os.path.join(ROOT, "include", "idefix_gb300.h"))
    objs = []
    cmds = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if _needs(o, [s] + headers):
            cmds.append([nvcc(), *ARCH, *NVFLAGS, *extra, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True, errors="replace")
        return cmd, r

    # the longest units (the sweeps and the persistent kernels) are listed first
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if _needs(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


def reference_src():
    """the reference's src/ tree: $IDEFIX_SRC, else a `reference/` checkout
    beside this repository; None where neither exists (the reference harness
    is then not built and the tests that need it skip)"""
    ref_src = os.environ.get("IDEFIX_SRC") or os.path.join(os.path.dirname(ROOT), "reference", "src")
    return ref_src if os.path.isdir(ref_src) else None


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "libofx.so"], check=True)
    ref_src = reference_src()
    if ref_src:
        subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                        f"IDEFIX_SRC={ref_src}"], check=True)


if __name__ == "__main__":
    build_library(verbose="-v" in sys.argv)
    build_oracle()
    print(LIB)
