"""Build recipe for the native libraries (no cmake; a few translation units in parallel).

  libgbsa.so        CUDA kernels for sm_103a + the C-ABI (include/gbsa.h)
  libgbsa_synth.so  seeded synthetic data generator (host C++)
  oracle/liboracle.so  CPU oracle (test infrastructure; built here so the tests,
                    smoke() and the benchmark's CPU baseline find it)
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

from ._build_paths import CSRC_DIR, GBSA_SO, INCLUDE_DIR, ORACLE_DIR, ORACLE_SO, PKG_DIR, SYNTH_SO

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE_DIR, "-I" + CSRC_DIR,
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout)
        raise RuntimeError(f"build step failed: {cmd[0]} … {cmd[-1]}")
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(force=False, verbose=False):
    cu = sorted(glob.glob(os.path.join(CSRC_DIR, "*.cu")))
    hdrs = sorted(glob.glob(os.path.join(CSRC_DIR, "*.cuh")) + glob.glob(os.path.join(CSRC_DIR, "*.h"))
                  + [os.path.join(INCLUDE_DIR, "gbsa.h")])
    objdir = os.path.join(PKG_DIR, "_build")
    os.makedirs(objdir, exist_ok=True)
    jobs = []

    def obj_of(src):
        return os.path.join(objdir, os.path.basename(src) + ".o")

    with ThreadPoolExecutor(max_workers=max(4, os.cpu_count() or 4)) as ex:
        futs = []
        for src in cu:
            o = obj_of(src)
            if force or not _newer(o, [src] + hdrs):
                futs.append(ex.submit(_run, [NVCC] + ARCH + NVCC_FLAGS + ["-c", src, "-o", o]))
        synth_src = os.path.join(CSRC_DIR, "synth.cpp")
        if force or not _newer(SYNTH_SO, [synth_src]):
            futs.append(ex.submit(_run, [CXX] + CXX_FLAGS + ["-shared", "-pthread", synth_src, "-o", SYNTH_SO]))
        osrc = [os.path.join(ORACLE_DIR, "oracle.cpp")]
        if force or not _newer(ORACLE_SO, osrc + [os.path.join(ORACLE_DIR, "oracle.h"), os.path.join(INCLUDE_DIR, "gbsa.h")]):
            futs.append(ex.submit(_run, [CXX] + CXX_FLAGS + ["-shared", "-pthread"] + osrc + ["-o", ORACLE_SO]))
        for f in futs:
            out = f.result()
            if verbose and out:
                print(out)
    objs = [obj_of(s) for s in cu]
    if force or not _newer(GBSA_SO, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", GBSA_SO] + objs + ["-lcudart"])
    return GBSA_SO


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", GBSA_SO)
