"""Builds libblqh_gpu.so in-tree from blqh_gb300/csrc/*.cu for sm_103a.

One translation unit per nvcc process, compiled in parallel, then linked with
nvcc -shared. Host code uses portable flags only (the library is also built on
aarch64 hosts). Usage: python -m blqh_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libblqh_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libblqh_gpu.so")
    return p


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                     glob.glob(os.path.join(HERE, "..", "include", "*.h")))
    objs, jobs = [], []
    for s in sources:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    build_dropin(force)
    return LIB


DROPIN = os.path.join(HERE, "dropin")
DROPIN_LIB = os.path.join(HERE, "libblqh_dropin.so")
DROPIN_SPIN = os.path.join(HERE, "dropin_spin")
DROPIN_SPIN_LIB = os.path.join(HERE, "libblqh_dropin_spin.so")
DROPIN_MONO = os.path.join(HERE, "dropin_mono")
DROPIN_MONO_LIB = os.path.join(HERE, "libblqh_dropin_mono.so")


def _build_cxx_lib(out: str, srcs: list, inc: str, force: bool) -> str:
    deps = srcs + [LIB] + glob.glob(os.path.join(inc, "*.h")) + glob.glob(os.path.join(DROPIN, "*.h")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    if force or _stale(out, deps):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++11", "-fPIC", "-shared", "-I", inc, "-o", out,
               *srcs, "-L", HERE, "-lblqh_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("drop-in build failed: " + os.path.basename(out))
    return out


def build_dropin(force: bool = False) -> str:
    """libblqh_dropin.so / libblqh_dropin_spin.so / libblqh_dropin_mono.so: the reference's basis /
    lhamil / hamil classes (spinless, spinful and monolayer models) over the C ABI."""
    mat = os.path.join(DROPIN, "matrix.cpp")
    _build_cxx_lib(DROPIN_SPIN_LIB, [os.path.join(DROPIN_SPIN, "dropin_spin.cpp"), mat], DROPIN_SPIN, force)
    _build_cxx_lib(DROPIN_MONO_LIB, [os.path.join(DROPIN_MONO, "dropin_mono.cpp"), mat], DROPIN_MONO, force)
    return _build_cxx_lib(DROPIN_LIB, [os.path.join(DROPIN, "dropin.cpp"), mat], DROPIN, force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
