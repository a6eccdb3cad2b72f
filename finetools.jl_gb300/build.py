"""Builds libfegpu.so (the CUDA library behind include/fegpu.h) in-tree.

Each translation unit is compiled in parallel with nvcc for sm_103a only; the
shared object lands next to this file, where the ctypes binding loads it.
No cmake, no torch extension machinery: plain nvcc + g++.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfegpu.so")
LIB_CHECKED = os.path.join(HERE, "libfegpu_checked.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                     "-Xptxas", "-warn-spills" if os.environ.get("FEGPU_PTXAS_VERBOSE") else "-O3",
                     "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INCLUDE, "-I", CSRC,
             "-I", "/usr/local/cuda/include"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfegpu")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(jobs: int | None = None, verbose: bool = False, force: bool = False,
          device_checks: bool = False) -> str:
    """Builds libfegpu.so; device_checks=True builds libfegpu_checked.so, whose
    kernels check the indices they read and write (FEGPU_DEVICE_CHECKS)."""
    build_dir = BUILD + ("_checked" if device_checks else "")
    lib = LIB_CHECKED if device_checks else LIB
    defs = ["-DFEGPU_DEVICE_CHECKS"] if device_checks else []
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    cmds, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            extra = ["-Xptxas", "-v"] if verbose else []
            cmds.append([nvcc] + NVCC_FLAGS + defs + extra + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmds.append(["g++"] + CXX_FLAGS + defs + ["-c", src, "-o", obj])
    if cmds:
        jobs = jobs or min(len(cmds), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(jobs) as ex:
            for log in ex.map(_compile, cmds):
                if verbose and log:
                    sys.stderr.write(log)
    if cmds or not os.path.exists(lib) or any(
            os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        tmp = lib + ".tmp"
        _compile([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv,
                device_checks="--device-checks" in sys.argv))
