"""Build script for the Base_GB300 libraries.

Produces, in-tree:
  rajaperf_gb300/lib/libb200.so            sm_103a kernel library (C ABI, include/b200.h)
  rajaperf_gb300/lib/librajaperf_gb300.so  host layer (C ABI, include/rajaperf_gb300.h)
  rajaperf_gb300/bin/rajaperf-gb300        suite driver for the Base_GB300 variant

Every CUDA translation unit is compiled with
  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo
in parallel; objects are rebuilt only when a source or header is newer.
Run: python -m rajaperf_gb300.build  (or __graft_entry__.build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(ROOT, "_build", "obj")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _cuda_libdir(home: str) -> str:
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(home, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(home, "lib64")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {os.path.basename(cmd[-1])}")


def _check_arch_stamp() -> None:
    """Objects and libraries from another host architecture are discarded."""
    import platform
    stamp = os.path.join(ROOT, "_build", "ARCH")
    arch = platform.machine()
    old = open(stamp).read().strip() if os.path.exists(stamp) else None
    if old != arch:
        for d in (OBJ, LIB, BIN):
            shutil.rmtree(d, ignore_errors=True)
        os.makedirs(os.path.dirname(stamp), exist_ok=True)
        with open(stamp, "w") as f:
            f.write(arch + "\n")


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    _check_arch_stamp()
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    libdir = _cuda_libdir(home)
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)

    b200_dir = os.path.join(CSRC, "b200")
    host_dir = os.path.join(CSRC, "host")
    b200_hdrs = glob.glob(os.path.join(b200_dir, "*.cuh")) + [os.path.join(INCLUDE, "b200.h")]
    host_hdrs = (glob.glob(os.path.join(host_dir, "**", "*.hpp"), recursive=True)
                 + glob.glob(os.path.join(INCLUDE, "*.h")))

    jobs_list = []
    b200_objs = []
    for src in sorted(glob.glob(os.path.join(b200_dir, "*.cu"))):
        obj = os.path.join(OBJ, "b200_" + os.path.basename(src) + ".o")
        b200_objs.append(obj)
        if _newer(obj, [src] + b200_hdrs):
            jobs_list.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17",
                              "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", b200_dir,
                              "-c", src, "-o", obj])
    host_objs = []
    for src in sorted(glob.glob(os.path.join(host_dir, "**", "*.cpp"), recursive=True)):
        rel = os.path.relpath(src, host_dir).replace(os.sep, "_")
        obj = os.path.join(OBJ, "host_" + rel + ".o")
        if os.path.basename(src) == "driver.cpp":
            driver_obj = obj
        else:
            host_objs.append(obj)
        if _newer(obj, [src] + host_hdrs):
            jobs_list.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall",
                              "-I", INCLUDE, "-I", host_dir,
                              "-I", os.path.join(home, "include"),
                              "-c", src, "-o", obj])

    workers = jobs or min(32, (os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        futs = [ex.submit(_run, cmd) for cmd in jobs_list]
        for f in futs:
            f.result()

    libb200 = os.path.join(LIB, "libb200.so")
    if _newer(libb200, b200_objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", libb200, *b200_objs,
              f"-Xlinker", f"-rpath={libdir}"])
    libhost = os.path.join(LIB, "librajaperf_gb300.so")
    if _newer(libhost, host_objs + [libb200]):
        _run(["g++", "-shared", "-o", libhost, *host_objs, "-L", LIB, "-lb200",
              "-L", libdir, "-lcudart", f"-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{libdir}"])
    exe = os.path.join(BIN, "rajaperf-gb300")
    if _newer(exe, [driver_obj, libhost]):
        _run(["g++", "-o", exe, driver_obj, "-L", LIB, "-lrajaperf_gb300", "-lb200",
              "-L", libdir, "-lcudart", "-Wl,-rpath,$ORIGIN/../lib",
              f"-Wl,-rpath,{libdir}"])
    if verbose:
        print(f"built {libb200}\n      {libhost}\n      {exe}")
    return {"libb200": libb200, "libhost": libhost, "exe": exe}


if __name__ == "__main__":
    build(verbose=True)
