"""Builds the suite with the Base_GB300 variant registered as INTEGRATION.md
describes -- a recipe of the test infrastructure, run where the suite's
checkout exists.

INTEGRATION.md holds the maintainer's changes as blocks, each after a
marker comment:

    <!-- patch: <file> before|after "<anchor>" -->   insert the next code block
                                                     before / after the first
                                                     line containing <anchor>
    <!-- file: <file> -->                            the next code block is a
                                                     new file

This script copies every source directory of the suite that a block touches
(so that the suite's same-directory includes see the patched headers), applies
the blocks in document order, writes the new files, and compiles the sources
the oracle build compiles (ref_build/Makefile's SRCS) plus the new files and
integration_main.cpp against the patched tree, linking libb200.so and the
CUDA runtime.  Outputs go under oracle/_ref/integration/ only (git-ignored).

    python oracle/ref_build/integration.py [REF]   -> prints the executable path
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref", "integration")

MARK = re.compile(r'<!-- (patch|file): (\S+)(?: (before|after) "((?:[^"\\]|\\.)*)")? -->')


def parse_blocks(md_text: str):
    """[(kind, file, where, anchor, code)] in document order."""
    blocks = []
    lines = md_text.splitlines()
    i = 0
    while i < len(lines):
        m = MARK.fullmatch(lines[i].strip())
        if not m:
            i += 1
            continue
        kind, path, where, anchor = m.groups()
        anchor = anchor.encode().decode("unicode_escape") if anchor is not None else None
        j = i + 1
        while not lines[j].startswith("```"):
            j += 1
        k = j + 1
        while not lines[k].startswith("```"):
            k += 1
        blocks.append((kind, path, where, anchor, "\n".join(lines[j + 1:k]) + "\n"))
        i = k + 1
    return blocks


def apply_patch(text: str, where: str, anchor: str, code: str, what: str) -> str:
    lines = text.splitlines(keepends=True)
    for n, ln in enumerate(lines):
        if anchor in ln:
            at = n if where == "before" else n + 1
            return "".join(lines[:at]) + code + "".join(lines[at:])
    raise RuntimeError(f"{what}: anchor {anchor!r} not found")


def ref_root(arg: str | None) -> str:
    if arg:
        return arg
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build(ref: str | None = None) -> str:
    ref = ref_root(ref)
    if not os.path.isdir(os.path.join(ref, "src", "common")):
        raise FileNotFoundError(f"no suite checkout at {ref}")
    blocks = parse_blocks(open(os.path.join(ROOT, "INTEGRATION.md")).read())
    src = os.path.join(OUT, "src")
    shutil.rmtree(OUT, ignore_errors=True)
    os.makedirs(src)
    dirs = sorted({os.path.dirname(b[1]) for b in blocks})
    for d in dirs:
        shutil.copytree(os.path.join(ref, "src", d), os.path.join(src, d))
    for kind, path, where, anchor, code in blocks:
        target = os.path.join(src, path)
        if kind == "file":
            with open(target, "w") as f:
                f.write(code)
            continue
        text = open(target).read()
        with open(target, "w") as f:
            f.write(apply_patch(text, where, anchor, code, path))

    srcs = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-srcs"],
                          capture_output=True, text=True, check=True).stdout.split()
    srcs += [b[1] for b in blocks if b[0] == "file"]
    home = cuda_home()
    lib = os.path.join(ROOT, "rajaperf_gb300", "lib")
    flags = ["-O1", "-std=c++17", "-w", "-DRAJA_PERFSUITE_ENABLE_GB300", "-I", src,
             "-I", os.path.join(HERE, "shim"), "-I", os.path.join(ref, "src"),
             "-I", os.path.join(ROOT, "include"), "-I", os.path.join(home, "include")]
    objdir = os.path.join(OUT, "obj")
    jobs = []
    for rel in srcs:
        patched = os.path.join(src, rel)
        path = patched if os.path.exists(patched) else os.path.join(ref, "src", rel)
        jobs.append((path, os.path.join(objdir, rel.replace("/", "_") + ".o")))
    for own in ("ref_registry.cpp", "integration_main.cpp"):
        jobs.append((os.path.join(HERE, own), os.path.join(objdir, own + ".o")))
    os.makedirs(objdir)

    def compile_one(job):
        r = subprocess.run(["g++", *flags, "-c", job[0], "-o", job[1]], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {job[0]}:\n{r.stderr[-4000:]}")

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(compile_one, jobs))
    exe = os.path.join(OUT, "rajaperf_ref_gb300")
    cudalib = next(d for d in (os.path.join(home, s) for s in ("lib64", "lib",
                   "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"))
                   if os.path.exists(os.path.join(d, "libcudart.so")))
    r = subprocess.run(["g++", "-o", exe, *[j[1] for j in jobs], "-L", lib, "-lb200",
                        f"-Wl,-rpath,{lib}", "-L", cudalib, "-lcudart", f"-Wl,-rpath,{cudalib}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking:\n{r.stderr[-4000:]}")
    return exe


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
