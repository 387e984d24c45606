"""Tries to compile the suite's own Base_CUDA sources (K-Cuda.cpp of every
covered kernel) for sm_103a with the oracle build's stand-in headers, and
records per kernel whether it builds and, if not, the first error.  A recipe
of the test infrastructure; outputs go to oracle/_ref/cuda_build.json only.

The suite's CUDA variants are written against RAJA's CUDA back end
(RAJA::forall with cuda_exec policies, RAJA::ReduceSum/ReduceMinLoc,
RAJA::kernel, camp resources), and the RAJA submodule is absent from the
checkout, so the stand-ins under shim/ (made for the host-only Base_Seq
build) do not cover them; this probe documents how far each file gets.

    python oracle/ref_build/cuda_probe.py [REF]
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")

KERNELS = ["stream/COPY", "stream/MUL", "stream/ADD", "stream/TRIAD", "stream/DOT",
           "lcals/HYDRO_1D", "lcals/HYDRO_2D", "lcals/EOS", "lcals/FIRST_DIFF",
           "lcals/INT_PREDICT", "lcals/FIRST_MIN", "apps/DEL_DOT_VEC_2D", "apps/VOL3D",
           "apps/ENERGY", "apps/PRESSURE", "polybench/POLYBENCH_JACOBI_2D",
           "polybench/POLYBENCH_HEAT_3D", "polybench/POLYBENCH_FDTD_2D",
           "polybench/POLYBENCH_GEMM", "polybench/POLYBENCH_3MM", "algorithm/SCAN",
           "algorithm/REDUCE_SUM"]


def ref_root(arg: str | None) -> str:
    if arg:
        return arg
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def first_error(text: str) -> str:
    for ln in text.splitlines():
        if "error" in ln:
            # drop the checkout's path prefix so the record names files by
            # their path in the suite's tree
            return ln.split("/src/", 1)[-1].strip()[:240]
    return text.strip().splitlines()[-1][:240] if text.strip() else "unknown"


def probe(ref: str | None = None) -> dict:
    ref = ref_root(ref)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(os.path.join(OUT, "cuda_obj"), exist_ok=True)

    def one(k):
        src = os.path.join(ref, "src", k + "-Cuda.cpp")
        obj = os.path.join(OUT, "cuda_obj", k.replace("/", "_") + ".o")
        r = subprocess.run([nvcc, "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
                            "-std=c++17", "-DRAJA_ENABLE_CUDA", "--expt-extended-lambda",
                            "-I", os.path.join(HERE, "shim"), "-I", os.path.join(ref, "src"),
                            "-c", src, "-o", obj], capture_output=True, text=True)
        return k, {"builds": r.returncode == 0,
                   "first_error": None if r.returncode == 0 else first_error(r.stderr)}

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        res = dict(ex.map(one, KERNELS))
    with open(os.path.join(OUT, "cuda_build.json"), "w") as f:
        json.dump(res, f, indent=1)
    return res


if __name__ == "__main__":
    out = probe(sys.argv[1] if len(sys.argv) > 1 else None)
    for k, v in out.items():
        print(f"{k}: {'builds' if v['builds'] else 'does not build: ' + v['first_error']}")
