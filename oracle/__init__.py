"""CPU oracle for the Base_GB300 kernels -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package.  It wraps two things:

* liboracle.so: a plain-C restatement (oracle.c) of the RAJA Performance
  Suite's Base_Seq / Base_OpenMP variants for the hot-path kernels;
* oracle/_ref/rajaperf_ref: the suite's own Base_Seq code compiled from the
  suite's sources (ref_build/Makefile).  It exists only where the suite
  checkout is present; its outputs are committed as tests/golden fixtures,
  which pin the restatement.
"""
from __future__ import annotations

import ctypes
import json
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# one library per host architecture, so a copy made on another machine is
# never loaded by mistake
LIB_PATH = os.path.join(HERE, f"liboracle.{platform.machine()}.so")
REF_EXE = os.path.join(HERE, "_ref", "rajaperf_ref")


class OracleOpts(ctypes.Structure):
    _fields_ = [("size", ctypes.c_double), ("reps", ctypes.c_long),
                ("init_mode", ctypes.c_int), ("threads", ctypes.c_int),
                ("seed", ctypes.c_ulonglong), ("lo", ctypes.c_double),
                ("hi", ctypes.c_double), ("tsteps", ctypes.c_long),
                ("variant", ctypes.c_int), ("skip_checksum", ctypes.c_int),
                ("num_bins", ctypes.c_long), ("bin_algo", ctypes.c_int),
                ("halo_width", ctypes.c_long), ("halo_num_vars", ctypes.c_long)]


class OracleResult(ctypes.Structure):
    _fields_ = [("checksum", ctypes.c_double), ("checksum_residual", ctypes.c_double),
                ("actual_size", ctypes.c_longlong), ("reps", ctypes.c_longlong),
                ("its_per_rep", ctypes.c_longlong), ("kernels_per_rep", ctypes.c_longlong),
                ("bytes_per_rep", ctypes.c_longlong), ("flops_per_rep", ctypes.c_longlong),
                ("time_s", ctypes.c_double), ("status", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compiles liboracle.so (and oracle/_ref when the suite sources exist)."""
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.run(["cc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp",
                        "-shared", "-fPIC", src, "-o", LIB_PATH, "-lm"], check=True)
    return LIB_PATH


def build_ref(ref_root: str | None = None) -> str | None:
    """Builds the suite's own Base_Seq code into oracle/_ref when the suite
    checkout is available; returns the executable path or None."""
    if not ref_root:
        # the recipe resolves the checkout (RAJAPERF_REF, else its default)
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C",
                            os.path.join(HERE, "ref_build"), "print-ref"],
                           capture_output=True, text=True)
        ref_root = r.stdout.strip() if r.returncode == 0 else ""
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src", "common")):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref_build"),
                    f"REF={ref_root}"], check=True)
    return REF_EXE if os.path.exists(REF_EXE) else None


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_run.argtypes = [ctypes.c_char_p, ctypes.POINTER(OracleOpts),
                                 ctypes.POINTER(OracleResult)]
        L.oracle_run.restype = ctypes.c_int
        L.oracle_checksum.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                                      ctypes.POINTER(ctypes.c_double)]
        L.oracle_checksum.restype = ctypes.c_double
        L.oracle_checksum_i64.argtypes = L.oracle_checksum.argtypes
        L.oracle_checksum_i64.restype = ctypes.c_double
        L.oracle_uniform_value.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                           ctypes.c_double, ctypes.c_double]
        L.oracle_uniform_value.restype = ctypes.c_double
        L.oracle_first_min_planted_index.argtypes = [ctypes.c_uint64, ctypes.c_int64]
        L.oracle_first_min_planted_index.restype = ctypes.c_int64
        P, I, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
        for name, args in {
            "oracle_hydro_2d_rep": [P] * 11 + [D, D, I, I],
            "oracle_del_dot_vec_2d_rep": [P] * 6 + [I, I, D, D],
            "oracle_vol3d_rep": [P] * 4 + [D, I, I, I, I],
            "oracle_energy_rep": [P] * 15 + [D, D, D, D, I],
            "oracle_jacobi_2d": [P, P, I, I],
            "oracle_heat_3d": [P, P, I, I],
            "oracle_fdtd_2d": [P, P, P, P, I, I, I],
            "oracle_scan_f64": [P, P, I],
            "oracle_scan_i64": [P, P, I],
            "oracle_gemm": [P, P, P, I, I, I, D, D],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = None
        _lib = L
    return _lib


def run(kernel: str, size: float = -1, reps: int = 1, init: str = "reference",
        seed: int = 4793, lo: float = 0.5, hi: float = 1.5, tsteps: int = -1,
        threads: int = 0, variant: int = 0, skip_checksum: bool = False,
        num_bins: int = 10, bin_algo: str = "RunsRandomSizes", halo_width: int = 1,
        halo_num_vars: int = 3) -> dict:
    """Runs one kernel with the suite's Base_Seq (threads=0) or Base_OpenMP
    semantics and returns its checksum, sizes and rep-loop time."""
    algos = ["Random", "RunsRandomSizes", "RunsEvenSizes", "Single"]
    o = OracleOpts(size=float(size), reps=int(reps),
                   init_mode=1 if init == "uniform" else 0, threads=int(threads),
                   seed=int(seed), lo=float(lo), hi=float(hi), tsteps=int(tsteps),
                   variant=int(variant), skip_checksum=1 if skip_checksum else 0,
                   num_bins=int(num_bins), bin_algo=algos.index(bin_algo),
                   halo_width=int(halo_width), halo_num_vars=int(halo_num_vars))
    r = OracleResult()
    st = lib().oracle_run(kernel.encode(), ctypes.byref(o), ctypes.byref(r))
    if st != 0:
        raise RuntimeError(f"oracle_run({kernel}) failed with status {st}")
    return {"checksum": r.checksum, "checksum_residual": r.checksum_residual,
            "actual_size": r.actual_size, "reps": r.reps, "its_per_rep": r.its_per_rep,
            "kernels_per_rep": r.kernels_per_rep, "bytes_per_rep": r.bytes_per_rep,
            "flops_per_rep": r.flops_per_rep, "time_s": r.time_s}


def checksum(arr, scale: float = 1.0) -> float:
    """The suite's checksum (DataUtils.cpp:600-621) of a numpy array."""
    import numpy as np
    a = np.ascontiguousarray(arr)
    if a.dtype == np.int64:
        return lib().oracle_checksum_i64(a.ctypes.data, a.size, scale, None)
    a = np.ascontiguousarray(a, dtype=np.float64)
    return lib().oracle_checksum(a.ctypes.data, a.size, scale, None)


def run_ref(kernel: str, size: int, reps: int, extra=()) -> dict:
    """Runs the suite's own Base_Seq code (oracle/_ref) for one kernel;
    `extra` are further suite options (e.g. --multi_reduce_num_bins 100)."""
    out = subprocess.run([REF_EXE, kernel, str(size), str(reps), *map(str, extra)],
                         check=True, capture_output=True, text=True).stdout
    line = [ln for ln in out.splitlines() if ln.startswith("{")][-1]
    return json.loads(line)


def call(name: str, *args) -> None:
    """Calls an oracle building block; numpy arrays are passed by address
    (they must be contiguous and of the declared element type)."""
    conv = []
    for a in args:
        if hasattr(a, "ctypes"):
            conv.append(a.ctypes.data)
        else:
            conv.append(a)
    getattr(lib(), name)(*conv)
