"""ctypes bindings to the Base_GB300 libraries.

* ``b200()``: libb200.so, the sm_103a kernel library (include/b200.h);
* ``host()``: librajaperf_gb300.so, the C++ suite layer (include/rajaperf_gb300.h);
* ``run_suite(args)``: runs the suite for a command line through the host
  layer and returns one dict per kernel and tuning.

The libraries are built in-tree by ``rajaperf_gb300.build.build()``.  Loading
raises ``RuntimeError`` when they are missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_DIR = os.path.join(PKG, "lib")
BIN_DIR = os.path.join(PKG, "bin")
LIBB200 = os.path.join(LIB_DIR, "libb200.so")
LIBHOST = os.path.join(LIB_DIR, "librajaperf_gb300.so")
DRIVER = os.path.join(BIN_DIR, "rajaperf-gb300")
INCLUDE = os.path.join(ROOT, "include")

B200_OK = 0
B200_ERR_INVALID_ARG = 1
B200_ERR_LAUNCH = 2
B200_ERR_TIMEOUT = 3
B200_ERR_WORKSPACE = 4
B200_ERR_UNSUPPORTED = 5


class Tune(ctypes.Structure):
    """b200_tune (include/b200.h)."""
    _fields_ = [("block_size", ctypes.c_int32), ("items", ctypes.c_int32),
                ("vec", ctypes.c_int32), ("grid_blocks", ctypes.c_int32),
                ("tile_x", ctypes.c_int32), ("tile_y", ctypes.c_int32),
                ("tile_z", ctypes.c_int32), ("time_block", ctypes.c_int32),
                ("algo", ctypes.c_int32), ("wait_limit_us", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 2)]


class Caps(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("sm_count", ctypes.c_int32),
                ("cc_major", ctypes.c_int32), ("cc_minor", ctypes.c_int32),
                ("global_mem_bytes", ctypes.c_int64), ("l2_bytes", ctypes.c_int64),
                ("max_smem_per_block_optin", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RpResult(ctypes.Structure):
    """rp_result (include/rajaperf_gb300.h)."""
    _fields_ = [("kernel", ctypes.c_char * 64), ("variant", ctypes.c_char * 32),
                ("tuning", ctypes.c_char * 64), ("checksum", ctypes.c_double),
                ("checksum_residual", ctypes.c_double), ("min_time_s", ctypes.c_double),
                ("avg_time_s", ctypes.c_double), ("max_time_s", ctypes.c_double),
                ("reps", ctypes.c_int64), ("actual_size", ctypes.c_int64),
                ("its_per_rep", ctypes.c_int64), ("kernels_per_rep", ctypes.c_int64),
                ("bytes_per_rep", ctypes.c_int64), ("flops_per_rep", ctypes.c_int64),
                ("passes", ctypes.c_int32), ("failed", ctypes.c_int32),
                ("h2d_bytes_per_rep", ctypes.c_int64), ("d2h_bytes_per_rep", ctypes.c_int64)]


class RpBatchResult(ctypes.Structure):
    _fields_ = [("kernels", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("reps", ctypes.c_int64), ("launches_per_rep", ctypes.c_int64),
                ("launch_time_s", ctypes.c_double), ("graph_time_s", ctypes.c_double),
                ("graph_serial_time_s", ctypes.c_double)]


_C_TYPES = {
    "double": ctypes.c_double, "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64,
    "size_t": ctypes.c_size_t, "int": ctypes.c_int, "int32_t": ctypes.c_int32,
    "b200_stream_t": ctypes.c_void_p, "void": None,
}


def _ctype(decl: str):
    """ctypes type of one C parameter/return declaration from b200.h."""
    d = decl.replace("const ", "").strip()
    if d.startswith("char*") or d == "char *":
        return ctypes.c_char_p
    if "b200_tune*" in d.replace(" ", ""):
        return ctypes.POINTER(Tune)
    if "b200_caps*" in d.replace(" ", ""):
        return ctypes.POINTER(Caps)
    if "*" in d:
        return ctypes.c_void_p  # device or host address passed as an integer
    base = d.split()[0]
    if base not in _C_TYPES:
        raise ValueError(f"unmapped C type in b200.h: {decl!r}")
    return _C_TYPES[base]


def parse_signatures(header: str = "b200.h") -> dict:
    """{name: (argtypes, restype)} for every function declared in a header."""
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    sigs = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b((?:b200|rp)_\w+)\s*\(([^;{]*?)\)\s*;",
                         text, flags=re.S):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        ret = ret.replace("const char*", "char*").replace("const char *", "char*")
        restype = ctypes.c_char_p if ret.endswith("char*") else _ctype(ret)
        args = []
        if params and params != "void":
            for prm in params.split(","):
                prm = " ".join(prm.split())
                # drop the parameter name
                tname = re.sub(r"\b\w+$", "", prm).strip() if not prm.endswith("*") else prm
                args.append(_ctype(tname))
        sigs[name] = (args, restype)
    return sigs


_b200 = None
_host = None


def _require(path: str) -> None:
    if not os.path.exists(path):
        raise RuntimeError(
            f"{os.path.basename(path)} is not built ({path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` -- the Base_GB300 "
            "path has no CPU fallback")


def b200() -> ctypes.CDLL:
    """Loads libb200.so with typed entry points."""
    global _b200
    if _b200 is None:
        _require(LIBB200)
        lib = ctypes.CDLL(LIBB200)
        for name, (args, res) in parse_signatures("b200.h").items():
            fn = getattr(lib, name, None)
            if fn is None:
                raise RuntimeError(f"{LIBB200} does not export {name} (declared in b200.h)")
            fn.argtypes = args
            fn.restype = res
        _b200 = lib
    return _b200


def host() -> ctypes.CDLL:
    """Loads librajaperf_gb300.so (the suite layer)."""
    global _host
    if _host is None:
        _require(LIBHOST)
        lib = ctypes.CDLL(LIBHOST)
        lib.rp_last_error.argtypes = []
        lib.rp_last_error.restype = ctypes.c_char_p
        lib.rp_run.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                               ctypes.POINTER(RpResult), ctypes.c_int,
                               ctypes.POINTER(ctypes.c_int)]
        lib.rp_run.restype = ctypes.c_int
        lib.rp_graph_batch.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                       ctypes.POINTER(RpBatchResult)]
        lib.rp_graph_batch.restype = ctypes.c_int
        _host = lib
    return _host


def last_error() -> str:
    return b200().b200_last_error_string().decode()


def check(status: int, what: str = "b200 call") -> None:
    if status != B200_OK:
        raise RuntimeError(f"{what} failed ({status}): {last_error()}")


def _argv(args: list[str]):
    full = ["rajaperf-gb300"] + [str(a) for a in args]
    arr = (ctypes.c_char_p * len(full))(*[a.encode() for a in full])
    return len(full), arr


def run_suite(args: list[str], capacity: int = 256) -> list[dict]:
    """Runs the Base_GB300 suite for a command line; one dict per kernel x
    tuning.  Raises RuntimeError on bad input or a failed kernel."""
    lib = host()
    argc, argv = _argv(args)
    out = (RpResult * capacity)()
    count = ctypes.c_int(0)
    st = lib.rp_run(argc, argv, out, capacity, ctypes.byref(count))
    if st != 0:
        raise RuntimeError(f"rp_run failed ({st}): {lib.rp_last_error().decode()}")
    res = []
    for r in out[:count.value]:
        res.append({
            "kernel": r.kernel.decode(), "variant": r.variant.decode(),
            "tuning": r.tuning.decode(), "checksum": r.checksum,
            "checksum_residual": r.checksum_residual, "min_time_s": r.min_time_s,
            "avg_time_s": r.avg_time_s, "max_time_s": r.max_time_s, "reps": r.reps,
            "actual_size": r.actual_size, "its_per_rep": r.its_per_rep,
            "kernels_per_rep": r.kernels_per_rep, "bytes_per_rep": r.bytes_per_rep,
            "flops_per_rep": r.flops_per_rep, "passes": r.passes,
            "h2d_bytes_per_rep": r.h2d_bytes_per_rep, "d2h_bytes_per_rep": r.d2h_bytes_per_rep})
    return res


def graph_batch(args: list[str]) -> dict:
    """Runs --graph-batch for a command line (args must contain it)."""
    lib = host()
    argc, argv = _argv(args)
    out = RpBatchResult()
    st = lib.rp_graph_batch(argc, argv, ctypes.byref(out))
    if st != 0:
        raise RuntimeError(f"rp_graph_batch failed ({st}): {lib.rp_last_error().decode()}")
    return {"kernels": out.kernels, "reps": out.reps,
            "launches_per_rep": out.launches_per_rep,
            "launch_time_s": out.launch_time_s, "graph_time_s": out.graph_time_s,
            "graph_serial_time_s": out.graph_serial_time_s}


def declared_functions(header: str) -> list[str]:
    """Function names declared in one of the include/*.h headers."""
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:b200|rp)_[a-z0-9_]+)\s*\(", text)))
