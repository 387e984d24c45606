#!/usr/bin/env python3
"""Benchmark of the Base_GB300 loop-kernel hot path.

Metric: geomean over the workload's kernels of achieved HBM bandwidth as a
fraction of the measured copy peak (percent), bandwidth being the suite's
Bytes/rep divided by the time of one rep (scripts/caliper_graph/plot.py:15-31
of the suite).  One "step" runs every kernel of the workload once.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload bandwidth_stencil|stream]

* value: kernels timed with CUDA events on the launching stream, inputs
  resident in HBM, L2 flushed before every kernel (a 256 MiB write, then two
  256 MiB reads of another buffer so no dirty flush lines remain).
* e2e: the same metric through the Base_GB300 suite layer (rp_run) with the
  kernels' arrays in pinned host memory (--host-data): every rep moves its
  inputs from host memory and its outputs back inside the timed region.
* cpu_baseline / --impl reference: the suite's Base_OpenMP loops (the CPU
  oracle's restatement) on all host cores, one rep per kernel at full size.
Under torchrun (N>1) every rank runs its own replica (the path has no data
exchange); value is summed over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
BF16_FALLBACK_TFLOPS = 1900.0
L2_FLUSH_BYTES = 256 << 20


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]),
                "bf16_tflops": float(d.get("bf16_tflops", BF16_FALLBACK_TFLOPS)),
                "source": "measured"}
    return {"hbm_gbs": HBM_FALLBACK_GBS, "bf16_tflops": BF16_FALLBACK_TFLOPS,
            "source": "fallback"}


def load_traffic() -> dict:
    """Per-kernel DRAM bytes per launch from committed ncu summaries."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


# --------------------------------------------------------------------------
# workload cases
# --------------------------------------------------------------------------

class Case:
    """One kernel of the workload: device buffers, one rep, and the suite's
    Bytes/rep and FLOPs/rep for it."""
    name = ""
    launches = 1
    flops_per_rep = 0

    def __init__(self, torch, rp, seed):
        self.torch = torch
        self.rp = rp
        self.L = rp.b200()
        self.seed = seed
        self.stream_id = 0

    def uniform(self, n, lo=0.5, hi=1.5):
        t = self.torch.empty(n, dtype=self.torch.float64, device="cuda")
        self.rp.check(self.L.b200_init_uniform(t.data_ptr(), n, self.seed, self.stream_id,
                                               lo, hi, None), "init")
        self.stream_id += 1
        return t

    def zeros(self, n, dtype=None):
        return self.torch.zeros(n, dtype=dtype or self.torch.float64, device="cuda")

    # launch shape: a b200_tune from the committed tuning table, or None
    # (the library default); cases with a reduction workspace re-size it
    tp = None

    def set_tune(self, tune):
        self.tune = tune
        self.tp = None if tune is None else ctypes.byref(tune)
        if getattr(self, "ws_kind", None) == "reduce":
            self.ws_bytes = self.L.b200_reduce_workspace_bytes(self.n, self.tp)
            self.ws = self.torch.zeros(self.ws_bytes, dtype=self.torch.uint8, device="cuda")

    # subclasses define bytes_per_rep and run(stream)


def _stream_cases():
    class Triad(Case):
        name = "Stream_TRIAD"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.zeros(n)
            self.b = self.uniform(n)
            self.c = self.uniform(n)
            self.bytes_per_rep = 24 * n

        def run(self, s):
            return self.L.b200_stream_triad(self.a.data_ptr(), self.b.data_ptr(),
                                            self.c.data_ptr(), 0.5, self.n, self.tp, s)

    class Copy(Case):
        name = "Stream_COPY"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.c = self.zeros(n)
            self.bytes_per_rep = 16 * n

        def run(self, s):
            return self.L.b200_stream_copy(self.a.data_ptr(), self.c.data_ptr(), self.n,
                                           self.tp, s)

    class Mul(Case):
        name = "Stream_MUL"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.b = self.zeros(n)
            self.c = self.uniform(n)
            self.bytes_per_rep = 16 * n

        def run(self, s):
            return self.L.b200_stream_mul(self.b.data_ptr(), self.c.data_ptr(), 0.5, self.n,
                                          self.tp, s)

    class Add(Case):
        name = "Stream_ADD"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.b = self.uniform(n)
            self.c = self.zeros(n)
            self.bytes_per_rep = 24 * n

        def run(self, s):
            return self.L.b200_stream_add(self.a.data_ptr(), self.b.data_ptr(),
                                          self.c.data_ptr(), self.n, self.tp, s)

    class Dot(Case):
        name = "Stream_DOT"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.b = self.uniform(n)
            self.acc = self.zeros(1)
            self.ws_kind = "reduce"
            self.ws_bytes = self.L.b200_reduce_workspace_bytes(n, None)
            self.ws = self.zeros(self.ws_bytes, dtype=torch.uint8)
            self.bytes_per_rep = 16 * n + 16

        def run(self, s):
            return self.L.b200_stream_dot(self.a.data_ptr(), self.b.data_ptr(), self.n, 0.0,
                                          self.acc.data_ptr(), self.ws.data_ptr(),
                                          self.ws_bytes, self.tp, s)

    return {"Stream_COPY": Copy, "Stream_MUL": Mul, "Stream_ADD": Add,
            "Stream_TRIAD": Triad, "Stream_DOT": Dot}


def _ddv_mesh(np, rzmax, seed):
    """ADomain(rzmax, 2) of apps/AppsData.hpp with jittered node positions
    and the real-zone list (AppsData.cpp:56-151)."""
    npnl, npnr = 2, 1
    imin = jmin = npnl
    imax = jmax = npnl + rzmax - 1
    jp = imax + 1 - imin + npnl + npnr
    nnalls = jp * (jmax + 1 - jmin + npnl + npnr)
    ii, jj = np.meshgrid(np.arange(jp), np.arange(nnalls // jp))
    rng = np.random.default_rng(seed)
    x = (ii * 0.2 + 0.2 * rng.uniform(-0.1, 0.1, ii.shape)).ravel()
    y = (jj * 0.1 + 0.1 * rng.uniform(-0.1, 0.1, jj.shape)).ravel()
    zi, zj = np.meshgrid(np.arange(imin, imax), np.arange(jmin, jmax))
    zones = (zi + zj * jp).ravel().astype(np.int64)
    n_real_nodes = (imax + 1 - imin) * (jmax + 1 - jmin)
    return x, y, zones, jp, nnalls, n_real_nodes


def _bandwidth_cases():
    import numpy as np

    class Hydro2D(Case):
        name = "Lcals_HYDRO_2D"
        launches = 2

        def __init__(self, torch, rp, seed, size):
            super().__init__(torch, rp, seed)
            self.jn = self.kn = int(math.sqrt(size) + math.sqrt(2) - 1)
            n = self.kn * self.jn
            self.arr = [self.uniform(n) for _ in range(11)]
            kn, jn = self.kn, self.jn
            self.bytes_per_rep = (8 * (4 * n + 4 * n + 4 * (kn - 2) * (jn - 2)) +
                                  8 * 6 * (kn - 2) * (jn - 2))
            self.flops_per_rep = 44 * (kn - 2) * (jn - 2)
            # ncu: BODY1 10 per point (its divisions and products run on the
            # integer and FP32 pipes), BODY2+BODY3 14 per point (6 of its 8
            # differences on the integer pipes)
            self.fp64_instr_per_rep = 24 * (kn - 2) * (jn - 2)

        def run(self, s):
            a = [t.data_ptr() for t in self.arr]
            return self.L.b200_lcals_hydro_2d(*a, 0.0041, 0.0037, self.kn, self.jn, self.tp, s)

    class Eos(Case):
        name = "Lcals_EOS"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.x = self.zeros(n + 7)
            self.y, self.z, self.u = (self.uniform(n + 7) for _ in range(3))
            self.bytes_per_rep = 16 * n + 8 * (n + 7) + 8 * n
            self.flops_per_rep = 16 * n
            # two of the eight FMAs per element on the integer pipes
            self.fp64_instr_per_rep = 6 * n

        def run(self, s):
            return self.L.b200_lcals_eos(self.x.data_ptr(), self.y.data_ptr(), self.z.data_ptr(),
                                         self.u.data_ptr(), 0.0979, 0.1958, 0.0979, self.n,
                                         self.tp, s)

    class FirstDiff(Case):
        name = "Lcals_FIRST_DIFF"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.x = self.zeros(n + 1)
            self.y = self.uniform(n + 1)
            self.bytes_per_rep = 8 * (n + 1) + 8 * n
            self.flops_per_rep = n
            self.fp64_instr_per_rep = n

        def run(self, s):
            return self.L.b200_lcals_first_diff(self.x.data_ptr(), self.y.data_ptr(), self.n,
                                                self.tp, s)

    class FirstMin(Case):
        name = "Lcals_FIRST_MIN"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.x = self.uniform(n)
            planted = int(np.random.default_rng(seed).integers(0, n))
            self.x[planted] = -0.5
            self.loc = self.zeros(1, dtype=torch.int64)
            self.ws_kind = "reduce"
            self.ws_bytes = self.L.b200_reduce_workspace_bytes(n, None)
            self.ws = self.zeros(self.ws_bytes, dtype=torch.uint8)
            self.bytes_per_rep = 8 + 8 + 8 * n + 8 + 8
            self.flops_per_rep = 0
            self.fp64_instr_per_rep = 0

        def run(self, s):
            return self.L.b200_lcals_first_min(self.x.data_ptr(), self.n, 0.5, 0,
                                               self.loc.data_ptr(), None, self.ws.data_ptr(),
                                               self.ws_bytes, self.tp, s)

    class DelDotVec2D(Case):
        name = "Apps_DEL_DOT_VEC_2D"

        def __init__(self, torch, rp, seed, size):
            super().__init__(torch, rp, seed)
            rzmax = int(math.sqrt(size) + 1 + math.sqrt(2) - 1)
            x, y, zones, self.jp, nn, n_real_nodes = _ddv_mesh(np, rzmax, seed)
            self.x = torch.from_numpy(x).cuda()
            self.y = torch.from_numpy(y).cuda()
            self.zones = torch.from_numpy(zones).cuda()
            self.nz = zones.size
            self.xdot, self.ydot = self.uniform(nn), self.uniform(nn)
            self.div = self.zeros(nn)
            self.bytes_per_rep = 8 * self.nz + 4 * 8 * n_real_nodes + 8 * self.nz
            self.flops_per_rep = 54 * self.nz
            # 27 per zone: of the 30 adds and 3 FMAs, the first add of six
            # corner sums runs on the integer pipes, as do the halves,
            # divisions, standalone products and + ptiny
            self.fp64_instr_per_rep = 27 * self.nz

        def run(self, s):
            return self.L.b200_apps_del_dot_vec_2d(
                self.x.data_ptr(), self.y.data_ptr(), self.xdot.data_ptr(),
                self.ydot.data_ptr(), self.div.data_ptr(), self.zones.data_ptr(), self.nz,
                self.jp, 1e-20, 0.5, self.tp, s)

    class Jacobi2D(Case):
        name = "Polybench_JACOBI_2D"

        def __init__(self, torch, rp, seed, size, tsteps=50):
            super().__init__(torch, rp, seed)
            N = self.N = int(math.sqrt(size) + 2 + math.sqrt(2) - 1)
            self.tsteps = tsteps
            self.launches = 2 * tsteps
            self.A, self.B = self.uniform(N * N), self.uniform(N * N)
            self.bytes_per_rep = (8 * (N * N - 4) * 2 + 8 * (N - 2) * (N - 2) * 2) * tsteps
            self.flops_per_rep = tsteps * 10 * (N - 2) * (N - 2)
            # per point and half-step: three of the four adds on the FP64 pipe
            # (the first add and the product by 0.2 run on the integer pipes)
            self.fp64_instr_per_rep = tsteps * 6 * (N - 2) * (N - 2)

        def run(self, s):
            return self.L.b200_polybench_jacobi_2d(self.A.data_ptr(), self.B.data_ptr(), self.N,
                                                   self.tsteps, self.tp, s)

    class Heat3D(Case):
        name = "Polybench_HEAT_3D"

        def __init__(self, torch, rp, seed, size, tsteps=20):
            super().__init__(torch, rp, seed)
            N = self.N = int(round(size ** (1.0 / 3.0)) + 2 + 3 ** (1.0 / 3.0) - 1)
            self.tsteps = tsteps
            self.launches = 2 * tsteps
            self.A, self.B = self.uniform(N ** 3), self.uniform(N ** 3)
            inner = (N - 2) ** 3
            self.bytes_per_rep = (8 * (N ** 3 - 12 * (N - 2) - 8) * 2 + 8 * inner * 2) * tsteps
            self.flops_per_rep = tsteps * 30 * inner
            # per point and half-step: 9 adds, 2.5 of them (5 of the 6
            # differences b(+1) - 2a of two planes) on the integer pipes
            self.fp64_instr_per_rep = tsteps * 13 * inner

        def run(self, s):
            return self.L.b200_polybench_heat_3d(self.A.data_ptr(), self.B.data_ptr(), self.N,
                                                 self.tsteps, self.tp, s)

    class Fdtd2D(Case):
        name = "Polybench_FDTD_2D"

        def __init__(self, torch, rp, seed, size, tsteps=40):
            super().__init__(torch, rp, seed)
            nx = ny = self.nx = self.ny = int(math.sqrt(size) + 1 + math.sqrt(2) - 1)
            self.tsteps = tsteps
            self.launches = 2 * tsteps
            self.hz = self.zeros(nx * ny)
            self.ex, self.ey = self.uniform(nx * ny), self.uniform(nx * ny)
            self.fict = self.uniform(tsteps)
            rd = 8 * (1 + (nx - 1) * ny + nx * ny + nx * (ny - 1) + nx * ny +
                      (nx - 1) * (ny - 1) + (nx - 1) * ny + nx * (ny - 1))
            wr = 8 * (ny + (nx - 1) * ny + nx * (ny - 1) + (nx - 1) * (ny - 1))
            self.bytes_per_rep = (rd + wr) * tsteps
            self.flops_per_rep = tsteps * (3 * (nx - 1) * ny + 3 * nx * (ny - 1) +
                                           5 * (nx - 1) * (ny - 1))
            # FP64-pipe instructions: 2 per ey and ex update, 4 per hz update
            self.fp64_instr_per_rep = tsteps * (2 * (nx - 1) * ny + 2 * nx * (ny - 1) +
                                                4 * (nx - 1) * (ny - 1))
            # one launch per time step (tile-edge snapshots in the workspace)
            self.launches = 1 + tsteps
            self.ws_bytes = self.L.b200_fdtd_2d_workspace_bytes(nx, ny)
            self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device="cuda")

        def run(self, s):
            return self.L.b200_polybench_fdtd_2d_ws(self.ex.data_ptr(), self.ey.data_ptr(),
                                                    self.hz.data_ptr(), self.fict.data_ptr(),
                                                    self.nx, self.ny, self.tsteps,
                                                    self.ws.data_ptr(), self.ws_bytes, self.tp, s)

    class ScanI64(Case):
        name = "Algorithm_SCAN"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.x = torch.empty(n, dtype=torch.int64, device="cuda")
            rp.check(self.L.b200_init_uniform_i64(self.x.data_ptr(), n, seed, 0, 0, 100, None))
            self.y = self.zeros(n, dtype=torch.int64)
            self.ws_bytes = self.L.b200_scan_workspace_bytes(n)
            self.ws = self.zeros(self.ws_bytes, dtype=torch.uint8)
            self.bytes_per_rep = 16 * n
            self.flops_per_rep = n
            self.fp64_instr_per_rep = 0

        def run(self, s):
            return self.L.b200_algorithm_scan_i64(self.x.data_ptr(), self.y.data_ptr(), self.n,
                                                  0, self.ws.data_ptr(), self.ws_bytes, self.tp, s)

    return {"Lcals_HYDRO_2D": Hydro2D, "Lcals_EOS": Eos, "Lcals_FIRST_DIFF": FirstDiff,
            "Lcals_FIRST_MIN": FirstMin, "Apps_DEL_DOT_VEC_2D": DelDotVec2D,
            "Polybench_JACOBI_2D": Jacobi2D, "Polybench_HEAT_3D": Heat3D,
            "Polybench_FDTD_2D": Fdtd2D, "Algorithm_SCAN": ScanI64}


# --------------------------------------------------------------------------
# every 1-D kernel at 2^27 elements
# --------------------------------------------------------------------------

# FP64-pipe instructions per element, as ncu counts them for these kernels
# (sm__inst_executed_pipe_fp64 x 32 / elements; DADD/DMUL/DFMA, double
# compares, the divides' and exp's FP64 steps), and the suite's Bytes/rep per
# element.  A kernel with fewer FP64 instructions per byte than
# the GPU's balance point (FP64 instruction rate / HBM copy rate) is
# HBM-bound; the others are bounded by the FP64 pipe first.
BW27 = {
    # kernel: (bytes/elem, fp64 instr/elem, arrays (name, length factor, init), scalars)
    "Stream_COPY": (16, 0), "Stream_MUL": (16, 1), "Stream_ADD": (24, 1),
    "Stream_TRIAD": (24, 1), "Stream_DOT": (16, 1), "Basic_DAXPY": (24, 1),
    "Basic_INIT3": (40, 1), "Basic_MULADDSUB": (40, 3), "Lcals_HYDRO_1D": (24, 3),
    "Lcals_EOS": (32, 6), "Lcals_FIRST_DIFF": (16, 1), "Lcals_INT_PREDICT": (88, 9),
    "Lcals_FIRST_MIN": (8, 0), "Lcals_DIFF_PREDICT": (160, 9), "Lcals_PLANCKIAN": (40, 16),
    "Apps_PRESSURE": (48, 6), "Apps_ENERGY": (216, 18), "Algorithm_SCAN": (16, 0),
    "Algorithm_REDUCE_SUM": (8, 1), "Algorithm_MEMSET": (8, 0), "Algorithm_MEMCPY": (16, 0),
    "Basic_INDEXLIST": (10, 0), "Algorithm_HISTOGRAM": (8, 0), "Basic_MULTI_REDUCE": (16, 1),
}


def bw27_run(torch, rp, name, n, seed):
    """Allocates one kernel's arrays (uniform [0.5, 1.5) on the device) and
    returns (run(stream) -> status, keep-alive list)."""
    L = rp.b200()
    sid = [0]

    def u(m):
        t = torch.empty(m, dtype=torch.float64, device="cuda")
        rp.check(L.b200_init_uniform(t.data_ptr(), m, seed, sid[0], 0.5, 1.5, None), "init")
        sid[0] += 1
        return t

    def z(m, dtype=torch.float64):
        return torch.zeros(m, dtype=dtype, device="cuda")

    P = lambda t: t.data_ptr()
    if name == "Stream_COPY":
        a, c = u(n), z(n)
        return (lambda s: L.b200_stream_copy(P(a), P(c), n, None, s)), [a, c]
    if name == "Stream_MUL":
        b, c = z(n), u(n)
        return (lambda s: L.b200_stream_mul(P(b), P(c), 0.5, n, None, s)), [b, c]
    if name == "Stream_ADD":
        a, b, c = u(n), u(n), z(n)
        return (lambda s: L.b200_stream_add(P(a), P(b), P(c), n, None, s)), [a, b, c]
    if name == "Stream_TRIAD":
        a, b, c = z(n), u(n), u(n)
        return (lambda s: L.b200_stream_triad(P(a), P(b), P(c), 0.5, n, None, s)), [a, b, c]
    if name == "Stream_DOT":
        a, b, acc = u(n), u(n), z(1)
        wb = L.b200_reduce_workspace_bytes(n, None)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_stream_dot(P(a), P(b), n, 0.0, P(acc), P(ws), wb, None, s)), \
            [a, b, acc, ws]
    if name == "Basic_DAXPY":
        y, x = z(n), u(n)
        return (lambda s: L.b200_basic_daxpy(P(y), P(x), 0.5, n, None, s)), [y, x]
    if name in ("Basic_INIT3", "Basic_MULADDSUB"):
        o1, o2, o3, i1, i2 = z(n), z(n), z(n), u(n), u(n)
        fn = L.b200_basic_init3 if name == "Basic_INIT3" else L.b200_basic_muladdsub
        return (lambda s: fn(P(o1), P(o2), P(o3), P(i1), P(i2), n, None, s)), \
            [o1, o2, o3, i1, i2]
    if name == "Lcals_HYDRO_1D":
        x, y, zz = z(n + 12), u(n + 12), u(n + 12)
        return (lambda s: L.b200_lcals_hydro_1d(P(x), P(y), P(zz), 0.0979, 0.1958, 0.0979, n,
                                                None, s)), [x, y, zz]
    if name == "Lcals_EOS":
        x, y, zz, uu = z(n + 7), u(n + 7), u(n + 7), u(n + 7)
        return (lambda s: L.b200_lcals_eos(P(x), P(y), P(zz), P(uu), 0.0979, 0.1958, 0.0979, n,
                                           None, s)), [x, y, zz, uu]
    if name == "Lcals_FIRST_DIFF":
        x, y = z(n + 1), u(n + 1)
        return (lambda s: L.b200_lcals_first_diff(P(x), P(y), n, None, s)), [x, y]
    if name == "Lcals_INT_PREDICT":
        px = u(13 * n)
        return (lambda s: L.b200_lcals_int_predict(P(px), 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7,
                                                   0.8, n, None, s)), [px]
    if name == "Lcals_FIRST_MIN":
        x = u(n)
        x[n // 3] = -0.5
        loc = z(1, torch.int64)
        wb = L.b200_reduce_workspace_bytes(n, None)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_lcals_first_min(P(x), n, 0.5, 0, P(loc), None, P(ws), wb,
                                                 None, s)), [x, loc, ws]
    if name == "Lcals_DIFF_PREDICT":
        px, cx = z(14 * n), u(14 * n)
        return (lambda s: L.b200_lcals_diff_predict(P(px), P(cx), n, None, s)), [px, cx]
    if name == "Lcals_PLANCKIAN":
        x, y, uu, v, w = u(n), z(n), u(n), u(n), z(n)
        return (lambda s: L.b200_lcals_planckian(P(x), P(y), P(uu), P(v), P(w), n, None, s)), \
            [x, y, uu, v, w]
    if name == "Apps_PRESSURE":
        comp, bvc, pn, eo, vn = u(n), z(n), z(n), u(n), u(n)
        return (lambda s: L.b200_apps_pressure(P(comp), P(bvc), P(pn), P(eo), P(vn), 0.5,
                                               1e-7, 0.0, 1.2, n, None, s)), \
            [comp, bvc, pn, eo, vn]
    if name == "Apps_ENERGY":
        arrs = [z(n)] + [u(n) for _ in range(4)] + [z(n)] + [u(n) for _ in range(9)]
        return (lambda s: L.b200_apps_energy(*[P(t) for t in arrs], 1.1, 1e-7, 0.0, 1e-7, n,
                                             None, s)), arrs
    if name == "Algorithm_SCAN":
        x = torch.empty(n, dtype=torch.int64, device="cuda")
        rp.check(L.b200_init_uniform_i64(P(x), n, seed, 0, 0, 100, None))
        y = z(n, torch.int64)
        wb = L.b200_scan_workspace_bytes(n)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_algorithm_scan_i64(P(x), P(y), n, 0, P(ws), wb, None, s)), \
            [x, y, ws]
    if name == "Algorithm_REDUCE_SUM":
        x, out = u(n), z(1)
        wb = L.b200_reduce_workspace_bytes(n, None)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_algorithm_reduce_sum(P(x), n, 0.0, P(out), P(ws), wb, None,
                                                      s)), [x, out, ws]
    if name == "Algorithm_MEMSET":
        x = z(n)
        return (lambda s: L.b200_algorithm_memset(P(x), 0.0, n, None, s)), [x]
    if name == "Algorithm_MEMCPY":
        x, y = u(n), z(n)
        return (lambda s: L.b200_algorithm_memcpy(P(x), P(y), n, None, s)), [x, y]
    if name == "Basic_INDEXLIST":
        x = u(n)
        x.sub_(1.0)  # uniform [-0.5, 0.5): about half the items selected
        lst = z(n, torch.int32)
        ln = z(1, torch.int64)
        wb = L.b200_indexlist_workspace_bytes(n)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_basic_indexlist(P(x), P(lst), n, P(ln), P(ws), wb, None, s)), \
            [x, lst, ln, ws]
    if name in ("Algorithm_HISTOGRAM", "Basic_MULTI_REDUCE"):
        nb = 10
        bins = torch.empty(n, dtype=torch.int64, device="cuda")
        rp.check(L.b200_init_uniform_i64(P(bins), n, seed, 7, 0, nb, None))
        if name == "Algorithm_HISTOGRAM":
            cinit, cnt = z(nb, torch.int64), z(nb, torch.int64)
            return (lambda s: L.b200_algorithm_histogram(P(bins), n, nb, P(cinit), P(cnt), None,
                                                         s)), [bins, cinit, cnt]
        data, vinit, vals = u(n), z(nb), z(nb)
        wb = L.b200_multi_reduce_workspace_bytes(n, nb)
        ws = z(wb, torch.uint8)
        return (lambda s: L.b200_basic_multi_reduce(P(bins), P(data), n, nb, P(vinit), P(vals),
                                                    P(ws), wb, None, s)), \
            [bins, data, vinit, vals, ws]
    raise KeyError(name)


def measure_bw27(torch, rp, stream, peaks, fp64_instr_rate, seed, n=1 << 27, steps=5,
                 warmup=3, only=None):
    """Times every 1-D kernel at n elements (inputs far larger than L2, so no
    flush is needed) and reports GB/s against the copy peak, the kernel's
    bound (HBM or FP64 pipe) and geomeans over all kernels and over the
    HBM-bound ones."""
    s = stream.cuda_stream
    balance = fp64_instr_rate / (peaks["hbm_gbs"] * 1e9)  # FP64 instr per byte
    rows = []
    for name, (bpe, ipe) in BW27.items():
        if only and name not in only and name.split("_", 1)[1] not in only:
            continue
        run, keep = bw27_run(torch, rp, name, n, seed)
        for _ in range(warmup):
            rp.check(run(s), name)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        torch.cuda.synchronize()
        for e0, e1 in ev:
            e0.record(stream)
            rp.check(run(s), name)
            e1.record(stream)
        torch.cuda.synchronize()
        t = sorted(e0.elapsed_time(e1) for e0, e1 in ev)[len(ev) // 2] / 1e3
        gbs = bpe * n / t / 1e9
        bound = "hbm" if ipe / bpe <= balance else "fp64"
        # the kernel's own ceiling: HBM time or FP64-pipe time, whichever is longer
        t_floor = max(bpe * n / (peaks["hbm_gbs"] * 1e9), ipe * n / fp64_instr_rate)
        rows.append({"kernel": name, "ms": round(t * 1e3, 4), "gbs": round(gbs, 1),
                     "pct_hbm": round(100 * gbs / peaks["hbm_gbs"], 2), "bound": bound,
                     "fp64_instr_per_byte": round(ipe / bpe, 4),
                     "pct_of_own_bound": round(100 * t_floor / t, 2)})
        # the arrays go back to torch's cache, not to the driver: memory the
        # driver takes back is cleaned in the background, which took 18-30%
        # of the bandwidth of the kernel timed next (measured after the 14 GB
        # of INT_PREDICT's arrays), so no cache is emptied between kernels
        del run, keep
    hbm_rows = [r for r in rows if r["bound"] == "hbm"]
    return {
        "n": n, "balance_fp64_instr_per_byte": round(balance, 4),
        "geomean_pct_hbm_all": round(geomean([r["pct_hbm"] for r in rows]), 2),
        "geomean_pct_hbm_hbm_bound": round(geomean([r["pct_hbm"] for r in hbm_rows]), 2),
        "geomean_pct_of_own_bound_all": round(geomean([r["pct_of_own_bound"] for r in rows]),
                                              2),
        "per_kernel": rows,
    }


# workload -> list of (kernel, size, oracle kwargs for the CPU baseline)
WORKLOADS = {
    "bandwidth_stencil": {
        "description": "FP64, uniform [0.5,1.5) from a seed: HYDRO_2D 4096x4096; EOS, "
                       "FIRST_DIFF, FIRST_MIN (planted minimum) N=2^24; DEL_DOT_VEC_2D "
                       "4096x4096 mesh jittered by up to 0.1 cell; JACOBI_2D N=4096, 50 "
                       "tsteps; HEAT_3D 256^3, 20 tsteps; SCAN int64 in [0,100), N=2^26",
        "kernels": [("Lcals_HYDRO_2D", 4096 * 4096), ("Lcals_EOS", 1 << 24),
                    ("Lcals_FIRST_DIFF", 1 << 24), ("Lcals_FIRST_MIN", 1 << 24),
                    ("Apps_DEL_DOT_VEC_2D", 4096 * 4096), ("Polybench_JACOBI_2D", 4094 * 4094),
                    ("Polybench_HEAT_3D", 254 ** 3), ("Algorithm_SCAN", 1 << 26)],
    },
    "stream": {
        "description": "Stream COPY/MUL/ADD/TRIAD/DOT, FP64, N=2^27 per array",
        "kernels": [("Stream_COPY", 1 << 27), ("Stream_MUL", 1 << 27),
                    ("Stream_ADD", 1 << 27), ("Stream_TRIAD", 1 << 27),
                    ("Stream_DOT", 1 << 27)],
    },
    "large": {
        "description": "FP64, uniform [0.5,1.5) from a seed: Stream COPY/MUL/ADD/TRIAD at "
                       "2^28 (2 GiB per array); HEAT_3D 768^3, 100 tsteps; FDTD_2D 8192x8192, "
                       "100 tsteps; JACOBI_2D 16384x16384, 40 tsteps",
        "kernels": [("Stream_COPY", 1 << 28), ("Stream_MUL", 1 << 28),
                    ("Stream_ADD", 1 << 28), ("Stream_TRIAD", 1 << 28),
                    ("Polybench_HEAT_3D", 766 ** 3), ("Polybench_FDTD_2D", 8191 * 8192),
                    ("Polybench_JACOBI_2D", 16382 * 16382)],
        "params": {"Polybench_HEAT_3D": {"tsteps": 100}, "Polybench_FDTD_2D": {"tsteps": 100},
                   "Polybench_JACOBI_2D": {"tsteps": 40}},
    },
}
DEFAULT_WORKLOAD = "bandwidth_stencil"


def workload_kernels(workload, only=None):
    ks = WORKLOADS[workload]["kernels"]
    if only:
        ks = [(k, n) for k, n in ks if k in only or k.split("_", 1)[1] in only]
    return ks


TUNING_TABLE = os.path.join(ROOT, "rajaperf_gb300", "tuning", "gb300.txt")
# kernels whose table entry was measured for a different form than the bench
# runs (SCAN's entry is for the suite's default FP64 scan; the bench times the
# int64 scan)
TABLE_SKIP = {"Algorithm_SCAN"}


def load_tuning_table(rp, path=TUNING_TABLE):
    """{(kernel, size): b200_tune} from a tuning table (the suite layer's
    --tuning-table format; exact-size entries, as the autotuner writes)."""
    table = {}
    if not os.path.exists(path):
        return table
    fields = {"block": "block_size", "items": "items", "vec": "vec", "grid": "grid_blocks",
              "tile_x": "tile_x", "tile_y": "tile_y", "tile_z": "tile_z",
              "time_block": "time_block", "algo": "algo"}
    for ln in open(path):
        ln = ln.split("#", 1)[0].split()
        if len(ln) < 3:
            continue
        t = rp.Tune()
        for kv in ln[3:]:
            k, v = kv.split("=")
            setattr(t, fields[k], int(v))
        table[(ln[0], int(ln[1]))] = t
    return table


def build_cases(torch, rp, workload, seed, only=None, table=None):
    registry = {}
    registry.update(_stream_cases())
    registry.update(_bandwidth_cases())
    params = WORKLOADS[workload].get("params", {})
    cases = []
    for k, n in workload_kernels(workload, only):
        c = registry[k](torch, rp, seed, n, **params.get(k, {}))
        if table and k not in TABLE_SKIP and (k, n) in table:
            c.set_tune(table[(k, n)])
        cases.append(c)
    return cases


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------

class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------

def combine_ranks(dist, step_s, value, device):
    """Whole-job figures of N replicas: the slowest rank's step time and the
    sum of the per-rank metric (every rank ran the full workload)."""
    import torch
    t = torch.tensor([step_s], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    v = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(v, op=dist.ReduceOp.SUM)
    return float(t.item()), float(v.item())


def geomean(xs):
    xs = [x for x in xs if x > 0]
    return math.exp(sum(math.log(x) for x in xs) / len(xs)) if xs else 0.0


def run_gpu(args, rank, world):
    import torch
    import rajaperf_gb300 as rp

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    peaks = load_peaks()
    traffic = load_traffic()
    table = load_tuning_table(rp) if args.tuning_table else {}
    cases = build_cases(torch, rp, args.workload, args.seed + rank, args.kernels, table)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    # L2 flush before every kernel: a write of a 256 MiB buffer evicts the
    # kernel's inputs and outputs, then two reads of a second 256 MiB buffer
    # evict the flush's own dirty lines, so that their write-back to HBM is
    # not charged to the timed kernel (at 2^24 elements it would add up to
    # ~128 MB of writes to a kernel that moves 134-268 MB).  One read was not
    # enough: FIRST_MIN at 2^24 took 31.4 us after write + one read, 28.7 us
    # after write + two reads, 27.2 us back to back with no flush at all.
    flush_w = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    flush_r = torch.zeros(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    fp64 = measure_fp64_peak(torch, rp, stream)

    def l2_flush():
        flush_w.zero_()
        flush_r.sum()
        flush_r.sum()

    def one_step(timed_events=None):
        for i, c in enumerate(cases):
            l2_flush()
            if timed_events is not None:
                timed_events[i][0].record(stream)
            rp.check(c.run(s), c.name)
            if timed_events is not None:
                timed_events[i][1].record(stream)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in cases] for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = rp.b200().b200_launch_count()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        one_step(ev[k])
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = rp.b200().b200_launch_count() - launches0
    clocks = sampler.stop()
    if dist:
        dist.barrier()

    per_kernel = []
    for i, c in enumerate(cases):
        ms = [ev[k][i][0].elapsed_time(ev[k][i][1]) for k in range(args.steps)]
        avg_s = sum(ms) / len(ms) / 1e3
        gbs = c.bytes_per_rep / avg_s / 1e9
        gfs = c.flops_per_rep / avg_s / 1e9
        fi = getattr(c, "fp64_instr_per_rep", None)
        per_kernel.append({"kernel": c.name, "ms": avg_s * 1e3, "gbs": gbs,
                           "frac": gbs / peaks["hbm_gbs"], "bytes": c.bytes_per_rep,
                           "gflops": gfs, "fp64_frac": gfs / fp64["gflops"],
                           # FP64-pipe instructions (ncu counts) / time / peak rate
                           "fp64_pipe_frac": (round(fi / avg_s / fp64["fma_per_s"], 4)
                                              if fi is not None else None),
                           "launches": c.launches})
    step_s = sum(p["ms"] for p in per_kernel) / 1e3
    value = 100.0 * geomean([p["frac"] for p in per_kernel])

    # e2e through the suite layer with host-resident data
    e2e = None if args.no_e2e else run_e2e(torch, rp, args, peaks)

    dom = max(per_kernel, key=lambda p: p["ms"])
    tr = traffic.get(dom["kernel"])
    # per launch: the rep's algorithmic bytes and time divided by its launches
    roofline = {"bound": "hbm", "kernel": dom["kernel"], "achieved": round(dom["gbs"], 1),
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(dom["gbs"] / peaks["hbm_gbs"], 4),
                "traffic": (tr["bytes_per_launch"] if tr else None),
                "algorithmic_bytes_per_launch": dom["bytes"] // dom["launches"],
                "launch_ms": round(dom["ms"] / dom["launches"], 4),
                "traffic_source": (tr["source"] if tr else None),
                "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json copy peak)"
                               if peaks["source"] == "measured" else "fallback",
                "fp64": {"achieved_gflops": round(dom["gflops"], 1),
                         "peak_gflops": round(fp64["gflops"], 1),
                         "frac": round(dom["fp64_frac"], 4),
                         "pipe_frac": dom.get("fp64_pipe_frac"),
                         "peak_source": "measured in this run: max of the DFMA probe and "
                                        "native FP64 GEMM 2048^3 (FMA = 2 flops)",
                         "probe_gflops": fp64["probe_gflops"],
                         "dgemm_gflops": fp64["dgemm_gflops"]}}
    return {
        "value": value, "step_s": step_s, "per_kernel": per_kernel, "e2e": e2e,
        "roofline": roofline, "clocks": clocks, "launches": launches, "wall_s": wall,
        "world": world, "dist": dist, "fp64": fp64,
    }


def measure_fp8_peak(torch, n=8192):
    """Dense e4m3 GEMM throughput of cuBLASLt (torch._scaled_mm, FP32 scales,
    bf16 out) at n^3, best of 10: the denominator for the split GEMM's FP8
    tensor work.  None where torch lacks the call."""
    try:
        a = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn)
        b = torch.randn(n, n, device="cuda").to(torch.float8_e4m3fn).t()
        one = torch.ones((), device="cuda")
        f = lambda: torch._scaled_mm(a, b, scale_a=one, scale_b=one, out_dtype=torch.bfloat16)
        for _ in range(3):
            f()
        best = None
        for _ in range(10):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            best = t if best is None else min(best, t)
        del a, b
        torch.cuda.empty_cache()
        return round(2.0 * n ** 3 / best / 1e12, 1)
    except (RuntimeError, AttributeError, TypeError):
        return None


def measure_gemm(torch, rp, stream, sizes=(1024, 4096, 8192), seed=4793):
    """Square C = 1.5*A*B + 1.2*C, entries uniform in [-1, 1): native FP64
    (b200_gemm_f64) against split precision (b200_gemm_split: the default
    e4m3 tcgen05 engine with paired digit weights, the single-weight e4m3 and
    bf16 tcgen05 engines and the legacy mma.sync engine), TFLOP/s at 2*N^3 and the split result's relative Frobenius error
    against the native FP64 result and cuBLAS FP64; plus a variant with rows
    of A scaled by 2^k, k in [-20, 20]."""
    import ctypes
    L = rp.b200()
    s = stream.cuda_stream
    legacy = rp.Tune(algo=1)  # the mma.sync engine, for comparison
    bf16 = rp.Tune(algo=2)    # the same digits on bf16 tensor cores
    single = rp.Tune(algo=3)  # e4m3, one digit weight per 128x128 MMA
    slices = 10  # the library default (b200_gemm_split)
    pairs = slices * (slices + 1) // 2  # slice products formed per C element
    out = []
    for n in sizes:
        g = torch.Generator(device="cuda").manual_seed(seed + n)
        A = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        B = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        C0 = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        ws_bytes = max(L.b200_gemm_split_workspace_bytes(n, n, n, t)
                       for t in (None, ctypes.byref(legacy), ctypes.byref(bf16)))
        ws = torch.zeros(ws_bytes, dtype=torch.uint8, device="cuda")
        res = {"n": n}

        def split(tune):
            return lambda C: L.b200_gemm_split(A.data_ptr(), B.data_ptr(), C.data_ptr(), n, n,
                                               n, 1.5, 1.2, ws.data_ptr(), ws_bytes, tune, s)
        for name, fn in (("native", lambda C: L.b200_gemm_f64(A.data_ptr(), B.data_ptr(),
                                                             C.data_ptr(), n, n, n, 1.5, 1.2,
                                                             None, s)),
                         ("split", split(None)),
                         ("split_e4m3_single_weight", split(ctypes.byref(single))),
                         ("split_bf16", split(ctypes.byref(bf16))),
                         ("split_mma_sync", split(ctypes.byref(legacy)))):
            C = C0.clone()
            rp.check(fn(C), name)  # warm-up
            reps = 1 if (name in ("native", "split_mma_sync") and n >= 8192) else 3
            best = None
            for _ in range(reps):
                C = C0.clone()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rp.check(fn(C), name)
                e1.record(stream)
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1) / 1e3
                best = t if best is None else min(best, t)
            res[f"{name}_ms"] = round(best * 1e3, 3)
            res[f"{name}_tflops"] = round(2.0 * n ** 3 / best / 1e12, 3)
            res[f"C_{name}"] = C
        err = (res["C_split"] - res["C_native"]).norm() / res["C_native"].norm()
        res["rel_err_vs_fp64"] = float(err)
        # an independent FP64 result: cuBLAS DGEMM through torch.matmul
        ref = torch.addmm(C0, A, B, beta=1.2, alpha=1.5)
        rn = ref.norm()
        res["rel_err_split_vs_cublas_fp64"] = float((res["C_split"] - ref).norm() / rn)
        res["rel_err_native_vs_cublas_fp64"] = float((res["C_native"] - ref).norm() / rn)
        res["split_fp8_equals_split_bf16"] = bool(torch.equal(res["C_split"],
                                                              res["C_split_bf16"]))
        del ref
        res["speedup"] = round(res["split_tflops"] / res["native_tflops"], 2)
        res["speedup_vs_bf16_engine"] = round(res["split_tflops"] / res["split_bf16_tflops"], 2)
        res["speedup_vs_mma_sync"] = round(res["split_tflops"] / res["split_mma_sync_tflops"], 2)
        # tensor work actually issued: `pairs` slice products of 2*n^3 each
        # (e4m3 for the default engine, bf16 for the bf16 engine)
        res["split_fp8_work_tflops"] = round(res["split_tflops"] * pairs, 1)
        res["split_bf16_work_tflops"] = round(res["split_bf16_tflops"] * pairs, 1)
        res["split_equals_single_weight"] = bool(torch.equal(res["C_split"],
                                                             res["C_split_e4m3_single_weight"]))
        del res["C_split"], res["C_native"], res["C_split_mma_sync"], res["C_split_bf16"]
        del res["C_split_e4m3_single_weight"]
        if n == sizes[-1] or n <= 4096:
            # row-scaled variant (accuracy only)
            k = torch.randint(-20, 21, (n, 1), device="cuda", generator=g).to(torch.float64)
            As = A * torch.exp2(k)
            Cn, Cs = C0.clone(), C0.clone()
            rp.check(L.b200_gemm_f64(As.data_ptr(), B.data_ptr(), Cn.data_ptr(), n, n, n, 1.5,
                                     1.2, None, s))
            rp.check(L.b200_gemm_split(As.data_ptr(), B.data_ptr(), Cs.data_ptr(), n, n, n,
                                       1.5, 1.2, ws.data_ptr(), ws_bytes, None, s))
            torch.cuda.synchronize()
            res["row_scaled_rel_err"] = float((Cs - Cn).norm() / Cn.norm())
        st = L.b200_workspace_status(ws.data_ptr(), ws_bytes, s)
        res["workspace_status"] = "ok" if st == 0 else f"error {st}: {rp.last_error()}"
        out.append(res)
        del A, B, C0, ws
        torch.cuda.empty_cache()
    out.append(measure_gemm_suite_shape(torch, rp, stream, sizes[-1], seed))
    return out


def measure_gemm_suite_shape(torch, rp, stream, n, seed):
    """The suite's own GEMM shape (POLYBENCH_GEMM.cpp: nk = 1.2 ni) at ni = nj
    = n: C = A*B with K = 1.2 n (9830 at n = 8192, two exact FP32 chunks),
    split precision against native FP64 and cuBLAS FP64."""
    L = rp.b200()
    s = stream.cuda_stream
    k = int(1.2 * n)
    g = torch.Generator(device="cuda").manual_seed(seed + 7 * n)
    A = torch.rand(n, k, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand(k, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    wb = L.b200_gemm_split_workspace_bytes(n, n, k, None)
    ws = torch.zeros(wb, dtype=torch.uint8, device="cuda")
    res = {"m": n, "n": n, "k": k, "shape": "suite GEMM (nk = 1.2 ni)"}
    Cs = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    Cn = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    for name, C, fn in (("split", Cs, lambda: L.b200_gemm_split(
                            A.data_ptr(), B.data_ptr(), Cs.data_ptr(), n, n, k, 1.0, 0.0,
                            ws.data_ptr(), wb, None, s)),
                        ("native", Cn, lambda: L.b200_gemm_f64(
                            A.data_ptr(), B.data_ptr(), Cn.data_ptr(), n, n, k, 1.0, 0.0,
                            None, s))):
        rp.check(fn(), name)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rp.check(fn(), name)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        res[f"{name}_ms"] = round(t * 1e3, 3)
        res[f"{name}_tflops"] = round(2.0 * n * n * k / t / 1e12, 3)
    ref = torch.matmul(A, B)
    rn = ref.norm()
    res["rel_err_split_vs_cublas_fp64"] = float((Cs - ref).norm() / rn)
    res["rel_err_native_vs_cublas_fp64"] = float((Cn - ref).norm() / rn)
    res["rel_err_split_vs_native"] = float((Cs - Cn).norm() / Cn.norm())
    res["speedup"] = round(res["split_tflops"] / res["native_tflops"], 2)
    st = L.b200_workspace_status(ws.data_ptr(), wb, s)
    res["workspace_status"] = "ok" if st == 0 else f"error {st}: {rp.last_error()}"
    del A, B, Cs, Cn, ref, ws
    torch.cuda.empty_cache()
    return res


def measure_3mm(torch, rp, stream, n=2048, seed=4793):
    """Polybench 3MM, square N: E = A*B, F = C*D, G = E*F with entries uniform
    in [-1, 1); native FP64 (b200_polybench_3mm) against three split-precision
    products (b200_gemm_split, alpha 1, beta 0), TFLOP/s at 3 * 2 N^3 and the
    split G's relative Frobenius error against the native G."""
    L = rp.b200()
    s = stream.cuda_stream
    g = torch.Generator(device="cuda").manual_seed(seed + 3 * n)
    A, B, C, D = (torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
                  for _ in range(4))
    E, F, G = (torch.zeros(n, n, dtype=torch.float64, device="cuda") for _ in range(3))
    Es, Fs, Gs = (torch.zeros(n, n, dtype=torch.float64, device="cuda") for _ in range(3))
    wb = L.b200_gemm_split_workspace_bytes(n, n, n, None)
    ws = torch.zeros(wb, dtype=torch.uint8, device="cuda")
    P = lambda t: t.data_ptr()

    def native():
        return L.b200_polybench_3mm(P(A), P(B), P(C), P(D), P(E), P(F), P(G), n, n, n, n, n,
                                    None, s)

    def split():
        for x, y, z in ((A, B, Es), (C, D, Fs), (Es, Fs, Gs)):
            rc = L.b200_gemm_split(P(x), P(y), P(z), n, n, n, 1.0, 0.0, P(ws), wb, None, s)
            if rc != 0:
                return rc
        return 0

    res = {"n": n}
    for name, fn in (("native", native), ("split", split)):
        rp.check(fn(), name)  # warm-up
        best = None
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rp.check(fn(), name)
            e1.record(stream)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            best = t if best is None else min(best, t)
        res[f"{name}_ms"] = round(best * 1e3, 3)
        res[f"{name}_tflops"] = round(3 * 2.0 * n ** 3 / best / 1e12, 3)
    res["rel_err_vs_fp64"] = float((Gs - G).norm() / G.norm())
    res["speedup"] = round(res["split_tflops"] / res["native_tflops"], 2)
    del A, B, C, D, E, F, G, Es, Fs, Gs, ws
    torch.cuda.empty_cache()
    return res


BATCH_KERNELS = ["Stream_COPY", "Stream_MUL", "Stream_ADD", "Stream_TRIAD", "Stream_DOT",
                 "Lcals_HYDRO_1D", "Lcals_HYDRO_2D", "Lcals_EOS", "Lcals_FIRST_DIFF",
                 "Lcals_INT_PREDICT", "Lcals_FIRST_MIN", "Apps_DEL_DOT_VEC_2D", "Apps_VOL3D",
                 "Apps_ENERGY", "Apps_PRESSURE", "Basic_DAXPY", "Basic_INIT3",
                 "Basic_MULADDSUB", "Lcals_DIFF_PREDICT", "Lcals_PLANCKIAN"]


def measure_graph_batch(rp, seed, reps=100):
    """The 20-kernel small-size suite: sizes log-uniform in [2^12, 2^18] per
    kernel (seeded), FP64 uniform [0.5, 1.5) data, `reps` reps.  The whole
    group's rep loop runs once as individual library calls and as one
    captured CUDA graph (one branch per kernel, branches concurrent; also a
    single-chain graph), with the library's default launch shapes and again
    with shapes the autotuner measured for these kernels and sizes."""
    import random
    import tempfile
    rng = random.Random(seed)
    sizes = {k: int(round(2.0 ** rng.uniform(12.0, 18.0))) for k in BATCH_KERNELS}
    base = ["--graph-batch", str(reps), "-k", *BATCH_KERNELS, "--size-map",
            *[f"{k}={n}" for k, n in sizes.items()], "--init", "uniform", "--seed", str(seed)]
    out = {"kernels": len(BATCH_KERNELS), "reps": reps, "sizes": sizes}
    with tempfile.TemporaryDirectory() as tmp:
        table = os.path.join(tmp, "autotuned.txt")
        for label, extra in (("default_shapes", []), ("autotuned", ["--autotune", table])):
            r = rp.graph_batch(base + extra)
            out[label] = {
                "launch_time_ms": round(r["launch_time_s"] * 1e3, 3),
                "graph_time_ms": round(r["graph_time_s"] * 1e3, 3),
                "graph_serial_time_ms": round(r["graph_serial_time_s"] * 1e3, 3),
                "per_rep_launch_us": round(r["launch_time_s"] / reps * 1e6, 2),
                "per_rep_graph_us": round(r["graph_time_s"] / reps * 1e6, 2),
                "launches_per_rep": r["launches_per_rep"],
                "speedup": round(r["launch_time_s"] / r["graph_time_s"], 2),
                "speedup_serial_graph": round(r["launch_time_s"] / r["graph_serial_time_s"], 2),
            }
        shapes = {}
        for line in open(table):
            f = line.split("#", 1)[0].split()
            if f:
                shapes[f[0]] = " ".join(f[3:]) or "default"
        out["autotuned"]["shapes"] = shapes
    return out


def measure_fp64_peak(torch, rp, stream):
    """FP64 FMA rate of this GPU, measured two ways in this run: the library's
    DFMA probe (independent FMA chains, best of 4) and the native FP64 GEMM
    (b200_gemm_f64, 2048^3, best of 3: all DFMA).  The higher of the two is
    the FP64 peak the FP64-bound kernels are measured against."""
    import ctypes
    L = rp.b200()
    out = torch.empty(int(L.b200_probe_dfma_threads()), dtype=torch.float64, device="cuda")
    cnt = ctypes.c_int64(0)
    probe = 0.0
    for _ in range(4):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rp.check(L.b200_probe_dfma(out.data_ptr(), 512, ctypes.byref(cnt), stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        probe = max(probe, cnt.value / (e0.elapsed_time(e1) / 1e3))
    n = 2048
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g)
    B = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g)
    C = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    gemm = 0.0
    for _ in range(4):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rp.check(L.b200_gemm_f64(A.data_ptr(), B.data_ptr(), C.data_ptr(), n, n, n, 1.0, 0.0,
                                 None, stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        gemm = max(gemm, float(n) ** 3 / (e0.elapsed_time(e1) / 1e3))
    best = max(probe, gemm)
    return {"fma_per_s": best, "gflops": 2.0 * best / 1e9,
            "probe_gflops": round(2.0 * probe / 1e9, 1), "dgemm_gflops": round(2.0 * gemm / 1e9, 1)}


# suite options of the e2e leg per kernel (tuning, time steps)
E2E_SUITE_ARGS = {"Polybench_JACOBI_2D": ["-t", "default", "--polybench_tsteps", 50],
                  "Polybench_HEAT_3D": ["-t", "default", "--polybench_tsteps", 20],
                  "Polybench_FDTD_2D": ["-t", "default", "--polybench_tsteps", 100],
                  "Algorithm_SCAN": ["-t", "int64"]}


def host_link_info(torch):
    """Copy-engine rates between pinned host memory and the device (256 MiB,
    best of 3) and the host's NUMA layout, recorded beside the e2e number."""
    nb = 256 << 20
    h = torch.empty(nb, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nb, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nb, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nb, dtype=torch.uint8, device="cuda")

    def best(fn):
        t = 1e9
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            t = min(t, e0.elapsed_time(e1) / 1e3)
        return t

    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def both():
        cur = torch.cuda.current_stream()
        s1.wait_stream(cur)
        s2.wait_stream(cur)
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)
        cur.wait_stream(s1)
        cur.wait_stream(s2)

    info = {"h2d_gbs": round(nb / best(lambda: d.copy_(h, non_blocking=True)) / 1e9, 1),
            "d2h_gbs": round(nb / best(lambda: h2.copy_(d, non_blocking=True)) / 1e9, 1),
            "both_directions_gbs_each": round(nb / best(both) / 1e9, 1)}
    try:
        nodes = sorted(x for x in os.listdir("/sys/devices/system/node") if x.startswith("node"))
        info["numa_nodes"] = len(nodes)
        info["cpus_of_numa_nodes"] = {n: open(f"/sys/devices/system/node/{n}/cpulist").read().strip()
                                      for n in nodes}
    except OSError:
        pass
    del h, h2, d, d2
    return info


def run_e2e(torch, rp, args, peaks):
    """The metric end to end through the Base_GB300 suite layer (rp_run, the
    path a user of the suite calls) with host-resident data (--host-data):
    the kernels' arrays live in pinned host memory and every rep's timed
    work includes moving its inputs from host memory and its outputs back --
    streaming kernels (EOS, FIRST_DIFF, FIRST_MIN, the int64 SCAN) read and
    write host memory themselves, the others (HYDRO_2D, DEL_DOT_VEC_2D,
    JACOBI_2D, HEAT_3D) copy their arrays in and out around each rep.  Time
    per rep = the suite's rep-loop time / reps."""
    reps = max(2, min(args.steps, 5))
    fr, per, h2d, d2h = [], [], 0, 0
    for kname, size in workload_kernels(args.workload, args.kernels):
        opts = E2E_SUITE_ARGS.get(kname, ["-t", "default"])
        table = ["--tuning-table", TUNING_TABLE] if args.tuning_table else []
        r = rp.run_suite(["--size", size, "--checkrun", reps, "-k", kname, "--init", "uniform",
                          "--seed", args.seed, "--host-data", "--disable-warmup", *table,
                          *opts])[0]
        t = r["min_time_s"] / r["reps"]
        f = r["bytes_per_rep"] / t / 1e9 / peaks["hbm_gbs"]
        fr.append(f)
        h2d += r["h2d_bytes_per_rep"]
        d2h += r["d2h_bytes_per_rep"]
        per.append({"kernel": kname, "ms": round(t * 1e3, 4), "frac": round(f, 5),
                    "h2d_bytes": r["h2d_bytes_per_rep"], "d2h_bytes": r["d2h_bytes_per_rep"],
                    "checksum": r["checksum"]})
    return {"value": round(100.0 * geomean(fr), 3), "unit": "%",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "path": "rp_run --host-data (the Base_GB300 suite layer, arrays in pinned host "
                    "memory)",
            "link": host_link_info(torch), "per_kernel": per}


# --------------------------------------------------------------------------
# CPU arms
# --------------------------------------------------------------------------

def cpu_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_cpu(workload, seed, threads, peaks, only=None):
    """The suite's Base_OpenMP loops (oracle restatement), one rep per kernel
    at the workload's full size; returns the metric and per-kernel times."""
    import oracle
    oracle.build()
    fr, per = [], []
    for kname, size in workload_kernels(workload, only):
        kw = dict(WORKLOAD_ORACLE_ARGS.get(kname, {}))
        kw.update(WORKLOADS[workload].get("params", {}).get(kname, {}))
        r = oracle.run(kname, size=size, reps=1, init="uniform", seed=seed,
                       threads=threads, skip_checksum=True, **kw)
        gbs = r["bytes_per_rep"] / max(r["time_s"], 1e-9) / 1e9
        fr.append(gbs / peaks["hbm_gbs"])
        per.append({"kernel": kname, "s": r["time_s"], "gbs": gbs})
    return 100.0 * geomean(fr), per


# oracle arguments of the CPU baseline per kernel (time steps, int64 scan)
WORKLOAD_ORACLE_ARGS = {"Polybench_JACOBI_2D": {"tsteps": 50},
                        "Polybench_HEAT_3D": {"tsteps": 20},
                        "Algorithm_SCAN": {"variant": 1}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=4793)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tuning-table", type=int, default=1,
                    help="1 (default): launch shapes from rajaperf_gb300/tuning/gb300.txt "
                         "(autotuned on GB300 for these sizes); 0: library defaults")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the host-buffer end-to-end leg")
    ap.add_argument("--kernels", type=lambda s: s.split(","), default=None,
                    help="comma list: run only these kernels of the workload")
    ap.add_argument("--gemm", choices=["auto", "on", "off"], default="auto",
                    help="split-precision vs native FP64 GEMM leg (auto: on for one "
                         "rank and the default workload without --kernels)")
    ap.add_argument("--gemm-sizes", type=lambda s: [int(x) for x in s.split(",")],
                    default=[1024, 4096, 8192], help="square sizes of the GEMM leg")
    ap.add_argument("--extras", choices=["auto", "on", "off", "bw", "batch"], default="auto",
                    help="every 1-D kernel at 2^27 elements and the 20-kernel graph batch "
                         "(auto: on for one rank and the default workload without "
                         "--kernels)")
    ap.add_argument("--bw-size", type=int, default=1 << 27,
                    help="element count of the all-kernels bandwidth leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    peaks = load_peaks()
    desc = WORKLOADS[args.workload]["description"]
    config = {"workload": args.workload, "description": desc,
              "kernels": [k for k, _ in workload_kernels(args.workload, args.kernels)],
              "l2": "flushed before every kernel: 256 MiB write, then two 256 MiB reads "
                    "of a second buffer (no dirty flush lines left to write back)",
              "init": f"uniform [0.5,1.5) seed {args.seed}",
              "launch_shapes": ("rajaperf_gb300/tuning/gb300.txt (autotuned on GB300)"
                                if args.tuning_table else "library defaults")}
    metric = "geomean % of measured HBM copy peak over kernels (suite Bytes/rep)"

    if args.impl == "reference":
        if rank != 0:
            return
        cores = cpu_cores()
        vals, per = [], []
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            v, per = run_cpu(args.workload, args.seed, cores, peaks, args.kernels)
            vals.append(v)
        wall = time.perf_counter() - t0
        v = sum(vals) / len(vals)
        line = {"impl": "reference", "metric": metric, "value": round(v, 4), "unit": "%",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(1e3 * wall / max(1, args.steps), 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": round(v, 4), "unit": "%", "cores": cores,
                                 "kind": "port",
                                 "sample": "suite Base_OpenMP loops (C restatement), one rep "
                                           "per kernel at full size",
                                 "per_kernel": per},
                "e2e": {"value": round(v, 4), "unit": "%", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    res = run_gpu(args, rank, world)
    dist = res.pop("dist")
    gemm = mm3 = None
    if args.gemm == "on" or (args.gemm == "auto" and not args.kernels and world == 1):
        import torch
        import rajaperf_gb300 as rp
        gemm = measure_gemm(torch, rp, torch.cuda.current_stream(), sizes=args.gemm_sizes)
        mm3 = measure_3mm(torch, rp, torch.cuda.current_stream())
        fp8_peak = measure_fp8_peak(torch)
        for row in gemm:
            row["cublaslt_fp8_dense_tflops"] = fp8_peak
            if fp8_peak and "split_fp8_work_tflops" in row:
                row["split_fp8_work_frac_of_cublaslt_fp8"] = round(
                    row["split_fp8_work_tflops"] / fp8_peak, 3)
            if "split_bf16_work_tflops" in row:
                row["split_bf16_work_frac_of_measured_bf16"] = round(
                    row["split_bf16_work_tflops"] / peaks["bf16_tflops"], 3)
    bw27 = batch = None
    extras = args.extras
    if extras == "auto":
        extras = "on" if (not args.kernels and world == 1) else "off"
    if extras in ("on", "bw") and rank == 0:
        import torch
        import rajaperf_gb300 as rp
        bw27 = measure_bw27(torch, rp, torch.cuda.current_stream(), peaks,
                            res["fp64"]["fma_per_s"], args.seed, n=args.bw_size)
    if extras in ("on", "batch") and rank == 0:
        import rajaperf_gb300 as rp
        batch = measure_graph_batch(rp, args.seed)
    value = res["value"]
    if dist:
        res["step_s"], value = combine_ranks(dist, res["step_s"], value, "cuda")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cores = cpu_cores()
        cv, per = run_cpu(args.workload, args.seed, cores, peaks, args.kernels)
        cpu = {"value": round(cv, 4), "unit": "%", "cores": cores, "kind": "port",
               "sample": "suite Base_OpenMP loops (C restatement), one rep per kernel at "
                         "the workload's full size", "per_kernel": per}
    line = {
        "metric": metric, "value": round(value, 3), "unit": "%", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(res["step_s"] * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config, "e2e": res["e2e"], "roofline": res["roofline"],
        "cpu_baseline": cpu, "clocks": res["clocks"], "gpu_launches": res["launches"],
        "fp64_peak_gflops": round(res["fp64"]["gflops"], 1),
        "gemm_split_vs_fp64": gemm,
        "3mm_split_vs_fp64": mm3,
        "bandwidth_all_1d": bw27,
        "graph_batch": batch,
        "per_kernel": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in p.items()}
                       for p in res["per_kernel"]],
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
