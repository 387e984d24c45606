#!/usr/bin/env python3
"""Benchmark of the Base_GB300 loop-kernel hot path.

Metric: geomean over the workload's kernels of achieved HBM bandwidth as a
fraction of the measured copy peak (percent), bandwidth being the suite's
Bytes/rep divided by the time of one rep (scripts/caliper_graph/plot.py:15-31
of the suite).  One "step" runs every kernel of the workload once.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload bandwidth_stencil|stream]

* value: kernels timed with CUDA events on the launching stream, inputs
  resident in HBM, L2 flushed (a 256 MiB write) before every kernel.
* e2e: the same metric through the C ABI with host buffers: each step copies
  the kernel's inputs from pinned host memory, runs it and reads the
  result back, all inside the timed region.
* cpu_baseline / --impl reference: the suite's Base_OpenMP loops (the CPU
  oracle's restatement) on all host cores, one rep per kernel at full size.
Under torchrun (N>1) every rank runs its own replica (the path has no data
exchange); value is summed over ranks.
"""
from __future__ import annotations

import argparse
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
L2_FLUSH_BYTES = 256 << 20


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": HBM_FALLBACK_GBS, "source": "fallback"}


def load_traffic() -> dict:
    """Per-kernel DRAM bytes per launch from committed ncu summaries."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    return json.load(open(p)) if os.path.exists(p) else {}


# --------------------------------------------------------------------------
# workload cases
# --------------------------------------------------------------------------

class Case:
    """One kernel of the workload: device buffers, one rep, bytes per rep."""
    name = ""
    launches = 1

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

    # subclasses define: inputs (list of device tensors copied H2D in e2e),
    # outputs (tensors read back in e2e), bytes_per_rep, run(stream)
    def inputs(self):
        return []

    def outputs(self):
        return []


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

        def inputs(self):
            return [self.b, self.c]

        def outputs(self):
            return [self.a]

        def run(self, s):
            return self.L.b200_stream_triad(self.a.data_ptr(), self.b.data_ptr(),
                                            self.c.data_ptr(), 0.5, self.n, None, s)

    class Copy(Case):
        name = "Stream_COPY"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.c = self.zeros(n)
            self.bytes_per_rep = 16 * n

        def inputs(self):
            return [self.a]

        def outputs(self):
            return [self.c]

        def run(self, s):
            return self.L.b200_stream_copy(self.a.data_ptr(), self.c.data_ptr(), self.n,
                                           None, s)

    class Mul(Case):
        name = "Stream_MUL"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.b = self.zeros(n)
            self.c = self.uniform(n)
            self.bytes_per_rep = 16 * n

        def inputs(self):
            return [self.c]

        def outputs(self):
            return [self.b]

        def run(self, s):
            return self.L.b200_stream_mul(self.b.data_ptr(), self.c.data_ptr(), 0.5, self.n,
                                          None, s)

    class Add(Case):
        name = "Stream_ADD"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.b = self.uniform(n)
            self.c = self.zeros(n)
            self.bytes_per_rep = 24 * n

        def inputs(self):
            return [self.a, self.b]

        def outputs(self):
            return [self.c]

        def run(self, s):
            return self.L.b200_stream_add(self.a.data_ptr(), self.b.data_ptr(),
                                          self.c.data_ptr(), self.n, None, s)

    class Dot(Case):
        name = "Stream_DOT"

        def __init__(self, torch, rp, seed, n):
            super().__init__(torch, rp, seed)
            self.n = n
            self.a = self.uniform(n)
            self.b = self.uniform(n)
            self.acc = self.zeros(1)
            self.ws_bytes = self.L.b200_reduce_workspace_bytes(n, None)
            self.ws = self.zeros(self.ws_bytes, dtype=torch.uint8)
            self.bytes_per_rep = 16 * n + 16

        def inputs(self):
            return [self.a, self.b]

        def outputs(self):
            return [self.acc]

        def run(self, s):
            return self.L.b200_stream_dot(self.a.data_ptr(), self.b.data_ptr(), self.n, 0.0,
                                          self.acc.data_ptr(), self.ws.data_ptr(),
                                          self.ws_bytes, None, s)

    return {"Stream_COPY": Copy, "Stream_MUL": Mul, "Stream_ADD": Add,
            "Stream_TRIAD": Triad, "Stream_DOT": Dot}


# workload -> list of (kernel, size, oracle kwargs for the CPU baseline)
WORKLOADS = {
    "stream": {
        "description": "Stream COPY/MUL/ADD/TRIAD/DOT, FP64, N=2^27 per array",
        "kernels": [("Stream_COPY", 1 << 27), ("Stream_MUL", 1 << 27),
                    ("Stream_ADD", 1 << 27), ("Stream_TRIAD", 1 << 27),
                    ("Stream_DOT", 1 << 27)],
    },
}
DEFAULT_WORKLOAD = "stream"


def build_cases(torch, rp, workload, seed):
    registry = {}
    registry.update(_stream_cases())
    cases = []
    for kname, size in WORKLOADS[workload]["kernels"]:
        if kname in registry:
            cases.append(registry[kname](torch, rp, seed, size))
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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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
    cases = build_cases(torch, rp, args.workload, args.seed + rank)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def one_step(timed_events=None):
        for i, c in enumerate(cases):
            flush.zero_()
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
        per_kernel.append({"kernel": c.name, "ms": avg_s * 1e3, "gbs": gbs,
                           "frac": gbs / peaks["hbm_gbs"], "bytes": c.bytes_per_rep})
    step_s = sum(p["ms"] for p in per_kernel) / 1e3
    if dist:
        t = torch.tensor([step_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_s = float(t.item())
    value = 100.0 * geomean([p["frac"] for p in per_kernel])

    # e2e through the C ABI with host buffers
    e2e = run_e2e(torch, rp, cases, s, stream, args, peaks)

    dom = max(per_kernel, key=lambda p: p["ms"])
    tr = traffic.get(dom["kernel"])
    roofline = {"bound": "hbm", "kernel": dom["kernel"], "achieved": round(dom["gbs"], 1),
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(dom["gbs"] / peaks["hbm_gbs"], 4),
                "traffic": (tr["bytes_per_launch"] if tr else None),
                "algorithmic_bytes": dom["bytes"], "peak_source": peaks["source"]}
    return {
        "value": value, "step_s": step_s, "per_kernel": per_kernel, "e2e": e2e,
        "roofline": roofline, "clocks": clocks, "launches": launches, "wall_s": wall,
        "world": world, "dist": dist,
    }


def run_e2e(torch, rp, cases, s, stream, args, peaks):
    """Host buffers -> H2D -> kernel -> D2H, timed with events."""
    host_in = [[x.cpu().pin_memory() for x in c.inputs()] for c in cases]
    host_out = [[torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in c.outputs()]
                for c in cases]
    h2d = sum(x.numel() * x.element_size() for hs in host_in for x in hs)
    d2h = sum(x.numel() * x.element_size() for hs in host_out for x in hs)
    steps = max(1, min(args.steps, 5))
    times = [[0.0] * len(cases) for _ in range(steps)]
    for k in range(-1, steps):
        for i, c in enumerate(cases):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for dst, src in zip(c.inputs(), host_in[i]):
                dst.copy_(src, non_blocking=True)
            rp.check(c.run(s), c.name)
            for dst, src in zip(host_out[i], c.outputs()):
                dst.copy_(src, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= 0:
                times[k][i] = e0.elapsed_time(e1) / 1e3
    fr = []
    for i, c in enumerate(cases):
        avg = sum(times[k][i] for k in range(steps)) / steps
        fr.append(c.bytes_per_rep / avg / 1e9 / peaks["hbm_gbs"])
    return {"value": round(100.0 * geomean(fr), 3), "unit": "% of HBM peak",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}


# --------------------------------------------------------------------------
# CPU arms
# --------------------------------------------------------------------------

def cpu_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_cpu(workload, seed, threads, peaks):
    """The suite's Base_OpenMP loops (oracle restatement), one rep per kernel
    at the workload's full size; returns the metric and per-kernel times."""
    import oracle
    oracle.build()
    fr, per = [], []
    for kname, size in WORKLOADS[workload]["kernels"]:
        kw = dict(WORKLOAD_ORACLE_ARGS.get(kname, {}))
        r = oracle.run(kname, size=size, reps=1, init="uniform", seed=seed,
                       threads=threads, skip_checksum=True, **kw)
        gbs = r["bytes_per_rep"] / max(r["time_s"], 1e-9) / 1e9
        fr.append(gbs / peaks["hbm_gbs"])
        per.append({"kernel": kname, "s": r["time_s"], "gbs": gbs})
    return 100.0 * geomean(fr), per


WORKLOAD_ORACLE_ARGS = {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=4793)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    peaks = load_peaks()
    desc = WORKLOADS[args.workload]["description"]
    config = {"workload": args.workload, "description": desc,
              "kernels": [k for k, _ in WORKLOADS[args.workload]["kernels"]],
              "l2": "flushed (256 MiB write) before every kernel",
              "init": f"uniform [0.5,1.5) seed {args.seed}"}
    metric = "geomean % of measured HBM copy peak over kernels (suite Bytes/rep)"

    if args.impl == "reference":
        if rank != 0:
            return
        cores = cpu_cores()
        vals, per = [], []
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            v, per = run_cpu(args.workload, args.seed, cores, peaks)
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
    value = res["value"]
    if dist:
        import torch
        t = torch.tensor([value], device="cuda", dtype=torch.float64)
        dist.all_reduce(t)
        value = float(t.item())
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cores = cpu_cores()
        cv, per = run_cpu(args.workload, args.seed, cores, peaks)
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
        "per_kernel": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in p.items()}
                       for p in res["per_kernel"]],
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
