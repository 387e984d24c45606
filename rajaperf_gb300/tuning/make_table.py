"""Measures the GB300 tuning table for the benchmark's problem sizes.

Runs the suite layer's autotuner (--autotune) for every kernel and size of
the bandwidth/stencil workload, the Stream TRIAD/DOT case at N = 1e6, and
the large set, and writes the winners, one entry per kernel and size, as a
tuning table that --tuning-table loads:

    python -m rajaperf_gb300.tuning.make_table rajaperf_gb300/tuning/gb300.txt

Needs a GB300 (the candidates are timed as graph replays with CUDA events).
"""
from __future__ import annotations

import datetime
import os
import sys
import tempfile

# (kernel, --size, further suite options)
CASES = [
    ("Stream_TRIAD", 1000000, []), ("Stream_DOT", 1000000, []),
    ("Lcals_HYDRO_2D", 4096 * 4096, []), ("Lcals_EOS", 1 << 24, []),
    ("Lcals_FIRST_DIFF", 1 << 24, []), ("Lcals_FIRST_MIN", 1 << 24, []),
    ("Apps_DEL_DOT_VEC_2D", 4096 * 4096, []),
    ("Polybench_JACOBI_2D", 4094 * 4094, ["--polybench_tsteps", 50]),
    ("Algorithm_SCAN", 1 << 26, ["-t", "int64"]),
    ("Stream_COPY", 1 << 28, []), ("Stream_MUL", 1 << 28, []),
    ("Stream_ADD", 1 << 28, []), ("Stream_TRIAD", 1 << 28, []),
    ("Polybench_FDTD_2D", 8191 * 8192, ["--polybench_tsteps", 10]),
    ("Polybench_JACOBI_2D", 16382 * 16382, ["--polybench_tsteps", 4]),
]


def main(out_path: str) -> None:
    root = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, root)
    import rajaperf_gb300 as rp
    import torch
    lines = []
    with tempfile.TemporaryDirectory() as tmp:
        for n, (kernel, size, opts) in enumerate(CASES):
            path = os.path.join(tmp, f"t{n}.txt")
            rp.run_suite(["--size", size, "--checkrun", 1, "-k", kernel, "--init", "uniform",
                          "--disable-warmup", "--autotune", path, *opts])
            if os.path.exists(path):
                lines += [ln.rstrip("\n") for ln in open(path)
                          if ln.strip() and not ln.startswith("#")]
    name = torch.cuda.get_device_name(0)
    head = [f"# GB300 tuning table: autotuned launch shapes for the benchmark sizes",
            f"# device: {name}; measured {datetime.date.today().isoformat()} by",
            "# python -m rajaperf_gb300.tuning.make_table (the suite's --autotune per",
            "# kernel and size; candidates timed as graph replays, best of three)",
            "# <Group_KERNEL> <min_size> <max_size> key=value ...   # measured times"]
    with open(out_path, "w") as f:
        f.write("\n".join(head + lines) + "\n")
    print(out_path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "gb300.txt")
