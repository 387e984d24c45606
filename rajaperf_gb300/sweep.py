"""Problem-size sweep over one or more suite executables, in the layout of the
suite's own scripts/sweep_size.sh: for every executable i a directory
RAJAPerf_<i>, for every size (size-min, size-min * ratio, ... up to size-max)
a directory SIZE_<size, 9 digits> inside it, where the executable runs with
`--size <size>` plus the extra arguments and writes its reports; its output
goes to raja-perf-sweep.txt there, preceded by the command line.

    python -m rajaperf_gb300.sweep -x rajaperf_gb300/bin/rajaperf-gb300 \\
        [-x other-exe ...] [--size-min 10000] [--size-max 1000000] \\
        [--size-ratio 2] [-- <suite arguments>]

The defaults are the suite script's (10000 .. 1000000, ratio 2).  Checks as
there: sizes positive, ratio above 1, min not above max, every executable an
existing executable file, and no RAJAPerf_<i> directory already present.
With --summary FILE the per-size timing reports (RAJAPerf-timing-Average.csv,
the suite's name: each kernel's run time in seconds, averaged over passes)
are gathered into one CSV: size, executable, kernel, variant-tuning, seconds.
"""
import argparse
import csv
import os
import subprocess
import sys


def sizes(size_min, size_max, ratio):
    s = size_min
    while s <= size_max:
        yield s
        s *= ratio


def parse(argv):
    extra = []
    if "--" in argv:
        i = argv.index("--")
        argv, extra = argv[:i], argv[i + 1:]
    ap = argparse.ArgumentParser(prog="python -m rajaperf_gb300.sweep",
                                 description="problem-size sweep (suite layout)")
    ap.add_argument("-x", "--executable", action="append", default=[], dest="executables")
    ap.add_argument("-m", "--size-min", type=int, default=10000)
    ap.add_argument("-M", "--size-max", type=int, default=1000000)
    ap.add_argument("-r", "--size-ratio", type=int, default=2)
    ap.add_argument("--summary", default=None,
                    help="write one CSV of the timing reports over every size")
    args = ap.parse_args(argv)
    args.extra = extra
    return args


def check(args):
    if args.size_min <= 0:
        return f"Invalid size-min: {args.size_min}"
    if args.size_max <= 0:
        return f"Invalid size-max: {args.size_max}"
    if args.size_ratio <= 1:
        return f"Invalid size-ratio: {args.size_ratio}"
    if args.size_min > args.size_max:
        return f"Invalid sizes size-min: {args.size_min}, size-max: {args.size_max}"
    if not args.executables:
        return "No executable given (-x)"
    for exe in args.executables:
        if not os.path.isfile(exe):
            return f"Executable not found: {exe}"
        if not os.access(exe, os.X_OK):
            return f"Executable not executable: {exe}"
    for i in range(len(args.executables)):
        if os.path.exists(f"RAJAPerf_{i}"):
            return f"Directory exists: RAJAPerf_{i}"
    return None


def read_timing(path):
    """(kernel, column, seconds) rows of a suite timing CSV: line 1 title, line
    2 variants, line 3 tunings, then one row per kernel ("Not run" skipped)."""
    with open(path) as f:
        rows = [[c.strip() for c in r] for r in csv.reader(f)]
    if len(rows) < 3:
        return []
    variants, tunings = rows[1][1:], rows[2][1:]
    out = []
    for r in rows[3:]:
        if not r or not r[0]:
            continue
        for v, t, cell in zip(variants, tunings, r[1:]):
            try:
                out.append((r[0], f"{v}-{t}", float(cell)))
            except ValueError:
                pass
    return out


def main(argv=None):
    args = parse(sys.argv[1:] if argv is None else argv)
    print("Running sweep with executables: " + " ".join(args.executables))
    print(f"Sweeping from size {args.size_min} to {args.size_max} with ratio {args.size_ratio}")
    print("extra args to executables are: " + " ".join(args.extra))
    err = check(args)
    if err:
        print(err, file=sys.stderr)
        return 1
    exes = [os.path.abspath(e) for e in args.executables]
    for i in range(len(exes)):
        os.mkdir(f"RAJAPerf_{i}")
    summary = []
    rc = 0
    for size in sizes(args.size_min, args.size_max, args.size_ratio):
        for i, exe in enumerate(exes):
            d = os.path.join(f"RAJAPerf_{i}", f"SIZE_{size:09d}")
            os.mkdir(d)
            cmd = [exe, "--size", str(size)] + args.extra
            line = " ".join(cmd)
            print(line)
            with open(os.path.join(d, "raja-perf-sweep.txt"), "w") as log:
                log.write(line + "\n")
                log.flush()
                r = subprocess.run(cmd, cwd=d, stdout=log, stderr=subprocess.STDOUT)
            rc = rc or r.returncode
            t = os.path.join(d, "RAJAPerf-timing-Average.csv")
            if args.summary and os.path.exists(t):
                summary += [(size, i, k, col, sec) for k, col, sec in read_timing(t)]
    if args.summary:
        with open(args.summary, "w", newline="") as f:
            w = csv.writer(f)
            w.writerow(["size", "executable", "kernel", "variant-tuning", "mean_runtime_s"])
            w.writerows(summary)
    return rc


if __name__ == "__main__":
    sys.exit(main())
