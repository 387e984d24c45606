"""The problem-size sweep (rajaperf_gb300/sweep.py), in the layout of the
suite's scripts/sweep_size.sh: directories RAJAPerf_<i>/SIZE_<9 digits>, one
run per size and executable with --size and the extra arguments, the output
in raja-perf-sweep.txt after the command line, and the script's checks.  A
stand-in executable (a shell script) records its arguments and writes a
timing report in the suite's layout, so no GPU is needed."""
import csv
import os
import stat
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = """#!/bin/sh
echo "args: $@"
size=$2
printf 'Mean Runtime Report (sec.) , , \\n' > RAJAPerf-timing-Average.csv
printf 'Kernel   , Base_GB300 , Base_GB300\\n' >> RAJAPerf-timing-Average.csv
printf 'Kernel   , default    , graph     \\n' >> RAJAPerf-timing-Average.csv
printf 'Stream_TRIAD , 0.%06d , Not run\\n' "$size" >> RAJAPerf-timing-Average.csv
"""


def run(tmp_path, *args):
    return subprocess.run([sys.executable, "-m", "rajaperf_gb300.sweep", *args], cwd=tmp_path,
                          capture_output=True, text=True,
                          env=dict(os.environ, PYTHONPATH=ROOT))


@pytest.fixture
def fake(tmp_path):
    p = tmp_path / "fake-exe"
    p.write_text(FAKE)
    p.chmod(p.stat().st_mode | stat.S_IXUSR)
    return str(p)


def test_layout_and_arguments(tmp_path, fake):
    r = run(tmp_path, "-x", fake, "-x", fake, "-m", "1000", "-M", "9000", "-r", "3",
            "--summary", "sum.csv", "--", "-k", "Stream_TRIAD", "--checkrun", "2")
    assert r.returncode == 0, r.stderr
    assert "Sweeping from size 1000 to 9000 with ratio 3" in r.stdout
    for i in (0, 1):
        got = sorted(os.listdir(tmp_path / f"RAJAPerf_{i}"))
        assert got == ["SIZE_000001000", "SIZE_000003000", "SIZE_000009000"]
        log = (tmp_path / f"RAJAPerf_{i}" / "SIZE_000003000" / "raja-perf-sweep.txt").read_text()
        first, second = log.splitlines()[:2]
        assert first == f"{fake} --size 3000 -k Stream_TRIAD --checkrun 2"
        assert second == "args: --size 3000 -k Stream_TRIAD --checkrun 2"
    rows = list(csv.reader(open(tmp_path / "sum.csv")))
    assert rows[0] == ["size", "executable", "kernel", "variant-tuning", "mean_runtime_s"]
    body = [(int(a), int(b), c, d, float(e)) for a, b, c, d, e in rows[1:]]
    assert (3000, 1, "Stream_TRIAD", "Base_GB300-default", 0.003) in body
    assert len(body) == 6  # "Not run" cells are skipped


@pytest.mark.parametrize("args,msg", [
    (["-m", "0"], "Invalid size-min: 0"),
    (["-M", "-5"], "Invalid size-max: -5"),
    (["-r", "1"], "Invalid size-ratio: 1"),
    (["-m", "100", "-M", "10"], "Invalid sizes size-min: 100, size-max: 10"),
    (["-x", "no-such-exe"], "Executable not found: no-such-exe"),
])
def test_checks(tmp_path, fake, args, msg):
    base = [] if "-x" in args else ["-x", fake]
    r = run(tmp_path, *base, *args)
    assert r.returncode == 1 and msg in r.stderr
    assert not (tmp_path / "RAJAPerf_0").exists()


def test_refuses_an_existing_directory(tmp_path, fake):
    (tmp_path / "RAJAPerf_0").mkdir()
    r = run(tmp_path, "-x", fake, "-m", "10", "-M", "10")
    assert r.returncode == 1 and "Directory exists: RAJAPerf_0" in r.stderr
