"""Every Base_GB300 kernel through the C++ suite layer (the rajaperf-gb300
driver's code path) against the RAJA Performance Suite's own Base_Seq
checksums (tests/golden/ref_checksums.json), for the "default" (one library
call per rep) and "graph" (rep loop replayed as a CUDA graph) tunings.

Tolerances: relative 1e-12 for element-wise and stencil kernels; exact for
FIRST_MIN's location; for the sums (DOT, REDUCE_SUM, SCAN) the reassociation
bound (n + log2 n + reps) * 2^-53 * sum|terms| relative to the checksum."""
import csv
import json
import math
import os

import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu

RECORDS = json.load(open(gu.GOLDEN))["records"]
KERNELS = sorted({r["kernel"] for r in RECORDS})
SUMS = {"Stream_DOT", "Algorithm_REDUCE_SUM", "Algorithm_SCAN", "Basic_MULTI_REDUCE"}


def _check(kernel, rec, got):
    what = f"{kernel} size={rec['size']} reps={rec['reps']}"
    assert got["actual_size"] == rec["actual_size"], what
    assert got["bytes_per_rep"] == rec["bytes_per_rep"], what
    assert got["flops_per_rep"] == rec["flops_per_rep"], what
    want = rec["checksum"]
    if kernel == "Lcals_FIRST_MIN":
        assert got["checksum"] == want, what
    elif kernel in SUMS:
        n = max(rec["actual_size"], 1)
        bound = (n + math.ceil(math.log2(n + 1)) + rec["reps"]) * gu.U * abs(want) + 1e-300
        assert abs(got["checksum"] - want) <= bound, (what, got["checksum"], want)
    else:
        gu.assert_close_rel(got["checksum"], want, what=what)


@pytest.mark.parametrize("kernel", KERNELS)
def test_kernel_matches_suite_base_seq(kernel):
    for rec in [r for r in RECORDS if r["kernel"] == kernel]:
        res = rp.run_suite(["--size", rec["size"], "--checkrun", rec["reps"], "-k", kernel,
                            "-t", "default", "graph", "--disable-warmup",
                            *rec.get("args", [])])
        assert {r["tuning"] for r in res} == {"default", "graph"}, res
        for r in res:
            _check(kernel, rec, r)


@pytest.mark.parametrize("kernel", ["Polybench_GEMM", "Polybench_3MM"])
def test_split_precision_tunings_match_base_seq(kernel):
    for rec in [r for r in RECORDS if r["kernel"] == kernel]:
        res = rp.run_suite(["--size", rec["size"], "--checkrun", rec["reps"], "-k", kernel,
                            "-t", "split_fp8", "split_fp8_graph", "split_bf16",
                            "--disable-warmup"])
        assert len(res) == 3
        for r in res:
            _check(kernel, rec, r)


def test_tuning_table_shapes(tmp_path):
    """Non-default launch shapes from a tuning table keep the checksums."""
    table = tmp_path / "tune.txt"
    lines = [f"{k} 0 -1 block=128 items=2" for k in KERNELS] + ["# comment"]
    table.write_text("\n".join(lines) + "\n")
    for kernel in ["Stream_TRIAD", "Lcals_EOS", "Apps_ENERGY", "Lcals_FIRST_MIN",
                   "Stream_DOT", "Lcals_HYDRO_2D", "Apps_VOL3D"]:
        rec = [r for r in RECORDS if r["kernel"] == kernel and r["size"] == 65537][0]
        res = rp.run_suite(["--size", rec["size"], "--checkrun", rec["reps"], "-k", kernel,
                            "-t", "default", "--disable-warmup", "--tuning-table", str(table)])
        _check(kernel, rec, res[0])


def test_npasses_average_checksum():
    rec = [r for r in RECORDS if r["kernel"] == "Stream_TRIAD" and r["size"] == 1000][0]
    res = rp.run_suite(["--size", 1000, "--checkrun", rec["reps"], "-k", "Stream_TRIAD",
                        "-t", "default", "--npasses", 3, "--disable-warmup"])
    assert res[0]["passes"] == 3
    _check("Stream_TRIAD", rec, res[0])


def test_uniform_mode_matches_oracle():
    import oracle
    for kernel, size, reps in [("Lcals_HYDRO_2D", 4096, 2), ("Apps_DEL_DOT_VEC_2D", 4096, 1),
                               ("Lcals_FIRST_MIN", 100003, 2), ("Polybench_JACOBI_2D", 4096, 1),
                               ("Polybench_HEAT_3D", 4096, 1), ("Lcals_EOS", 100000, 1)]:
        res = rp.run_suite(["--size", size, "--checkrun", reps, "-k", kernel, "-t", "default",
                            "--init", "uniform", "--seed", 11, "--disable-warmup"])
        want = oracle.run(kernel, size=size, reps=reps, init="uniform", seed=11)
        if kernel == "Lcals_FIRST_MIN":
            assert res[0]["checksum"] == want["checksum"]
            assert want["checksum"] == oracle.lib().oracle_first_min_planted_index(11, 100003)
        else:
            gu.assert_close_rel(res[0]["checksum"], want["checksum"], what=kernel)


def test_polybench_tsteps_override():
    import oracle
    for kernel in ["Polybench_JACOBI_2D", "Polybench_HEAT_3D", "Polybench_FDTD_2D"]:
        res = rp.run_suite(["--size", 2000, "--checkrun", 1, "-k", kernel, "-t", "default",
                            "--polybench_tsteps", 7, "--disable-warmup"])
        want = oracle.run(kernel, size=2000, reps=1, tsteps=7)
        gu.assert_close_rel(res[0]["checksum"], want["checksum"], what=kernel)
        assert res[0]["bytes_per_rep"] == want["bytes_per_rep"]


def test_scan_int64_exact():
    import oracle
    for size in [1, 4095, 4096, 4097, 1 << 20, 3_000_001]:
        res = rp.run_suite(["--size", size, "--checkrun", 2, "-k", "Algorithm_SCAN",
                            "-t", "int64", "int64_graph", "--init", "uniform", "--seed", 5,
                            "--disable-warmup"])
        want = oracle.run("Algorithm_SCAN", size=size, reps=2, init="uniform", seed=5,
                          variant=1)
        for r in res:
            assert r["checksum"] == want["checksum"], (size, r["tuning"])


def test_bad_command_lines():
    with pytest.raises(RuntimeError, match="unknown kernel"):
        rp.run_suite(["-k", "NoSuchKernel"])
    with pytest.raises(RuntimeError, match="exclusive"):
        rp.run_suite(["--size", 10, "--sizefact", 2])
    with pytest.raises(RuntimeError, match="not available"):
        rp.run_suite(["-v", "Base_CUDA"])


def test_autotune_table_and_graph_batch(tmp_path):
    """--autotune measures shapes for the selected kernels at their sizes,
    writes a table --tuning-table reads back, and the graph batch runs with
    it; checksums with the tuned shapes still match Base_Seq."""
    table = tmp_path / "autotuned.txt"
    kernels = ["Stream_TRIAD", "Stream_DOT", "Lcals_FIRST_MIN", "Lcals_EOS", "Lcals_HYDRO_2D",
               "Algorithm_SCAN", "Polybench_JACOBI_2D"]
    b = rp.graph_batch(["--graph-batch", 5, "-k", *kernels, "--size", 65537,
                        "--autotune", str(table)])
    assert b["kernels"] == len(kernels) and b["reps"] == 5
    assert b["launch_time_s"] > 0 and b["graph_time_s"] > 0 and b["launches_per_rep"] > 0
    entries = [ln.split("#", 1)[0].split() for ln in table.read_text().splitlines()]
    tuned = {e[0] for e in entries if e}
    # every kernel with more than one candidate shape gets an entry (JACOBI_2D:
    # rows per thread of its column-segment kernel)
    assert tuned == set(kernels), tuned
    for e in entries:
        if e:
            assert e[1] == e[2] and all("=" in kv for kv in e[3:]), e
    for kernel in ["Stream_TRIAD", "Stream_DOT", "Lcals_FIRST_MIN", "Lcals_EOS",
                   "Polybench_JACOBI_2D"]:
        rec = [r for r in RECORDS if r["kernel"] == kernel and r["size"] == 65537][0]
        res = rp.run_suite(["--size", rec["size"], "--checkrun", rec["reps"], "-k", kernel,
                            "-t", "default", "--disable-warmup", "--tuning-table", str(table)])
        _check(kernel, rec, res[0])


def test_report_files(tmp_path):
    """-od writes the suite's report set: timing and speedup CSVs per
    --npasses-combiners entry, the checksum report whose difference column
    is against the first tuning run, the FOM report and the kernel details."""
    out = tmp_path / "rep"
    res = rp.run_suite(["--size", 65537, "--checkrun", 2, "-k", "Stream_TRIAD", "Stream_DOT",
                        "-t", "default", "graph", "--disable-warmup", "--npasses", 2,
                        "--npasses-combiners", "Average", "Minimum", "--refvar", "Base_GB300",
                        "-od", str(out), "-of", "R"])
    names = sorted(p.name for p in out.iterdir())
    assert names == sorted(["R-timing-Average.csv", "R-timing-Minimum.csv",
                            "R-speedup-Average.csv", "R-speedup-Minimum.csv", "R-checksum.txt",
                            "R-fom.csv", "R-kernels.csv", "R-roofline.json"])
    timing = (out / "R-timing-Average.csv").read_text().splitlines()
    assert timing[0].startswith("Mean Runtime Report (sec.) ")
    assert [c.strip() for c in timing[2].split(" , ")[1:]] == ["default", "graph"]
    speed = (out / "R-speedup-Average.csv").read_text().splitlines()
    for row in speed[3:]:
        vals = [float(c) for c in row.split(" , ")[1:]]
        assert vals[0] == 1.0 and vals[1] > 0
    ck = (out / "R-checksum.txt").read_text()
    for r in res:
        assert f"Base_GB300-{r['tuning']}" in ck
    fom = (out / "R-fom.csv").read_text().splitlines()
    assert "base_ref" in fom[3]
    with pytest.raises(RuntimeError, match="not available"):
        rp.run_suite(["--size", 100, "-k", "Stream_TRIAD", "--refvar", "Base_Seq"])


def test_size_sweep_runs_the_suite(tmp_path):
    """rajaperf_gb300.sweep with the suite executable: one run per size, each
    writing its timing report where the sweep gathers it."""
    import subprocess
    import sys
    exe = os.path.join(ROOT, "rajaperf_gb300", "bin", "rajaperf-gb300")
    r = subprocess.run([sys.executable, "-m", "rajaperf_gb300.sweep", "-x", exe, "-m", "4096",
                        "-M", "16384", "-r", "4", "--summary", "sum.csv", "--", "-k",
                        "Stream_TRIAD", "Lcals_FIRST_DIFF", "--checkrun", "2"],
                       cwd=tmp_path, capture_output=True, text=True,
                       env=dict(os.environ, PYTHONPATH=ROOT))
    assert r.returncode == 0, r.stdout + r.stderr
    for size in (4096, 16384):
        d = tmp_path / "RAJAPerf_0" / f"SIZE_{size:09d}"
        assert (d / "RAJAPerf-timing-Average.csv").exists()
    rows = list(csv.reader(open(tmp_path / "sum.csv")))[1:]
    kernels = {(int(s), k) for s, _, k, _, _ in rows}
    assert kernels == {(s, k) for s in (4096, 16384) for k in ("Stream_TRIAD", "Lcals_FIRST_DIFF")}
    assert all(float(v) > 0 for *_, v in rows)
