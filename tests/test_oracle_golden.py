"""The CPU oracle against the RAJA Performance Suite's own Base_Seq results.

tests/golden/ref_checksums.json holds checksums, sizes and Bytes/FLOPs per
rep produced by the suite's own code (oracle/_ref, see make_golden.py).  The
C restatement must reproduce every record bit for bit; where the suite
build is present in this checkout, it is also compared live.
"""
import json
import os

import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_checksums.json")
RECORDS = json.load(open(GOLDEN))["records"]


def option_kwargs(args):
    """oracle.run keywords for a record's further suite options."""
    kw = {}
    for opt, val in zip(args[::2], args[1::2]):
        if opt == "--multi_reduce_num_bins":
            kw["num_bins"] = int(val)
        elif opt == "--multi_reduce_bin_assignment_algorithm":
            kw["bin_algo"] = val
        elif opt == "--halo_width":
            kw["halo_width"] = int(val)
        elif opt == "--halo_num_vars":
            kw["halo_num_vars"] = int(val)
        else:
            raise KeyError(opt)
    return kw


@pytest.mark.parametrize("rec", RECORDS,
                         ids=lambda r: f"{r['kernel']}-{r['size']}x{r['reps']}"
                                       + ("-" + "-".join(r["args"][1::2]) if "args" in r else ""))
def test_oracle_matches_suite_base_seq(rec):
    r = oracle.run(rec["kernel"], size=rec["size"], reps=rec["reps"],
                   **option_kwargs(rec.get("args", [])))
    assert r["actual_size"] == rec["actual_size"]
    assert r["bytes_per_rep"] == rec["bytes_per_rep"]
    assert r["flops_per_rep"] == rec["flops_per_rep"]
    # The golden value is the suite's long double checksum printed with 21
    # digits; the oracle's rounds to the same double.
    assert r["checksum"] == rec["checksum"], (r["checksum"], rec["checksum"])


def test_known_answers_stream_1e6():
    """The suite's CPU-runnable Stream case (N=1e6, 5 reps)."""
    assert oracle.run("Stream_TRIAD", size=1000000, reps=5)["checksum"] == 135.91984956172908
    assert oracle.run("Stream_DOT", size=1000000, reps=5)["checksum"] == 99999.933449605887


@pytest.mark.skipif(not os.path.exists(oracle.REF_EXE), reason="suite build not present")
@pytest.mark.parametrize("kernel", sorted({r["kernel"] for r in RECORDS}))
def test_oracle_matches_live_suite_build(kernel):
    for size, reps in [(2000, 2), (4097, 1)]:
        if kernel in ("Polybench_GEMM", "Polybench_3MM") and size > 2000:
            continue
        ref = oracle.run_ref(kernel, size, reps)
        mine = oracle.run(kernel, size=size, reps=reps)
        assert mine["checksum"] == ref["checksum"]


def test_openmp_variant_agrees_with_seq():
    """Base_OpenMP restatement vs Base_Seq: identical for element-wise
    kernels, within reassociation bounds for reductions and the scan."""
    for k in ["Stream_TRIAD", "Lcals_EOS", "Apps_ENERGY", "Lcals_HYDRO_2D",
              "Polybench_JACOBI_2D", "Lcals_FIRST_MIN"]:
        a = oracle.run(k, size=20000, reps=2)
        b = oracle.run(k, size=20000, reps=2, threads=4)
        assert a["checksum"] == b["checksum"], k
    for k in ["Stream_DOT", "Algorithm_REDUCE_SUM", "Algorithm_SCAN"]:
        a = oracle.run(k, size=20000, reps=2)
        b = oracle.run(k, size=20000, reps=2, threads=4)
        assert abs(a["checksum"] - b["checksum"]) <= 1e-10 * abs(a["checksum"]), k


def test_uniform_mode_is_seeded():
    a = oracle.run("Stream_TRIAD", size=1000, reps=1, init="uniform", seed=7)
    b = oracle.run("Stream_TRIAD", size=1000, reps=1, init="uniform", seed=7)
    c = oracle.run("Stream_TRIAD", size=1000, reps=1, init="uniform", seed=8)
    assert a["checksum"] == b["checksum"] != c["checksum"]
    v = [oracle.lib().oracle_uniform_value(7, 0, i, 0.5, 1.5) for i in range(1000)]
    assert min(v) >= 0.5 and max(v) < 1.5


def test_scan_int64_exact():
    r = oracle.run("Algorithm_SCAN", size=100000, reps=1, init="uniform", variant=1)
    assert r["checksum"] > 0
