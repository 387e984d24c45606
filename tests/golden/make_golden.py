"""Regenerates tests/golden/ref_checksums.json from the RAJA Performance
Suite's own Base_Seq code (oracle/_ref/rajaperf_ref, built from the suite's
sources by oracle/ref_build/Makefile).

Run where the suite checkout exists:
    python tests/golden/make_golden.py [/path/to/RAJAPerf]
Each record is one `rajaperf_ref <kernel> <size> <reps>` run: the suite's
checksum (printed with 21 significant digits), actual problem size, reps,
Bytes/rep and FLOPs/rep.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

KERNELS = [
    "Stream_COPY", "Stream_MUL", "Stream_ADD", "Stream_TRIAD", "Stream_DOT",
    "Basic_DAXPY", "Basic_INIT3", "Basic_MULADDSUB",
    "Lcals_HYDRO_1D", "Lcals_HYDRO_2D", "Lcals_EOS", "Lcals_FIRST_DIFF",
    "Lcals_INT_PREDICT", "Lcals_FIRST_MIN", "Lcals_DIFF_PREDICT", "Lcals_PLANCKIAN",
    "Apps_DEL_DOT_VEC_2D", "Apps_VOL3D", "Apps_ENERGY", "Apps_PRESSURE",
    "Polybench_JACOBI_2D", "Polybench_HEAT_3D", "Polybench_FDTD_2D",
    "Polybench_GEMM", "Polybench_3MM",
    "Algorithm_SCAN", "Algorithm_REDUCE_SUM",
    "Basic_INDEXLIST", "Basic_INDEXLIST_3LOOP", "Basic_MULTI_REDUCE",
    "Algorithm_MEMSET", "Algorithm_MEMCPY", "Algorithm_HISTOGRAM",
    "Comm_HALO_PACKING", "Comm_HALO_PACKING_FUSED",
]
CASES = [(1, 1), (31, 2), (1000, 3), (10000, 2), (65537, 1)]
EXTRA = {
    # the suite's own CPU-runnable Stream case: N = 1e6
    "Stream_TRIAD": [(1000000, 5)],
    "Stream_DOT": [(1000000, 5)],
}
# further suite options per record: the bin counts and layouts of HISTOGRAM
# and MULTI_REDUCE (--multi_reduce_num_bins, --multi_reduce_bin_assignment_algorithm)
BIN_CASES = [(nb, algo, size) for nb, algo in ((1, "Single"), (7, "Random"), (100, "RunsEvenSizes"),
                                               (100, "Random"), (3000, "RunsRandomSizes"))
             for size in (1000, 65537)]
OPTION_CASES = {
    k: [(size, 2, ["--multi_reduce_num_bins", str(nb),
                   "--multi_reduce_bin_assignment_algorithm", algo])
        for nb, algo, size in BIN_CASES]
    for k in ("Algorithm_HISTOGRAM", "Basic_MULTI_REDUCE")
}
# halo width and variable count of HALO_PACKING(_FUSED)
for _k in ("Comm_HALO_PACKING", "Comm_HALO_PACKING_FUSED"):
    OPTION_CASES[_k] = [(size, 2, ["--halo_width", str(w), "--halo_num_vars", str(nv)])
                        for w, nv in ((2, 1), (3, 4)) for size in (1000, 65537)]


def main() -> None:
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    exe = oracle.build_ref(ref_root)
    if not exe:
        sys.exit("suite sources not found; nothing generated")
    records = []
    for k in KERNELS:
        for size, reps in CASES + EXTRA.get(k, []):
            if k in ("Polybench_GEMM", "Polybench_3MM") and size > 10000:
                continue
            r = oracle.run_ref(k, size, reps)
            records.append({"kernel": k, "size": size, "reps": reps,
                            "checksum": r["checksum"], "actual_size": r["actual_size"],
                            "bytes_per_rep": r["bytes_per_rep"],
                            "flops_per_rep": r["flops_per_rep"]})
        for size, reps, args in OPTION_CASES.get(k, []):
            r = oracle.run_ref(k, size, reps, args)
            records.append({"kernel": k, "size": size, "reps": reps, "args": args,
                            "checksum": r["checksum"], "actual_size": r["actual_size"],
                            "bytes_per_rep": r["bytes_per_rep"],
                            "flops_per_rep": r["flops_per_rep"]})
    out = os.path.join(HERE, "ref_checksums.json")
    with open(out, "w") as f:
        json.dump({"generator": "oracle/_ref/rajaperf_ref (suite Base_Seq, x86-64 g++ -O2 "
                                "-ffp-contract=off)",
                   "records": records}, f, indent=1)
    print(f"wrote {len(records)} records to {out}")


if __name__ == "__main__":
    main()
