"""The committed GB300 tuning table (rajaperf_gb300/tuning/gb300.txt, written
by rajaperf_gb300/tuning/make_table.py from the suite's --autotune on a
GB300): it parses in the suite layer and in bench.py, and it has an entry
for every kernel and size of the bandwidth/stencil workload."""
import os

import bench
import rajaperf_gb300 as rp

TABLE = os.path.join(os.path.dirname(rp.PKG), "rajaperf_gb300", "tuning", "gb300.txt")


def test_table_parses_in_the_suite_layer():
    res = rp.run_suite(["--tuning-table", TABLE, "--dryrun", "-k", "Stream_TRIAD"])
    assert res == []


def test_table_covers_the_workload():
    table = bench.load_tuning_table(rp, TABLE)
    for kernel, size in bench.workload_kernels("bandwidth_stencil"):
        # HEAT_3D has one launch shape (the autotuner has nothing to choose)
        if kernel in bench.TABLE_SKIP or kernel == "Polybench_HEAT_3D":
            continue
        assert (kernel, size) in table, kernel
    t = table[("Polybench_JACOBI_2D", 4094 * 4094)]
    assert t.items in (1, 2, 4, 8)
