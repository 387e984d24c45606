"""--host-data: the suite layer with the kernels' arrays in pinned host memory
(the suite's CudaPinned data space).  Streaming kernels run on the host
arrays directly; iterating and gathering kernels copy their arrays in and
out around every rep.  Either way the results are the device-memory run's:
the checksums must match it (bit for bit where the same kernel runs; the
FP64 scan runs its one-CTA-per-tile form on host memory, within the
reassociation bound), and the reported bytes per rep are the arrays a rep
moves across the host link."""
import math

import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

# kernel, --size, extra options, tuning, bit-identical to the device run
CASES = [
    ("Stream_TRIAD", 100003, [], "default", True),
    ("Stream_COPY", 100003, [], "default", True),
    ("Stream_MUL", 100003, [], "default", True),
    ("Stream_ADD", 100003, [], "default", True),
    ("Stream_DOT", 100003, [], "default", True),
    ("Lcals_EOS", 1 << 20, [], "default", True),
    ("Lcals_FIRST_DIFF", 1 << 20, [], "default", True),
    ("Lcals_FIRST_MIN", 1 << 20, [], "default", True),
    ("Lcals_HYDRO_2D", 512 * 512, [], "default", True),
    ("Apps_DEL_DOT_VEC_2D", 512 * 512, [], "default", True),
    ("Polybench_JACOBI_2D", 510 * 510, ["--polybench_tsteps", 5], "default", True),
    ("Polybench_HEAT_3D", 62 ** 3, ["--polybench_tsteps", 4], "default", True),
    ("Algorithm_SCAN", 1 << 20, [], "int64", True),
    ("Algorithm_SCAN", 1 << 20, [], "default", False),
]


@pytest.mark.parametrize("kernel,size,opts,tuning,exact", CASES,
                         ids=[f"{c[0]}-{c[3]}" for c in CASES])
@pytest.mark.parametrize("init", ["reference", "uniform"])
def test_host_data_matches_device_run(kernel, size, opts, tuning, exact, init):
    args = ["--size", size, "--checkrun", 3, "-k", kernel, "-t", tuning, "graph"
            if tuning == "default" else "int64_graph", "--init", init, "--disable-warmup",
            *opts]
    dev = {r["tuning"]: r for r in rp.run_suite(args)}
    host = {r["tuning"]: r for r in rp.run_suite(args + ["--host-data"])}
    assert dev.keys() == host.keys()
    for t, h in host.items():
        d = dev[t]
        if exact:
            assert h["checksum"] == d["checksum"], (kernel, t, h["checksum"], d["checksum"])
        else:
            n = d["actual_size"]
            bound = (n + math.ceil(math.log2(n)) + 3) * gu.U * abs(d["checksum"]) * 4
            assert abs(h["checksum"] - d["checksum"]) <= bound
        assert d["h2d_bytes_per_rep"] == 0 and d["d2h_bytes_per_rep"] == 0
        assert h["h2d_bytes_per_rep"] > 0 and h["d2h_bytes_per_rep"] > 0
        assert h["avg_time_s"] > 0


def test_host_data_bytes_per_rep():
    n = 1 << 20
    r = rp.run_suite(["--size", n, "--checkrun", 1, "-k", "Lcals_FIRST_DIFF", "-t", "default",
                      "--host-data", "--disable-warmup"])[0]
    assert r["h2d_bytes_per_rep"] == 8 * (n + 1) and r["d2h_bytes_per_rep"] == 8 * n
    r = rp.run_suite(["--size", 510 * 510, "--checkrun", 1, "-k", "Polybench_JACOBI_2D",
                      "-t", "default", "--host-data", "--disable-warmup"])[0]
    assert r["h2d_bytes_per_rep"] == r["d2h_bytes_per_rep"] == 2 * 8 * 512 * 512


def test_host_data_unsupported_kernel_fails_loudly():
    with pytest.raises(RuntimeError, match="no --host-data form"):
        rp.run_suite(["--size", 1000, "--checkrun", 1, "-k", "Apps_VOL3D", "--host-data",
                      "--disable-warmup"])
    with pytest.raises(RuntimeError, match="does not combine"):
        rp.run_suite(["--graph-batch", 2, "-k", "Stream_TRIAD", "--host-data"])
