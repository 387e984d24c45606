"""Parity at the benchmarked sizes.

The bandwidth/stencil workload that bench.py times (HYDRO_2D 4096^2;
EOS, FIRST_DIFF and FIRST_MIN at 2^24; DEL_DOT_VEC_2D on a jittered 4096^2
mesh; JACOBI_2D N=4096 for 50 time steps; HEAT_3D 256^3 for 20 time steps;
the int64 SCAN at 2^26), all from uniform [0.5, 1.5) data with seed 4793,
runs here through the Base_GB300 suite layer (rp_run, the rajaperf-gb300
driver's path) and its checksums are compared with the CPU oracle's
Base_OpenMP restatement of the suite's loops on the same inputs:
relative 1e-12 for the FP64 kernels, exact for FIRST_MIN's location and the
int64 scan.  These sizes exercise the integer-pipe fast paths of the FP64
kernels (the FP64-free division, products and exponent moves) on every
point the benchmark computes.

Also here: the Stream TRIAD/DOT case at N=1,000,000 with alpha = 0.5 and
b, c uniform in [0, 1), and one two-step case of each large stencil
(JACOBI_2D 16384^2, HEAT_3D 768^3, FDTD_2D 8192^2), compared element by
element with the oracle's loops run on a host copy of the same inputs."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import oracle
import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

SEED = 4793

# (kernel, --size, tuning, suite options, oracle options, comparison)
WORKLOAD = [
    ("Lcals_HYDRO_2D", 4096 * 4096, "default", [], {}, "rel"),
    ("Lcals_EOS", 1 << 24, "default", [], {}, "rel"),
    ("Lcals_FIRST_DIFF", 1 << 24, "default", [], {}, "rel"),
    ("Lcals_FIRST_MIN", 1 << 24, "default", [], {}, "exact"),
    ("Apps_DEL_DOT_VEC_2D", 4096 * 4096, "default", [], {}, "rel"),
    ("Polybench_JACOBI_2D", 4094 * 4094, "default", ["--polybench_tsteps", 50],
     {"tsteps": 50}, "rel"),
    ("Polybench_HEAT_3D", 254 ** 3, "default", ["--polybench_tsteps", 20],
     {"tsteps": 20}, "rel"),
    ("Algorithm_SCAN", 1 << 26, "int64", [], {"variant": 1}, "exact"),
]


def _cores():
    return len(os.sched_getaffinity(0))


@pytest.mark.parametrize("kernel,size,tuning,opts,okw,cmp", WORKLOAD,
                         ids=[w[0] for w in WORKLOAD])
def test_bench_workload_matches_oracle(kernel, size, tuning, opts, okw, cmp):
    # the two host checksums (suite layer, oracle) run concurrently
    with cf.ThreadPoolExecutor(1) as ex:
        fut = ex.submit(oracle.run, kernel, size=size, reps=1, init="uniform", seed=SEED,
                        threads=_cores(), **okw)
        res = rp.run_suite(["--size", size, "--checkrun", 1, "-k", kernel, "-t", tuning,
                            "--init", "uniform", "--seed", SEED, "--disable-warmup", *opts])
        want = fut.result()
    assert len(res) == 1, res
    got = res[0]
    assert got["actual_size"] == want["actual_size"]
    assert got["bytes_per_rep"] == want["bytes_per_rep"]
    if cmp == "exact":
        assert got["checksum"] == want["checksum"], (kernel, got["checksum"], want["checksum"])
    else:
        gu.assert_close_rel(got["checksum"], want["checksum"], what=kernel)
    if kernel == "Lcals_FIRST_MIN":
        assert want["checksum"] == oracle.lib().oracle_first_min_planted_index(SEED, size)


def _uniform(n, stream_id, lo=0.5, hi=1.5, seed=SEED):
    torch = gu.torch_cuda()
    t = torch.empty(n, dtype=torch.float64, device="cuda")
    rp.check(rp.b200().b200_init_uniform(t.data_ptr(), n, seed, stream_id, lo, hi, None),
             "b200_init_uniform")
    return t


def test_triad_dot_1e6_alpha_half():
    """cfg1: a = b + 0.5 c and sum b c at N = 1e6, b, c uniform in [0, 1).
    0.5 c is exact, so TRIAD is bit-exact; DOT within the reassociation bound."""
    torch = gu.torch_cuda()
    L = rp.b200()
    n = 1_000_000
    db, dc = _uniform(n, 1, 0.0, 1.0), _uniform(n, 2, 0.0, 1.0)
    da = torch.zeros(n, dtype=torch.float64, device="cuda")
    s = gu.stream()
    rp.check(L.b200_stream_triad(da.data_ptr(), db.data_ptr(), dc.data_ptr(), 0.5, n, None, s),
             "b200_stream_triad")
    wsb = L.b200_reduce_workspace_bytes(n, None)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    rp.check(L.b200_stream_dot(db.data_ptr(), dc.data_ptr(), n, 0.0, acc.data_ptr(),
                               ws.data_ptr(), wsb, None, s), "b200_stream_dot")
    b, c, a = gu.host(db), gu.host(dc), gu.host(da)
    assert np.array_equal(a, b + 0.5 * c)
    prod = b * c
    want = float(np.sum(prod))
    assert abs(float(gu.host(acc)[0]) - want) <= gu.reduction_bound(n, 1, float(np.sum(prod)))
    # the suite's checksum of the TRIAD output (scale 0.001 * 1e6 / N)
    assert oracle.checksum(a, 0.001) == oracle.checksum(b + 0.5 * c, 0.001)


def _ulp_max(got, want):
    return int(np.max(gu.ulp_diff(got, want))) if got.size else 0


@pytest.mark.parametrize("kernel", ["Polybench_JACOBI_2D", "Polybench_HEAT_3D",
                                    "Polybench_FDTD_2D"])
def test_large_stencils_two_steps(kernel):
    """The large-set stencils at full size for two time steps, element by
    element against the oracle's loops on a host copy of the same inputs.
    JACOBI_2D is bit-exact (no operation can contract); HEAT_3D and FDTD_2D
    differ from the unfused oracle by the device's FMA contractions only
    (within 1e-12 relative)."""
    torch = gu.torch_cuda()
    L = rp.b200()
    s = gu.stream()
    ts = 2
    if kernel == "Polybench_JACOBI_2D":
        N = 16384
        dA, dB = _uniform(N * N, 10), _uniform(N * N, 11)
        A, B = gu.host(dA), gu.host(dB)
        rp.check(L.b200_polybench_jacobi_2d(dA.data_ptr(), dB.data_ptr(), N, ts, None, s),
                 "b200_polybench_jacobi_2d")
        oracle.call("oracle_jacobi_2d", A, B, N, ts)
        pairs = [(gu.host(dA), A), (gu.host(dB), B)]
        exact = True
    elif kernel == "Polybench_HEAT_3D":
        N = 768
        dA, dB = _uniform(N ** 3, 20), _uniform(N ** 3, 21)
        A, B = gu.host(dA), gu.host(dB)
        rp.check(L.b200_polybench_heat_3d(dA.data_ptr(), dB.data_ptr(), N, ts, None, s),
                 "b200_polybench_heat_3d")
        oracle.call("oracle_heat_3d", A, B, N, ts)
        pairs = [(gu.host(dA), A), (gu.host(dB), B)]
        exact = False
    else:
        nx = ny = 8192
        d = [_uniform(nx * ny, 30 + k) for k in range(3)]
        df = _uniform(ts, 33)
        ex, ey, hz = (gu.host(t) for t in d)
        fict = gu.host(df)
        rp.check(L.b200_polybench_fdtd_2d(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                          df.data_ptr(), nx, ny, ts, None, s),
                 "b200_polybench_fdtd_2d")
        oracle.call("oracle_fdtd_2d", ex, ey, hz, fict, nx, ny, ts)
        pairs = [(gu.host(t), w) for t, w in zip(d, (ex, ey, hz))]
        exact = False
    for got, want in pairs:
        if exact:
            assert np.array_equal(got, want), _ulp_max(got, want)
        else:
            # relative to each value, floored at 1e-3 of the largest value so
            # that results of cancellation (FDTD's differences near zero) are
            # held to the error of the operands they came from
            floor = 1e-3 * float(np.max(np.abs(want)))
            err = np.abs(got - want) / np.maximum(np.abs(want), floor)
            assert float(np.max(err)) <= gu.REL_TOL, (float(np.max(err)), _ulp_max(got, want))
