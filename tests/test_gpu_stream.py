"""Stream group on the GPU: suite checksums against the suite's own Base_Seq
results, and element-wise checks of the C ABI (include/b200.h)."""
import ctypes

import numpy as np
import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

STREAM = ["Stream_COPY", "Stream_MUL", "Stream_ADD", "Stream_TRIAD", "Stream_DOT"]


@pytest.mark.parametrize("kernel", STREAM)
def test_suite_checksum_matches_base_seq(kernel):
    for rec in gu.golden(kernel):
        res = rp.run_suite(["--size", rec["size"], "--checkrun", rec["reps"],
                            "-k", kernel, "--disable-warmup"])
        assert {r["tuning"] for r in res} >= {"default", "graph"}
        for r in res:
            assert r["actual_size"] == rec["actual_size"]
            assert r["bytes_per_rep"] == rec["bytes_per_rep"]
            assert r["flops_per_rep"] == rec["flops_per_rep"]
            what = f"{kernel} {rec['size']}x{rec['reps']} {r['tuning']}"
            if kernel == "Stream_DOT":
                # sum |a_i b_i| ~ checksum / reps for these positive inputs
                bound = gu.reduction_bound(rec["actual_size"], rec["reps"],
                                           abs(rec["checksum"]))
                assert abs(r["checksum"] - rec["checksum"]) <= bound, what
            else:
                gu.assert_close_rel(r["checksum"], rec["checksum"], what=what)


def _arrays(n, seed=1):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 255, 256, 1023, 4099, 1 << 20])
@pytest.mark.parametrize("offset", [0, 1])
def test_triad_elementwise(n, offset):
    torch = gu.torch_cuda()
    b, c = _arrays(n + offset)
    db, dc = gu.dev(b), gu.dev(c)
    da = torch.zeros(n + offset, dtype=torch.float64, device="cuda")
    alpha = 0.0978987899
    esz = 8 * offset
    gu.rp.check(rp.b200().b200_stream_triad(da.data_ptr() + esz, db.data_ptr() + esz,
                                            dc.data_ptr() + esz, alpha, n, None,
                                            gu.stream()), "triad")
    got = gu.host(da)[offset:]
    want = b[offset:] + alpha * c[offset:]
    # a fused multiply-add rounds once: at most 1 ulp from the two-step form
    assert np.all(gu.ulp_diff(got, want) <= 1)


@pytest.mark.parametrize("n", [1, 7, 4096, 100003])
def test_copy_mul_add_elementwise(n):
    torch = gu.torch_cuda()
    a, b = _arrays(n, 3)
    da, db = gu.dev(a), gu.dev(b)
    dc = torch.zeros(n, dtype=torch.float64, device="cuda")
    L = rp.b200()
    rp.check(L.b200_stream_copy(da.data_ptr(), dc.data_ptr(), n, None, gu.stream()))
    assert np.array_equal(gu.host(dc), a)
    rp.check(L.b200_stream_mul(dc.data_ptr(), db.data_ptr(), 0.25, n, None, gu.stream()))
    assert np.array_equal(gu.host(dc), 0.25 * b)
    rp.check(L.b200_stream_add(da.data_ptr(), db.data_ptr(), dc.data_ptr(), n, None,
                               gu.stream()))
    assert np.array_equal(gu.host(dc), a + b)


@pytest.mark.parametrize("block,items", [(64, 1), (128, 2), (256, 4), (512, 8), (1024, 4)])
def test_triad_tunings(block, items):
    torch = gu.torch_cuda()
    n = 300007
    b, c = _arrays(n, 5)
    db, dc = gu.dev(b), gu.dev(c)
    da = torch.zeros(n, dtype=torch.float64, device="cuda")
    t = rp.Tune(block_size=block, items=items)
    rp.check(rp.b200().b200_stream_triad(da.data_ptr(), db.data_ptr(), dc.data_ptr(), 2.0,
                                         n, ctypes.byref(t), gu.stream()))
    assert np.all(gu.ulp_diff(gu.host(da), b + 2.0 * c) <= 1)


def _dot(a, b, n, init=0.0, tune=None, accum=None):
    torch = gu.torch_cuda()
    L = rp.b200()
    tp = ctypes.byref(tune) if tune is not None else None
    ws_bytes = L.b200_reduce_workspace_bytes(n, tp)
    ws = torch.zeros(ws_bytes, dtype=torch.uint8, device="cuda")
    acc = accum if accum is not None else torch.zeros(1, dtype=torch.float64, device="cuda")
    rp.check(L.b200_stream_dot(a.data_ptr(), b.data_ptr(), n, init, acc.data_ptr(),
                               ws.data_ptr(), ws_bytes, tp, gu.stream()), "dot")
    return acc, ws


@pytest.mark.parametrize("n", [0, 1, 2, 3, 1000, 65537, 1 << 22])
def test_dot_value_and_determinism(n):
    a, b = _arrays(n, 11)
    da, db = gu.dev(a), gu.dev(b)
    acc, ws = _dot(da, db, n, init=0.5)
    v1 = float(gu.host(acc)[0])
    want = 0.5 + float(np.sum(a * b))
    assert abs(v1 - want) <= gu.reduction_bound(n, 1, float(np.sum(np.abs(a * b))) + 0.5)
    # the workspace is reusable and the tree is fixed: repeat adds the same
    acc2, _ = _dot(da, db, n, init=0.5)
    assert float(gu.host(acc2)[0]) == v1
    # accumulation into the same device scalar, as the rep loop does
    _dot(da, db, n, init=0.5, accum=acc)
    assert float(gu.host(acc)[0]) == v1 + v1


def test_dot_misaligned_and_tunings():
    n = 123457
    a, b = _arrays(n + 1, 13)
    da, db = gu.dev(a), gu.dev(b)
    torch = gu.torch_cuda()
    sa = da[1:]
    sb = db[1:]
    acc, _ = _dot(sa, sb, n)
    want = float(np.sum(a[1:] * b[1:]))
    assert abs(float(gu.host(acc)[0]) - want) <= gu.reduction_bound(n, 1, want)
    for blk, it in [(128, 1), (512, 8)]:
        acc, _ = _dot(da, db, n, tune=rp.Tune(block_size=blk, items=it))
        want = float(np.sum(a[:n] * b[:n]))
        assert abs(float(gu.host(acc)[0]) - want) <= gu.reduction_bound(n, 1, want)


def test_argument_errors():
    torch = gu.torch_cuda()
    L = rp.b200()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    assert L.b200_stream_triad(None, x.data_ptr(), x.data_ptr(), 1.0, 16, None, None) == \
        rp.B200_ERR_INVALID_ARG
    assert "bad args" in rp.last_error()
    assert L.b200_stream_copy(x.data_ptr(), x.data_ptr(), -1, None, None) == \
        rp.B200_ERR_INVALID_ARG
    bad = rp.Tune(block_size=96)
    assert L.b200_stream_triad(x.data_ptr(), x.data_ptr(), x.data_ptr(), 1.0, 16,
                               ctypes.byref(bad), None) == rp.B200_ERR_INVALID_ARG
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    ws = torch.zeros(8, dtype=torch.uint8, device="cuda")
    assert L.b200_stream_dot(x.data_ptr(), x.data_ptr(), 16, 0.0, acc.data_ptr(),
                             ws.data_ptr(), 8, None, None) == rp.B200_ERR_WORKSPACE


def test_init_kernels_bit_exact():
    torch = gu.torch_cuda()
    import oracle
    L = rp.b200()
    n = 100001
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    rp.check(L.b200_init_reference(d.data_ptr(), n, 0.1, gu.stream()))
    i = np.arange(n, dtype=np.float64)
    assert np.array_equal(gu.host(d), 0.1 * (i + 1.1) / (i + 1.12345))
    rp.check(L.b200_init_uniform(d.data_ptr(), n, 99, 3, 0.5, 1.5, gu.stream()))
    got = gu.host(d)
    want = np.array([oracle.lib().oracle_uniform_value(99, 3, k, 0.5, 1.5)
                     for k in range(0, n, 997)])
    assert np.array_equal(got[::997], want)
    di = torch.empty(n, dtype=torch.int64, device="cuda")
    rp.check(L.b200_init_uniform_i64(di.data_ptr(), n, 5, 1, 0, 100, gu.stream()))
    gi = gu.host(di)
    assert gi.min() >= 0 and gi.max() < 100


def test_launch_counter_counts():
    torch = gu.torch_cuda()
    L = rp.b200()
    x = torch.zeros(1 << 16, dtype=torch.float64, device="cuda")
    c0 = L.b200_launch_count()
    rp.check(L.b200_stream_copy(x.data_ptr(), x.data_ptr(), 1 << 16, None, None))
    assert L.b200_launch_count() == c0 + 1


def test_device_caps():
    caps = rp.Caps()
    rp.check(rp.b200().b200_device_caps(ctypes.byref(caps)))
    assert caps.sm_count > 0 and caps.cc_major >= 10
