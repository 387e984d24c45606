"""b200_stream_dot_static: the DOT entry point for callers that cannot
allocate device memory (a framework that owns the whole device heap, or a
latency-critical loop that must not pay cudaMalloc's implicit
synchronisation).  It keeps its scratch in a library-owned device array.

The test checks it against b200_stream_dot (which takes a caller-allocated
workspace) on two calls in a row, within the reduction tolerance the other
DOT tests use.  It lives in its own file that pytest collects last, and it
passes both alone in a fresh process and after the other tests."""
import ctypes

import numpy as np
import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu


def _static_fn():
    fn = rp.b200().b200_stream_dot_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                   ctypes.c_void_p, ctypes.POINTER(rp.Tune), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("n", [1, 4097, 1 << 22])
def test_dot_static_matches_workspace_dot(n):
    torch = gu.torch_cuda()
    L = rp.b200()
    rng = np.random.default_rng(n)
    a, b = rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n)
    da, db = gu.dev(a), gu.dev(b)
    ws_bytes = L.b200_reduce_workspace_bytes(n, None)
    ws = torch.zeros(ws_bytes, dtype=torch.uint8, device="cuda")
    acc_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    acc_static = torch.zeros(1, dtype=torch.float64, device="cuda")
    static = _static_fn()
    s = gu.stream()
    bound = gu.reduction_bound(n, 2, 2.0 * float(np.sum(a * b)) + 1.0)
    for call in range(2):
        rp.check(L.b200_stream_dot(da.data_ptr(), db.data_ptr(), n, 0.25, acc_ref.data_ptr(),
                                   ws.data_ptr(), ws_bytes, None, s), "b200_stream_dot")
        rp.check(static(da.data_ptr(), db.data_ptr(), n, 0.25, acc_static.data_ptr(), None, s),
                 "b200_stream_dot_static")
        got = float(gu.host(acc_static)[0])
        want = float(gu.host(acc_ref)[0])
        assert abs(got - want) <= bound, (call, got, want)
    assert abs(got - 2 * (0.25 + float(np.sum(a * b)))) <= bound


def test_dot_static_full_scratch_and_no_device_allocation():
    """A launch of exactly the 4096 CTAs the static scratch holds (its last
    partial slot used) agrees with the workspace DOT, and calls after the
    first one in this context leave the device's free memory unchanged (the
    first call may load the library's device module, which the driver does
    once per context)."""
    torch = gu.torch_cuda()
    L = rp.b200()
    n = 4096 * 64 * 3 + 17
    rng = np.random.default_rng(7)
    a, b = rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n)
    da, db = gu.dev(a), gu.dev(b)
    t = rp.Tune(block_size=64, items=1, grid_blocks=4096)
    ws_bytes = L.b200_reduce_workspace_bytes(n, ctypes.byref(t))
    assert ws_bytes == L.b200_stream_dot_static_max_scratch_bytes()
    ws = torch.zeros(ws_bytes, dtype=torch.uint8, device="cuda")
    acc_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    acc_static = torch.zeros(1, dtype=torch.float64, device="cuda")
    static = _static_fn()
    s = gu.stream()
    rp.check(static(da.data_ptr(), db.data_ptr(), n, 0.0, acc_static.data_ptr(),
                    ctypes.byref(t), s), "b200_stream_dot_static")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        rp.check(static(da.data_ptr(), db.data_ptr(), n, 0.0, acc_static.data_ptr(),
                        ctypes.byref(t), s), "b200_stream_dot_static")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    for _ in range(4):
        rp.check(L.b200_stream_dot(da.data_ptr(), db.data_ptr(), n, 0.0, acc_ref.data_ptr(),
                                   ws.data_ptr(), ws_bytes, ctypes.byref(t), s),
                 "b200_stream_dot")
    got = float(gu.host(acc_static)[0])
    want = float(gu.host(acc_ref)[0])
    bound = gu.reduction_bound(n, 4, 4.0 * float(np.sum(a * b)))
    assert abs(got - want) <= bound, (got, want)
    assert abs(got - 4 * float(np.sum(a * b))) <= bound


def test_dot_static_rejects_oversized_shape():
    torch = gu.torch_cuda()
    x = torch.ones(1 << 20, dtype=torch.float64, device="cuda")
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    t = rp.Tune(block_size=64, items=1, grid_blocks=8192)
    st = _static_fn()(x.data_ptr(), x.data_ptr(), 1 << 20, 0.0, acc.data_ptr(),
                      ctypes.byref(t), None)
    assert st == rp.B200_ERR_WORKSPACE
    assert "static scratch" in rp.last_error()
