"""Device-side wait limits and their report.

The scan, index-list and split-GEMM kernels bound every wait (mbarrier
phases, predecessor tiles in the lookback) and record a wait that gives up
in their workspace's error word; b200_workspace_status() reports it as
B200_ERR_TIMEOUT and clears the workspace, and the suite layer fails the run.

To make a lookback wait run out without faulting or hanging anything, the
tests mark the first tile tickets of a zeroed scan workspace as taken
before the call: the persistent kernel then draws tiles from that ticket on
(its tile ids stay below the tile count), and the first drawn tile's
lookback waits for predecessors that no CTA processes, until the short
limit set in b200_tune.wait_limit_us (1 ms) runs out.  Every other wait of
the launch is bounded by the same limit, so the launch ends within a few
milliseconds; the call's results are invalid, the status says so, and the
next call on the cleared workspace is correct again."""
import ctypes

import numpy as np
import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

TILE = 4096  # items per tile of the persistent scan and index-list kernels


def _ws(nbytes):
    torch = gu.torch_cuda()
    return torch.zeros(int(nbytes), dtype=torch.uint8, device="cuda")


def _take_tickets(ws, k):
    # header word 0: low 32 bits = tickets taken, high 32 bits = launch epoch
    torch = gu.torch_cuda()
    torch.cuda.synchronize()
    ws[:8].view(torch.int64)[0] += k
    torch.cuda.synchronize()


def test_scan_wait_runs_out_and_is_reported():
    torch = gu.torch_cuda()
    L = rp.b200()
    n = 64 * TILE
    x = np.random.default_rng(1).integers(0, 100, n).astype(np.int64)
    dx = gu.dev(x)
    dy = torch.zeros(n, dtype=torch.int64, device="cuda")
    wb = L.b200_scan_workspace_bytes(n)
    ws = _ws(wb)
    s = gu.stream()
    # a normal call first: status OK
    rp.check(L.b200_algorithm_scan_i64(dx.data_ptr(), dy.data_ptr(), n, 0, ws.data_ptr(), wb,
                                       None, s), "scan")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_OK
    want = np.concatenate(([0], np.cumsum(x)[:-1]))
    assert np.array_equal(gu.host(dy), want)
    # three tickets taken before the call: tile 3's lookback cannot finish
    _take_tickets(ws, 3)
    t = rp.Tune(wait_limit_us=1000)
    rp.check(L.b200_algorithm_scan_i64(dx.data_ptr(), dy.data_ptr(), n, 0, ws.data_ptr(), wb,
                                       ctypes.byref(t), s), "scan (stalled)")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_ERR_TIMEOUT
    assert "gave up" in rp.last_error()
    assert int(gu.host(ws).max()) == 0  # cleared for the next call
    # the next call on the cleared workspace is correct and reports OK
    dy.zero_()
    rp.check(L.b200_algorithm_scan_i64(dx.data_ptr(), dy.data_ptr(), n, 0, ws.data_ptr(), wb,
                                       ctypes.byref(t), s), "scan")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_OK
    assert np.array_equal(gu.host(dy), want)


def test_indexlist_wait_runs_out_and_is_reported():
    torch = gu.torch_cuda()
    L = rp.b200()
    n = 40 * TILE + 123
    x = np.random.default_rng(2).uniform(-1.0, 1.0, n)
    dx = gu.dev(x)
    dl = torch.zeros(n, dtype=torch.int32, device="cuda")
    dlen = torch.zeros(1, dtype=torch.int64, device="cuda")
    wb = L.b200_indexlist_workspace_bytes(n)
    ws = _ws(wb)
    s = gu.stream()
    _take_tickets(ws, 5)
    t = rp.Tune(wait_limit_us=1000)
    rp.check(L.b200_basic_indexlist(dx.data_ptr(), dl.data_ptr(), n, dlen.data_ptr(),
                                    ws.data_ptr(), wb, ctypes.byref(t), s), "indexlist (stalled)")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_ERR_TIMEOUT
    rp.check(L.b200_basic_indexlist(dx.data_ptr(), dl.data_ptr(), n, dlen.data_ptr(),
                                    ws.data_ptr(), wb, ctypes.byref(t), s), "indexlist")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_OK
    idx = np.nonzero(x < 0)[0]
    assert int(gu.host(dlen)[0]) == idx.size
    assert np.array_equal(gu.host(dl)[:idx.size], idx.astype(np.int32))


def test_workspace_status_ok_after_split_gemm_and_rejects_small_workspace():
    torch = gu.torch_cuda()
    L = rp.b200()
    m = n = k = 256
    rng = np.random.default_rng(3)
    A, B = rng.uniform(-1, 1, (m, k)), rng.uniform(-1, 1, (k, n))
    dA, dB = gu.dev(A.ravel()), gu.dev(B.ravel())
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    wb = L.b200_gemm_split_workspace_bytes(m, n, k, None)
    ws = _ws(wb)
    s = gu.stream()
    t = rp.Tune(wait_limit_us=200000)
    rp.check(L.b200_gemm_split(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k, 1.0, 0.0,
                               ws.data_ptr(), wb, ctypes.byref(t), s), "gemm_split")
    assert L.b200_workspace_status(ws.data_ptr(), wb, s) == rp.B200_OK
    got = gu.host(dC).reshape(m, n)
    assert np.linalg.norm(got - A @ B) <= 1e-13 * np.linalg.norm(A @ B)
    assert L.b200_workspace_status(ws.data_ptr(), 128, s) == rp.B200_ERR_INVALID_ARG


@pytest.mark.parametrize("kernel,tuning", [("Algorithm_SCAN", "int64"),
                                           ("Basic_INDEXLIST", "default")])
def test_suite_run_fails_on_device_timeout(kernel, tuning):
    """rp_run marks the run failed (RP_ERR_RUN) with the timeout message; the
    same command line without the stall passes.  (The FP64 scan's default,
    the one-CTA-per-tile kernel, refuses the stall: its tile ids could pass
    the tile count.)"""
    args = ["--size", 50 * TILE, "--checkrun", 2, "-k", kernel, "-t", tuning,
            "--disable-warmup", "--wait-limit-us", 1000]
    with pytest.raises(RuntimeError, match="device-side wait timed out"):
        rp.run_suite(args + ["--inject-lookback-stall", 3])
    res = rp.run_suite(args[:-2] + ["--wait-limit-us", 200000])
    assert len(res) == 1 and res[0]["tuning"] == tuning


def test_stall_refused_by_the_tile_kernel():
    with pytest.raises(RuntimeError, match="needs the pipelined"):
        rp.run_suite(["--size", 50 * TILE, "--checkrun", 1, "-k", "Algorithm_SCAN", "-t",
                      "default", "--disable-warmup", "--inject-lookback-stall", 3])
