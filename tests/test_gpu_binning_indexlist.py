"""MEMSET, MEMCPY, INDEXLIST, HISTOGRAM and MULTI_REDUCE through the C ABI
against direct numpy references, on inputs the suite's own set-up never
produces: empty and ragged sizes, misaligned pointers, lists that are empty
or full, bins outside the range (skipped), non-zero initial counts/values,
bin counts above the shared-memory paths.  Integer results are exact;
MULTI_REDUCE sums are within the reassociation bound, and bit-identical run
to run on the deterministic path (<= 96 bins)."""
import ctypes

import numpy as np
import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu


def lib():
    return rp.b200()


def zeros(n, dtype):
    torch = gu.torch_cuda()
    return torch.zeros(max(int(n), 1), dtype=dtype, device="cuda")


@pytest.mark.parametrize("n", [0, 1, 2, 7, 4096, 100003])
@pytest.mark.parametrize("offset", [0, 1])
def test_memset_memcpy(n, offset):
    torch = gu.torch_cuda()
    x = torch.full((n + 2,), -7.0, dtype=torch.float64, device="cuda")
    rp.check(lib().b200_algorithm_memset(x.data_ptr() + 8 * offset, 2.5, n, None, gu.stream()))
    h = gu.host(x)
    assert np.all(h[offset:offset + n] == 2.5)
    assert np.all(h[:offset] == -7.0) and np.all(h[offset + n:] == -7.0)
    src = gu.dev(np.arange(n + 2, dtype=np.float64))
    dst = torch.full((n + 2,), -1.0, dtype=torch.float64, device="cuda")
    rp.check(lib().b200_algorithm_memcpy(src.data_ptr() + 8 * offset,
                                         dst.data_ptr() + 8 * offset, n, None, gu.stream()))
    d = gu.host(dst)
    assert np.array_equal(d[offset:offset + n], np.arange(offset, offset + n, dtype=np.float64))
    assert np.all(d[offset + n:] == -1.0)


@pytest.mark.parametrize("algo", [0, 1])
@pytest.mark.parametrize("case", ["empty", "none", "all", "random", "sparse", "ragged",
                                  "many_tiles", "one_pair", "special"])
def test_indexlist(case, algo):
    """algo 0: the persistent ring kernel (x aligned); algo 1: one CTA per
    tile.  many_tiles runs several tiles per SM through the ring."""
    torch = gu.torch_cuda()
    rng = np.random.default_rng(5)
    n = {"empty": 0, "ragged": 4096 * 7 + 123, "many_tiles": 4096 * 152 * 5 + 77,
         "one_pair": 2}.get(case, 1 << 20)
    x = rng.uniform(-1, 1, n)
    if case == "none":
        x = np.abs(x) + 0.1
    elif case == "all":
        x = -np.abs(x) - 0.1
    elif case == "sparse":
        x = np.abs(x) + 0.1
        x[rng.integers(0, n, 37)] = -1.0
    elif case == "special":  # x < 0 is tested on the integer pipe: IEEE semantics
        neg_nan = np.frombuffer(np.uint64(0xFFF8000000000001).tobytes(), dtype=np.float64)[0]
        vals = np.array([-0.0, 0.0, np.nan, neg_nan, -np.inf, np.inf, -5e-324, 5e-324,
                         -1.7976931348623157e308, 2.2250738585072014e-308])
        x[rng.integers(0, n, 4000)] = vals[rng.integers(0, vals.size, 4000)]
    dx = gu.dev(x) if n else zeros(1, torch.float64)
    lst = torch.full((max(n, 1),), -5, dtype=torch.int32, device="cuda")
    ln = zeros(1, torch.int64)
    wsb = lib().b200_indexlist_workspace_bytes(n)
    ws = zeros(wsb, torch.uint8)
    for _ in range(2):  # the workspace is reused
        rp.check(lib().b200_basic_indexlist(dx.data_ptr(), lst.data_ptr(), n, ln.data_ptr(),
                                            ws.data_ptr(), wsb, ctypes.byref(rp.Tune(algo=algo)),
                                            gu.stream()))
        want = np.nonzero(x < 0.0)[0]
        got_len = int(gu.host(ln)[0])
        assert got_len == want.size
        got = gu.host(lst)
        assert np.array_equal(got[:want.size], want.astype(np.int32))
        assert np.all(got[want.size:n] == -5)  # entries past the count untouched
    assert int(gu.host(ws[16:20]).view(np.uint32)[0]) == 0
    assert int(gu.host(ws[0:4]).view(np.uint32)[0]) == 0  # ticket count reset


@pytest.mark.parametrize("n", [4096, 8193, 4096 * 5, 4096 * 4 * 152 + 4095,
                               4096 * (4 * 152 * 2 + 1), 4096 * 24 * 152 + 17])
@pytest.mark.parametrize("offset", [0, 1])
def test_indexlist_run_and_slot_edges(n, offset):
    """The persistent kernel draws runs of 4 consecutive tiles: one tile,
    a run plus one, exactly one run per CTA plus a ragged tile, two runs per
    CTA plus one, and more tiles than a CTA's 24 slots hold, so slots and
    stages wrap; offset 1 makes x unaligned (the one-CTA-per-tile kernel)."""
    torch = gu.torch_cuda()
    rng = np.random.default_rng(n + offset)
    x = rng.uniform(-1, 1, n + offset)
    x[rng.integers(0, n + offset, 64)] = -0.0  # never selected
    dx = gu.dev(x)
    lst = torch.full((n,), -5, dtype=torch.int32, device="cuda")
    ln = zeros(1, torch.int64)
    wsb = lib().b200_indexlist_workspace_bytes(n)
    ws = zeros(wsb, torch.uint8)
    for _ in range(2):
        rp.check(lib().b200_basic_indexlist(dx.data_ptr() + 8 * offset, lst.data_ptr(), n,
                                            ln.data_ptr(), ws.data_ptr(), wsb, None,
                                            gu.stream()))
        want = np.nonzero(x[offset:] < 0.0)[0]
        assert int(gu.host(ln)[0]) == want.size
        got = gu.host(lst)
        assert np.array_equal(got[:want.size], want.astype(np.int32))
        assert np.all(got[want.size:] == -5)
    assert lib().b200_workspace_status(ws.data_ptr(), wsb, gu.stream()) == rp.B200_OK


@pytest.mark.parametrize("num_bins", [1, 10, 1000, 20000])
@pytest.mark.parametrize("layout", ["runs", "random"])
def test_histogram(num_bins, layout):
    torch = gu.torch_cuda()
    rng = np.random.default_rng(num_bins)
    n = 300007
    if layout == "runs":
        bins = np.sort(rng.integers(0, num_bins, n))
    else:
        bins = rng.integers(0, num_bins, n)
    bins[rng.integers(0, n, 50)] = num_bins + 3   # out of range: skipped
    bins[rng.integers(0, n, 50)] = -1
    init = rng.integers(0, 1000, num_bins).astype(np.uint64)
    db = gu.dev(bins.astype(np.int64))
    dinit = gu.dev(init.astype(np.int64))
    counts = zeros(num_bins, torch.int64)
    for _ in range(2):
        rp.check(lib().b200_algorithm_histogram(db.data_ptr(), n, num_bins, dinit.data_ptr(),
                                                counts.data_ptr(), None, gu.stream()))
        ok = (bins >= 0) & (bins < num_bins)
        want = init + np.bincount(bins[ok], minlength=num_bins).astype(np.uint64)
        assert np.array_equal(gu.host(counts).view(np.uint64)[:num_bins], want)


@pytest.mark.parametrize("num_bins", [1, 10, 96, 97, 500])
def test_multi_reduce(num_bins):
    torch = gu.torch_cuda()
    rng = np.random.default_rng(num_bins + 1)
    n = 400003
    bins = rng.integers(0, num_bins, n)
    bins[rng.integers(0, n, 20)] = num_bins  # out of range: skipped
    data = rng.uniform(0, 1, n)
    init = rng.uniform(-1, 1, num_bins)
    db, dd, dinit = gu.dev(bins.astype(np.int64)), gu.dev(data), gu.dev(init)
    vals = zeros(num_bins, torch.float64)
    wsb = lib().b200_multi_reduce_workspace_bytes(n, num_bins)
    ws = zeros(wsb, torch.uint8)
    runs = []
    for _ in range(2):
        rp.check(lib().b200_basic_multi_reduce(db.data_ptr(), dd.data_ptr(), n, num_bins,
                                               dinit.data_ptr(), vals.data_ptr(), ws.data_ptr(),
                                               wsb, None, gu.stream()))
        runs.append(gu.host(vals)[:num_bins].copy())
    ok = bins < num_bins
    want = init + np.bincount(bins[ok], weights=data[ok], minlength=num_bins)
    absum = np.abs(init) + np.bincount(bins[ok], weights=np.abs(data[ok]), minlength=num_bins)
    bound = (n + 64) * gu.U * absum
    assert np.all(np.abs(runs[0] - want) <= bound)
    if num_bins <= 96:
        assert np.array_equal(runs[0], runs[1])  # deterministic path


def test_bad_args_rejected():
    torch = gu.torch_cuda()
    x = zeros(16, torch.float64)
    assert lib().b200_algorithm_histogram(x.data_ptr(), 4, 0, x.data_ptr(), x.data_ptr(),
                                          None, None) == rp.B200_ERR_INVALID_ARG
    assert lib().b200_basic_indexlist(x.data_ptr(), x.data_ptr(), 1 << 31, x.data_ptr(),
                                      x.data_ptr(), 1 << 20, None, None) == rp.B200_ERR_INVALID_ARG
    assert lib().b200_basic_indexlist(x.data_ptr(), x.data_ptr(), 100, x.data_ptr(),
                                      x.data_ptr(), 8, None, None) == rp.B200_ERR_WORKSPACE


class HaloSeg(ctypes.Structure):
    _fields_ = [("var", ctypes.c_void_p), ("list", ctypes.c_void_p),
                ("buffer", ctypes.c_void_p), ("len", ctypes.c_int64)]


def test_halo_packing_segments():
    """Packs read the variables before any unpack of the same call writes
    them; empty segments are skipped; the largest segment tables work."""
    torch = gu.torch_cuda()
    rng = np.random.default_rng(9)
    nvar, size = 3, 5000
    var_h = [rng.uniform(-1, 1, size) for _ in range(nvar)]
    var_d = [gu.dev(v.copy()) for v in var_h]
    lens = [0, 1, 17, 1000, 3000]
    pack, unpack, keep, expect_buf = [], [], [], []
    cells = rng.permutation(size)  # disjoint unpack targets
    pos = 0
    for k, n in enumerate(lens * 40):  # 200 segments per direction
        v = k % nvar
        plist = rng.integers(0, size, n).astype(np.int32)
        ulist = cells[pos:pos + min(n, 20)].astype(np.int32)
        pos = (pos + len(ulist)) % (size - 20)
        pl, ul = gu.dev(plist), gu.dev(ulist)
        pb = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
        ub = gu.dev(rng.uniform(5, 6, max(len(ulist), 1)))
        keep += [pl, ul, pb, ub]
        pack.append(HaloSeg(var_d[v].data_ptr(), pl.data_ptr(), pb.data_ptr(), n))
        unpack.append(HaloSeg(var_d[v].data_ptr(), ul.data_ptr(), ub.data_ptr(), len(ulist)))
        expect_buf.append((pb, var_h[v][plist]))
    P = (HaloSeg * len(pack))(*pack)
    U = (HaloSeg * len(unpack))(*unpack)
    rp.check(lib().b200_comm_halo_packing(ctypes.addressof(P), len(pack), ctypes.addressof(U),
                                          len(unpack), None, gu.stream()))
    for pb, want in expect_buf:  # packed from the values before the unpacks
        assert np.array_equal(gu.host(pb)[:want.size], want)
    want_vars = [v.copy() for v in var_h]
    for k, seg in enumerate(unpack):
        if seg.len:
            ul = gu.host(keep[4 * k + 1])[:seg.len]
            ub = gu.host(keep[4 * k + 3])[:seg.len]
            want_vars[k % nvar][ul] = ub
    for v in range(nvar):
        assert np.array_equal(gu.host(var_d[v]), want_vars[v])
    too_many = (HaloSeg * 257)()
    assert lib().b200_comm_halo_packing(ctypes.addressof(too_many), 257, None, 0, None,
                                        None) == rp.B200_ERR_INVALID_ARG
