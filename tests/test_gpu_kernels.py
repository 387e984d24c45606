"""Element-wise checks of the C ABI against the CPU oracle on random inputs,
including inputs the suite's own data never produce (signed ENERGY
compression, ties and negative zeros for FIRST_MIN, ragged sizes)."""
import ctypes

import numpy as np
import pytest

import oracle
import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu


def close(got, want, rtol=1e-12):
    got = np.asarray(got)
    want = np.asarray(want)
    scale = max(float(np.max(np.abs(want))) if want.size else 0.0, 1e-300)
    assert np.all(np.abs(got - want) <= rtol * np.maximum(np.abs(want), scale * 1e-3)), \
        float(np.max(np.abs(got - want)))


def dev(a):
    return gu.dev(a)


def ws(nbytes):
    torch = gu.torch_cuda()
    return torch.zeros(max(int(nbytes), 1), dtype=torch.uint8, device="cuda")


L = None


def lib():
    global L
    if L is None:
        L = rp.b200()
    return L


@pytest.mark.parametrize("kn,jn", [(3, 3), (5, 7), (64, 65), (257, 300)])
def test_hydro_2d(kn, jn):
    rng = np.random.default_rng(kn * 1000 + jn)
    arrs = [rng.uniform(0.5, 1.5, kn * jn) for _ in range(11)]
    d = [dev(a) for a in arrs]
    rp.check(lib().b200_lcals_hydro_2d(*[t.data_ptr() for t in d], 0.0041, 0.0037, kn, jn,
                                       None, gu.stream()))
    ref = [a.copy() for a in arrs]
    oracle.call("oracle_hydro_2d_rep", *ref, 0.0041, 0.0037, kn, jn)
    for g, w in zip(d, ref):
        close(gu.host(g), w)


def test_del_dot_vec_2d_irregular_zones():
    rng = np.random.default_rng(3)
    jp, nn = 37, 37 * 40
    x, y, xd, yd = (rng.uniform(0.5, 1.5, nn) for _ in range(4))
    div = np.zeros(nn)
    zones = rng.permutation(np.arange(0, nn - jp - 1))[:500].astype(np.int64)
    # keep every device buffer referenced until the kernel has run: a
    # temporary's memory would be handed to the next allocation
    dd, dx, dy, dxd, dyd, dz = dev(div), dev(x), dev(y), dev(xd), dev(yd), dev(zones)
    rp.check(lib().b200_apps_del_dot_vec_2d(dx.data_ptr(), dy.data_ptr(), dxd.data_ptr(),
                                            dyd.data_ptr(), dd.data_ptr(), dz.data_ptr(),
                                            zones.size, jp, 1e-20, 0.5, None, gu.stream()))
    oracle.call("oracle_del_dot_vec_2d_rep", x, y, xd, yd, div, zones, zones.size, jp,
                1e-20, 0.5)
    close(gu.host(dd), div)


@pytest.mark.parametrize("int_adds", [2, 4, 6, 8])
def test_del_dot_vec_2d_integer_pipe_adds_bit_identical(int_adds):
    """Corner sums opened on the integer pipes (tile_z = 1 + count): the same
    bits as the FP64-pipe form on a mesh of positive coordinates and fields
    (the fast path) and on signed fields with zeros (the fallback)."""
    rng = np.random.default_rng(17 + int_adds)
    jp, rows = 301, 120
    nn = jp * rows
    ii, jj = np.meshgrid(np.arange(jp), np.arange(rows))
    for signed in (False, True):
        x = (ii.ravel() * 0.2 + rng.uniform(-0.02, 0.02, nn))
        y = (jj.ravel() * 0.1 + rng.uniform(-0.01, 0.01, nn))
        lo = -1.5 if signed else 0.5
        xd, yd = rng.uniform(lo, 1.5, nn), rng.uniform(lo, 1.5, nn)
        if signed:
            xd[rng.integers(0, nn, 30)] = 0.0
        zones = np.arange(0, nn - jp - 1, dtype=np.int64)
        zones = zones[(zones % jp) != jp - 1]
        out = []
        for tz in (1, 1 + int_adds):
            div = np.zeros(nn)
            dd, dx, dy, dxd, dyd, dz = dev(div), dev(x), dev(y), dev(xd), dev(yd), dev(zones)
            rp.check(lib().b200_apps_del_dot_vec_2d(
                dx.data_ptr(), dy.data_ptr(), dxd.data_ptr(), dyd.data_ptr(), dd.data_ptr(),
                dz.data_ptr(), zones.size, jp, 1e-20, 0.5, ctypes.byref(rp.Tune(tile_z=tz)),
                gu.stream()))
            out.append(gu.host(dd))
        assert np.array_equal(out[0], out[1])


def test_vol3d_random_mesh():
    rng = np.random.default_rng(4)
    jp, kp = 11, 11 * 13
    nn = kp * 9
    x, y, z = (rng.uniform(0.0, 3.0, nn) for _ in range(3))
    vol = np.zeros(nn)
    ib, ie = 5, nn - kp - jp - 2
    dv, dx, dy, dz = dev(vol), dev(x), dev(y), dev(z)
    rp.check(lib().b200_apps_vol3d(dx.data_ptr(), dy.data_ptr(), dz.data_ptr(),
                                   dv.data_ptr(), 1.0 / 12, jp, kp, ib, ie, None, gu.stream()))
    oracle.call("oracle_vol3d_rep", x, y, z, vol, 1.0 / 12, jp, kp, ib, ie)
    close(gu.host(dv), vol, rtol=1e-10)


@pytest.mark.parametrize("n", [1, 33, 10007])
def test_energy_all_branches(n):
    rng = np.random.default_rng(n)
    arrs = [rng.uniform(0.1, 1.5, n) for _ in range(15)]
    arrs[2] = rng.uniform(-1.0, 1.0, n)       # delvc: both signs
    arrs[12] = rng.uniform(-1.0, 1.0, n)      # ql_old
    arrs[5] = np.zeros(n)                     # q_new
    arrs[0] = np.zeros(n)                     # e_new
    arrs[11][::7] = -5.0                      # pbvc: drive ssc <= tiny
    # zeros and subnormals in delvc and work: the exponent-move products and
    # the integer-pipe division by 6 fall back to the FP64 pipe for them
    arrs[2][::11] = 0.0
    arrs[2][5::13] = 3e-310
    arrs[7][::17] = 0.0
    arrs[7][3::19] = -2e-309
    scal = (0.3, 0.01, -0.5, 0.02)
    d = [dev(a) for a in arrs]
    rp.check(lib().b200_apps_energy(*[t.data_ptr() for t in d], *scal, n, None, gu.stream()))
    ref = [a.copy() for a in arrs]
    oracle.call("oracle_energy_rep", *ref, *scal, n)
    close(gu.host(d[0]), ref[0], rtol=1e-11)
    close(gu.host(d[5]), ref[5], rtol=1e-11)


def test_pressure_clamps():
    n = 5000
    rng = np.random.default_rng(9)
    comp = rng.uniform(-1.2, 1.0, n)
    eold = rng.uniform(-1.0, 1.0, n)
    vnew = rng.uniform(0.0, 2.0, n)
    bvc = np.zeros(n)
    pnew = np.zeros(n)
    cls, p_cut, pmin, eosvmax = 0.2, 0.01, -0.05, 1.7
    db, dp, dc, de, dvn = dev(bvc), dev(pnew), dev(comp), dev(eold), dev(vnew)
    rp.check(lib().b200_apps_pressure(dc.data_ptr(), db.data_ptr(), dp.data_ptr(),
                                      de.data_ptr(), dvn.data_ptr(), cls, p_cut,
                                      pmin, eosvmax, n, None, gu.stream()))
    b = cls * (comp + 1.0)
    p = b * eold
    p = np.where(np.abs(p) < p_cut, 0.0, p)
    p = np.where(vnew >= eosvmax, 0.0, p)
    p = np.where(p < pmin, pmin, p)
    assert np.array_equal(gu.host(db), b)
    close(gu.host(dp), p)


@pytest.mark.parametrize("N,ts", [(3, 1), (10, 3), (129, 5)])
def test_jacobi_heat(N, ts):
    rng = np.random.default_rng(N)
    A, B = rng.uniform(0.5, 1.5, N * N), rng.uniform(0.5, 1.5, N * N)
    dA, dB = dev(A), dev(B)
    rp.check(lib().b200_polybench_jacobi_2d(dA.data_ptr(), dB.data_ptr(), N, ts, None,
                                            gu.stream()))
    oracle.call("oracle_jacobi_2d", A, B, N, ts)
    close(gu.host(dA), A)
    close(gu.host(dB), B)
    M = max(3, N // 4)
    A3, B3 = rng.uniform(0.5, 1.5, M ** 3), rng.uniform(0.5, 1.5, M ** 3)
    dA3, dB3 = dev(A3), dev(B3)
    rp.check(lib().b200_polybench_heat_3d(dA3.data_ptr(), dB3.data_ptr(), M, ts, None,
                                          gu.stream()))
    oracle.call("oracle_heat_3d", A3, B3, M, ts)
    close(gu.host(dA3), A3)
    close(gu.host(dB3), B3)


@pytest.mark.parametrize("nx,ny,ts", [(1, 1, 1), (2, 5, 2), (33, 65, 4), (200, 130, 3)])
def test_fdtd_2d(nx, ny, ts):
    rng = np.random.default_rng(nx + ny)
    ex, ey, hz = (rng.uniform(0.5, 1.5, nx * ny) for _ in range(3))
    fict = rng.uniform(0.5, 1.5, ts)
    d = [dev(a) for a in (ex, ey, hz)]
    df = dev(fict)
    rp.check(lib().b200_polybench_fdtd_2d(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                          df.data_ptr(), nx, ny, ts, None, gu.stream()))
    oracle.call("oracle_fdtd_2d", ex, ey, hz, fict, nx, ny, ts)
    for g, w in zip(d, (ex, ey, hz)):
        close(gu.host(g), w)


@pytest.mark.parametrize("rows", [8, 16, 32])
@pytest.mark.parametrize("nx,ny,ts", [(1, 1, 2), (1, 7, 2), (7, 1, 3), (2, 2, 1), (33, 129, 3),
                                     (32, 128, 2), (64, 256, 4), (100, 300, 5), (257, 1000, 3)])
def test_fdtd_2d_one_launch_per_step(nx, ny, ts, rows):
    """The fused step (one launch per time step, tile edges from snapshots) is
    bit-identical to the two-launch form, tiles cut across rows and columns
    and partial last tiles included, and the workspace needs no zeroing."""
    rng = np.random.default_rng(nx * 1000 + ny)
    ex, ey, hz = (rng.uniform(0.5, 1.5, nx * ny) for _ in range(3))
    fict = rng.uniform(0.5, 1.5, ts)
    d1 = [dev(a) for a in (ex, ey, hz)]
    d2 = [dev(a) for a in (ex, ey, hz)]
    df = dev(fict)
    rp.check(lib().b200_polybench_fdtd_2d(d1[0].data_ptr(), d1[1].data_ptr(), d1[2].data_ptr(),
                                          df.data_ptr(), nx, ny, ts, None, gu.stream()))
    wb = lib().b200_fdtd_2d_workspace_bytes(nx, ny)
    torch = gu.torch_cuda()
    w = torch.full((wb,), 0x7F, dtype=torch.uint8, device="cuda")
    t = rp.Tune(tile_y=rows)
    rp.check(lib().b200_polybench_fdtd_2d_ws(d2[0].data_ptr(), d2[1].data_ptr(), d2[2].data_ptr(),
                                             df.data_ptr(), nx, ny, ts, w.data_ptr(), wb,
                                             ctypes.byref(t), gu.stream()))
    for a, b in zip(d1, d2):
        assert np.array_equal(gu.host(a), gu.host(b))
    oracle.call("oracle_fdtd_2d", ex, ey, hz, fict, nx, ny, ts)
    for g, w_ in zip(d2, (ex, ey, hz)):
        close(gu.host(g), w_)


def test_fdtd_2d_ws_rejects_small_workspace():
    torch = gu.torch_cuda()
    x = torch.zeros(64 * 64, dtype=torch.float64, device="cuda")
    wb = lib().b200_fdtd_2d_workspace_bytes(64, 64)
    assert lib().b200_polybench_fdtd_2d_ws(x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                                           64, 64, 1, x.data_ptr(), wb - 8, None,
                                           None) == rp.B200_ERR_WORKSPACE


SCAN_TUNES = {"default": dict(), "ring": dict(algo=2), "tile4096": dict(algo=1, items=16),
              "tile8192": dict(algo=1, items=32)}


@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 8191, 8193, 100003, 1 << 21,
                               152 * 4096 * 3 + 1000])
@pytest.mark.parametrize("kind", sorted(SCAN_TUNES))
def test_scan_f64_and_i64(n, kind):
    """The pipelined persistent kernel and the one-tile-per-CTA kernel with
    both tile sizes; the calls alternate kernels on one workspace, which the
    epoch-tagged statuses and the ticket reset must tolerate."""
    rng = np.random.default_rng(n)
    x = rng.uniform(0.0, 1.0, n)
    xi = rng.integers(0, 100, n).astype(np.int64)
    wsb = lib().b200_scan_workspace_bytes(n)
    w = ws(wsb)
    torch = gu.torch_cuda()
    dy = torch.zeros(n, dtype=torch.float64, device="cuda")
    dyi = torch.zeros(n, dtype=torch.int64, device="cuda")
    dx, dxi = dev(x), dev(xi)
    t = rp.Tune(**SCAN_TUNES[kind])
    other = rp.Tune(algo=1, items=16) if kind in ("default", "ring") else rp.Tune(algo=2)
    for rep in range(3):  # the workspace is reused across calls
        rp.check(lib().b200_algorithm_scan(dx.data_ptr(), dy.data_ptr(), n, 0.25,
                                           w.data_ptr(), wsb, ctypes.byref(other), gu.stream()))
        rp.check(lib().b200_algorithm_scan(dx.data_ptr(), dy.data_ptr(), n, 0.25,
                                           w.data_ptr(), wsb, ctypes.byref(t), gu.stream()))
        rp.check(lib().b200_algorithm_scan_i64(dxi.data_ptr(), dyi.data_ptr(), n, 7,
                                               w.data_ptr(), wsb, ctypes.byref(t), gu.stream()))
        want_i = 7 + np.concatenate([[0], np.cumsum(xi)[:-1]])
        assert np.array_equal(gu.host(dyi), want_i)
        want = np.zeros(n)
        oracle.call("oracle_scan_f64", x, want, n)
        want += 0.25
        got = gu.host(dy)
        assert np.all(np.abs(got - want) <= (n + 64) * gu.U * (np.abs(want) + 0.25))
    hdr = gu.host(w)[:24].view(np.uint32)
    assert hdr[4] == 0, "lookback wait gave up"
    assert hdr[0] == 0, "ticket count not reset"


@pytest.mark.parametrize("n", [8192 * 3 + 5, 1 << 20])
def test_scan_misaligned_pointers(n):
    """x and y one element past a 16-byte boundary: the 8-byte load/store
    path; results must match the vector path's exactly (int64)."""
    torch = gu.torch_cuda()
    rng = np.random.default_rng(n)
    xi = rng.integers(0, 100, n + 1).astype(np.int64)
    dx = dev(xi)
    dy = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    wsb = lib().b200_scan_workspace_bytes(n)
    w = ws(wsb)
    rp.check(lib().b200_algorithm_scan_i64(dx.data_ptr() + 8, dy.data_ptr() + 8, n, 3,
                                           w.data_ptr(), wsb, None, gu.stream()))
    want = 3 + np.concatenate([[0], np.cumsum(xi[1:])[:-1]])
    got = gu.host(dy)[1:]
    assert np.array_equal(got, want)
    assert gu.host(dy)[0] == 0  # nothing written before y


@pytest.mark.parametrize("case", ["planted", "ties", "first", "last", "negzero", "tiny",
                                  "nan", "inf"])
def test_first_min_exact(case):
    n = 1 << 20 if case != "tiny" else 1
    rng = np.random.default_rng(1)
    x = rng.uniform(0.5, 1.5, n)
    if case == "planted":
        x[123457] = -1e10
    elif case == "ties":
        x[999] = x[5000] = x[777777] = -2.0
    elif case == "first":
        x[0] = -3.0
        x[100] = -3.0
    elif case == "last":
        x[-1] = -1.0
    elif case == "negzero":
        x[:] = 1.0
        x[4000] = 0.0
        x[300] = -0.0
    elif case == "nan":
        x[10:1000] = np.nan
        x[77777] = -7.0
    elif case == "inf":
        x[5] = np.inf
        x[6000] = -np.inf
        x[7000] = -np.inf
    # strict '<' scan from (x[0], 0), as the suite's loop
    finite = np.where(np.isnan(x), np.inf, x)
    cand = int(np.argmin(finite))
    want = cand if finite[cand] < x[0] else 0
    torch = gu.torch_cuda()
    loc = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    val = torch.zeros(1, dtype=torch.float64, device="cuda")
    wsb = lib().b200_reduce_workspace_bytes(n, None)
    w = ws(wsb)
    dx = dev(x)
    for _ in range(2):
        rp.check(lib().b200_lcals_first_min(dx.data_ptr(), n, float(x[0]), 0,
                                            loc.data_ptr(), val.data_ptr(), w.data_ptr(), wsb,
                                            None, gu.stream()))
        assert int(gu.host(loc)[0]) == want
        got_val = float(gu.host(val)[0])
        assert got_val == float(x[want]) or (np.isnan(got_val) and np.isnan(x[want]))


@pytest.mark.parametrize("n", [(1 << 20) + 4095, (1 << 20) + 1, 3 * (1 << 20) + 17])
@pytest.mark.parametrize("case", ["tail", "last_tile", "tie_tile_tail", "tie_ctas", "uniform"])
@pytest.mark.parametrize("tune", ["default", "grid7", "algo1", "unaligned"])
def test_first_min_tails(n, case, tune):
    """Sizes past 2^20 that are not multiples of 4096 (and odd): the minimum in
    the ragged end, ties between distant tiles and between a tile and the end,
    the default grid, a 7-CTA grid (long grid-stride loops), an algo tuning and
    an unaligned start (8-byte loads instead of pairs)."""
    rng = np.random.default_rng(n + len(case))
    x = rng.uniform(0.5, 1.5, n)
    whole = (n // 4096) * 4096
    if case == "tail":
        x[n - 1] = -1.0
    elif case == "last_tile":
        x[whole - 1] = -1.0
        x[n - 1] = -1.0
    elif case == "tie_tile_tail":
        x[n - 1] = -1.0
        x[4096 * 3 + 5] = -1.0
    elif case == "tie_ctas":
        for i in (4096 * 200 + 7, 4096 * 1 + 4095, 4096 * 5 + 2, whole - 4096):
            x[i] = -4.0
    torch = gu.torch_cuda()
    loc = torch.full((1,), -2, dtype=torch.int64, device="cuda")
    val = torch.zeros(1, dtype=torch.float64, device="cuda")
    wsb = lib().b200_reduce_workspace_bytes(n, None)
    w = ws(wsb)
    dx = dev(x)
    ptr, m, xs = dx.data_ptr(), n, x
    t = None
    if tune == "grid7":
        t = rp.Tune(grid_blocks=7)
    elif tune == "algo1":
        t = rp.Tune(algo=1)
    elif tune == "unaligned":
        ptr, m, xs = ptr + 8, n - 1, x[1:]
    want = int(np.argmin(xs))
    want = want if xs[want] < xs[0] else 0
    for _ in range(3):
        rp.check(lib().b200_lcals_first_min(ptr, m, float(xs[0]), 0, loc.data_ptr(),
                                            val.data_ptr(), w.data_ptr(), wsb,
                                            ctypes.byref(t) if t is not None else None,
                                            gu.stream()))
        assert int(gu.host(loc)[0]) == want
        assert float(gu.host(val)[0]) == float(xs[want])


@pytest.mark.parametrize("n", [0, 1, 1000, 1 << 22])
def test_reduce_sum(n):
    rng = np.random.default_rng(n)
    x = rng.uniform(0.5, 1.5, n)
    torch = gu.torch_cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    wsb = lib().b200_reduce_workspace_bytes(n, None)
    w = ws(wsb)
    dx = dev(x)
    rp.check(lib().b200_algorithm_reduce_sum(dx.data_ptr() if n else 0, n, 1.5,
                                             out.data_ptr(), w.data_ptr(), wsb, None,
                                             gu.stream()))
    got = float(gu.host(out)[0])
    want = 1.5 + float(np.sum(x))
    assert abs(got - want) <= gu.reduction_bound(max(n, 1), 1, want)


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (7, 5, 3), (64, 64, 64), (100, 130, 77),
                                   (257, 129, 300)])
def test_gemm_f64(m, n, k):
    rng = np.random.default_rng(m * n * k)
    A, B, C = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n), rng.uniform(-1, 1, m * n)
    dA, dB, dC = dev(A), dev(B), dev(C)
    rp.check(lib().b200_gemm_f64(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k,
                                 1.5, 1.2, None, gu.stream()))
    want = 1.5 * (A.reshape(m, k) @ B.reshape(k, n)) + 1.2 * C.reshape(m, n)
    bound = (k + 2) * gu.U * (1.5 * (np.abs(A.reshape(m, k)) @ np.abs(B.reshape(k, n))) +
                              1.2 * np.abs(C.reshape(m, n)))
    assert np.all(np.abs(gu.host(dC).reshape(m, n) - want) <= bound)


@pytest.mark.parametrize("fn,args", [
    ("b200_lcals_eos", 8), ("b200_lcals_hydro_1d", 7), ("b200_lcals_first_diff", 3),
])
def test_null_pointer_rejected(fn, args):
    f = getattr(lib(), fn)
    argv = [None] * (len(f.argtypes))
    for i, t in enumerate(f.argtypes):
        if t is ctypes.c_double:
            argv[i] = 1.0
        elif t in (ctypes.c_int64, ctypes.c_long):
            argv[i] = 16
    assert f(*argv) == rp.B200_ERR_INVALID_ARG


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_integer_pipe_fp64_is_bit_exact(op):
    """The integer-pipe add/sub/mul used by the mixed-pipe stencils, the
    exponent-shift products by 0.5, 0.125 and 2 of DEL_DOT_VEC_2D and HEAT_3D,
    the FP64-free division of HYDRO_2D and DEL_DOT_VEC_2D, INDEXLIST's integer
    x < 0 test, the integer-pipe multiply of JACOBI_2D, HYDRO_2D and
    DEL_DOT_VEC_2D, DEL_DOT_VEC_2D's + ptiny, JACOBI_2D's close-exponent
    integer add, HEAT_3D's signed one and EOS's integer-pipe FMA, against the FP64 pipe on 16M operands (every class of
    double; 64M for the division)."""
    torch = gu.torch_cuda()
    bad = torch.zeros(1, dtype=torch.int64, device="cuda")
    n = (1 << 26) if op == 6 else (1 << 24)
    rp.check(lib().b200_f64emu_selftest(n, 12345 + op, op, bad.data_ptr(), gu.stream()))
    assert int(gu.host(bad)[0]) == 0


@pytest.mark.parametrize("N,ts", [(3, 1), (37, 2), (300, 3), (1031, 2)])
@pytest.mark.parametrize("int_adds", [0, 4, 8, 9, 10, 12])
@pytest.mark.parametrize("mul_fp64", [False, True])
@pytest.mark.parametrize("rows", [2, 4])
def test_jacobi_integer_pipe_adds_bit_identical(N, ts, int_adds, mul_fp64, rows):
    """Integer-pipe adds per four points (tile_z = 1 + count) and the product
    by 0.2 on either pipe (tile_y 2: FP64): bit-identical to the suite's loop
    in the oracle, on data of one sign (the fast path) and on signed data
    with zeros (the native fallback)."""
    rng = np.random.default_rng(N + 11 * int_adds + rows + 3 * mul_fp64)
    for signed in (False, True):
        lo = -1.5 if signed else 0.5
        A, B = rng.uniform(lo, 1.5, N * N), rng.uniform(lo, 1.5, N * N)
        if signed:
            A[rng.integers(0, N * N, 20)] = 0.0
        dA, dB = dev(A), dev(B)
        t = rp.Tune(items=rows, tile_z=1 + int_adds, tile_y=2 if mul_fp64 else 1)
        rp.check(lib().b200_polybench_jacobi_2d(dA.data_ptr(), dB.data_ptr(), N, ts,
                                                ctypes.byref(t), gu.stream()))
        oracle.call("oracle_jacobi_2d", A, B, N, ts)
        assert np.array_equal(gu.host(dA), A) and np.array_equal(gu.host(dB), B)


@pytest.mark.parametrize("N,ts", [(3, 1), (4, 1), (19, 2), (66, 3)])
@pytest.mark.parametrize("subs2", [0, 1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("planes", [2, 4])
def test_heat_integer_pipe_differences_bit_identical(N, ts, subs2, planes):
    """HEAT_3D with each thread walking `planes` planes (tile_x) and `subs2`
    of the six differences b(+1) - 2a of two planes on the integer pipes
    (tile_z = 1 + subs2): bit-identical to the suite's loop in the oracle on
    positive data (the fast path, cancellations of any depth), on signed data
    with zeros (the thread fallback) and on a plateau (exact zeros)."""
    rng = np.random.default_rng(N + 5 * subs2 + 31 * planes)
    for data in ("positive", "signed", "plateau"):
        if data == "plateau":
            A, B = np.full(N ** 3, 1.0), np.full(N ** 3, 1.0)
            A[rng.integers(0, N ** 3, 30)] = 1.5
        else:
            lo = -1.5 if data == "signed" else 0.5
            A, B = rng.uniform(lo, 1.5, N ** 3), rng.uniform(lo, 1.5, N ** 3)
            if data == "signed":
                A[rng.integers(0, N ** 3, 20)] = 0.0
        dA, dB = dev(A), dev(B)
        t = rp.Tune(tile_x=planes, tile_z=1 + subs2)
        rp.check(lib().b200_polybench_heat_3d(dA.data_ptr(), dB.data_ptr(), N, ts,
                                              ctypes.byref(t), gu.stream()))
        oracle.call("oracle_heat_3d", A, B, N, ts)
        assert np.array_equal(gu.host(dA), A) and np.array_equal(gu.host(dB), B), data


def test_heat_integer_pipe_bad_counts_rejected():
    torch = gu.torch_cuda()
    d = torch.zeros(27, dtype=torch.float64, device="cuda")
    for tx, tz in ((2, 8), (1, 1), (3, 1), (8, 1)):
        t = rp.Tune(tile_x=tx, tile_z=tz)
        assert lib().b200_polybench_heat_3d(d.data_ptr(), d.data_ptr(), 3, 1, ctypes.byref(t),
                                            gu.stream()) == rp.B200_ERR_INVALID_ARG


@pytest.mark.parametrize("N,ts", [(3, 1), (37, 2), (300, 3)])
@pytest.mark.parametrize("shape", [(5, 4, 10), (1, 1, 3), (9, 2, 1), (4, 1, 7)])
def test_jacobi_mixed_pipes_bit_identical(N, ts, shape):
    rng = np.random.default_rng(N * 7 + shape[0])
    A, B = rng.uniform(0.5, 1.5, N * N), rng.uniform(0.5, 1.5, N * N)
    dA1, dB1, dA2, dB2 = dev(A), dev(B), dev(A), dev(B)
    rp.check(lib().b200_polybench_jacobi_2d(dA1.data_ptr(), dB1.data_ptr(), N, ts, None,
                                            gu.stream()))
    t = rp.Tune(algo=shape[0], tile_y=shape[1], tile_z=shape[2])
    rp.check(lib().b200_polybench_jacobi_2d(dA2.data_ptr(), dB2.data_ptr(), N, ts,
                                            ctypes.byref(t), gu.stream()))
    assert np.array_equal(gu.host(dA1), gu.host(dA2))
    assert np.array_equal(gu.host(dB1), gu.host(dB2))


@pytest.mark.parametrize("N,ts", [(3, 1), (20, 2), (70, 2)])
@pytest.mark.parametrize("shape", [(5, 2, 5, 32), (1, 1, 2, 3), (9, 1, 1, 7), (3, 3, 1, 5)])
def test_heat_mixed_pipes_bit_identical(N, ts, shape):
    rng = np.random.default_rng(N * 11 + shape[0])
    A, B = rng.uniform(0.5, 1.5, N ** 3), rng.uniform(0.5, 1.5, N ** 3)
    dA1, dB1, dA2, dB2 = dev(A), dev(B), dev(A), dev(B)
    rp.check(lib().b200_polybench_heat_3d(dA1.data_ptr(), dB1.data_ptr(), N, ts, None,
                                          gu.stream()))
    t = rp.Tune(algo=shape[0], tile_y=shape[1], tile_z=shape[2], tile_x=shape[3])
    rp.check(lib().b200_polybench_heat_3d(dA2.data_ptr(), dB2.data_ptr(), N, ts,
                                          ctypes.byref(t), gu.stream()))
    assert np.array_equal(gu.host(dA1), gu.host(dA2))
    assert np.array_equal(gu.host(dB1), gu.host(dB2))


@pytest.mark.parametrize("case", ["plateau", "subnormal", "mixed"])
def test_heat_exponent_shift_special_values(case):
    """The default HEAT_3D kernel scales by 0.125 with an integer exponent move
    and rewrites a thread's points with FP64 products when a term is zero,
    subnormal or non-finite; its results must equal the all-FP64-pipe
    kernel's (algo 1: no emulated warps) bit for bit on such data."""
    N, ts = 34, 2
    rng = np.random.default_rng(7)
    A = np.full(N ** 3, 1.0)
    B = np.full(N ** 3, 1.0)
    if case == "plateau":          # exactly zero Laplacian terms almost everywhere
        A[rng.integers(0, N ** 3, 40)] = 1.5
    elif case == "subnormal":      # terms and results below the normal range
        A = rng.uniform(0.5, 1.5, N ** 3) * 1e-308
        B = rng.uniform(0.5, 1.5, N ** 3) * 1e-308
    else:
        A = rng.uniform(0.5, 1.5, N ** 3)
        A[: N ** 3 // 2] = 0.75
        A[rng.integers(0, N ** 3, 100)] = 4e-310
    dA1, dB1, dA2, dB2 = dev(A), dev(B), dev(A), dev(B)
    rp.check(lib().b200_polybench_heat_3d(dA1.data_ptr(), dB1.data_ptr(), N, ts, None,
                                          gu.stream()))
    t = rp.Tune(algo=1)
    rp.check(lib().b200_polybench_heat_3d(dA2.data_ptr(), dB2.data_ptr(), N, ts,
                                          ctypes.byref(t), gu.stream()))
    assert np.array_equal(gu.host(dA1).view(np.int64), gu.host(dA2).view(np.int64))
    assert np.array_equal(gu.host(dB1).view(np.int64), gu.host(dB2).view(np.int64))


@pytest.mark.parametrize("case", ["zeros", "subnormal", "mixed"])
def test_jacobi_integer_multiply_special_values(case):
    """The default JACOBI_2D kernel multiplies by 0.2 on the integer pipe and
    rewrites a thread's points natively when a sum is zero, subnormal or
    non-finite; its results must equal the all-FP64-pipe kernel's (algo 1:
    no emulated warps) bit for bit on such data."""
    N, ts = 70, 3
    rng = np.random.default_rng(11)
    if case == "zeros":
        A = np.zeros(N * N)
        A[rng.integers(0, N * N, 30)] = 1.0
    elif case == "subnormal":
        A = rng.uniform(0.5, 1.5, N * N) * 1e-310
    else:
        A = rng.uniform(0.5, 1.5, N * N)
        A[: N * N // 3] = 0.0
        A[rng.integers(0, N * N, 50)] = 3e-309
    B = rng.uniform(0.5, 1.5, N * N)
    dA1, dB1, dA2, dB2 = dev(A), dev(B), dev(A), dev(B)
    rp.check(lib().b200_polybench_jacobi_2d(dA1.data_ptr(), dB1.data_ptr(), N, ts, None,
                                            gu.stream()))
    t = rp.Tune(algo=1)
    rp.check(lib().b200_polybench_jacobi_2d(dA2.data_ptr(), dB2.data_ptr(), N, ts,
                                            ctypes.byref(t), gu.stream()))
    assert np.array_equal(gu.host(dA1).view(np.int64), gu.host(dA2).view(np.int64))
    assert np.array_equal(gu.host(dB1).view(np.int64), gu.host(dB2).view(np.int64))


def close_special(got, want, rtol=1e-12):
    """NaNs and infinities in the same places (infinities with the same
    sign), the finite values within rtol."""
    got, want = np.asarray(got), np.asarray(want)
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN positions differ"
    inf = np.isinf(want)
    assert np.array_equal(np.isinf(got), inf), "infinity positions differ"
    assert np.array_equal(got[inf], want[inf]), "infinity signs differ"
    fin = np.isfinite(want)
    if fin.any():
        close(got[fin], want[fin], rtol)


@pytest.mark.parametrize("kh", [2, 4, 6, 8])
@pytest.mark.parametrize("kn,jn", [(3, 3), (9, 70), (131, 257)])
def test_hydro_2d_integer_pipe_differences_bit_identical(kh, kn, jn):
    """BODY2 with `kh` of its eight differences on the integer pipes
    (tile_z = 1 + kh): every output bit-identical to the FP64-pipe kernel
    (tile_z = 1), on positive data (the fast path) and on signed data with
    zeros, subnormals and equal neighbours (the voted FP64 redo)."""
    rng = np.random.default_rng(kh * 7 + kn + jn)
    for data in ("positive", "special"):
        arrs = [rng.uniform(0.5 if data == "positive" else -1.5, 1.5, kn * jn) for _ in range(11)]
        if data == "special":
            zz, zr = arrs[8], arrs[5]
            zz[rng.integers(0, kn * jn, 40)] = 0.0
            zr[rng.integers(0, kn * jn, 40)] = 3e-310
            zz[1::7] = zz[0::7][: len(zz[1::7])]              # equal neighbours: exact zeros
        outs = []
        for tz in (1, 1 + kh):
            d = [dev(a) for a in arrs]
            t = rp.Tune(tile_z=tz)
            rp.check(lib().b200_lcals_hydro_2d(*[x.data_ptr() for x in d], 0.0041, 0.0037, kn, jn,
                                               ctypes.byref(t), gu.stream()))
            outs.append([gu.host(x) for x in d])
        for g, w in zip(outs[1], outs[0]):
            assert np.array_equal(g.view(np.int64), w.view(np.int64)), data


def test_hydro_2d_integer_pipe_long_columns():
    """More than 64 interior rows per thread (kn - 2 > 64 x 65535 with jn = 3):
    the launcher falls back to the FP64-pipe differences (one redo bit per
    point would not fit), and the results equal the FP64-pipe kernel's."""
    kn, jn = 64 * 65535 + 2 + 700, 3
    rng = np.random.default_rng(99)
    arrs = [rng.uniform(0.5, 1.5, kn * jn) for _ in range(11)]
    outs = []
    for tz in (1, 7):
        d = [dev(a) for a in arrs]
        t = rp.Tune(tile_z=tz)
        rp.check(lib().b200_lcals_hydro_2d(*[x.data_ptr() for x in d], 0.0041, 0.0037, kn, jn,
                                           ctypes.byref(t), gu.stream()))
        outs.append([gu.host(x) for x in d])
        del d
    for g, w in zip(outs[1], outs[0]):
        assert np.array_equal(g.view(np.int64), w.view(np.int64))


def test_hydro_2d_bad_difference_count_rejected():
    torch = gu.torch_cuda()
    d = torch.zeros(9, dtype=torch.float64, device="cuda")
    for tz in (2, 10):
        t = rp.Tune(tile_z=tz)
        assert lib().b200_lcals_hydro_2d(*([d.data_ptr()] * 11), 0.1, 0.1, 3, 3, ctypes.byref(t),
                                         gu.stream()) == rp.B200_ERR_INVALID_ARG


@pytest.mark.parametrize("kf,items,block", [(1, 2, 128), (2, 2, 128), (3, 2, 128), (2, 1, 256),
                                             (2, 4, 512), (2, 8, 128), (3, 8, 256)])
@pytest.mark.parametrize("n", [1, 7, 4097, 100003])
def test_eos_integer_pipe_fmas_bit_identical(kf, items, block, n):
    """EOS with `kf` of each element's eight FMAs on the integer pipes
    (tile_z = 1 + kf): bit-identical to the FP64-pipe kernel (tile_z = 1) on
    the suite's kind of data (positive; the fast path), on signed data with
    zeros and subnormals (the redo after the loop) and with coefficients
    that put some addends below their products."""
    rng = np.random.default_rng(kf * 31 + items * 7 + block + n)
    for data, coef in (("positive", (0.0979, 0.1958, 0.0979)), ("special", (0.0979, 0.1958, 0.0979)),
                       ("positive", (3.5e9, 2.1e-3, 7.0))):
        lo = 0.5 if data == "positive" else -1.5
        y, z, u = (rng.uniform(lo, 1.5, n + 7) for _ in range(3))
        if data == "special":
            z[rng.integers(0, n + 7, max(1, n // 50))] = 0.0
            u[rng.integers(0, n + 7, max(1, n // 50))] = 2e-310
        outs = []
        for tz in (1, 1 + kf):
            dx, dy, dz, du = dev(np.zeros(n + 7)), dev(y), dev(z), dev(u)
            t = rp.Tune(tile_z=tz, items=items if tz > 1 else 0, block_size=block if tz > 1 else 0)
            rp.check(lib().b200_lcals_eos(dx.data_ptr(), dy.data_ptr(), dz.data_ptr(), du.data_ptr(),
                                          *coef, n, ctypes.byref(t), gu.stream()))
            outs.append(gu.host(dx))
        assert np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64)), (data, coef)


def test_hydro_2d_division_special_values():
    """BODY1 divides without the FP64 pipe and falls back to the FP64 divide
    for zero, subnormal and non-finite operands or quotients: zero
    denominators (+-inf and 0/0) and subnormal numerators must come out as
    the suite's loop gives them."""
    kn, jn = 70, 67
    rng = np.random.default_rng(21)
    arrs = [rng.uniform(0.5, 1.5, kn * jn) for _ in range(11)]
    za, zb, zm, zp, zq, zr = arrs[0], arrs[1], arrs[2], arrs[3], arrs[4], arrs[5]
    zm[rng.integers(0, kn * jn, 300)] = 0.0          # zero denominators
    zp[rng.integers(0, kn * jn, 200)] = zq[0] * 0.0  # zero numerator terms
    zr[rng.integers(0, kn * jn, 100)] = 1e-310       # subnormal factors
    d = [dev(a) for a in arrs]
    rp.check(lib().b200_lcals_hydro_2d(*[t.data_ptr() for t in d], 0.0041, 0.0037, kn, jn,
                                       None, gu.stream()))
    ref = [a.copy() for a in arrs]
    oracle.call("oracle_hydro_2d_rep", *ref, 0.0041, 0.0037, kn, jn)
    for g, w in zip(d[:2], ref[:2]):  # za, zb: BODY1's quotients
        close_special(gu.host(g), w)


def test_del_dot_vec_2d_division_special_values():
    """Degenerate zones (equal corners: zero area with ptiny 0, zero y sums)
    take the FP64 divide: +-inf and NaN where the suite's loop gives them."""
    rng = np.random.default_rng(22)
    jp, nn = 37, 37 * 40
    x, y, xd, yd = (rng.uniform(0.5, 1.5, nn) for _ in range(4))
    x[rng.integers(0, nn, 150)] = 0.0
    y[rng.integers(0, nn, 150)] = 0.0
    x[:jp * 4] = 1.0   # the first rows: equal corners, zero area
    y[:jp * 4] = 0.0   # and zero y sums
    div = np.zeros(nn)
    zones = np.arange(0, nn - jp - 1).astype(np.int64)
    dd, dx, dy, dxd, dyd, dz = dev(div), dev(x), dev(y), dev(xd), dev(yd), dev(zones)
    rp.check(lib().b200_apps_del_dot_vec_2d(dx.data_ptr(), dy.data_ptr(), dxd.data_ptr(),
                                            dyd.data_ptr(), dd.data_ptr(), dz.data_ptr(),
                                            zones.size, jp, 0.0, 0.5, None, gu.stream()))
    oracle.call("oracle_del_dot_vec_2d_rep", x, y, xd, yd, div, zones, zones.size, jp, 0.0, 0.5)
    # Zones whose area cancels between two equal nonzero products are left
    # out: there the FMA-contracted GPU area keeps the products' rounding
    # residual while the suite's loop (each product rounded) gets exactly 0.
    c1, c2, c3, c4 = zones + 1, zones + 1 + jp, zones + jp, zones
    xi = 0.5 * (x[c1] + x[c2] - x[c3] - x[c4])
    xj = 0.5 * (x[c2] + x[c3] - x[c4] - x[c1])
    yi = 0.5 * (y[c1] + y[c2] - y[c3] - y[c4])
    yj = 0.5 * (y[c2] + y[c3] - y[c4] - y[c1])
    cancel = (xi * yj == xj * yi) & (xi * yj != 0.0)
    keep = np.ones(nn, dtype=bool)
    keep[zones[cancel]] = False
    assert keep.sum() > nn // 2
    close_special(gu.host(dd)[keep], div[keep])


def test_planckian_division_special_values():
    """u / v and x / (exp(y) - 1) without the FP64 pipe, with the FP64 divide
    for zero, subnormal and non-finite cases (v = 0, u = v = 0, huge y)."""
    rng = np.random.default_rng(23)
    n = 50000
    x, u, v = rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n), rng.uniform(0.5, 1.5, n)
    v[rng.integers(0, n, 300)] = 0.0
    u[rng.integers(0, n, 300)] = 0.0
    u[rng.integers(0, n, 300)] = 1e-310
    v[rng.integers(0, n, 300)] = 1e-3     # exp(y) overflows for large u / v
    u[rng.integers(0, n, 300)] = 900.0
    dx, du, dv = dev(x), dev(u), dev(v)
    torch = gu.torch_cuda()
    dy = torch.zeros(n, dtype=torch.float64, device="cuda")
    dw = torch.zeros(n, dtype=torch.float64, device="cuda")
    rp.check(lib().b200_lcals_planckian(dx.data_ptr(), dy.data_ptr(), du.data_ptr(),
                                        dv.data_ptr(), dw.data_ptr(), n, None, gu.stream()))
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        want_y = u / v
        want_w = x / (np.exp(want_y) - 1.0)
    close_special(gu.host(dy), want_y)            # a quotient: correctly rounded both ways
    close_special(gu.host(dw), want_w, rtol=1e-14)  # exp may differ in the last bit
