"""Every 1-D kernel at 2^27 elements (the size of the suite-wide bandwidth
figure), checked where a full host checksum would take minutes: element-wise
outputs at sampled windows (and the first and last window) against the
kernels' formulas (the suite's K.hpp macros, as the oracle restates them) on
the same inputs; ENERGY through the oracle's own rep on the gathered
elements; reductions and the scan against full-array references on the
device.  Tolerances: relative 1e-12 element-wise (nvcc contracts a*b+c into
FMA; numpy rounds each operation), exact for FIRST_MIN and the int64 scan,
the reassociation bound for the sums."""
import ctypes

import numpy as np
import pytest

import oracle
import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

N = 1 << 27
W = 512          # window length
WINDOWS = 48     # random windows, plus the first and the last


def lib():
    return rp.b200()


class Arrays:
    """Device arrays filled uniform [0.5, 1.5) by the library's generator."""

    def __init__(self, seed):
        self.seed = seed
        self.sid = 0
        self.keep = []

    def u(self, m):
        torch = gu.torch_cuda()
        t = torch.empty(m, dtype=torch.float64, device="cuda")
        rp.check(lib().b200_init_uniform(t.data_ptr(), m, self.seed, self.sid, 0.5, 1.5, None))
        self.sid += 1
        self.keep.append(t)
        return t

    def z(self, m, dtype=None):
        torch = gu.torch_cuda()
        t = torch.zeros(m, dtype=dtype or torch.float64, device="cuda")
        self.keep.append(t)
        return t


def starts(n, seed):
    rng = np.random.default_rng(seed)
    s = list(rng.integers(0, n - W, WINDOWS)) + [0, n - W]
    return [int(x) for x in s]


def win(t, s, length=W, offset=0):
    return gu.host(t[s + offset: s + offset + length])


def close(got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert np.all(np.abs(got - want) <= 1e-12 * np.maximum(np.abs(want), 1e-300)), \
        float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300)))


ELEMENTWISE = ["Stream_COPY", "Stream_MUL", "Stream_ADD", "Stream_TRIAD", "Basic_DAXPY",
               "Basic_INIT3", "Basic_MULADDSUB", "Lcals_HYDRO_1D", "Lcals_EOS",
               "Lcals_FIRST_DIFF", "Lcals_INT_PREDICT", "Lcals_DIFF_PREDICT",
               "Lcals_PLANCKIAN", "Apps_PRESSURE", "Apps_ENERGY"]


@pytest.mark.parametrize("kernel", ELEMENTWISE)
def test_elementwise_at_2e27(kernel):
    L, A, s = lib(), Arrays(27), gu.stream()
    n = N
    P = lambda t: t.data_ptr()
    q, r, t_ = 0.0979, 0.1958, 0.0979
    if kernel == "Stream_COPY":
        a, c = A.u(n), A.z(n)
        rp.check(L.b200_stream_copy(P(a), P(c), n, None, s))
        check = lambda st: close(win(c, st), win(a, st))
    elif kernel == "Stream_MUL":
        b, c = A.z(n), A.u(n)
        rp.check(L.b200_stream_mul(P(b), P(c), 0.5, n, None, s))
        check = lambda st: close(win(b, st), 0.5 * win(c, st))
    elif kernel == "Stream_ADD":
        a, b, c = A.u(n), A.u(n), A.z(n)
        rp.check(L.b200_stream_add(P(a), P(b), P(c), n, None, s))
        check = lambda st: close(win(c, st), win(a, st) + win(b, st))
    elif kernel == "Stream_TRIAD":
        a, b, c = A.z(n), A.u(n), A.u(n)
        rp.check(L.b200_stream_triad(P(a), P(b), P(c), 0.5, n, None, s))
        check = lambda st: close(win(a, st), win(b, st) + 0.5 * win(c, st))
    elif kernel == "Basic_DAXPY":
        y, x = A.z(n), A.u(n)
        rp.check(L.b200_basic_daxpy(P(y), P(x), 0.5, n, None, s))
        check = lambda st: close(win(y, st), 0.5 * win(x, st))
    elif kernel in ("Basic_INIT3", "Basic_MULADDSUB"):
        o1, o2, o3, i1, i2 = A.z(n), A.z(n), A.z(n), A.u(n), A.u(n)
        fn = L.b200_basic_init3 if kernel == "Basic_INIT3" else L.b200_basic_muladdsub
        rp.check(fn(P(o1), P(o2), P(o3), P(i1), P(i2), n, None, s))

        def check(st):
            x1, x2 = win(i1, st), win(i2, st)
            if kernel == "Basic_INIT3":
                for o in (o1, o2, o3):
                    close(win(o, st), -x1 - x2)
            else:
                close(win(o1, st), x1 * x2)
                close(win(o2, st), x1 + x2)
                close(win(o3, st), x1 - x2)
    elif kernel == "Lcals_HYDRO_1D":
        x, y, z = A.z(n + 12), A.u(n + 12), A.u(n + 12)
        rp.check(L.b200_lcals_hydro_1d(P(x), P(y), P(z), q, r, t_, n, None, s))

        def check(st):
            zz = win(z, st, W + 12)
            close(win(x, st), q + win(y, st) * (r * zz[10:10 + W] + t_ * zz[11:11 + W]))
    elif kernel == "Lcals_EOS":
        x, y, z, u = A.z(n + 7), A.u(n + 7), A.u(n + 7), A.u(n + 7)
        rp.check(L.b200_lcals_eos(P(x), P(y), P(z), P(u), q, r, t_, n, None, s))

        def check(st):
            uu = win(u, st, W + 7)
            U = [uu[k:k + W] for k in range(7)]
            want = (U[0] + r * (win(z, st) + r * win(y, st)) +
                    t_ * (U[3] + r * (U[2] + r * U[1]) + t_ * (U[6] + q * (U[5] + q * U[4]))))
            close(win(x, st), want)
    elif kernel == "Lcals_FIRST_DIFF":
        x, y = A.z(n + 1), A.u(n + 1)
        rp.check(L.b200_lcals_first_diff(P(x), P(y), n, None, s))

        def check(st):
            yy = win(y, st, W + 1)
            close(win(x, st), yy[1:] - yy[:-1])
    elif kernel == "Lcals_INT_PREDICT":
        px = A.u(13 * n)  # 13 planes of n
        dm = [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8]
        rp.check(L.b200_lcals_int_predict(P(px), *dm, n, None, s))

        def check(st):
            p = [win(px, st, offset=k * n) for k in range(13)]
            d22, d23, d24, d25, d26, d27, d28, c0 = dm
            want = (d28 * p[12] + d27 * p[11] + d26 * p[10] + d25 * p[9] + d24 * p[8] +
                    d23 * p[7] + d22 * p[6] + c0 * (p[4] + p[5]) + p[2])
            close(p[0], want)
    elif kernel == "Lcals_DIFF_PREDICT":
        px, cx = A.z(14 * n), A.u(14 * n)  # 14 planes of n each
        rp.check(L.b200_lcals_diff_predict(P(px), P(cx), n, None, s))

        def check(st):
            p = [np.zeros(W) for _ in range(14)]  # px starts at zero
            ar = win(cx, st, offset=4 * n)
            br = ar - p[4]; p[4] = ar
            cr = br - p[5]; p[5] = br
            ar = cr - p[6]; p[6] = cr
            br = ar - p[7]; p[7] = ar
            cr = br - p[8]; p[8] = br
            ar = cr - p[9]; p[9] = cr
            br = ar - p[10]; p[10] = ar
            cr = br - p[11]; p[11] = br
            p[13] = cr - p[12]; p[12] = cr
            for k in range(4, 14):
                close(win(px, st, offset=k * n), p[k])
    elif kernel == "Lcals_PLANCKIAN":
        x, y, u, v, w = A.u(n), A.z(n), A.u(n), A.u(n), A.z(n)
        rp.check(L.b200_lcals_planckian(P(x), P(y), P(u), P(v), P(w), n, None, s))

        def check(st):
            yy = win(u, st) / win(v, st)
            close(win(y, st), yy)
            close(win(w, st), win(x, st) / (np.exp(yy) - 1.0))
    elif kernel == "Apps_PRESSURE":
        comp, bvc, pn, eo, vn = A.u(n), A.z(n), A.z(n), A.u(n), A.u(n)
        cls, p_cut, pmin, eosvmax = 0.5, 0.9, 0.6, 1.3  # every clamp is taken somewhere
        rp.check(L.b200_apps_pressure(P(comp), P(bvc), P(pn), P(eo), P(vn), cls, p_cut, pmin,
                                      eosvmax, n, None, s))

        def check(st):
            b = cls * (win(comp, st) + 1.0)
            p = b * win(eo, st)
            p = np.where(np.abs(p) < p_cut, 0.0, p)
            p = np.where(win(vn, st) >= eosvmax, 0.0, p)
            p = np.where(p < pmin, pmin, p)
            close(win(bvc, st), b)
            close(win(pn, st), p)
    elif kernel == "Apps_ENERGY":
        arrs = [A.z(n)] + [A.u(n) for _ in range(4)] + [A.z(n)] + [A.u(n) for _ in range(9)]
        # delvc signed so both branch families run: delvc = u - 1 in [-0.5, 0.5)
        arrs[2].sub_(1.0)
        sc = (1.1, 0.55, 0.6, 0.05)
        rp.check(L.b200_apps_energy(*[P(t) for t in arrs], *sc, n, None, s))

        def check(st):
            h = [win(t, st) for t in arrs]
            e_new, q_new = np.zeros(W), np.zeros(W)
            oracle.call("oracle_energy_rep", e_new, *h[1:5], q_new, *h[6:], *sc, W)
            close(h[0], e_new)
            close(h[5], q_new)
    else:
        raise KeyError(kernel)
    torch = gu.torch_cuda()
    torch.cuda.synchronize()
    for st in starts(n, 5):
        check(st)


def test_reductions_and_scan_at_2e27():
    torch = gu.torch_cuda()
    L, A, s = lib(), Arrays(28), gu.stream()
    n = N
    P = lambda t: t.data_ptr()
    a, b = A.u(n), A.u(n)
    wb = L.b200_reduce_workspace_bytes(n, None)
    ws = A.z(wb, torch.uint8)
    acc = A.z(1)
    rp.check(L.b200_stream_dot(P(a), P(b), n, 0.0, P(acc), P(ws), wb, None, s))
    want = float(torch.dot(a, b))
    bound = (n + 64) * gu.U * float(torch.sum(a * b))
    assert abs(float(gu.host(acc)[0]) - want) <= bound
    out = A.z(1)
    rp.check(L.b200_algorithm_reduce_sum(P(a), n, 0.0, P(out), P(ws), wb, None, s))
    assert abs(float(gu.host(out)[0]) - float(torch.sum(a))) <= (n + 64) * gu.U * float(
        torch.sum(a))
    # FIRST_MIN: ties at two places, the first must win
    a[n - 5] = -3.0
    a[n // 3] = -3.0
    loc = A.z(1, torch.int64)
    rp.check(L.b200_lcals_first_min(P(a), n, 0.5, 0, P(loc), None, P(ws), wb, None, s))
    assert int(gu.host(loc)[0]) == n // 3
    # int64 scan, exact: the pipelined kernel and the one-tile-per-CTA kernel
    x = torch.empty(n, dtype=torch.int64, device="cuda")
    rp.check(L.b200_init_uniform_i64(P(x), n, 28, 0, 0, 100, None))
    y = A.z(n, torch.int64)
    swb = L.b200_scan_workspace_bytes(n)
    sws = A.z(swb, torch.uint8)
    want = torch.cumsum(x, 0) - x
    for tune in (dict(), dict(algo=1, items=16), dict(algo=1, items=32)):
        y.zero_()
        t = rp.Tune(**tune)
        rp.check(L.b200_algorithm_scan_i64(P(x), P(y), n, 0, P(sws), swb, ctypes.byref(t), s))
        assert bool(torch.equal(y, want))
    assert int(gu.host(sws[16:20]).view(np.uint32)[0]) == 0
