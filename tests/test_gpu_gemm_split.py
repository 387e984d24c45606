"""Split-precision FP64 GEMM (b200_gemm_split) against an FP64 reference.

The bound asked of it is a relative Frobenius error of 1e-13 against FP64;
the test states it per case, including rows scaled by 2^k, k in [-20, 20]
(the slicing is per row/column, so row scaling must not cost accuracy)."""
import ctypes

import numpy as np
import pytest

import rajaperf_gb300 as rp
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

REL_FROB = 1e-13


# 0 the default, 1 mma.sync, 2 tcgen05 on bf16 slices, 3 tcgen05 on e4m3 slices,
# 4 tcgen05 on e4m3 slices with paired digit weights (128 x 256 MMAs)
ENGINES = [0, 1, 2, 3, 4]


def run_split(A, B, C, alpha, beta, slices=None, engine=0):
    torch = gu.torch_cuda()
    m, k = A.shape
    n = B.shape[1]
    L = rp.b200()
    t = rp.Tune(items=slices or 0, algo=engine)
    tp = ctypes.byref(t)
    ws_bytes = L.b200_gemm_split_workspace_bytes(m, n, k, tp)
    # stale bytes everywhere but the 256-byte header, which a workspace
    # starts with zeroed (its error word is at byte 16)
    ws = torch.full((ws_bytes,), 0xAB, dtype=torch.uint8, device="cuda")
    ws[:256].zero_()
    dA, dB, dC = gu.dev(A.ravel()), gu.dev(B.ravel()), gu.dev(C.ravel())
    rp.check(L.b200_gemm_split(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k, alpha,
                               beta, ws.data_ptr(), ws_bytes, tp, gu.stream()), "gemm_split")
    got = gu.host(dC).reshape(m, n)
    if engine != 1:
        assert L.b200_workspace_status(ws.data_ptr(), ws_bytes, gu.stream()) == rp.B200_OK, \
            "a bounded wait gave up"
    return got


def reference(A, B, C, alpha, beta):
    # float128-free check: numpy FP64 matmul is itself accurate to ~k*u|A||B|,
    # well inside the 1e-13 target at these sizes
    return alpha * (A @ B) + beta * C


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (5, 7, 3), (128, 128, 32), (130, 257, 200),
                                   (256, 256, 1024), (64, 96, 8192), (384, 520, 700)])
def test_split_matches_fp64(m, n, k, engine):
    rng = np.random.default_rng(m + n + k)
    A, B, C = rng.uniform(-1, 1, (m, k)), rng.uniform(-1, 1, (k, n)), rng.uniform(-1, 1, (m, n))
    got = run_split(A, B, C, 1.5, 1.2, engine=engine)
    want = reference(A, B, C, 1.5, 1.2)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err <= REL_FROB, err


@pytest.mark.parametrize("engine", ENGINES)
def test_split_row_scaled(engine):
    rng = np.random.default_rng(7)
    m = n = 256
    k = 512
    A = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-20, 21, m))[:, None]
    B = rng.uniform(-1, 1, (k, n))
    C = rng.uniform(-1, 1, (m, n))
    got = run_split(A, B, C, 1.5, 1.2, engine=engine)
    want = reference(A, B, C, 1.5, 1.2)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err <= REL_FROB, err
    # per row, relative to that row's own scale
    row_err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert np.max(row_err) <= 10 * REL_FROB


@pytest.mark.parametrize("engine", ENGINES)
def test_split_nonnegative_worst_case_accumulation(engine):
    """All-positive data maximises the FP32 partial sums; the result must
    still meet the bound at the largest K the entry point accepts."""
    rng = np.random.default_rng(3)
    m = n = 64
    k = 8192
    A, B = rng.uniform(0, 1, (m, k)), rng.uniform(0, 1, (k, n))
    C = np.zeros((m, n))
    got = run_split(A, B, C, 1.0, 0.0, engine=engine)
    want = A @ B
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err <= REL_FROB, err


def test_split_fewer_slices_is_less_accurate():
    rng = np.random.default_rng(11)
    A, B = rng.uniform(-1, 1, (128, 256)), rng.uniform(-1, 1, (256, 128))
    C = np.zeros((128, 128))
    want = A @ B
    e4 = np.linalg.norm(run_split(A, B, C, 1.0, 0.0, slices=4) - want) / np.linalg.norm(want)
    e11 = np.linalg.norm(run_split(A, B, C, 1.0, 0.0) - want) / np.linalg.norm(want)
    assert e11 < e4
    assert 1e-9 < e4 < 1e-3


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("m,n,k,positive", [(64, 96, 8193, False), (130, 72, 9830, False),
                                            (32, 40, 20000, False), (64, 64, 9830, True),
                                            (16, 24, 24577, True)])
def test_split_k_beyond_one_chunk(m, n, k, positive, engine):
    """K above 8192 runs in chunks of at most 8192 whose exact FP32 sums are
    folded into the FP64 accumulator (the suite's GEMM shape has nk = 1.2 N,
    9830 at N = 8192).  The reference is formed in long double."""
    rng = np.random.default_rng(k + m)
    lo = 0.0 if positive else -1.0
    A, B = rng.uniform(lo, 1, (m, k)), rng.uniform(lo, 1, (k, n))
    C = rng.uniform(-1, 1, (m, n))
    got = run_split(A, B, C, 1.5, 1.2, engine=engine)
    want = (1.5 * (A.astype(np.longdouble) @ B.astype(np.longdouble))
            + 1.2 * C.astype(np.longdouble))
    err = float(np.linalg.norm((got - want).astype(np.float64)) /
                np.linalg.norm(want.astype(np.float64)))
    assert err <= REL_FROB, err


def test_split_rejects_too_large_k():
    torch = gu.torch_cuda()
    L = rp.b200()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    assert L.b200_gemm_split(x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 1, 64 * 8192 + 1,
                             1.0, 0.0, x.data_ptr(), 128, None, None) == rp.B200_ERR_INVALID_ARG


def test_engines_bit_identical_when_accumulation_is_exact():
    """For k <= 1024 every FP32 partial sum is an integer below 2^24, and the
    e4m3 and bf16 slices hold the same digits, so every engine forms the
    same weight sums and the same FP64 results."""
    rng = np.random.default_rng(21)
    A, B = rng.uniform(-1, 1, (200, 1024)), rng.uniform(-1, 1, (1024, 300))
    C = rng.uniform(-1, 1, (200, 300))
    got = [run_split(A, B, C, 0.75, -0.5, engine=e) for e in ENGINES]
    for e, g in zip(ENGINES[1:], got[1:]):
        assert np.array_equal(got[0], g), e


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("k,positive", [(8192, True), (8192, False), (20000, True)])
def test_integer_data_is_exact(engine, k, positive):
    """Integer A and B below 2^14: every slice product sum, every chunk fold
    and the final scaling are exact, so C = A B bit for bit (the products
    stay below 2^53).  The all-positive case drives the FP32 partial sums of
    a chunk (up to 8192 values of k) toward 2^24: any loss in the tensor
    cores' accumulation (of bf16 or e4m3 products) shows here."""
    rng = np.random.default_rng(k + 3 * positive)
    lo = 0 if positive else -(2 ** 14) + 1
    m, n = 136, 200
    A = rng.integers(lo, 2 ** 14, (m, k)).astype(np.float64)
    B = rng.integers(lo, 2 ** 14, (k, n)).astype(np.float64)
    want = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    got = run_split(A, B, np.zeros((m, n)), 1.0, 0.0, engine=engine)
    assert np.array_equal(got, want), float(np.max(np.abs(got - want)))


@pytest.mark.parametrize("slices", [3, 7, 11, 12])
def test_slice_counts_agree_across_engines(slices):
    """Odd slice counts leave the last digit weight without a partner in the
    paired engine; even and odd counts must give every engine the same
    result (k <= 8192: one exact chunk, the same FP64 fold order)."""
    rng = np.random.default_rng(slices)
    A, B = rng.uniform(-1, 1, (136, 700)), rng.uniform(-1, 1, (700, 264))
    C = rng.uniform(-1, 1, (136, 264))
    got = [run_split(A, B, C, 1.25, 0.5, slices=slices, engine=e) for e in (2, 3, 4)]
    assert np.array_equal(got[0], got[1]) and np.array_equal(got[0], got[2])
    want = reference(A, B, C, 1.25, 0.5)
    err = np.linalg.norm(got[0] - want) / np.linalg.norm(want)
    assert err <= max(REL_FROB, 20 * 32.0 ** -slices), err


def test_split_rejects_unknown_engine():
    torch = gu.torch_cuda()
    L = rp.b200()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    t = rp.Tune(algo=9)
    assert L.b200_gemm_split(x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 1, 1, 1.0, 0.0,
                             x.data_ptr(), 128, ctypes.byref(t), None) == rp.B200_ERR_INVALID_ARG
