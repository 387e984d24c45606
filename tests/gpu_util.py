"""Helpers shared by the GPU tests: device buffers (torch is only the
allocator here), the golden records and the checksum tolerances."""
import json
import math
import os

import numpy as np

import rajaperf_gb300 as rp

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_checksums.json")
U = 2.0 ** -53

# Relative checksum tolerance for FP64 element-wise and stencil kernels.
REL_TOL = 1e-12


def golden(kernel):
    return [r for r in json.load(open(GOLDEN))["records"] if r["kernel"] == kernel]


def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("CUDA device required")
    return torch


def dev(arr):
    """numpy -> device tensor (same dtype)."""
    torch = torch_cuda()
    return torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")


def host(t):
    torch = torch_cuda()
    torch.cuda.synchronize()
    return t.cpu().numpy()


def stream():
    return torch_cuda().cuda.current_stream().cuda_stream


def reduction_bound(n, reps, sum_abs):
    """|seq - tree| for a sum of n terms repeated `reps` times."""
    return (n + math.ceil(math.log2(max(n, 2))) + reps) * U * sum_abs


def assert_close_rel(got, want, rel=REL_TOL, what=""):
    assert abs(got - want) <= rel * max(abs(want), 1e-300), \
        f"{what}: got {got!r} want {want!r} rel {abs(got - want) / max(abs(want), 1e-300):.3e}"


def ulp_diff(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ai = a.view(np.int64)
    bi = b.view(np.int64)
    ai = np.where(ai < 0, np.int64(-(2 ** 63)) - ai, ai)
    bi = np.where(bi < 0, np.int64(-(2 ** 63)) - bi, bi)
    return np.abs(ai - bi)
