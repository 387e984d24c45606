"""Host-side argument checks of the C ABI's tuning fields: every call here
returns B200_ERR_INVALID_ARG before any CUDA call (the checks come first in
each entry point), so the test runs without a GPU.  The pointers are
stand-ins that are never dereferenced.  Skipped where a GPU is visible: the
GPU tests cover the same rejections with real buffers."""
import ctypes

import pytest

import rajaperf_gb300 as rp

FAKE = 16  # a non-null stand-in pointer


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible: the GPU tests cover these rejections")
    return rp.b200()


def tune(**kw):
    return ctypes.byref(rp.Tune(**kw))


def expect_invalid(status, what):
    assert status == rp.B200_ERR_INVALID_ARG, (what, status, rp.last_error())


def test_heat_3d_tuning_rejected(lib):
    for t in (dict(tile_x=3), dict(tile_x=8), dict(tile_z=8), dict(tile_x=2, tile_z=9)):
        expect_invalid(lib.b200_polybench_heat_3d(FAKE, FAKE, 3, 1, tune(**t), None), t)


def test_jacobi_2d_tuning_rejected(lib):
    for t in (dict(items=3), dict(tile_z=7), dict(tile_z=2), dict(items=4, tile_z=14)):
        expect_invalid(lib.b200_polybench_jacobi_2d(FAKE, FAKE, 3, 1, tune(**t), None), t)


def test_hydro_2d_tuning_rejected(lib):
    for t in (dict(tile_z=2), dict(tile_z=4), dict(tile_z=10), dict(block_size=100)):
        expect_invalid(lib.b200_lcals_hydro_2d(*([FAKE] * 11), 0.1, 0.1, 3, 3, tune(**t), None), t)


def test_eos_tuning_rejected(lib):
    for t in (dict(tile_z=5), dict(tile_z=3, items=3), dict(tile_z=2, items=16)):
        expect_invalid(lib.b200_lcals_eos(FAKE, FAKE, FAKE, FAKE, 0.1, 0.2, 0.1, 16, tune(**t),
                                          None), t)


def test_del_dot_vec_2d_tuning_rejected(lib):
    for t in (dict(tile_z=4), dict(tile_z=8), dict(tile_z=10)):
        expect_invalid(lib.b200_apps_del_dot_vec_2d(FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, 8, 3,
                                                    1e-20, 0.5, tune(**t), None), t)


def test_rejections_name_the_field(lib):
    lib.b200_polybench_heat_3d(FAKE, FAKE, 3, 1, tune(tile_x=3), None)
    assert "tile_x" in rp.last_error()
    lib.b200_lcals_eos(FAKE, FAKE, FAKE, FAKE, 0.1, 0.2, 0.1, 16, tune(tile_z=5), None)
    assert "tile_z" in rp.last_error()
