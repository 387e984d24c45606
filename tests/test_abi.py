"""The C-ABI libraries load and export every function their headers declare
(no GPU needed: nothing is called)."""
import ctypes

import pytest

import rajaperf_gb300 as rp


def test_libb200_exports_header():
    names = rp.declared_functions("b200.h")
    assert "b200_stream_triad" in names
    lib = rp.b200()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_exports_header():
    names = rp.declared_functions("rajaperf_gb300.h")
    assert {"rp_run", "rp_last_error", "rp_graph_batch"} <= set(names)
    lib = rp.host()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    names = rp.declared_functions("b200.h")
    sigs = rp.parse_signatures("b200.h")
    assert set(names) == set(sigs), set(names) ^ set(sigs)
    args, res = sigs["b200_stream_triad"]
    assert len(args) == 7 and res is ctypes.c_int
    args, res = sigs["b200_apps_energy"]
    assert len(args) == 22
    assert sigs["b200_last_error_string"] == ([], ctypes.c_char_p)
    assert sigs["b200_reduce_workspace_bytes"][1] is ctypes.c_size_t


def test_tune_struct_layout():
    assert ctypes.sizeof(rp.Tune) == 12 * 4
    assert ctypes.sizeof(rp.RpResult) == 64 + 32 + 64 + 5 * 8 + 6 * 8 + 8 + 2 * 8


def test_struct_sizes_match_the_headers(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets."""
    import subprocess
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "b200.h"\n#include "rajaperf_gb300.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(b200_tune), sizeof(rp_result), '
        'offsetof(rp_result, h2d_bytes_per_rep), offsetof(b200_tune, wait_limit_us), '
        'sizeof(rp_batch_result)); return 0; }\n')
    exe = tmp_path / "sizes"
    subprocess.run(["cc", "-I", rp.INCLUDE, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [ctypes.sizeof(rp.Tune), ctypes.sizeof(rp.RpResult),
                   rp.RpResult.h2d_bytes_per_rep.offset, rp.Tune.wait_limit_us.offset,
                   ctypes.sizeof(rp.RpBatchResult)]
