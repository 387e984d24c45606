"""The suite itself with Base_GB300 registered: oracle/ref_build/integration.py
applies INTEGRATION.md's blocks to copies of the suite's sources, writes its
TRIAD-GB300.cpp and DOT-GB300.cpp, and compiles and links the suite's common
layer and kernels against the patched headers and libb200.so.  The built
driver then reports that the suite's own TRIAD and DOT classes define the
Base_GB300 variant with the documented tunings.  Needs the suite's checkout
(the recipe finds it); without it the test is skipped.  Running the variant
needs a GPU as well (integration_main.cpp's --run), which this CPU test does
not use."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_build"))


def test_suite_builds_with_the_gb300_variant():
    import integration
    ref = integration.ref_root(os.environ.get("RAJAPERF_REF"))
    if not os.path.isdir(os.path.join(ref, "src", "common")):
        pytest.skip("the suite's checkout is not available here")
    if not os.path.exists(os.path.join(ROOT, "rajaperf_gb300", "lib", "libb200.so")):
        pytest.skip("libb200.so is not built")
    exe = integration.build(ref)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    line = [ln for ln in out.splitlines() if ln.startswith("{")][-1]
    got = json.loads(line)
    for k in ("Stream_TRIAD", "Stream_DOT"):
        assert got[k]["gb300_defined"] is True
        assert got[k]["gb300_tunings"] == ["default"]


def test_integration_blocks_parse():
    """Every marker of INTEGRATION.md is followed by a code block and names a
    file of the suite's source tree."""
    import integration
    blocks = integration.parse_blocks(open(os.path.join(ROOT, "INTEGRATION.md")).read())
    kinds = [b[0] for b in blocks]
    assert kinds.count("file") == 2 and kinds.count("patch") >= 10
    for kind, path, where, anchor, code in blocks:
        assert path.split("/")[0] in ("common", "stream")
        assert code.strip()
        if kind == "patch":
            assert where in ("before", "after") and anchor
