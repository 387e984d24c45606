"""Layouts of the suite's report files, written by the host layer's report
writers (rajaperf_gb300/csrc/host/common/Reports.cpp) for a fixed table of
results: the timing and speedup CSVs (the suite's Executor::writeCSVReport,
common/Executor.cpp:901-997), the checksum report with its difference column
(writeChecksumReport, :1281-1512), the FOM report (writeFOMReport,
:1000-1278, groups as getFOMGroups, :1618-1647) and the kernel details
(writeKernelInfoSummary, :508-642).  The writers need no GPU; this test
compiles them with a small driver (tests/report_layout_main.cpp)."""
import math
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMMON = os.path.join(ROOT, "rajaperf_gb300", "csrc", "host", "common")

VARIANTS = ["Base_GB300", "RAJA_GB300"]
TUNINGS = [["default", "graph", "int64"], ["default"]]
# kernel -> per column (variant, tuning): None (not defined) or
# (run, tot, min, max, checksum); npasses = 2
TABLE = {
    "Stream_TRIAD": [(True, 0.5, 0.24, 0.26, 135.91984956172908),
                     (True, 0.25, 0.12, 0.13, 135.91984956172908), None,
                     (True, 0.6, 0.29, 0.31, 135.919849561729)],
    "Algorithm_SCAN": [(True, 2.0, 0.9, 1.1, 4.5), (False, 0, 0, 0, 0),
                       (True, 1.0, 0.5, 0.5, 4.25), None],
}
KERNELS = ["Stream_TRIAD", "Algorithm_SCAN"]
COLS = [(v, t) for v, ts in zip(VARIANTS, TUNINGS) for t in ts]


@pytest.fixture(scope="module")
def reports(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("rep") / "report_layout")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", COMMON,
                    os.path.join(ROOT, "tests", "report_layout_main.cpp"),
                    os.path.join(COMMON, "Reports.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    sections, name = {}, None
    for line in out.splitlines():
        if line.startswith("@@ "):
            name = line[3:]
            sections[name] = []
        else:
            sections[name].append(line)
    return sections


def _csv_expected(title, prec, value):
    kw = max(len("Kernel  "), *map(len, KERNELS)) + 1
    widths = [max(prec + 2, len(v), len(t)) for v, t in COLS]
    lines = [title + " , " * len(COLS),
             "Kernel  ".ljust(kw) + "".join(" , " + v.ljust(w) for (v, _), w in zip(COLS, widths)),
             "Kernel  ".ljust(kw) + "".join(" , " + t.ljust(w) for (_, t), w in zip(COLS, widths))]
    for k in KERNELS:
        row = k.ljust(kw)
        for c, w in zip(range(len(COLS)), widths):
            x = value(k, c)
            row += " , " + ("Not run" if x is None else f"{x:.{prec}f}").rjust(w)
        lines.append(row)
    return lines


def test_timing_reports(reports):
    avg = _csv_expected("Mean Runtime Report (sec.) ", 6,
                        lambda k, c: None if TABLE[k][c] is None else TABLE[k][c][1] / 2)
    assert reports["timing-Average"] == avg
    mn = _csv_expected("Min Runtime Report (sec.) ", 6,
                       lambda k, c: None if TABLE[k][c] is None else TABLE[k][c][2])
    assert reports["timing-Minimum"] == mn


def test_speedup_report(reports):
    def speedup(k, c):
        ref, cell = TABLE[k][0], TABLE[k][c]
        if ref is None or cell is None:
            return None
        tv = cell[1] / 2
        return (ref[1] / 2) / tv if tv > 0 else 0.0
    want = _csv_expected("Mean Speedup Report (T_ref/T_var): ref var = Base_GB300 ", 3, speedup)
    assert reports["speedup-Average"] == want


def test_checksum_report_difference_column(reports):
    lines = reports["checksum"]
    assert lines[0] == "=" * 99 and lines[1] == "Checksum Report " and lines[2] == "=" * 99
    assert lines[4] == "." * 56
    assert lines[5].split() == ["Variants", "Checksum", "Checksum", "Diff"]
    assert "(vs. first variant listed)" in lines[6]
    assert lines[7] == "-" * 88
    nw = max(max(map(len, KERNELS)), max(len(v) + 1 + len(t) for v, t in COLS)) + 1
    for k in KERNELS:
        i = lines.index(k.ljust(nw))
        assert lines[i + 1] == "." * 56
        first = next(cell[4] for cell in TABLE[k] if cell is not None and cell[0])
        j = i + 2
        for (v, t), cell in zip(COLS, TABLE[k]):
            if cell is None:
                continue  # the kernel lacks this tuning: not listed
            line = lines[j]
            j += 1
            assert line.startswith(f"{v}-{t}".ljust(nw)), line
            fields = line[nw:].split()
            if not cell[0]:
                assert fields == ["Not", "Run", "Not", "Run"]
                continue
            assert len(line[nw:nw + 28].rstrip()) <= 28
            ck, diff = float(fields[0]), float(fields[1])
            assert math.isclose(ck, cell[4], rel_tol=1e-15)
            # the difference is formed in long double from the long double
            # checksums: equal to the double difference within a few ulps
            # of the checksum
            assert abs(diff - (first - cell[4])) <= 4 * 2.0 ** -52 * abs(first)
            if cell[4] == first:
                assert diff == 0.0
        assert lines[j] == "" and lines[j + 1] == "-" * 55


def test_fom_report(reports):
    lines = reports["fom"]
    ncols = len(COLS)
    assert lines[0].startswith("FOM Report : signed speedup(-)/slowdown(+) for each PM")
    assert lines[0].endswith(" , " * (2 * ncols))
    assert lines[1].startswith("'OVER_TOL' in column to right")
    fw = max(16, *(len(v) + 1 + len(t) for v, t in COLS))
    kw = max(len("Kernel  "), *map(len, KERNELS)) + 1
    assert lines[2] == "Kernel  ".ljust(kw) + "".join(
        " , " + f"{v}-{t}".ljust(fw) + ",        " for v, t in COLS)
    rows = {ln[:kw].strip(): ln[kw:] for ln in lines[3:5]}
    for k in KERNELS:
        # fixed-width blocks: " , " + value (fw, left) + a 9-character tag
        blk = 3 + fw + 9
        assert len(rows[k]) == ncols * blk, rows[k]
        cells = [rows[k][i * blk + 3:(i + 1) * blk] for i in range(ncols)]
        assert all(rows[k][i * blk:i * blk + 3] == " , " for i in range(ncols))
        base = None
        for c, cell in enumerate(TABLE[k]):
            val, tag = cells[c][:fw].strip(), cells[c][fw:]
            if cell is None or not cell[0]:
                assert (val, tag) == ("0", ",        ")
                continue
            if base is None:
                base = cell[1]
                assert tag == ",base_ref" and float(val) == 0.0
                continue
            p = (cell[1] - base) / base
            assert float(val) == pytest.approx(p, abs=0.005)
            assert tag == (",OVER_TOL" if p > 0.1 else ",        ")
    summary = [ln[:kw].strip() for ln in lines[5:]]
    assert summary == ["", "Col Min", "Col Max", "Col Avg", "Col Std Dev"]


def test_kernel_info(reports):
    lines = reports["kernels"]
    assert lines[0] == "Kernels run without MPI"
    heads = ["Problem size", "Reps", "Iterations/rep", "Kernels/rep", "Bytes/rep", "FLOPS/rep",
             "BytesRead/rep", "BytesWritten/rep", "BytesAtomicModifyWritten/rep"]
    assert [h.strip() for h in lines[1].split(" , ")] == ["Kernels"] + heads
    assert lines[2].split(" , ")[0].strip() == "Stream_TRIAD"
    assert [int(x) for x in lines[2].split(" , ")[1:]] == [1000000, 1000, 1000000, 1, 24000000,
                                                          2000000, 16000000, 8000000, 0]
    assert [int(x) for x in lines[3].split(" , ")[1:]] == [67108864, 100, 67108864, 1,
                                                          1073741824, 67108864, 536870912,
                                                          536870912, 0]
    # columns as wide as their heading or the value's digits, plus 3
    col = lines[1].split(" , ")
    assert len(col[1]) == max(len("Problem size"), int(math.log10(67108864))) + 3
    assert len(col[5]) == max(len("Bytes/rep"), int(math.log10(1073741824))) + 3
    assert len(col[0]) == len("Algorithm_SCAN") + 2
