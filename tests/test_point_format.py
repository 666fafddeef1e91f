"""The command line's point output (csrc/point_format.cpp) byte for byte
against the oracle's restatement of the reference's formatter
(src/output_formatter.cpp:7-105), on the CPU: escapes, field markers, -y
with an explicit %y, -z with -fs/-fe, escaped percent signs in the
before/between/after texts, trailing backslashes and percent signs."""

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
POINTS = [(1, "0", 0), (-3, "12", 7), (5, "0", 2), (-1234567, "98765432109876543210", 3)]

CASES = [
    # (points, ordinates, conjugates, format, before, between, after)
    (True, True, True, "", "", "", ""),
    (True, False, True, "", "", "", ""),
    (True, True, False, "", "", "", ""),
    (False, True, True, "", "S", "M", "E\\n"),
    (True, True, True, "%x,%y,%z", "[", ";", "]"),
    (True, False, True, "%x %y %q %%\\%\\t|", "", "", ""),
    (True, True, True, "%\\%x%", "\\%a\\q\\", "%x\\n", "\\%\\t"),
    (True, True, True, "\x01%x\x01\\\\%y\\", "", "\\n--\\n", ""),
    (True, True, True, "%z%z%y%x%\x01%\\n", "\\", "\\\\", "%"),
    (True, True, True, "no fields at all", "", "", ""),
    (True, True, True, "%", "", "", ""),
    (True, True, True, "\\", "", "", ""),
    (True, False, True, "%y%y", "a", "b", "c"),
]


@pytest.fixture(scope="module")
def printer(tmp_path_factory):
    exe = tmp_path_factory.mktemp("fmt") / "point_format_check"
    build = subprocess.run(
        ["g++", "-O1", "-std=c++17", f"-I{ROOT / 'ratpoints-gpu_gb300' / 'csrc'}",
         str(ROOT / "tests" / "cpp" / "point_format_check.cpp"),
         str(ROOT / "ratpoints-gpu_gb300" / "csrc" / "point_format.cpp"), "-o", str(exe)],
        capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    return exe


@pytest.mark.parametrize("case", CASES, ids=[repr(c[3:])[:40] for c in CASES])
def test_printer_matches_oracle(printer, oracle, case):
    points, ordinates, conjugates, fmt, before, between, after = case
    stdin = "".join(f"{x} {y} {z}\n" for x, y, z in POINTS)
    got = subprocess.run([str(printer), "1" if points else "0", "1" if ordinates else "0",
                          "1" if conjugates else "0", fmt, before, between, after],
                         input=stdin.encode(), capture_output=True)
    assert got.returncode == 0
    o = oracle.Options(print_points=points, print_y=ordinates, format=fmt, before=before,
                       between=between, after=after)
    f = oracle.Formatter(o)
    for x, y, z in POINTS:
        f.point_pair(x, y, z, conjugates)
    f.finish()
    assert got.stdout == f.text().encode()
