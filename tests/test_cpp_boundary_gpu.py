"""The C++ drop-in boundary at link level: a C++ caller of the reference's
run_modular_sieve (include/sieve.hpp:43-47) is compiled with g++ against
include/ratpoints_gpu/sieve.hpp, linked with librpgpu, and run.  The program
(tests/cpp/run_modular_sieve_check.cpp) restates the reference's own boundary
test (tests/test_sieve_streaming.cpp:45-81): every site of the dense curve's
box arrives exactly once, including a stream that outgrows the first
survivor buffer and a square-denominator range."""

import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def test_cpp_caller_links_and_streams_every_site(rpg, tmp_path):
    lib_dir = Path(rpg.LIBRARY).parent
    exe = tmp_path / "run_modular_sieve_check"
    build = subprocess.run(
        ["g++", "-O2", "-std=c++17", f"-I{ROOT / 'include'}",
         str(ROOT / "tests" / "cpp" / "run_modular_sieve_check.cpp"), "-o", str(exe),
         f"-L{lib_dir}", "-lrpgpu", f"-Wl,-rpath,{lib_dir}", "-pthread"],
        capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    assert "all cases hold" in run.stdout
