"""Build the reference's host mock backend (its CPU path) from its sources.

Checker and baseline infrastructure, not product.  The reference's host
program (src/main.cpp, command_line.cpp, exact_polynomial.cpp,
output_formatter.cpp, point_search.cpp, gpu_devices.cpp) with its CPU test
double tests/mock_backend.cpp in place of src/sieve.cu, compiled unchanged
where they lie in the reference tree, as the reference's Makefile does for
`make test-host` (Makefile:35-36, 80-82).  The mock enumerates every site of
each batch and checks each one exactly with GMP, on one thread per mock
device.  GMP's development headers are absent here, so this project's
declaration shim (oracle/ref_cpu/gmp_shim: the documented C interface and a
small mpz_class/mpq_class) stands in for gmp.h/gmpxx.h, linked against the
system's libgmp.so.10.  Output: oracle/_ref/mock_ratpoints_gpu (git-ignored).
Runs only where the reference tree exists: --reference PATH, else the
RPG_REFERENCE_TREE environment variable, else the tree's mount point in the
build container (/root/reference).

    python oracle/ref_cpu/build_mock.py [--reference PATH]
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref" / "mock_ratpoints_gpu"
SOURCES = ["src/main.cpp", "src/command_line.cpp", "src/exact_polynomial.cpp",
           "src/output_formatter.cpp", "src/point_search.cpp", "src/gpu_devices.cpp",
           "tests/mock_backend.cpp"]


def build(reference: Path) -> Path | None:
    if not all((reference / s).exists() for s in SOURCES):
        return None
    inputs = [reference / s for s in SOURCES] + list((HERE / "gmp_shim").glob("*.h"))
    if OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in inputs):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_name(f"mock_ratpoints_gpu.{os.getpid()}.tmp")
    subprocess.run(["g++", "-std=c++14", "-O2", "-pthread", f"-I{HERE / 'gmp_shim'}",
                    f"-I{reference / 'tests' / 'mock_cuda'}", f"-I{reference / 'include'}",
                    *[str(reference / s) for s in SOURCES], "-o", str(tmp), "-l:libgmp.so.10"],
                   check=True)
    os.replace(tmp, OUT)
    return OUT


def main():
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference",
                        default=os.environ.get("RPG_REFERENCE_TREE", "/root/reference"))
    args = parser.parse_args()
    try:
        out = build(Path(args.reference))
    except (subprocess.CalledProcessError, OSError) as error:
        print(f"reference host mock: not built ({error})")
        return 0
    print(f"reference host mock: {out}" if out else
          f"reference host mock: not built (no reference tree at {args.reference})")
    return 0


if __name__ == "__main__":
    sys.exit(main())
