"""Compile the reference's GPU sieve (src/sieve.cu) into a cubin for sm_103a.

Baseline infrastructure, not product: the cubin holds the reference's own
basis_kernel and sieve_kernel, compiled unchanged from the reference tree into
oracle/_ref/ref_sieve.cubin (git-ignored).  ref_driver.cpp loads it through
the CUDA driver API and restates the reference's host driver
(src/sieve.cu:390-580) so the reference kernels can be timed and their
survivor sets compared on a GPU host that has no reference sources.

Runs only where the reference tree exists (default /root/reference); the
cubin it leaves is architecture-specific to the GPU, not to the host CPU.

    python oracle/ref_gpu/build_ref.py [--reference PATH]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref" / "ref_sieve.cubin"


def build(reference: Path) -> Path | None:
    source = reference / "src" / "sieve.cu"
    if not source.exists():
        return None
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= source.stat().st_mtime:
        return OUT
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run([nvcc, "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-O3",
                    "-std=c++14", f"-I{reference / 'include'}", f"-I{reference / 'src'}",
                    str(source), "-o", str(tmp)], check=True)
    os.replace(tmp, OUT)
    return OUT


def main():
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference", default="/root/reference")
    args = parser.parse_args()
    out = build(Path(args.reference))
    print(out if out else "reference tree not present; cubin not built")
    return 0


if __name__ == "__main__":
    sys.exit(main())
