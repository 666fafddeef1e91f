"""Compile the reference's GPU sieve (src/sieve.cu) into a cubin for sm_103a.

Baseline infrastructure, not product: the cubin holds the reference's own
basis_kernel and sieve_kernel, compiled unchanged from the reference tree into
oracle/_ref/ref_sieve.cubin (git-ignored).  ref_driver.cpp loads it through
the CUDA driver API and restates the reference's host driver
(src/sieve.cu:390-580) so the reference kernels can be timed and their
survivor sets compared on a GPU host that has no reference sources.

Runs only where the reference tree exists: --reference PATH, else the
RPG_REFERENCE_TREE environment variable, else the tree's mount point in the
build container (/root/reference).  It prints what it did (built, up to
date, or not built and why); the cubin it leaves is specific to the GPU
architecture, not to the host CPU, so it travels with the checkout.

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
    parser.add_argument("--reference",
                        default=os.environ.get("RPG_REFERENCE_TREE", "/root/reference"))
    args = parser.parse_args()
    before = OUT.stat().st_mtime if OUT.exists() else None
    out = build(Path(args.reference))
    if out:
        state = "up to date" if before == out.stat().st_mtime else "built"
        print(f"reference cubin: {out} ({state} from {args.reference})")
    elif OUT.exists():
        print(f"reference cubin: {OUT} (prebuilt; no reference tree at {args.reference})")
    else:
        print(f"reference cubin: not built (no reference tree at {args.reference}); "
              "the tests that compare with the reference's kernels will skip")
    return 0


if __name__ == "__main__":
    sys.exit(main())
