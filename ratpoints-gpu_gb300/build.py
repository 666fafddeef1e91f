"""Build librpgpu.so and the ratpoints_gpu executable in-tree for sm_103a.

Compiles the CUDA sources with nvcc (one -gencode, compute_103a/sm_103a) and
the host C++ sources with g++, in parallel, then links
    ratpoints-gpu_gb300/lib/librpgpu.so
    ratpoints-gpu_gb300/bin/ratpoints_gpu
Objects go to ratpoints-gpu_gb300/_build/.  Runs unchanged on x86_64 and
aarch64 hosts (no architecture-specific host flags).

    python ratpoints-gpu_gb300/build.py [--force] [--jobs N]
"""

from __future__ import annotations

import argparse
import concurrent.futures as futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIB_DIR = PACKAGE / "lib"
BIN_DIR = PACKAGE / "bin"
LIBRARY = LIB_DIR / "librpgpu.so"
EXECUTABLE = BIN_DIR / "ratpoints_gpu"

CUDA_SOURCES = ["sieve.cu", "noalloc.cu", "batch.cu", "preverify.cu", "selftest.cu", "probe.cu"]
CXX_SOURCES = ["bigint.cpp", "exact.cpp", "plan.cpp", "search.cpp", "cli.cpp", "point_format.cpp", "capi.cpp",
               "serve.cpp", "compat_sieve.cpp", "tune.cpp"]
MAIN_SOURCE = "ratpoints_gpu_main.cpp"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _includes():
    return [f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{cuda_home() / 'include'}"]


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").rglob("*.h*"))


def _run(cmd):
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"command failed ({result.returncode}): {' '.join(map(str, cmd))}\n"
                           f"{result.stdout}\n{result.stderr}")
    return result


def compile_commands():
    nvcc = str(cuda_home() / "bin" / "nvcc")
    jobs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        cmd = [nvcc, GENCODE, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-Xptxas", "-v", *_includes(), "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append((obj, [CSRC / src], cmd))
    for src in CXX_SOURCES + [MAIN_SOURCE]:
        obj = BUILD / (src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wextra",
               *_includes(), "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append((obj, [CSRC / src], cmd))
    return jobs


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    BIN_DIR.mkdir(exist_ok=True)
    headers = _headers()
    work = [(obj, cmd) for obj, deps, cmd in compile_commands()
            if force or _stale(obj, list(deps) + headers)]
    if work:
        with futures.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as pool:
            results = list(pool.map(lambda job: _run(job[1]), work))
        if verbose:
            for r in results:
                if r.stderr:
                    sys.stderr.write(r.stderr)
    objects = [BUILD / (s + ".o") for s in CUDA_SOURCES + CXX_SOURCES]
    nvcc = str(cuda_home() / "bin" / "nvcc")
    if force or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_name(f"librpgpu.{os.getpid()}.tmp.so")
        _run([nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objects),
              "-Xcompiler", "-pthread"])
        os.replace(tmp, LIBRARY)
    main_obj = BUILD / (MAIN_SOURCE + ".o")
    if force or _stale(EXECUTABLE, [main_obj, LIBRARY]):
        tmp = EXECUTABLE.with_name(f"ratpoints_gpu.{os.getpid()}.tmp")
        _run(["g++", "-o", str(tmp), str(main_obj), f"-L{LIB_DIR}", "-lrpgpu",
              "-Wl,-rpath,$ORIGIN/../lib", "-pthread"])
        os.replace(tmp, EXECUTABLE)
    return LIBRARY


def main():
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--jobs", type=int)
    parser.add_argument("--verbose", action="store_true")
    args = parser.parse_args()
    path = build(force=args.force, jobs=args.jobs, verbose=args.verbose)
    print(path)


if __name__ == "__main__":
    main()
