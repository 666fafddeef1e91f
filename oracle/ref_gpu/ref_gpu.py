"""Python handle on the reference's own GPU sieve kernels (baseline/checker).

Builds oracle/_build/libref_gpu.so from ref_driver.cpp and the oracle's C
helpers (linked against the CUDA driver API) and drives
oracle/_ref/ref_sieve.cubin, the reference's src/sieve.cu compiled unchanged
for sm_103a by build_ref.py.  Used by tests/ and bench.py only.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
CUBIN = ORACLE / "_ref" / "ref_sieve.cubin"
LIBRARY = ORACLE / "_build" / "libref_gpu.so"


def available() -> bool:
    return CUBIN.exists()


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    return Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")


def build(force: bool = False) -> Path:
    sources = [HERE / "ref_driver.cpp", ORACLE / "oracle.c"]
    if (not force and LIBRARY.exists()
            and all(LIBRARY.stat().st_mtime >= s.stat().st_mtime for s in sources)):
        return LIBRARY
    LIBRARY.parent.mkdir(exist_ok=True)
    cuda = _cuda_home()
    obj = LIBRARY.parent / f"oracle_c.{os.getpid()}.o"
    subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-c", str(ORACLE / "oracle.c"), "-o", str(obj)],
                   check=True)
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{cuda / 'include'}",
                    str(HERE / "ref_driver.cpp"), str(obj), f"-L{cuda / 'lib64' / 'stubs'}",
                    f"-L{cuda / 'targets' / 'sbsa-linux' / 'lib' / 'stubs'}", "-lcuda", "-pthread",
                    "-o", str(tmp)], check=True)
    obj.unlink()
    os.replace(tmp, LIBRARY)
    return LIBRARY


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        lib.rgd_error.restype = ctypes.c_char_p
        lib.rgd_open.argtypes = [ctypes.c_char_p]
        c_ull, c_dbl = ctypes.c_ulonglong, ctypes.c_double
        lib.rgd_run.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.c_longlong,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(c_ull), ctypes.POINTER(c_ull),
                                ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]
        if lib.rgd_open(str(CUBIN).encode()) != 0:
            raise RuntimeError(lib.rgd_error().decode())
        _lib = lib
    return _lib


def run(coefficients, bound, first, last, batch=65536, square=False):
    """Reference kernels over the box: dict with survivors, digest and timings."""
    lib = load()
    coeffs = [str(c) for c in coefficients]
    arr = (ctypes.c_char_p * len(coeffs))(*[c.encode() for c in coeffs])
    n = ctypes.c_ulonglong(0)
    digest = ctypes.c_ulonglong(0)
    sieve_ms, basis_ms, wall_ms = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    status = lib.rgd_run(arr, len(coeffs), int(bound), int(first), int(last), int(batch), int(square),
                         ctypes.byref(n), ctypes.byref(digest), ctypes.byref(sieve_ms),
                         ctypes.byref(basis_ms), ctypes.byref(wall_ms))
    if status != 0:
        raise RuntimeError(lib.rgd_error().decode())
    return {"survivors": n.value, "digest": digest.value, "sieve_ms": sieve_ms.value,
            "basis_ms": basis_ms.value, "wall_ms": wall_ms.value}
