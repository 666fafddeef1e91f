"""ctypes binding of librpgpu (include/ratpoints_gb300.h) for the Python test
and benchmark harness.  The product is the C++/CUDA library and the
ratpoints_gpu executable; this module only loads them.

Loading fails loudly (RuntimeError) when the library has not been built: there
is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
LIBRARY = PACKAGE / "lib" / "librpgpu.so"
ABI_VERSION = 3  # RPG_ABI_VERSION of include/ratpoints_gb300.h that these structures follow
EXECUTABLE = PACKAGE / "bin" / "ratpoints_gpu"
HEADER = ROOT / "include" / "ratpoints_gb300.h"

RPG_SIEVE_SQUARE_DENOMINATORS = 1
RPG_SIEVE_FAST_PLAN = 2
RPG_PLAN_REFERENCE = 0
RPG_PLAN_FAST = 1
RPG_SEARCH_HOST_VERIFY_ONLY = 1
STATUS_NAMES = {0: "RPG_OK", 1: "RPG_E_ARG", 2: "RPG_E_CUDA", 3: "RPG_E_OOM",
                4: "RPG_E_TIMEOUT", 5: "RPG_E_INTERNAL", 6: "RPG_E_NOT_SQUAREFREE"}


class RpgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


def build(force: bool = False):
    sys.path.insert(0, str(PACKAGE))
    try:
        import build as _build  # noqa: WPS433 - build step beside the sources
    finally:
        sys.path.pop(0)
    return _build.build(force=force)


class SieveStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in
                ("survivor_count", "word_count", "denominator_count", "launches")] + \
               [(name, ctypes.c_double) for name in
                ("basis_ms", "sieve_ms", "plan_ms", "workspace_ms", "basis_wall_ms",
                 "survivor_setup_ms", "verification_ms", "sieve_wall_ms", "initial_mask_bytes")] + \
               [(name, ctypes.c_uint64) for name in ("h2d_bytes", "d2h_bytes", "host_candidates")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Interval(ctypes.Structure):
    _fields_ = [("lower", ctypes.c_char_p), ("upper", ctypes.c_char_p)]


class SearchOptions(ctypes.Structure):
    _fields_ = [("coefficients", ctypes.POINTER(ctypes.c_char_p)),
                ("coefficient_count", ctypes.c_int32),
                ("numerator_bound", ctypes.c_int64),
                ("first", ctypes.c_int32), ("last", ctypes.c_int32),
                ("intervals", ctypes.POINTER(Interval)), ("interval_count", ctypes.c_int32),
                ("include_infinity", ctypes.c_int32), ("batch_size", ctypes.c_int32),
                ("square_denominators", ctypes.c_int32), ("plan", ctypes.c_int32),
                ("device", ctypes.c_int32), ("verify_threads", ctypes.c_int32),
                ("flags", ctypes.c_uint32)]


class FastPlanInfo(ctypes.Structure):
    _fields_ = [("class_prime", ctypes.c_int32), ("modulus_count", ctypes.c_int32),
                ("moduli", ctypes.c_int32 * 16), ("factors", (ctypes.c_int32 * 4) * 16),
                ("bits", ctypes.c_double), ("slots", ctypes.c_int32)]


class TuneReport(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("slots", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("candidate_rows", ctypes.c_int32 * 8), ("candidate_slots", ctypes.c_int32 * 8),
                ("candidate_ms", ctypes.c_double * 8), ("candidate_bits", ctypes.c_double * 8),
                ("sample_denominators", ctypes.c_int64), ("stored", ctypes.c_int32),
                ("key", ctypes.c_char * 96)]


class BatchStats(ctypes.Structure):
    _fields_ = ([(name, ctypes.c_uint64) for name in
                 ("curves", "wide_curves", "denominators", "survivors", "points", "launches",
                  "words", "table_words", "swept_words", "smem_bytes")] +
                [(name, ctypes.c_double) for name in
                 ("rectangle_sites", "plan_ms", "table_ms", "sieve_ms", "wide_ms", "narrow_ms",
                  "verify_ms", "wall_ms")] +
                [("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                 ("graph", ctypes.c_int32), ("host_candidates", ctypes.c_uint64),
                 ("items_per_kernel", ctypes.c_int32), ("items_from_cache", ctypes.c_int32)])

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchTuneReport(ctypes.Structure):
    _fields_ = [("items", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("candidate_items", ctypes.c_int32 * 8), ("candidate_ms", ctypes.c_double * 8),
                ("stored", ctypes.c_int32), ("key", ctypes.c_char * 96)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("memory_budget_bytes", ctypes.c_uint64), ("max_batch_curves", ctypes.c_int32)]


class RequestStats(ctypes.Structure):
    _fields_ = [("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double),
                ("rectangle_sites", ctypes.c_double), ("survivors", ctypes.c_uint64),
                ("points", ctypes.c_uint64), ("waves", ctypes.c_int32)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


CANDIDATE_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_int32), ctypes.c_size_t, ctypes.c_void_p)
POINT_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64,
                            ctypes.c_void_p)
BATCH_POINT_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_char_p,
                                  ctypes.c_int64, ctypes.c_void_p)
RPG_BATCH_NO_GRAPH = 1
RPG_BATCH_HOST_VERIFY_ONLY = 2

_lib = None


def load():
    """Load librpgpu.so; raises RuntimeError if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIBRARY.exists():
        raise RuntimeError(f"{LIBRARY} is not built; run python ratpoints-gpu_gb300/build.py")
    lib = ctypes.CDLL(str(LIBRARY))
    S = ctypes.c_int
    pp = ctypes.POINTER(ctypes.c_char_p)
    lib.rpg_sieve_run.restype = S
    lib.rpg_sieve_run.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_uint32, ctypes.c_int32, CANDIDATE_CB,
                                  ctypes.c_void_p, ctypes.POINTER(SieveStats)]
    lib.rpg_point_search.restype = S
    lib.rpg_point_search.argtypes = [ctypes.POINTER(SearchOptions), POINT_CB, ctypes.c_void_p,
                                     ctypes.POINTER(SieveStats)]
    lib.rpg_batch_search.restype = S
    lib.rpg_batch_search.argtypes = [ctypes.POINTER(SearchOptions), ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_uint32, BATCH_POINT_CB, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(BatchStats)]
    lib.rpg_server_create.restype = S
    lib.rpg_server_create.argtypes = [ctypes.POINTER(ServerOptions), ctypes.POINTER(ctypes.c_void_p)]
    lib.rpg_server_submit.restype = S
    lib.rpg_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(SearchOptions), ctypes.c_int32,
                                      ctypes.POINTER(ctypes.c_uint64)]
    lib.rpg_server_wait.restype = S
    lib.rpg_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, POINT_CB,
                                    ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                    ctypes.POINTER(RequestStats)]
    lib.rpg_server_destroy.restype = None
    lib.rpg_server_destroy.argtypes = [ctypes.c_void_p]
    lib.rpg_is_squarefree.restype = S
    lib.rpg_is_squarefree.argtypes = [pp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_square_root.restype = S
    lib.rpg_square_root.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_char_p, ctypes.c_size_t,
                                    ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_fast_plan.restype = S
    lib.rpg_fast_plan.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(FastPlanInfo)]
    lib.rpg_tune_fast_plan.restype = S
    lib.rpg_tune_fast_plan.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_uint32, ctypes.c_int32, ctypes.c_int64,
                                       ctypes.POINTER(TuneReport)]
    lib.rpg_tune_batch.restype = S
    lib.rpg_tune_batch.argtypes = [ctypes.POINTER(SearchOptions), ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(BatchTuneReport)]
    lib.rpg_batch_items.restype = S
    lib.rpg_batch_items.argtypes = [ctypes.POINTER(SearchOptions), ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_fast_shape.restype = S
    lib.rpg_fast_shape.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_preverify.restype = S
    lib.rpg_preverify.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                  ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_release_cached_resources.restype = S
    lib.rpg_release_cached_resources.argtypes = [ctypes.c_int32]
    lib.rpg_bounded_wait_selftest.restype = S
    lib.rpg_bounded_wait_selftest.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    lib.rpg_smem_read_probe.restype = S
    lib.rpg_smem_read_probe.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.rpg_cli_main.restype = ctypes.c_int32
    lib.rpg_cli_main.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p)]
    lib.rpg_session_create.restype = S
    lib.rpg_session_create.argtypes = [pp, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32,
                                       ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    lib.rpg_session_count.restype = S
    lib.rpg_session_count.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_double)]
    lib.rpg_session_work.restype = S
    lib.rpg_session_work.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(ctypes.c_uint32)]
    lib.rpg_session_plan.restype = S
    lib.rpg_session_plan.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                     ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_int32)]
    lib.rpg_session_destroy.restype = None
    lib.rpg_session_destroy.argtypes = [ctypes.c_void_p]
    lib.rpg_device_count.restype = ctypes.c_int32
    lib.rpg_abi_version.restype = ctypes.c_int32
    lib.rpg_last_error.restype = ctypes.c_char_p
    if lib.rpg_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{LIBRARY} has ABI version {lib.rpg_abi_version()}, this binding expects "
                           f"{ABI_VERSION}: rebuild it (python ratpoints-gpu_gb300/build.py)")
    _lib = lib
    return lib


def _check(status):
    if status != 0:
        raise RpgError(status, load().rpg_last_error().decode())


def _strings(values):
    arr = (ctypes.c_char_p * len(values))()
    for i, v in enumerate(values):
        arr[i] = str(v).encode()
    return arr


def coefficients_of(text_or_list):
    if isinstance(text_or_list, str):
        return text_or_list.split()
    return [str(c) for c in text_or_list]


def declared_functions():
    """Names of the functions include/ratpoints_gb300.h declares."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w ]*\*?\s*)\b(rpg_\w+)\s*\(", text, re.M)))


def sieve(coefficients, bound, first, last, square=False, plan="reference", device=-1):
    """Modular survivors as (a, d) int64/int32 arrays plus the stats dict."""
    lib = load()
    coeffs = coefficients_of(coefficients)
    chunks_a, chunks_d = [], []

    @CANDIDATE_CB
    def on_batch(a, d, n, _user):
        chunks_a.append(np.ctypeslib.as_array(a, shape=(n,)).copy())
        chunks_d.append(np.ctypeslib.as_array(d, shape=(n,)).copy())
        return 0

    flags = (RPG_SIEVE_SQUARE_DENOMINATORS if square else 0) | \
            (RPG_SIEVE_FAST_PLAN if plan == "fast" else 0)
    stats = SieveStats()
    _check(lib.rpg_sieve_run(_strings(coeffs), len(coeffs), int(bound), int(first), int(last),
                             flags, device, on_batch, None, ctypes.byref(stats)))
    a = np.concatenate(chunks_a) if chunks_a else np.zeros(0, np.int64)
    d = np.concatenate(chunks_d) if chunks_d else np.zeros(0, np.int32)
    return a, d, stats.as_dict()


def point_search(coefficients, bound, first, last, intervals=(), include_infinity=True,
                 batch_size=1 << 16, square=False, plan="fast", device=-1, verify_threads=0,
                 stop_after=None, preverify=True):
    """Verified points [(a, y, d)] in output order, plus the stats dict.
    preverify=False sends every modular survivor to the host's exact check."""
    lib = load()
    coeffs = coefficients_of(coefficients)
    points = []

    @POINT_CB
    def on_point(a, y, d, _user):
        points.append((a, int(y.decode()), d))
        return 0 if stop_after is not None and len(points) >= stop_after else 1

    opts = SearchOptions()
    keep = _fill_options(opts, coeffs, bound, first, last, intervals, include_infinity,
                         batch_size, square, plan, device, verify_threads)
    opts.flags = 0 if preverify else RPG_SEARCH_HOST_VERIFY_ONLY
    stats = SieveStats()
    _check(lib.rpg_point_search(ctypes.byref(opts), on_point, None, ctypes.byref(stats)))
    del keep
    return points, stats.as_dict()


def _fill_options(opts, coeffs, bound, first, last, intervals=(), include_infinity=True,
                  batch_size=1 << 16, square=False, plan="fast", device=-1, verify_threads=0):
    """Fill a SearchOptions; returns the ctypes buffers it points into (keep them alive)."""
    ivs = (Interval * max(1, len(intervals)))()
    for i, (lo, hi) in enumerate(intervals):
        ivs[i].lower = None if lo is None else str(lo).encode()
        ivs[i].upper = None if hi is None else str(hi).encode()
    cstr = _strings(coeffs)
    opts.coefficients = cstr
    opts.coefficient_count = len(coeffs)
    opts.numerator_bound = int(bound)
    opts.first, opts.last = int(first), int(last)
    opts.intervals = ivs
    opts.interval_count = len(intervals)
    opts.include_infinity = int(include_infinity)
    opts.batch_size = int(batch_size)
    opts.square_denominators = int(square)
    opts.plan = RPG_PLAN_FAST if plan == "fast" else RPG_PLAN_REFERENCE
    opts.device = device
    opts.verify_threads = verify_threads
    return (ivs, cstr)


def _batch_options(curves):
    """The curves as an rpg_search_options array (and the buffers it points to)."""
    arr = (SearchOptions * max(1, len(curves)))()
    keep = []
    for i, c in enumerate(curves):
        keep.append(_fill_options(arr[i], coefficients_of(c["coefficients"]), c["bound"],
                                  c["first"], c["last"], c.get("intervals", ()),
                                  c.get("include_infinity", True), square=c.get("square", False)))
    return arr, keep


def tune_batch(curves, device=-1):
    """Times the batch with 2,048, 8,192 and 32,768 work items per kernel
    (rpg_tune_batch) and returns {"items", "key", "stored", "candidates":
    [{"items", "ms"}, ...]}; the choice is kept in the RPG_TUNE_CACHE file when
    that environment variable is set."""
    arr, keep = _batch_options(curves)
    r = BatchTuneReport()
    _check(load().rpg_tune_batch(arr, len(curves), int(device), ctypes.byref(r)))
    del keep
    return {"items": r.items, "key": r.key.decode(), "stored": bool(r.stored),
            "candidates": [{"items": r.candidate_items[i], "ms": r.candidate_ms[i]}
                           for i in range(r.candidates)]}


def batch_items(curves):
    """(items per kernel, from_cache) a batch_search of these curves uses
    (host only)."""
    arr, keep = _batch_options(curves)
    items, cached = ctypes.c_int32(0), ctypes.c_int32(0)
    _check(load().rpg_batch_items(arr, len(curves), ctypes.byref(items), ctypes.byref(cached)))
    del keep
    return items.value, bool(cached.value)


def batch_search(curves, device=-1, graph=True, stop_after=None, preverify=True):
    """Search many curves in one batched pass.

    curves: list of dicts with keys coefficients, bound, first, last and
    optionally intervals, include_infinity, square.  Returns (points, status,
    survivors, stats): points[i] is curve i's [(a, y, d)] in the order
    point_search reports them (truncated to stop_after points when given).
    """
    lib = load()
    n = len(curves)
    arr, keep = _batch_options(curves)
    points = [[] for _ in range(n)]

    @BATCH_POINT_CB
    def on_point(i, a, y, d, _user):
        points[i].append((a, int(y.decode()), d))
        return 0 if stop_after is not None and len(points[i]) >= stop_after else 1

    status = (ctypes.c_int32 * max(1, n))()
    survivors = (ctypes.c_uint64 * max(1, n))()
    stats = BatchStats()
    flags = (0 if graph else RPG_BATCH_NO_GRAPH) | (0 if preverify else RPG_BATCH_HOST_VERIFY_ONLY)
    _check(lib.rpg_batch_search(arr, n, device, flags, on_point, None,
                                status, survivors, ctypes.byref(stats)))
    del keep
    return points, list(status)[:n], list(survivors)[:n], stats.as_dict()


class Server:
    """Serving loop (rpg_server_*): submit searches at any time, wait for answers.

    A request is a dict like batch_search's curves; wait() returns None on
    timeout, else (status, points, stats) with status the request's rpg_status
    (0, or e.g. 6 for a polynomial that is not squarefree).
    """

    def __init__(self, device=-1, lanes=2, memory_budget=8 << 30, max_batch_curves=1024):
        self._lib = load()
        opts = ServerOptions(device, lanes, memory_budget, max_batch_curves)
        handle = ctypes.c_void_p()
        _check(self._lib.rpg_server_create(ctypes.byref(opts), ctypes.byref(handle)))
        self._handle = handle

    def submit(self, curve, first_point_only=False):
        opts = SearchOptions()
        keep = _fill_options(opts, coefficients_of(curve["coefficients"]), curve["bound"],
                             curve["first"], curve["last"], curve.get("intervals", ()),
                             curve.get("include_infinity", True), square=curve.get("square", False))
        rid = ctypes.c_uint64()
        _check(self._lib.rpg_server_submit(self._handle, ctypes.byref(opts), int(first_point_only),
                                           ctypes.byref(rid)))
        del keep
        return rid.value

    def wait(self, request_id, timeout_ms=-1.0):
        points = []

        @POINT_CB
        def on_point(a, y, d, _user):
            points.append((a, int(y.decode()), d))
            return 1

        done = ctypes.c_int32(0)
        stats = RequestStats()
        status = self._lib.rpg_server_wait(self._handle, request_id, float(timeout_ms), on_point,
                                           None, ctypes.byref(done), ctypes.byref(stats))
        if not done.value:
            _check(status)
            return None
        return status, points, stats.as_dict()

    def close(self):
        if self._handle:
            self._lib.rpg_server_destroy(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def is_squarefree(coefficients):
    coeffs = coefficients_of(coefficients)
    out = ctypes.c_int32(-1)
    _check(load().rpg_is_squarefree(_strings(coeffs), len(coeffs), ctypes.byref(out)))
    return bool(out.value)


def fast_plan(coefficients, bound):
    """The single-curve fast plan for a curve and numerator bound (host only):
    {"class_prime", "moduli", "factors", "bits"}."""
    coeffs = coefficients_of(coefficients)
    info = FastPlanInfo()
    _check(load().rpg_fast_plan(_strings(coeffs), len(coeffs), int(bound), ctypes.byref(info)))
    n = info.modulus_count
    return {"class_prime": info.class_prime, "moduli": list(info.moduli[:n]),
            "factors": [[f for f in info.factors[i] if f] for i in range(n)], "bits": info.bits,
            "slots": info.slots}


def tune_fast_plan(coefficients, bound, first, last, square=False, device=-1, sample=1 << 17):
    """Times the fast plan's candidate shapes (rpg_tune_fast_plan) and returns
    {"rows", "slots", "key", "stored", "sample", "candidates": [{"rows",
    "slots", "ms", "bits"}, ...]}; the choice is kept in the RPG_TUNE_CACHE file
    when that environment variable is set."""
    coeffs = coefficients_of(coefficients)
    r = TuneReport()
    flags = RPG_SIEVE_SQUARE_DENOMINATORS if square else 0
    _check(load().rpg_tune_fast_plan(_strings(coeffs), len(coeffs), int(bound), int(first), int(last), flags,
                                     int(device), int(sample), ctypes.byref(r)))
    return {"rows": r.rows, "slots": r.slots, "key": r.key.decode(), "stored": bool(r.stored),
            "sample": r.sample_denominators,
            "candidates": [{"rows": r.candidate_rows[i], "slots": r.candidate_slots[i],
                            "ms": r.candidate_ms[i], "bits": r.candidate_bits[i]}
                           for i in range(r.candidates)]}


def fast_shape(coefficients, bound):
    """(rows, slots, from_cache) of the fast plan a sieve of this curve uses
    (host only): from_cache is True when a stored tuning result decides it."""
    coeffs = coefficients_of(coefficients)
    rows, slots, cached = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    _check(load().rpg_fast_shape(_strings(coeffs), len(coeffs), int(bound), ctypes.byref(rows),
                                 ctypes.byref(slots), ctypes.byref(cached)))
    return rows.value, slots.value, bool(cached.value)


def preverify(coefficients, a, b):
    """The device pre-verification test of site (a, b), evaluated on the host:
    False only if (a, b) cannot give a point."""
    coeffs = coefficients_of(coefficients)
    flag = ctypes.c_int32(-1)
    _check(load().rpg_preverify(_strings(coeffs), len(coeffs), int(a), int(b), ctypes.byref(flag)))
    return bool(flag.value)


def release_cached_resources(device=-1):
    """Frees the pooled streams and buffers that finished searches left for
    reuse on `device` (-1: every device)."""
    _check(load().rpg_release_cached_resources(int(device)))


def bounded_wait_selftest(polls, arrive, device=0):
    """Runs the bounded mbarrier wait self-test; raises RpgError with status
    RPG_E_TIMEOUT (4) when the wait gave up."""
    _check(load().rpg_bounded_wait_selftest(int(device), int(polls), int(bool(arrive))))


def smem_read_probe(iterations=4096, device=0):
    """Shared-memory read rate of the device: dict with gbs (GB/s),
    bytes_per_clock_per_sm and ms of the timed launch."""
    gbs, per_clk, ms = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    _check(load().rpg_smem_read_probe(int(device), int(iterations), ctypes.byref(gbs),
                                      ctypes.byref(per_clk), ctypes.byref(ms)))
    return {"gbs": gbs.value, "bytes_per_clock_per_sm": per_clk.value, "ms": ms.value}


def square_root(coefficients, a, b):
    coeffs = coefficients_of(coefficients)
    buf = ctypes.create_string_buffer(1 << 16)
    flag = ctypes.c_int32(-1)
    _check(load().rpg_square_root(_strings(coeffs), len(coeffs), int(a), int(b), buf,
                                  len(buf), ctypes.byref(flag)))
    return int(buf.value.decode()) if flag.value else None


class Session:
    """Device-resident tables; count() runs an event-timed counting pass."""

    def __init__(self, coefficients, bound, square=False, plan="reference", device=-1):
        lib = load()
        coeffs = coefficients_of(coefficients)
        flags = (RPG_SIEVE_SQUARE_DENOMINATORS if square else 0) | \
                (RPG_SIEVE_FAST_PLAN if plan == "fast" else 0)
        handle = ctypes.c_void_p()
        _check(lib.rpg_session_create(_strings(coeffs), len(coeffs), int(bound), flags, device,
                                      ctypes.byref(handle)))
        self._handle = handle

    def count(self, first, last, batch_size=1 << 16):
        n = ctypes.c_uint64(0)
        ms = ctypes.c_double(0)
        _check(load().rpg_session_count(self._handle, int(first), int(last), int(batch_size),
                                        ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def plan(self):
        """(class_prime, [small primes of the stage-1 rows]) of a fast-plan session."""
        cp = ctypes.c_int32(0)
        count = ctypes.c_int32(0)
        primes = (ctypes.c_int32 * 64)()
        _check(load().rpg_session_plan(self._handle, ctypes.byref(cp), primes, 64,
                                       ctypes.byref(count)))
        return cp.value, [primes[i] for i in range(count.value)]

    def work(self, first, last):
        """(64-site words swept, shared-memory bytes per swept word) of a pass."""
        words = ctypes.c_uint64(0)
        per = ctypes.c_uint32(0)
        _check(load().rpg_session_work(self._handle, int(first), int(last), ctypes.byref(words),
                                       ctypes.byref(per)))
        return words.value, per.value

    def close(self):
        if self._handle:
            load().rpg_session_destroy(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def cli(args, env=None, timeout=600, check=False):
    """Run the ratpoints_gpu executable; returns subprocess.CompletedProcess (bytes)."""
    if not EXECUTABLE.exists():
        raise RuntimeError(f"{EXECUTABLE} is not built; run python ratpoints-gpu_gb300/build.py")
    merged = dict(os.environ)
    merged.pop("RATPOINTS_GPU_BENCHMARK", None)
    merged.update(env or {})
    return subprocess.run([str(EXECUTABLE), *map(str, args)], capture_output=True,
                          timeout=timeout, env=merged, check=check)


def parse_metrics(stderr: bytes):
    """Key=value fields of the -v metrics line."""
    text = stderr.decode(errors="replace")
    line = re.search(r"^wall_ms=.*$", text, re.M)
    if not line:
        return None
    return {k: float(v) if "." in v else int(v)
            for k, v in re.findall(r"([a-z_]+)=([0-9.]+)", line.group())}
