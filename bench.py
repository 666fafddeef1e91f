"""Benchmark: Gsites/s of the bounded rational-point search on one GB300.

Workload (default): seeded random squarefree degree-6 curve with coefficients
uniform in [-2^32, 2^32), box a in [-5,000,000, 5,000,000], b in
[1, 5,000,000] (about 5e13 rectangle sites, 3.04e13 reduced pairs).

One step = one full sieve pass over the box with the per-curve tables already
resident on the device (value), timed with CUDA events on the sieve stream;
e2e = the same search through the C ABI rpg_point_search (coefficient strings
in, verified points out; planning, table build, host<->device copies and
exact verification inside the timed region), median of three searches after
two untimed ones.  Sites are counted as reduced pairs gcd(a, b) = 1, the
metric's definition; the rectangle count is in config.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference sieve (the
oracle port; the reference's own CPU path needs GMP headers and cannot be
built for the GPU host) on all host cores over a bounded sample of the same
workload.
"""

from __future__ import annotations

import argparse
import json
import os
import random
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "ratpoints-gpu_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "Gsites/s per GB300, batched vs plain, bit-exact point sets; p50/p99 latency"
UNIT = "Gsites/s"
C2_SEED = 5_000_000
HEIGHT = 5_000_000
DENOMINATORS = 5_000_000
BATCH = 1 << 16
SMS = 152
NOMINAL_SMEM_BYTES_PER_CLK = 128   # LDS bandwidth per SM, for comparison with the probe
# Dated ncu capture of one 65,536-denominator fast-plan launch of this workload
# (profiles/fast_sieve_kernel_c2.md gives the command): DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum) and the ALU-pipe share.  ncu
# runs every pass with a cold L2, so the DRAM figure is an upper bound for the
# timed launches, whose class tables stay in L2 between launches.
FAST_LAUNCH_PROFILE = {"dram_bytes": 43_845_120 + 71_424, "alu_pipe_frac": 0.554,
                       "issue_active_frac": 0.658,
                       "source": "profiles/fast_sieve_kernel_c2.md (ncu --set full, "
                                 "fast_sieve_kernel<7,3>, one launch)"}


def measured_hbm_gbs():
    """The machine's measured HBM copy bandwidth (GB/s), None if not recorded."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return None
REF_FAST_PRIMES = 10          # reference-plan primes read from shared memory per site


def c2_curve(seed=C2_SEED):
    """Seeded squarefree degree-6 curve, coefficients uniform in [-2^32, 2^32)."""
    import ratpoints_oracle as oracle

    rng = random.Random(seed)
    while True:
        coeffs = [rng.randrange(-(2**32), 2**32) for _ in range(7)]
        if coeffs[-1] != 0 and oracle.is_squarefree(coeffs):
            return [str(c) for c in coeffs]


def mobius(limit):
    """mu(n) for n <= limit: signs flipped by the primes up to sqrt(limit),
    zeros at their squares, and one more flip where a prime above sqrt(limit)
    is left over (at most one such factor fits)."""
    import numpy as np
    from math import isqrt

    root = isqrt(limit)
    small = np.ones(root + 1, dtype=bool)
    small[:2] = False
    for p in range(2, isqrt(root) + 1):
        if small[p]:
            small[p * p::p] = False
    mu = np.ones(limit + 1, dtype=np.int8)
    rest = np.arange(limit + 1, dtype=np.int64)
    for p in np.flatnonzero(small).tolist():
        mu[p::p] *= -1
        mu[p * p::p * p] = 0
        rest[p::p] //= p
    mu[rest > 1] *= -1
    mu[0] = 0
    return mu


def reduced_sites(height, last, mu=None, first=1):
    """#{(a, b): |a| <= height, first <= b <= last, gcd(a, b) = 1}
    = sum_d mu(d) (floor(last/d) - floor((first-1)/d)) (2 floor(height/d) + 1)."""
    import numpy as np

    mu = mobius(last) if mu is None else mu
    d = np.arange(1, last + 1, dtype=np.int64)
    multiples = last // d - (first - 1) // d
    terms = mu[1:last + 1].astype(np.int64) * multiples * (2 * (height // d) + 1)
    return int(terms.sum())


def rank_block(rank, per_rank):
    """Denominators [first, last] that `rank` sieves under weak scaling: each
    rank takes its own block of per_rank consecutive denominators."""
    return rank * per_rank + 1, (rank + 1) * per_rank


def sum_over_ranks(value, dist):
    """The ranks' integer counts added up."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([int(value)], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def max_over_ranks(value, dist):
    """The largest of the ranks' values (the step time of the slowest rank)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.file.flush()

    def summary(self):
        import statistics

        rows = []
        try:
            for line in Path(self.file.name).read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        sm_max = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, flag in zip(names, r[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        loaded = [s for s in sm if s > 0.5 * sm_max] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": sm_max,
                "reasons": sorted(reasons), "samples": len(rows)}


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def flush_l2(torch, buf, step):
    buf.fill_(step & 0xFF)
    torch.cuda.synchronize()


def cpu_baseline(coeffs, seconds=12.0):
    """Oracle port of the reference sieve on all host cores, bounded sample."""
    import ratpoints_oracle as oracle

    threads = os.cpu_count() or 1
    sieve = oracle.ModularSieve(coeffs, HEIGHT)
    t0 = time.perf_counter()
    sieve.count(1, threads, threads=threads)
    one = max(1e-3, time.perf_counter() - t0)
    k = max(threads, min(DENOMINATORS, int(threads * seconds / one)))
    t0 = time.perf_counter()
    survivors, _ = sieve.count(1, k, threads=threads)
    elapsed = time.perf_counter() - t0
    sieve.close()
    sites = reduced_sites(HEIGHT, k)
    return {"value": sites / elapsed / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle C restatement of the reference 32-prime word sieve, "
                      f"H={HEIGHT}, b in [1, {k}] ({sites} reduced sites, "
                      f"{survivors} modular survivors), {elapsed:.2f} s on {threads} threads"}


def reference_host_mock(threads=None):
    """The reference's own CPU path on the C1 configuration: its host program
    with the CPU mock backend (every site checked exactly with GMP), built from
    its unchanged sources by oracle/ref_cpu/build_mock.py where the reference
    tree exists; None elsewhere.  One mock device per thread."""
    import hashlib
    import statistics

    mock = ROOT / "oracle" / "_ref" / "mock_ratpoints_gpu"
    if not mock.exists():
        return None
    golden = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())["c1"]
    threads = threads or os.cpu_count() or 1
    env = dict(os.environ, RATPOINTS_TEST_DEVICE_COUNT=str(threads))
    env.pop("CUDA_VISIBLE_DEVICES", None)
    # at most 2,000,000 sites per mock worker (tests/mock_backend.cpp:106-108)
    batch = max(1, min(499, 2_000_000 // (2 * golden["height"] + 1)))
    cmd = [str(mock), golden["coefficients"], str(golden["height"]), "-du", str(golden["last"]),
           "--devices", "all", "--batch-size", str(batch)]
    times, same = [], True
    for _ in range(3):
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, env=env, timeout=600)
        times.append(time.perf_counter() - t0)
        same = same and r.returncode == 0 and hashlib.sha256(r.stdout).hexdigest() == golden["sha256"]
    wall = statistics.median(times)
    reduced = reduced_sites(golden["height"], golden["last"])
    return {"value": reduced / wall / 1e9, "unit": UNIT, "seconds": wall, "threads": threads,
            "stdout_matches_golden": same,
            "workload": f"C1: degree-6 curve, coefficients in [-50, 50], a in [-{golden['height']}, "
                        f"{golden['height']}], b in [1, {golden['last']}], default output; process "
                        "wall time, median of 3"}


def run_reference(args):
    coeffs = c2_curve()
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    values = []
    for _ in range(args.warmup):
        cpu_baseline(coeffs, seconds=3.0)
    for _ in range(args.steps):
        values.append(cpu_baseline(coeffs, seconds=args.cpu_seconds))
    value = sorted(v["value"] for v in values)[len(values) // 2]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {**values[-1], "value": value},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    mock = reference_host_mock()
    if mock is not None:
        line["reference_host_mock"] = mock
    print(json.dumps(line))


def _ref_gpu_module():
    sys.path.insert(0, str(ROOT / "oracle" / "ref_gpu"))
    import ref_gpu

    return ref_gpu


def reference_gpu(coeffs, denominators, rpg, steps=3):
    """The reference's own sieve kernels (src/sieve.cu compiled unchanged for
    sm_103a) over denominators [1, denominators] of the workload, with the
    reference's host loop restated: kernel event time, median of `steps`
    passes after a short warm-up; survivor multiset (count and digest)
    compared with this project's reference plan over the same box."""
    ref_gpu = _ref_gpu_module()
    import ratpoints_oracle as oracle

    if not ref_gpu.available():
        return {"unavailable": "reference cubin not built (needs the reference tree at build time)"}
    ref_gpu.run(coeffs, HEIGHT, 1, min(denominators, 4096))  # warm-up
    runs = [ref_gpu.run(coeffs, HEIGHT, 1, denominators) for _ in range(max(1, steps))]
    ref = sorted(runs, key=lambda r: r["sieve_ms"])[len(runs) // 2]
    a, d, _ = rpg.sieve(coeffs, HEIGHT, 1, denominators, plan="reference")
    digest = sum(oracle.mix_pair(x, y) for x, y in zip(a.tolist(), d.tolist())) % 2**64
    reduced = reduced_sites(HEIGHT, denominators)
    rect = (2 * HEIGHT + 1) * denominators
    return {"denominators": denominators, "steps": len(runs), "kernel_ms": ref["sieve_ms"],
            "basis_ms": ref["basis_ms"], "wall_ms": ref["wall_ms"],
            "value": reduced / (ref["sieve_ms"] / 1e3) / 1e9, "unit": UNIT,
            "rectangle_gsites_per_s": rect / (ref["sieve_ms"] / 1e3) / 1e9,
            "survivors": ref["survivors"],
            "survivor_set_matches_reference_plan": (len(a), digest) == (ref["survivors"],
                                                                        ref["digest"]),
            "note": "reference src/sieve.cu compiled for sm_103a, kernel event time; basis built "
                    "once (the reference rebuilds it per batch)"}


def record_curve_kernels(rpg, torch, flush, height=10 ** 7, denominators=10 ** 6, steps=3):
    """The record curve (the reference's own benchmark curve, a dense one) over
    a in [-H, H], b in [1, denominators]: the reference's kernels against this
    project's fast and reference plans, kernel time only (tables resident),
    median of `steps` passes; the reference plan's survivor count must equal
    the reference kernels'."""
    import workloads

    ref_gpu = _ref_gpu_module()
    reduced = workloads.reduced_sites(height, 1, denominators, workloads.mobius(denominators))
    out = {"workload": f"record curve, a in [-{height:g}, {height:g}], b in [1, {denominators:g}]",
           "reduced_sites": reduced}
    coeffs = workloads.RECORD_CURVE.split()
    for plan in ("fast", "reference"):
        session = rpg.Session(coeffs, height, plan=plan)
        session.count(1, min(denominators, 4096))
        times, counts = [], []
        for step in range(steps):
            flush_l2(torch, flush, step)
            n, ms = session.count(1, denominators)
            times.append(ms)
            counts.append(n)
        session.close()
        ms = sorted(times)[len(times) // 2]
        out[plan] = {"kernel_ms": ms, "value": reduced / (ms / 1e3) / 1e9, "unit": UNIT,
                     "survivors": counts[0]}
    if ref_gpu.available():
        ref_gpu.run(coeffs, height, 1, min(denominators, 4096))
        runs = [ref_gpu.run(coeffs, height, 1, denominators) for _ in range(steps)]
        ref = sorted(runs, key=lambda r: r["sieve_ms"])[len(runs) // 2]
        out["reference_kernels"] = {"kernel_ms": ref["sieve_ms"],
                                    "value": reduced / (ref["sieve_ms"] / 1e3) / 1e9, "unit": UNIT,
                                    "survivors": ref["survivors"]}
        out["survivor_count_matches_reference_plan"] = ref["survivors"] == out["reference"]["survivors"]
        out["ratio_fast"] = out["fast"]["value"] / out["reference_kernels"]["value"]
        out["ratio_same_survivors"] = out["reference"]["value"] / out["reference_kernels"]["value"]
    return out


def batch_benchmark(rpg, count=4096, plain_curves=4096, steps=2, shape="all", smem_peak_gbs=None,
                    tune=False):
    """Mixed many-curve batch: one batched pass against the plain per-curve
    loop of single-curve searches, same curves, points compared curve by curve.
    Both are timed end to end through the C ABI (coefficient strings in,
    verified points out).  shape "wide" / "narrow" keeps only the curves whose
    rows have at least / fewer than 2,048 words of 64 numerators (the two
    batch kernels), for per-kernel measurements.  With tune the batch's work
    items per kernel are tuned first (rpg_tune_batch, untimed, kept in the
    run's tuning cache)."""
    import workloads

    curves = workloads.mixed_batch(count)
    if shape != "all":
        wide = lambda c: (2 * c["bound"] + 64) // 64 >= 2048
        curves = [c for c in curves if wide(c) == (shape == "wide")]
        count = len(curves)
    mu = workloads.mobius(max(c["last"] for c in curves))
    reduced = [workloads.reduced_sites(c["bound"], c["first"], c["last"], mu) for c in curves]
    rect = [(2 * c["bound"] + 1) * (c["last"] - c["first"] + 1) for c in curves]
    tuning = rpg.tune_batch(curves) if tune else None
    rpg.batch_search(curves[:32])  # warm-up: module load, graph instantiation paths
    runs = []
    for _ in range(steps):
        t0 = time.perf_counter()
        points, status, survivors, stats = rpg.batch_search(curves)
        runs.append((time.perf_counter() - t0, points, stats))
    wall, points, stats = sorted(runs, key=lambda r: r[0])[len(runs) // 2]
    n_plain = min(plain_curves, count)
    t0 = time.perf_counter()
    plain = [rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"])[0]
             for c in curves[:n_plain]]
    plain_wall = time.perf_counter() - t0
    identical = all(a == b for a, b in zip(plain, points[:n_plain])) if n_plain else None
    total_reduced, plain_reduced = sum(reduced), sum(reduced[:n_plain])
    batched = total_reduced / wall / 1e9
    plain_value = plain_reduced / plain_wall / 1e9 if n_plain else None
    return {
        "shape": shape,
        "workload": f"{count} seeded squarefree curves: degree uniform in {{3,4,5,6,8,10}}, "
                    "coefficients random sign x random integer of bit length uniform in 8..64, "
                    "numerator bound A and denominator bound B independent, each log-uniform "
                    "in [1e3, 1e6]",
        "curves": count, "seed": 3, "reduced_sites": total_reduced, "rectangle_sites": sum(rect),
        "denominators": stats["denominators"],
        "batched": {"value": batched, "unit": UNIT, "wall_s": wall,
                    "kernel_value": total_reduced / (stats["sieve_ms"] / 1e3) / 1e9,
                    "sieve_ms": stats["sieve_ms"], "wide_kernel_ms": stats["wide_ms"],
                    "narrow_kernel_ms": stats["narrow_ms"], "table_ms": stats["table_ms"],
                    "plan_ms": stats["plan_ms"], "verify_ms": stats["verify_ms"],
                    "wide_curves": stats["wide_curves"], "survivors": stats["survivors"],
                    "points": stats["points"], "table_bytes": stats["table_words"] * 8,
                    "h2d_bytes": stats["h2d_bytes"], "d2h_bytes": stats["d2h_bytes"],
                    "graph": bool(stats["graph"]), "launches": stats["launches"],
                    "items_per_kernel": stats["items_per_kernel"],
                    "items_from_cache": bool(stats["items_from_cache"])},
        "items_tuning": None if tuning is None else {
            "key": tuning["key"], "chosen": tuning["items"],
            "candidates_ms": {str(c["items"]): round(c["ms"], 2) for c in tuning["candidates"]}},
        "plain_loop": {"value": plain_value, "unit": UNIT, "wall_s": plain_wall,
                       "curves": n_plain,
                       "note": "rpg_point_search (single-curve fast plan) called once per curve"},
        "speedup_vs_plain": batched / plain_value if plain_value else None,
        "roofline": None if not smem_peak_gbs else {
            "bound": "smem", "unit": "GB/s",
            "achieved": stats["smem_bytes"] / (stats["sieve_ms"] / 1e3) / 1e9,
            "peak": smem_peak_gbs,
            "frac": stats["smem_bytes"] / (stats["sieve_ms"] / 1e3) / 1e9 / smem_peak_gbs,
            "swept_words": stats["swept_words"], "smem_bytes": stats["smem_bytes"],
            "algorithmic": "8 B per stage-1 modulus of each curve's plan per swept 64-site word "
                           "(class words on the wide kernel, row words on the narrow one), both "
                           "kernels' time"},
        "points_identical": identical,
    }


def _loop(rpg, curves):
    """The plain per-curve loop: one single-curve search per curve."""
    t0 = time.perf_counter()
    pts = [rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"],
                            intervals=c.get("intervals", ()), square=c.get("square", False))[0]
           for c in curves]
    return time.perf_counter() - t0, pts


def restricted_benchmark(rpg, high_degree=256, cubics=32, plain_cubics=8):
    """High-degree curves with big coefficients restricted to x intervals, and
    cubics with square denominators: batched pass against the plain loop.
    Sites are those of the search boxes ((2A + 1) x denominators), whether or
    not the sieve sweeps them (interval narrowing skips rows' other numerators)."""
    import workloads

    out = {}
    curves = workloads.wide_degree(high_degree)
    box = sum((2 * c["bound"] + 1) * c["last"] for c in curves)
    rpg.batch_search(curves[:4])
    t0 = time.perf_counter()
    points, _, _, stats = rpg.batch_search(curves)
    wall = time.perf_counter() - t0
    plain_wall, plain = _loop(rpg, curves)
    out["high_degree_intervals"] = {
        "workload": f"{high_degree} curves, degree uniform in 12..40, coefficients of 100..256 bits, "
                    "A = B = 1e5, x in 3 random closed intervals",
        "box_sites": box, "batched": {"value": box / wall / 1e9, "unit": "rectangle Gsites/s",
                                      "wall_s": wall, "sieve_ms": stats["sieve_ms"],
                                      "points": stats["points"], "survivors": stats["survivors"]},
        "plain_loop": {"value": box / plain_wall / 1e9, "unit": "rectangle Gsites/s",
                       "wall_s": plain_wall, "note": "single-curve search of each curve: whole "
                                                     "rows swept, interval test on the host"},
        "speedup_vs_plain": plain_wall / wall,
        "points_identical": plain == points}
    if cubics > 0:
        cs = workloads.square_cubics(cubics)
        box = sum((2 * c["bound"] + 1) * c["last"] for c in cs)
        t0 = time.perf_counter()
        points, _, _, stats = rpg.batch_search(cs)
        wall = time.perf_counter() - t0
        n_plain = min(plain_cubics, cubics)
        plain_wall, plain = _loop(rpg, cs[:n_plain])
        plain_box = sum((2 * c["bound"] + 1) * c["last"] for c in cs[:n_plain])
        out["square_cubics"] = {
            "workload": f"{cubics} of the 256 cubics x^3 + alpha x + beta, alpha, beta uniform in "
                        "[-1e12, 1e12], denominators k^2 for k in [1, 46340], |a| <= 1e9",
            "box_sites": box,
            "batched": {"value": box / wall / 1e9, "unit": "rectangle Gsites/s", "wall_s": wall,
                        "sieve_ms": stats["sieve_ms"], "points": stats["points"],
                        "survivors": stats["survivors"]},
            "plain_loop": {"value": plain_box / plain_wall / 1e9, "unit": "rectangle Gsites/s",
                           "wall_s": plain_wall, "curves": n_plain},
            "points_identical": plain == points[:n_plain]}
    return out


def dense_curve_benchmark(rpg, height=10 ** 7):
    """The record curve (a dense curve: squares modulo most small primes, so
    many modular survivors) over a in [-H, H], b in [1, H] through the command
    line, with device pre-verification (default) and with every modular
    survivor checked on the host (--host-verify-only), both plans.  Each run's
    stdout SHA-256 is compared with the reference's published full-box output
    at H = 10^7."""
    import hashlib
    import workloads

    golden = json.loads((Path(__file__).resolve().parent / "tests" / "golden" / "golden.json").read_text())
    expected = next((g["sha256"] for g in golden["record_full"]
                     if g["height"] == height and g["last"] == height), None)
    rect = (2 * height + 1) * height
    reduced = workloads.reduced_sites(height, 1, height, workloads.mobius(height))
    runs = {}
    for plan in ("fast", "reference"):
        for mode, extra in (("device_preverify", []), ("host_verify_only", ["--host-verify-only"])):
            t0 = time.perf_counter()
            result = rpg.cli([workloads.RECORD_CURVE, height, "-v", "--sieve-plan", plan, *extra])
            wall = time.perf_counter() - t0
            m = rpg.parse_metrics(result.stderr) or {}
            runs[f"{plan}/{mode}"] = {
                "exit": result.returncode, "wall_s": wall, "value": reduced / wall / 1e9, "unit": UNIT,
                "internal_wall_ms": m.get("wall_ms"), "verification_ms": m.get("verification_ms"),
                "sieve_ms": m.get("sieve_ms"), "modular_survivors": m.get("survivors"),
                "exact_survivors": m.get("exact_survivors"),
                "sha256_matches_reference": hashlib.sha256(result.stdout).hexdigest() == expected}
    return {"workload": f"record curve, a in [-{height:g}, {height:g}], b in [1, {height:g}], "
                        "default output, through the ratpoints_gpu command line (process start, "
                        "table build, sieve, verification and output)",
            "reduced_sites": reduced, "rectangle_sites": rect, "runs": runs}


def serving_benchmark(rpg, count=1000, rate=200.0, lanes=2, check=40):
    """Poisson stream of requests into the serving loop: per-request latency
    (submit -> answer) percentiles and aggregate throughput over the stream."""
    import statistics
    import workloads

    stream = workloads.serving_stream(count, rate)
    mu = workloads.mobius(max(r["last"] for _, r, _ in stream))
    results = [None] * len(stream)
    with rpg.Server(lanes=lanes) as server:
        warm = server.submit(stream[0][1])
        server.wait(warm)
        ids = [None] * len(stream)
        t0 = time.perf_counter()

        def feed():
            for i, (at, req, first) in enumerate(stream):
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids[i] = server.submit(req, first)

        feeder = threading.Thread(target=feed)
        feeder.start()
        feeder.join()
        for i, rid in enumerate(ids):
            results[i] = server.wait(rid)
        wall = time.perf_counter() - t0
    lat = sorted(r[2]["latency_ms"] for r in results)
    pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))]
    queue = sorted(r[2]["queue_ms"] for r in results)
    qpct = lambda q: queue[min(len(queue) - 1, int(q * len(queue)))]
    # the slowest 1%: how much of their latency was queueing, and their waves
    tail = sorted(results, key=lambda r: r[2]["latency_ms"])[-max(1, len(results) // 100):]
    tail_info = {"requests": len(tail),
                 "mean_latency_ms": statistics.fmean(r[2]["latency_ms"] for r in tail),
                 "mean_queue_ms": statistics.fmean(r[2]["queue_ms"] for r in tail),
                 "mean_waves": statistics.fmean(r[2]["waves"] for r in tail),
                 "mean_rectangle_sites": statistics.fmean(r[2]["rectangle_sites"] for r in tail)}
    rect = sum(r[2]["rectangle_sites"] for r in results)
    reduced = 0
    for (_, req, _), r in zip(stream, results):
        searched = int(round(r[2]["rectangle_sites"] / (2 * req["bound"] + 1)))
        if searched:
            reduced += workloads.reduced_sites(req["bound"], req["first"], req["first"] + searched - 1, mu)
    rng = random.Random(1)
    sample = rng.sample(range(len(stream)), min(check, len(stream)))
    identical = all(
        results[i][1] == rpg.point_search(stream[i][1]["coefficients"], stream[i][1]["bound"],
                                          stream[i][1]["first"], stream[i][1]["last"],
                                          stop_after=1 if stream[i][2] else None)[0]
        for i in sample)
    return {"workload": f"{count} requests, Poisson arrivals at {rate:g}/s: degree uniform in 2..12, "
                        "coefficients of 16..128 bits, a in [-H, H], b in [1, H], H log-uniform in "
                        "[1e2, 1e6], 30% first point only",
            "lanes": lanes, "requests": count, "wall_s": wall,
            "p50_ms": pct(0.50), "p99_ms": pct(0.99), "mean_ms": statistics.fmean(lat),
            "max_ms": lat[-1], "queue_p50_ms": qpct(0.50), "queue_p99_ms": qpct(0.99),
            "slowest_1pct": tail_info, "offered_rate": rate,
            "value": reduced / wall / 1e9, "unit": UNIT,
            "rectangle_gsites_per_s": rect / wall / 1e9,
            "note": "throughput = reduced sites searched (first-point requests count the "
                    "denominators their waves covered) / stream wall time",
            "identical_to_single_search": {"checked": len(sample), "all": identical}}


def summary(line):
    """The headline comparisons, kept short and last on the line."""
    def r(x, nd=3):
        return None if x is None else round(float(x), nd)

    out = {"value": r(line["value"], 0), "e2e": r(line["e2e"]["value"], 0),
           "roofline_frac": r(line["roofline"]["frac"])}
    g = line.get("reference_gpu") or {}
    if g.get("value"):
        out["reference_kernels"] = {
            "denominators": g["denominators"], "value": r(g["value"], 0),
            "ratio_fast": r(line["value"] / g["value"], 1),
            "ratio_e2e": r(line["e2e"]["value"] / g["value"], 1),
            "ratio_same_survivors": r(line["reference_plan"]["value"] / g["value"], 2)
            if line.get("reference_plan") else None,
            "survivors_match": g.get("survivor_set_matches_reference_plan")}
    rc = line.get("record_curve_kernels") or {}
    if rc.get("ratio_fast"):
        out["record_curve_kernels"] = {"ratio_fast": r(rc["ratio_fast"], 2),
                                       "ratio_same_survivors": r(rc["ratio_same_survivors"], 2),
                                       "survivors_match": rc.get("survivor_count_matches_reference_plan")}
    b = line.get("batch") or {}
    if b:
        out["batch"] = {"speedup_vs_plain": r(b.get("speedup_vs_plain"), 2),
                        "points_identical": b.get("points_identical"),
                        "roofline_frac": r((b.get("roofline") or {}).get("frac")),
                        "items_per_kernel": (b.get("batched") or {}).get("items_per_kernel")}
    sv = line.get("serving") or {}
    if sv:
        out["serving"] = {"p50_ms": r(sv.get("p50_ms")), "p99_ms": r(sv.get("p99_ms")),
                          "identical": (sv.get("identical_to_single_search") or {}).get("all")}
        if sv.get("saturation"):
            out["serving"]["saturation"] = {k: r(sv["saturation"].get(k)) for k in
                                            ("value", "p50_ms", "p99_ms", "offered_rate")}
    dc = line.get("dense_curve") or {}
    if dc:
        out["dense_curve_sha_ok"] = all(v.get("sha256_matches_reference") for v in dc["runs"].values())
    rs = line.get("restricted") or {}
    if rs:
        out["restricted_identical"] = all(v.get("points_identical") for v in rs.values())
    at = line.get("autotune") or {}
    if at:
        out["autotune"] = {name: t["chosen"] for name, t in at.items()}
    cb = line.get("cpu_baseline") or {}
    if cb:
        out["cpu_baseline"] = {"value": r(cb.get("value")), "kind": cb.get("kind"),
                               "cores": cb.get("cores")}
    return out


def workload_config():
    rect = (2 * HEIGHT + 1) * DENOMINATORS
    return {"workload": "degree-6 curve, coefficients uniform in [-2^32, 2^32), "
                        "a in [-5e6, 5e6], b in [1, 5e6]",
            "height": HEIGHT, "denominators": DENOMINATORS, "batch": BATCH,
            "rectangle_sites": rect, "seed": C2_SEED,
            "l2": "256 MiB buffer written between timed steps (the fast plan's tables are "
                  "about 70 MB, the reference plan's 57 MB)"}


def main():
    parser = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=5)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--plan", choices=["reference", "fast"], default="fast")
    parser.add_argument("--reference-plan-steps", type=int, default=2)
    parser.add_argument("--reference-gpu-denominators", type=int, default=DENOMINATORS,
                        help="denominators of the box the reference's kernels sieve (0: skip)")
    parser.add_argument("--reference-gpu-steps", type=int, default=3,
                        help="timed passes of the reference's kernels (median reported)")
    parser.add_argument("--record-denominators", type=int, default=10 ** 6,
                        help="denominators of the record-curve kernel comparison (0: skip)")
    parser.add_argument("--denominators", type=int, default=DENOMINATORS)
    parser.add_argument("--e2e-steps", type=int, default=3, choices=range(1, 100), metavar="N",
                        help="timed searches through rpg_point_search (median reported)")
    parser.add_argument("--e2e-warmup", type=int, default=2, choices=range(0, 100), metavar="N",
                        help="untimed searches through rpg_point_search before them")
    parser.add_argument("--cpu-seconds", type=float, default=12.0)
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--tune", action=argparse.BooleanOptionalAction, default=True,
                        help="time the fast plan's candidate shapes first and use the fastest")
    parser.add_argument("--batch-curves", type=int, default=4096,
                        help="curves of the mixed batch (0: skip the batch measurement)")
    parser.add_argument("--batch-plain-curves", type=int, default=4096,
                        help="curves of the batch also run as a plain per-curve loop")
    parser.add_argument("--batch-shape", choices=["all", "wide", "narrow"], default="all",
                        help="keep only the batch curves of one kernel")
    parser.add_argument("--restricted", type=int, default=256,
                        help="high-degree interval-restricted curves (0: skip)")
    parser.add_argument("--square-cubics", type=int, default=32,
                        help="square-denominator cubics of the restricted searches (0: skip)")
    parser.add_argument("--serving-requests", type=int, default=1000,
                        help="requests of the serving stream (0: skip)")
    parser.add_argument("--saturation-rate", type=float, default=20000.0,
                        help="arrival rate (requests/s) of the serving saturation run")
    parser.add_argument("--dense-height", type=int, default=10 ** 7,
                        help="record-curve box height for the pre-verification runs (0: skip)")
    args = parser.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import ratpoints_gb300 as rpg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    rpg.build() if rank == 0 else None
    if dist:
        dist.barrier()
    rpg.load()
    coeffs = c2_curve()
    last = args.denominators
    tuning = None
    if args.tune:
        # the measured autotuner: candidate shapes of the fast plan timed on a
        # sample of this workload, the fastest kept in a tuning cache that the
        # sessions and searches below read (untimed)
        cache = Path(tempfile.mkdtemp(prefix="rpg_tune_")) / "fast_plan_shapes.json"
        os.environ["RPG_TUNE_CACHE"] = str(cache)
        tuning = {"c2": rpg.tune_fast_plan(coeffs, HEIGHT, 1, last, device=local, sample=1 << 17)}
        if args.record_denominators > 0 or args.dense_height > 0:
            import workloads
            tuning["record_curve"] = rpg.tune_fast_plan(workloads.RECORD_CURVE.split(), 10 ** 7, 1, 10 ** 7,
                                                        device=local, sample=20_000)
    # weak scaling: rank r sieves its own block of `last` denominators
    first_b, last_b = rank_block(rank, last)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def measure(plan, steps, warmup, sampler=None):
        session = rpg.Session(coeffs, HEIGHT, plan=plan, device=local)
        for step in range(warmup):
            flush_l2(torch, flush, step)
            session.count(first_b, last_b, BATCH)
        times, counts = [], []
        ctx = sampler if sampler is not None else _Null()
        with ctx:
            for step in range(steps):
                flush_l2(torch, flush, step)
                if dist:
                    dist.barrier()
                n, ms = session.count(first_b, last_b, BATCH)
                times.append(ms)
                counts.append(n)
        assert len(set(counts)) == 1, "survivor count changed between steps"
        words, per_word = session.work(first_b, last_b)
        session.close()
        step_ms = max_over_ranks(sum(times) / len(times), dist)
        return {"ms": step_ms, "survivors": counts[0], "words": words, "bytes_per_word": per_word}

    probe_clocks = ClockSampler(local)
    with probe_clocks:
        probe = rpg.smem_read_probe(device=local)
    probe_clock_mhz = probe_clocks.summary().get("sm_mhz")
    probe["sm_mhz"] = probe_clock_mhz
    clocks = ClockSampler(local)
    fast = measure(args.plan, args.steps, args.warmup, clocks)
    clock = clocks.summary()
    ref = None
    if args.plan != "reference" and args.reference_plan_steps > 0:
        ref = measure("reference", args.reference_plan_steps, 1)

    # sites of the whole job: every rank's own block
    reduced = sum_over_ranks(reduced_sites(HEIGHT, last_b, mobius(last_b), first=first_b), dist)
    rect = (2 * HEIGHT + 1) * last * world
    step_ms = fast["ms"]
    value = reduced / (step_ms / 1e3) / 1e9
    launches_per_step = (last + BATCH - 1) // BATCH

    # e2e through the C ABI: host strings in, verified points out
    e2e_times, e2e_stats, points = [], None, None
    for i in range(args.e2e_warmup + args.e2e_steps):
        t0 = time.perf_counter()
        points, e2e_stats = rpg.point_search(coeffs, HEIGHT, first_b, last_b, plan=args.plan,
                                             include_infinity=True)
        if i >= args.e2e_warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sorted(e2e_times)[len(e2e_times) // 2], dist)
    if rank != 0:
        return
    total_bytes = fast["words"] * fast["bytes_per_word"]
    achieved = total_bytes / (step_ms / 1e3) / 1e9
    sm_hz = (clock.get("sm_mhz") or probe_clock_mhz or 2070.0) * 1e6
    nominal = SMS * NOMINAL_SMEM_BYTES_PER_CLK * sm_hz / 1e9
    peak = probe["gbs"]
    launch_s = step_ms / launches_per_step / 1e3
    dram = FAST_LAUNCH_PROFILE["dram_bytes"] if args.plan == "fast" else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: seeded random squarefree degree-6 curve, "
                "coefficients uniform in [-2^32, 2^32)",
        "config": {**workload_config(), "denominators": last, "rectangle_sites": rect,
                   "reduced_sites": reduced, "plan": args.plan,
                   "rectangle_gsites_per_s": rect / (step_ms / 1e3) / 1e9,
                   "modular_survivors": fast["survivors"],
                   "words_swept_per_step": fast["words"]},
        "roofline": {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": dram,
                     "traffic_note": "DRAM bytes per 65,536-denominator launch from the dated ncu "
                                     f"capture in {FAST_LAUNCH_PROFILE['source']} (cold L2); the "
                                     "algorithmic shared-memory bytes per launch are "
                                     f"{total_bytes / launches_per_step:.3g}",
                     "algorithmic": f"{fast['bytes_per_word']} B of stage-1 shared-memory rows per "
                                    f"swept 64-site word x {fast['words']} words per step "
                                    f"/ {launches_per_step} launches",
                     "peak_source": "rpg_smem_read_probe in this run: lane-contiguous 64-bit shared "
                                    f"loads from every resident warp, {probe['gbs']:.0f} GB/s = "
                                    f"{probe['bytes_per_clock_per_sm']:.1f} B/clk/SM (nominal "
                                    f"{NOMINAL_SMEM_BYTES_PER_CLK} B/clk/SM x {SMS} SMs at the sampled "
                                    f"clock: {nominal:.0f} GB/s, frac {achieved / nominal:.3f})",
                     "int_pipe": {"alu_pipe_frac": FAST_LAUNCH_PROFILE["alu_pipe_frac"],
                                  "issue_active_frac": FAST_LAUNCH_PROFILE["issue_active_frac"],
                                  "source": FAST_LAUNCH_PROFILE["source"]} if args.plan == "fast" else None,
                     "hbm": None if dram is None or not measured_hbm_gbs() else {
                         "achieved": dram / launch_s / 1e9, "peak": measured_hbm_gbs(), "unit": "GB/s",
                         "frac": dram / launch_s / 1e9 / measured_hbm_gbs(),
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (STREAM-style copy)"}},
        "e2e": {"value": reduced / e2e_s / 1e9, "unit": UNIT,
                "seconds": e2e_s, "points": len(points),
                "h2d_bytes_per_step": int(e2e_stats.get("h2d_bytes", 0)) if e2e_stats else 0,
                "d2h_bytes_per_step": int(e2e_stats.get("d2h_bytes", 0)) if e2e_stats else 0,
                "breakdown_ms": {k: round(float(e2e_stats.get(k, 0)), 3) for k in
                                 ("plan_ms", "workspace_ms", "basis_wall_ms", "basis_ms", "sieve_ms",
                                  "sieve_wall_ms", "verification_ms")} if e2e_stats else None},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clock,
    }
    if tuning:
        line["autotune"] = {name: {"key": t["key"], "chosen": f"{t['rows']} rows x {t['slots']} slots",
                                   "sample_denominators": t["sample"],
                                   "candidates_ms": {f"{c['rows']}x{c['slots']}": round(c["ms"], 4)
                                                     for c in t["candidates"]}}
                            for name, t in tuning.items()}
    if args.reference_gpu_denominators > 0:
        line["reference_gpu"] = reference_gpu(coeffs, args.reference_gpu_denominators, rpg,
                                              args.reference_gpu_steps)
    if ref is not None:
        line["reference_plan"] = {
            "value": reduced / (ref["ms"] / 1e3) / 1e9, "unit": UNIT,
            "ms_per_step": ref["ms"], "modular_survivors": ref["survivors"],
            "note": "same kernel family with the reference's 32-prime plan: survivor set "
                    "identical to the reference implementation's"}
    if args.record_denominators > 0:
        line["record_curve_kernels"] = record_curve_kernels(rpg, torch, flush,
                                                            denominators=args.record_denominators)
    if args.batch_curves > 0:
        line["batch"] = batch_benchmark(rpg, args.batch_curves, args.batch_plain_curves,
                                        shape=args.batch_shape, smem_peak_gbs=peak, tune=args.tune)
    if args.restricted > 0:
        line["restricted"] = restricted_benchmark(rpg, args.restricted, args.square_cubics)
    if args.serving_requests > 0:
        line["serving"] = serving_benchmark(rpg, args.serving_requests)
        # the same stream offered far above what the device answers: the
        # sustained throughput and the latency at saturation
        sat = serving_benchmark(rpg, args.serving_requests, rate=args.saturation_rate, check=10)
        line["serving"]["saturation"] = {k: sat[k] for k in (
            "offered_rate", "requests", "wall_s", "value", "unit", "p50_ms", "p99_ms",
            "queue_p50_ms", "queue_p99_ms", "rectangle_gsites_per_s", "identical_to_single_search")}
    if args.dense_height > 0:
        line["dense_curve"] = dense_curve_benchmark(rpg, args.dense_height)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(coeffs, seconds=args.cpu_seconds)
    line["summary"] = summary(line)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
