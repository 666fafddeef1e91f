"""The reference plan against the reference's own CUDA kernels on the GPU.

oracle/_ref/ref_sieve.cubin is the reference's src/sieve.cu compiled unchanged
for sm_103a; oracle/ref_gpu drives it with a restatement of the reference's
host loop.  The survivor multiset of this project's reference plan must equal
the reference kernels' (count and order-independent digest), including the
streaming overflow path of the reference (dense curve).
"""

import random
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle" / "ref_gpu"))
import ref_gpu  # noqa: E402

if not ref_gpu.available():
    pytest.skip("reference cubin not built (needs the reference tree at build time)",
                allow_module_level=True)

RECORD = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800".split()


def compare(rpg, oracle, coeffs, bound, first, last, square=False, batch=65536):
    ref = ref_gpu.run(coeffs, bound, first, last, batch=batch, square=square)
    a, d, _ = rpg.sieve(coeffs, bound, first, last, square=square, plan="reference")
    digest = sum(oracle.mix_pair(x, y) for x, y in zip(a.tolist(), d.tolist())) % 2**64
    assert (len(a), digest) == (ref["survivors"], ref["digest"]), (coeffs[:2], bound, first, last)
    return ref


def test_dense_streaming_path(rpg, oracle, golden):
    ref = compare(rpg, oracle, golden["dense"]["coefficients"].split(), 5000, 1, 2)
    assert ref["survivors"] == 20002


def test_record_curve(rpg, oracle):
    compare(rpg, oracle, RECORD, 100_000, 1, 3000, batch=1000)


def test_c1_box(rpg, oracle, golden):
    compare(rpg, oracle, golden["c1"]["coefficients"].split(), 2000, 1, 2000, batch=499)


def test_square_denominators(rpg, oracle):
    compare(rpg, oracle, ["5", "-3", "0", "1"], 20000, 1, 4000, square=True)


def test_random_large_coefficients(rpg, oracle):
    rng = random.Random(37)
    coeffs = [str(rng.randint(-(2**128), 2**128)) for _ in range(11)]
    compare(rpg, oracle, coeffs, 30000, 100, 1100)


def test_c2_sample(rpg, oracle):
    import bench
    compare(rpg, oracle, bench.c2_curve(), 5_000_000, 1, 2048)


def test_c2_full_box(rpg, oracle):
    """The benchmark workload's whole box, a in [-5e6, 5e6], b in [1, 5e6]
    (5e13 sites): the reference kernels' survivor multiset equals this
    project's reference plan, and the command line's -v survivor count is the
    same number; the fast and reference plans print identical stdout."""
    import bench
    coeffs = bench.c2_curve()
    ref = compare(rpg, oracle, coeffs, 5_000_000, 1, 5_000_000)
    assert ref["survivors"] > 1000
    text = " ".join(coeffs)
    runs = {plan: rpg.cli([text, "5000000", "-v", "--sieve-plan", plan])
            for plan in ("reference", "fast")}
    for plan, result in runs.items():
        assert result.returncode == 0, (plan, result.stderr)
    assert runs["fast"].stdout == runs["reference"].stdout
    ref_metrics = rpg.parse_metrics(runs["reference"].stderr)
    fast_metrics = rpg.parse_metrics(runs["fast"].stderr)
    assert ref_metrics["survivors"] == ref["survivors"]
    assert ref_metrics["exact_survivors"] == fast_metrics["exact_survivors"]
    assert ref_metrics["denominators"] == fast_metrics["denominators"] == 5_000_000


def test_record_curve_at_full_height(rpg, oracle):
    # the record curve at its published height 10^7 (a dense curve: the
    # reference's fast launch overflows and its streaming rerun runs)
    compare(rpg, oracle, RECORD, 10_000_000, 1, 6000, batch=3000)


def planted_c2_curve(rpg, seed=77):
    """A squarefree curve of the benchmark's shape (degree 6, coefficients in
    [-2^32, 2^32)) with c0 chosen so that F(1, 1) = sum(c) is a square y^2:
    (1 : y : 1) is a point."""
    import math
    rng = random.Random(seed)
    while True:
        c = [rng.randrange(-(2**32), 2**32) for _ in range(7)]
        rest = sum(c[1:])
        y = math.isqrt(max(0, rest + 2**31))
        c[0] = y * y - rest
        if -(2**32) <= c[0] < 2**32 and c[6] != 0 and rpg.is_squarefree([str(v) for v in c]):
            return [str(v) for v in c], y


def test_c2_shape_with_points_full_box(rpg, oracle):
    """A curve of the benchmark's shape that has points, over the benchmark's
    whole box: the reference kernels' survivor multiset equals the reference
    plan's, both plans print the same non-empty stdout, and every printed
    point satisfies y^2 = F(a, b) exactly."""
    coeffs, y1 = planted_c2_curve(rpg)
    ref = compare(rpg, oracle, coeffs, 5_000_000, 1, 5_000_000)
    text = " ".join(coeffs)
    runs = {plan: rpg.cli([text, "5000000", "--sieve-plan", plan, "-i"]) for plan in ("reference", "fast")}
    assert runs["fast"].returncode == 0 and runs["reference"].returncode == 0
    assert runs["fast"].stdout == runs["reference"].stdout
    lines = runs["fast"].stdout.decode().splitlines()
    assert f"(1 : {y1} : 1)" in lines
    c = [int(v) for v in coeffs]
    for line in lines:
        a, y, b = (int(t) for t in line.strip("()").split(" : "))
        F = sum(ci * a**i * b**(6 - i) for i, ci in enumerate(c))
        assert y * y == F
    assert ref["survivors"] >= len(lines) // 2
