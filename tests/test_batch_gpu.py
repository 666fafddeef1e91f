"""Batched many-curve search: each curve's points are exactly the points of a
single-curve search of that curve (same order, infinity first), for curves on
the narrow (dense, warp per denominator) and the wide (class layout, CTA per
denominator) kernels, with and without the CUDA graph, with intervals, square
denominators, a first-point stop, failing curves in the mix, and a survivor
buffer too small for the first pass."""

import random

import pytest

pytestmark = pytest.mark.gpu


def random_curve(rng, degree, bits):
    while True:
        c = [str(rng.choice((-1, 1)) * rng.getrandbits(rng.randint(1, bits))) for _ in range(degree + 1)]
        if c[-1] == "0":
            c[-1] = "3"
        yield c


def mixed_curves(rng, n, heights, dens, degrees=(3, 4, 5, 6, 8, 10), bits=64):
    curves = []
    for _ in range(n):
        degree = rng.choice(degrees)
        coeffs = next(random_curve(rng, degree, rng.randint(min(8, bits), bits)))
        curves.append({"coefficients": coeffs, "bound": rng.randint(*heights),
                       "first": 1, "last": rng.randint(*dens)})
    return curves


def single(rpg, c, **kw):
    points, _ = rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"],
                                 intervals=c.get("intervals", ()),
                                 include_infinity=c.get("include_infinity", True),
                                 square=c.get("square", False), **kw)
    return points


def squarefree(rpg, curves):
    return [c for c in curves if rpg.is_squarefree(c["coefficients"])]


def test_batch_matches_oracle_small_boxes(rpg, oracle, golden):
    curves = [{"coefficients": golden["dense"]["coefficients"].split(), "bound": 300,
               "first": 1, "last": 40}]
    rng = random.Random(7)
    for _ in range(8):
        degree = rng.choice([1, 2, 3, 4, 5, 6])
        coeffs = [str(rng.randint(-20, 20)) for _ in range(degree + 1)]
        if coeffs[-1] == "0":
            coeffs[-1] = "1"
        curves.append({"coefficients": coeffs, "bound": rng.choice([30, 200, 700]),
                       "first": rng.randint(1, 20), "last": rng.randint(20, 60)})
    curves = squarefree(rpg, curves)
    points, status, _, stats = rpg.batch_search(curves)
    assert all(s == 0 for s in status)
    for c, got in zip(curves, points):
        expected = []
        o = oracle.Options(coefficients=c["coefficients"], height=c["bound"], first=c["first"],
                           last=c["last"])
        oracle.search(o, lambda a, y, d: expected.append((a, int(y), d)) or True)
        assert got == expected, c
    assert stats["curves"] == len(curves)


def test_batch_matches_single_search_mixed(rpg):
    rng = random.Random(2024)
    curves = mixed_curves(rng, 48, (100, 20000), (1, 3000))
    # wide rows (>= 2048 words of 64 numerators) with a few denominators each
    curves += mixed_curves(rng, 12, (70000, 400000), (1, 60))
    curves = squarefree(rpg, curves)
    points, status, survivors, stats = rpg.batch_search(curves)
    assert stats["wide_curves"] >= 6 and stats["curves"] - stats["wide_curves"] >= 20
    assert stats["graph"] == 1
    for c, got, s, n in zip(curves, points, status, survivors):
        assert s == 0
        assert got == single(rpg, c), c
        assert n >= sum(1 for p in got if p[2] != 0)


def test_batch_small_coefficients_many_points(rpg, golden):
    """Curves with many points on both kernels."""
    dense = golden["dense"]["coefficients"].split()
    curves = [{"coefficients": dense, "bound": b, "first": 1, "last": last}
              for b, last in ((1000, 500), (5000, 50), (150000, 12), (300000, 3))]
    rng = random.Random(5)
    for _ in range(10):
        coeffs = [str(rng.randint(-3, 3)) for _ in range(rng.choice([3, 4, 5, 6]) + 1)]
        coeffs[-1] = str(rng.choice([1, 4, 9]))
        curves.append({"coefficients": coeffs, "bound": rng.choice([500, 3000, 100000]),
                       "first": 1, "last": rng.choice([20, 200])})
    curves = squarefree(rpg, curves)
    points, status, _, stats = rpg.batch_search(curves)
    assert sum(len(p) for p in points) > 30
    for c, got in zip(curves, points):
        assert got == single(rpg, c), c


def test_graph_and_direct_launch_agree(rpg):
    rng = random.Random(99)
    curves = squarefree(rpg, mixed_curves(rng, 24, (50, 100000), (1, 400)))
    a = rpg.batch_search(curves, graph=True)
    b = rpg.batch_search(curves, graph=False)
    assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
    assert a[3]["graph"] == 1 and b[3]["graph"] == 0


def test_intervals_square_denominators_and_infinity(rpg, golden):
    dense = golden["dense"]["coefficients"].split()
    curves = [
        {"coefficients": dense, "bound": 4000, "first": 1, "last": 300,
         "intervals": [("-1.5", "-0.25"), ("0.5", "2e0")]},
        {"coefficients": dense, "bound": 200000, "first": 1, "last": 8,
         "intervals": [(None, "-3"), ("0.5", None)]},
        {"coefficients": dense, "bound": 3000, "first": 1, "last": 60, "square": True},
        {"coefficients": ["1", "0", "0", "1"], "bound": 100000, "first": 1, "last": 30,
         "square": True},
        {"coefficients": dense, "bound": 500, "first": 5, "last": 90, "include_infinity": False},
    ]
    points, status, _, _ = rpg.batch_search(curves)
    assert status == [0] * len(curves)
    for c, got in zip(curves, points):
        assert got == single(rpg, c), c


def test_failing_curves_do_not_disturb_the_rest(rpg, golden):
    dense = golden["dense"]["coefficients"].split()
    curves = [
        {"coefficients": dense, "bound": 800, "first": 1, "last": 50},
        {"coefficients": ["1", "2", "1"], "bound": 100, "first": 1, "last": 10},   # (x+1)^2
        {"coefficients": dense, "bound": 800, "first": 9, "last": 3},              # empty range
        {"coefficients": ["1", "x", "2"], "bound": 100, "first": 1, "last": 10},   # not an integer
        {"coefficients": dense, "bound": 90000, "first": 1, "last": 5},
    ]
    points, status, _, _ = rpg.batch_search(curves)
    assert status == [0, 6, 1, 1, 0]
    assert points[1] == points[2] == points[3] == []
    assert points[0] == single(rpg, curves[0])
    assert points[4] == single(rpg, curves[4])


def test_first_point_stop(rpg):
    rng = random.Random(3)
    curves = squarefree(rpg, mixed_curves(rng, 16, (100, 5000), (1, 200), bits=6))
    points, _, _, _ = rpg.batch_search(curves, stop_after=1)
    for c, got in zip(curves, points):
        assert got == single(rpg, c, stop_after=1)


def test_survivor_overflow_rerun(rpg, golden, monkeypatch):
    dense = golden["dense"]["coefficients"].split()
    curves = [{"coefficients": dense, "bound": 5000, "first": 1, "last": 100},
              {"coefficients": dense, "bound": 100000, "first": 1, "last": 6}]
    full, _, surv_full, _ = rpg.batch_search(curves)
    monkeypatch.setenv("RPG_BATCH_CAPACITY", "16")
    small, _, surv_small, stats = rpg.batch_search(curves)
    assert small == full and surv_small == surv_full
    assert stats["survivors"] > 16


def _decimal(a, d):
    """a/d as an exact decimal string when d divides a power of ten, else None."""
    k = 0
    while (10**k) % d and k < 12:
        k += 1
    if (10**k) % d:
        return None
    n = a * (10**k // d)
    sign = "-" if n < 0 else ""
    digits = str(abs(n)).rjust(k + 1, "0")
    return sign + (digits[:-k] + "." + digits[-k:] if k else digits)


def test_interval_narrowing_matches_single_search(rpg, golden):
    """Each denominator sweeps only the numerators of the x intervals: random
    unions of intervals, exact one-point intervals at known points, infinite
    and huge-exponent bounds, overlapping and unsorted intervals, and more
    intervals than the device narrows (whole rows, host filter only)."""
    dense = golden["dense"]["coefficients"].split()
    mordell = ["17", "0", "0", "1"]  # y^2 = x^3 + 17: many points with small denominators
    rng = random.Random(17)
    known = [p for p in single(rpg, {"coefficients": mordell, "bound": 6000, "first": 1, "last": 400})
             if p[2] != 0]
    exact = [s for s in (_decimal(a, d) for a, _, d in known) if s is not None]
    assert len(exact) >= 4
    curves = []
    for bound, last in ((6000, 400), (150000, 10)):
        curves.append({"coefficients": mordell, "bound": bound, "first": 1, "last": last,
                       "intervals": [(x, x) for x in exact[:4]]})
        curves.append({"coefficients": dense, "bound": bound, "first": 1, "last": last,
                       "intervals": [(None, "-2.5"), ("-3", "-1e0"), ("4e-1", "1e400"),
                                     ("-1e-400", "0")]})
        curves.append({"coefficients": dense, "bound": bound, "first": 1, "last": last,
                       "intervals": [(str(-i - 0.5), str(-i)) for i in range(10)]})
    # narrowed rows still long enough for the class-layout kernel
    for c in mixed_curves(rng, 4, (300000, 500000), (20, 60), bits=10):
        lo = rng.uniform(-9000, -5000)
        c["intervals"] = [(f"{lo:.2f}", f"{lo + 4000:.2f}"), ("15.5", f"{rng.uniform(6000, 9000):.3f}")]
        curves.append(c)
    for _ in range(24):
        c = mixed_curves(rng, 1, (200, 120000), (1, 300), bits=10)[0]
        ivs = []
        for _ in range(3):
            lo = rng.uniform(-8, 8)
            ivs.append((f"{lo:.4f}", f"{lo + rng.uniform(0, 3):.4f}"))
        c["intervals"] = ivs
        curves.append(c)
    curves = squarefree(rpg, curves)
    points, status, survivors, stats = rpg.batch_search(curves)
    assert all(s == 0 for s in status)
    assert stats["wide_curves"] >= 5 and stats["curves"] - stats["wide_curves"] >= 20
    for c, got in zip(curves, points):
        assert got == single(rpg, c), c
    full, _, full_survivors, _ = rpg.batch_search([dict(c, intervals=()) for c in curves[:2]])
    # one-point intervals sweep a few numerators per denominator: what survives
    # there is the points themselves and their unreduced multiples
    assert survivors[0] < full_survivors[0] and survivors[1] < full_survivors[1]


def test_huge_rows_searched_alone(rpg, golden):
    # numerator bounds above 2^17 words of 64 numerators go to the single-curve
    # kernel beside the batched ones; answers stay those of a single search
    rng = random.Random(21)
    curves = [{"coefficients": ["1", "-1", "0", "1"], "bound": 10 ** 7, "first": 1, "last": 300},
              {"coefficients": golden["record_curve"]["coefficients"].split(), "bound": 5 * 10 ** 6,
               "first": 2, "last": 120, "intervals": [(None, "-0.3333"), ("0.5", "7")]},
              {"coefficients": ["-2", "0", "1", "0", "1"], "bound": 9 * 10 ** 6, "first": 1, "last": 40,
               "square": True, "include_infinity": False}]
    curves += squarefree(rpg, mixed_curves(rng, 12, (100, 100000), (10, 400)))
    points, status, survivors, stats = rpg.batch_search(curves)
    assert all(s == 0 for s in status)
    assert stats["curves"] == len(curves)
    for c, got, n in zip(curves, points, survivors):
        expected, st = rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"],
                                        intervals=c.get("intervals", ()),
                                        include_infinity=c.get("include_infinity", True),
                                        square=c.get("square", False))
        assert got == expected, c["bound"]
    assert points[0] and points[1]


def test_survivor_counts_repeat(rpg):
    # work is handed out dynamically, so warps see the denominators in a
    # different order each run; survivors per curve must not depend on it
    rng = random.Random(77)
    curves = squarefree(rpg, mixed_curves(rng, 48, (50, 300000), (5, 2000), bits=24))
    first = rpg.batch_search(curves, preverify=False)
    for _ in range(2):
        again = rpg.batch_search(curves, preverify=False)
        assert again[2] == first[2]
        assert again[0] == first[0]


def _oracle_points(oracle, c):
    from fractions import Fraction

    ivs = [oracle.Interval(None if lo is None else Fraction(lo), None if hi is None else Fraction(hi))
           for lo, hi in c.get("intervals", ())]
    o = oracle.Options(coefficients=list(c["coefficients"]), height=c["bound"], first=c["first"],
                       last=c["last"], intervals=ivs,
                       include_infinity=c.get("include_infinity", True),
                       square=c.get("square", False))
    expected = []
    oracle.search(o, lambda a, y, d: expected.append((a, int(y), d)) or True)
    return expected


def test_wide_kernel_matches_oracle(rpg, oracle):
    """Curves whose rows have at least 2,048 words of 64 numerators (bound >=
    65,504) go to the class-layout wide kernel; each curve's points must equal
    the oracle's restatement of the reference pipeline (its 32-prime sieve and
    exact verification), with x intervals, square denominators and a first
    denominator above 1 in the mix."""
    mordell = ["17", "0", "0", "1"]          # y^2 = x^3 + 17
    cubic = ["1", "0", "0", "1"]             # y^2 = x^3 + 1
    curves = [
        {"coefficients": mordell, "bound": 70000, "first": 1, "last": 6},
        {"coefficients": mordell, "bound": 100000, "first": 2, "last": 5,
         "intervals": [("-3", "-1"), ("0.5", "5e1")]},
        {"coefficients": cubic, "bound": 90000, "first": 1, "last": 4, "square": True},
        {"coefficients": ["-2", "0", "1", "0", "1"], "bound": 66000, "first": 1, "last": 6,
         "square": True, "include_infinity": False},
    ]
    rng = random.Random(4242)
    while len(curves) < 12:
        degree = rng.choice([3, 4, 5, 6, 8])
        coeffs = [str(rng.randint(-9, 9)) for _ in range(degree + 1)]
        coeffs[-1] = str(rng.choice([1, 4, 9, -1]))
        c = {"coefficients": coeffs, "bound": rng.randint(65504, 160000), "first": 1,
             "last": rng.randint(2, 5)}
        if rng.random() < 0.4:
            lo = rng.uniform(-6, 2)
            c["intervals"] = [(f"{lo:.3f}", f"{lo + rng.uniform(0.5, 4):.3f}")]
        if rpg.is_squarefree(coeffs):
            curves.append(c)
    points, status, _, stats = rpg.batch_search(curves)
    assert status == [0] * len(curves)
    # x intervals narrow a curve's rows, which can send it to the narrow kernel
    assert stats["wide_curves"] >= sum(1 for c in curves if not c.get("intervals"))
    found = 0
    for c, got in zip(curves, points):
        expected = _oracle_points(oracle, c)
        assert got == expected, c
        found += len(expected)
    assert found >= 20


def test_denominator_primes_batch(rpg, oracle):
    """Even-degree curves whose leading coefficient is a non-square mod some
    small primes (c_6 = 3: 5, 7, 17; c_4 = -1: 3, 7, 11, 19): both batch
    kernels skip the denominators divisible by one, which hold no points;
    every curve's points equal the oracle's restatement of the reference
    pipeline."""
    sextic = ["9", "1", "0", "-3", "0", "1", "3"]
    quartic = ["4", "0", "-5", "0", "-1"]
    curves = [
        {"coefficients": sextic, "bound": 70000, "first": 1, "last": 40},
        {"coefficients": sextic, "bound": 3000, "first": 1, "last": 400},
        {"coefficients": quartic, "bound": 5000, "first": 1, "last": 300},
        {"coefficients": quartic, "bound": 80000, "first": 1, "last": 30, "square": True},
    ]
    assert all(rpg.is_squarefree(c["coefficients"]) for c in curves)
    points, status, _, stats = rpg.batch_search(curves)
    assert status == [0] * len(curves)
    assert stats["wide_curves"] == 2
    for c, got in zip(curves, points):
        assert got == _oracle_points(oracle, c), c
        assert all(d % 7 for _, _, d in got if d)
