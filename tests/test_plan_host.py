"""The fast plan's autotuner on the host (rpg_fast_plan, no GPU): the plan
chosen for the C2 curve, rows of large primes for the dense record curve,
well-formed moduli, and no filter that a known point fails."""

from fractions import Fraction

import pytest

RECORD = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800"


def is_prime(n):
    return n > 1 and all(n % f for f in range(2, int(n ** 0.5) + 1))


def well_formed(plan):
    assert 1 <= len(plan["moduli"]) <= 12
    seen = set()
    for m, factors in zip(plan["moduli"], plan["factors"]):
        assert m <= 1500 and factors
        product = 1
        for q in factors:
            assert is_prime(q) and q % 2 == 1 and q < 512
            assert q not in seen and q != plan["class_prime"]
            seen.add(q)
            product *= q
        assert product == m
    assert plan["class_prime"] in (1, 3, 5, 7, 11, 13)


def test_c2_plan(rpg):
    import bench
    plan = rpg.fast_plan(bench.c2_curve(), 5_000_000)
    well_formed(plan)
    # rows of small-prime products; class prime 7: its classes sweep 18 of
    # the 49 residue pairs (d, r) mod 7 (3 residues for each d prime to 7,
    # none for 7 | d: c_6 is not a square mod 7), against 12 of 25 mod 5
    # (f mod 3 is always a square); three staged denominators per CTA cost
    # it no filtering (13.3 bits)
    assert plan["class_prime"] == 7
    assert 6 <= len(plan["moduli"]) <= 8 and plan["bits"] > 13
    assert plan["slots"] == 3
    assert all(q < 128 for f in plan["factors"] for q in f)
    assert 61 in [q for f in plan["factors"] for q in f]


def test_dense_curve_gets_large_prime_rows(rpg):
    plan = rpg.fast_plan(RECORD, 10 ** 7)
    well_formed(plan)
    assert plan["class_prime"] == 1
    assert len(plan["moduli"]) >= 10 and plan["bits"] > 11
    assert plan["slots"] == 2  # three slots would cost it 1.5 bits
    assert all(len(f) == 1 and f[0] > 128 for f in plan["factors"])


def test_known_points_pass_every_row(rpg, golden):
    # the record curve's published points survive each stage-1 prime of its plan
    plan = rpg.fast_plan(RECORD, 10 ** 6)
    coeffs = [int(c) for c in RECORD.split()]
    primes = [q for f in plan["factors"] for q in f]
    n = len(coeffs) - 1
    for text in golden["record_curve"]["x"][:120]:
        x = Fraction(text)
        a, b = x.numerator, x.denominator
        F = sum(c * a ** i * b ** (n - i) for i, c in enumerate(coeffs))
        for q in primes:
            assert pow(F % q, (q - 1) // 2, q) in (0, 1), (text, q)


@pytest.mark.parametrize("height", [10, 10 ** 3, 10 ** 9])
def test_small_and_large_heights(rpg, height):
    for coeffs in ("1 0 1", "1 -1 0 1", "-3 5 -7 11 2", RECORD):
        well_formed(rpg.fast_plan(coeffs, height))


def test_argument_errors(rpg):
    with pytest.raises(rpg.RpgError):
        rpg.fast_plan("1 0 1", 0)
    with pytest.raises(rpg.RpgError):
        rpg.fast_plan("x 1", 10)


def test_huge_rows_keep_two_slots(rpg):
    # rows of more than 2^20 words: sweeping a denominator outlasts copying
    # its rows, so the larger two-slot row budget (stronger moduli) is kept
    plan = rpg.fast_plan("-9876543210 1234567 0 1", 10 ** 9)
    well_formed(plan)
    assert plan["slots"] == 2


def test_plans_match_the_regression_fixture(rpg):
    # tests/golden/plans.json (tests/golden/make_plans.py): the autotuner's
    # decisions for 60 seeded curves; speed-ups of the planner keep them
    import json
    from pathlib import Path

    rows = json.loads((Path(__file__).parent / "golden" / "plans.json").read_text())
    assert len(rows) == 60
    for row in rows:
        plan = rpg.fast_plan(row["coefficients"], row["height"])
        want = row["plan"]
        assert (plan["class_prime"], plan["moduli"], plan["factors"], plan["slots"]) == \
            (want["class_prime"], want["moduli"], want["factors"], want["slots"]), row
        assert plan["bits"] == pytest.approx(want["bits"], abs=1e-9)


def test_class_prime_minimises_the_swept_share(rpg):
    # the planner's class prime, checked by brute force: of the primes 3..13
    # whose classes keep at least 256 words and at most 256 classes per
    # denominator, the one whose classes sweep the smallest share of the
    # residue pairs (d, r) mod q (q | d admits every r != 0 only when c_n is a
    # square mod q or the degree is odd), if that share is below 2^-0.45
    import random

    rng = random.Random(99)
    squares64 = {v * v % 64 for v in range(64)}
    chosen = 0
    for _ in range(40):
        degree = rng.choice([3, 4, 5, 6, 8])
        coeffs = [rng.randint(-10 ** 9, 10 ** 9) for _ in range(degree + 1)]
        if coeffs[-1] == 0:
            coeffs[-1] = 7
        height = rng.choice([10 ** 6, 5 * 10 ** 6, 2 * 10 ** 7])
        plan = rpg.fast_plan(" ".join(map(str, coeffs)), height)

        def f_mod(x, q):
            return sum(c * pow(x, i, q) for i, c in enumerate(coeffs)) % q

        worst2 = 0
        for dd in range(64):
            count = 0
            for r in range(64):
                if dd % 2 == 0 and r % 2 == 0:
                    continue
                v = sum(c * pow(r, i, 64) * pow(dd, degree - i, 64) for i, c in enumerate(coeffs)) % 64
                if degree % 2:
                    v = v * dd % 64
                count += v in squares64
            worst2 = max(worst2, count)
        shares = {}
        for q in (3, 5, 7, 11, 13):
            if (2 * height + 1) / (64 * 64 * q) < 256:
                continue
            sq = {v * v % q for v in range(q)}
            admitted = sum(f_mod(x, q) in sq for x in range(q))
            lead = degree % 2 == 1 or coeffs[-1] % q in sq
            divides = q - 1 if lead else 0
            if worst2 * max(admitted, divides) > 256:
                continue
            shares[q] = ((q - 1) * admitted + divides) / (q * q)
        best = min(shares.values(), default=1.0)
        if best < 2 ** -0.45:
            assert plan["class_prime"] in shares and shares[plan["class_prime"]] == pytest.approx(best), \
                (coeffs, height, shares, plan["class_prime"])
            chosen += 1
        else:
            assert plan["class_prime"] == 1, (coeffs, height, shares)
    assert chosen >= 10
