"""Fast plan parity: its survivor set is exactly the reference plan's survivor
set intersected with the extra filters the fast plan documents (2-adic
classes mod 64 with gcd parity; f(a/d) a square mod each small prime the
per-curve plan chose, or gcd and the leading-coefficient test when the prime
divides d; and, for even degree, no denominator divisible by a prime p < 512
mod which the leading coefficient is not a square).  Every extra filter holds
for every point, so the point sets are equal."""

import math
import random

import pytest

pytestmark = pytest.mark.gpu

def plan_primes(rpg, coeffs, bound):
    with rpg.Session(coeffs, bound, plan="fast") as session:
        class_prime, primes = session.plan()
    return sorted(set(primes) | ({class_prime} if class_prime > 1 else set()))


def fast_filter(coeffs, small_primes):
    c = [int(x) for x in coeffs]
    n = len(c) - 1
    squares64 = {v * v % 64 for v in range(64)}
    sq = {q: {v * v % q for v in range(q)} for q in small_primes}
    lead_ok = {q: (n % 2 == 1) or (c[-1] % q in sq[q]) for q in small_primes}
    # denominator primes: c_n a nonzero non-square mod p, even degree
    odd_primes = [p for p in range(3, 512, 2) if all(p % f for f in range(3, int(p ** 0.5) + 1, 2))]
    denominator_primes = [] if n % 2 else [
        p for p in odd_primes if c[-1] % p and pow(c[-1] % p, (p - 1) // 2, p) == p - 1]

    def F_mod(a, d, m):
        value = sum(ci * pow(a, i, m) * pow(d, n - i, m) for i, ci in enumerate(c)) % m
        return value * d % m if n % 2 else value

    def passes(a, d):
        if d % 2 == 0 and a % 2 == 0:
            return False
        if any(d % p == 0 for p in denominator_primes):
            return False
        if F_mod(a % 64, d % 64, 64) not in squares64:
            return False
        for q in small_primes:
            if d % q == 0:
                if a % q == 0 or not lead_ok[q]:
                    return False
            else:
                x = a * pow(d, -1, q) % q
                fx = sum(ci * pow(x, i, q) for i, ci in enumerate(c)) % q
                if fx not in sq[q]:
                    return False
        return True

    return passes


def check(rpg, oracle, coeffs, bound, first, last, square=False):
    a, d, _ = rpg.sieve(coeffs, bound, first, last, square=square, plan="fast")
    got = sorted(zip(a.tolist(), d.tolist()), key=lambda t: (t[1], t[0]))
    assert len(got) == len(set(got))
    sieve = oracle.ModularSieve(coeffs, bound)
    ref = sieve.survivors(first, last, square)
    sieve.close()
    passes = fast_filter(coeffs, plan_primes(rpg, coeffs, bound))
    expected = [(x, y) for x, y in ref if passes(x, y)]
    assert got == expected, (coeffs, bound, first, last, len(got), len(expected))
    return got


def test_dense_curve_fast_plan(rpg, oracle, golden):
    dense = golden["dense"]
    check(rpg, oracle, dense["coefficients"].split(), 5000, 1, 2)


def test_fast_plan_small_boxes(rpg, oracle):
    rng = random.Random(41)
    for _ in range(10):
        degree = rng.choice([1, 2, 3, 4, 5, 6, 8])
        coeffs = [str(rng.randint(-30, 30)) for _ in range(degree + 1)]
        if coeffs[-1] == "0":
            coeffs[-1] = "4"
        bound = rng.choice([40, 300, 2000, 4097])
        first = rng.randint(1, 300)
        check(rpg, oracle, coeffs, bound, first, first + rng.randint(0, 80))


@pytest.mark.parametrize("bound", [1, 2, 63, 64, 65, 4095, 4096, 4097, 8191, 70000])
def test_fast_plan_class_edges(rpg, oracle, bound):
    # class word boundaries: 64 classes x words of 64 sites spaced 64 apart
    check(rpg, oracle, ["1", "3", "0", "-7", "2"], bound, 1, 30)
    check(rpg, oracle, ["0", "1", "0", "1"], bound, 1, 20)


def test_fast_plan_square_denominators(rpg, oracle):
    check(rpg, oracle, ["1", "-1", "0", "1"], 10, 1, 3, square=True)
    check(rpg, oracle, ["5", "-3", "0", "1"], 3000, 1, 200, square=True)


def test_fast_plan_divisible_denominators(rpg, oracle):
    coeffs = ["9", "1", "0", "-3", "0", "1", "4"]
    for d in (105, 3 * 5 * 7 * 11 * 13, 17 * 19 * 23, 509 * 3, 64 * 105):
        check(rpg, oracle, coeffs, 2000, d, d + 3)


def test_fast_plan_denominator_primes(rpg, oracle):
    # c_6 = 3 is not a square mod 5, 7 or 17: no denominator divisible by
    # one of them keeps a survivor, and the rest match the reference plan
    coeffs = ["9", "1", "0", "-3", "0", "1", "3"]
    got = check(rpg, oracle, coeffs, 2000, 1, 140)
    assert got and all(d % 5 and d % 7 and d % 17 for _, d in got)
    assert {d for _, d in got} & {1, 2, 3, 4, 11, 13}
    got = check(rpg, oracle, coeffs, 3000, 1, 60, square=True)
    assert got and all(d % 5 and d % 7 for _, d in got)


def test_fast_plan_small_buffers(rpg, oracle, golden, monkeypatch):
    monkeypatch.setenv("RPG_SURVIVOR_CAPACITY", "64")
    dense = golden["dense"]
    check(rpg, oracle, dense["coefficients"].split(), 5000, 1, 2)


def test_plan_choice_for_the_benchmark_curve(rpg):
    import bench
    coeffs = bench.c2_curve()
    with rpg.Session(coeffs, 5_000_000, plan="fast") as session:
        class_prime, primes = session.plan()
    # strong small primes for this curve: 5, 7, 11 (f(x) mod 3 is always a square)
    assert class_prime in (5, 7, 11)
    assert 3 not in primes and 13 not in primes and class_prime not in primes
    assert 61 in primes


def test_fast_plan_large_height(rpg, oracle):
    # class prime in use (long classes), last-word clipping per class
    check(rpg, oracle, ["247747600", "-985905640", "567207969", "2396040466", "52485681",
                        "-470135160", "82342800"], 3_000_003, 1, 40)


def test_fast_plan_keeps_every_point(rpg, oracle):
    # record curve: every published point survives the fast plan
    coeffs = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800".split()
    a, d, _ = rpg.sieve(coeffs, 10**5, 1, 3000, plan="fast")
    survivors = set(zip(a.tolist(), d.tolist()))
    points = [(x, y) for x, y in survivors
              if math.gcd(x, y) == 1 and oracle.square_root(coeffs, x, y) is not None]
    ra, rd, _ = rpg.sieve(coeffs, 10**5, 1, 3000, plan="reference")
    ref_points = [(x, y) for x, y in zip(ra.tolist(), rd.tolist())
                  if math.gcd(x, y) == 1 and oracle.square_root(coeffs, x, y) is not None]
    assert sorted(points) == sorted(ref_points) and len(points) > 50
    assert len(survivors) < len(ra)
