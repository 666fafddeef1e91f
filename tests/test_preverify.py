"""Device pre-verification test, evaluated on the host through rpg_preverify
(the same code the kernel runs): every point passes it, and it rejects
almost every site that is not a point.  No GPU needed."""

import math
import random

import pytest


def F(coeffs, a, b):
    n = len(coeffs)
    value = sum(c * a ** i * b ** (n - 1 - i) for i, c in enumerate(coeffs))
    return value * b if n % 2 == 0 else value


def is_point(coeffs, a, b):
    if math.gcd(a, b) != 1:
        return False
    v = F(coeffs, a, b)
    return v >= 0 and math.isqrt(v) ** 2 == v


CURVES = [
    [1, 0, 1],
    [1, 1, 0, 1],
    [1, 0, 1, 0, 1],
    [-3, 5, -7, 11, 2],
    [247747600, -985905640, 567207969, 2396040466, 52485681, -470135160, 82342800],
    [4, -37, -48, 27, 34, -28, 49],
    [1, -1, 0, 1],
]


@pytest.mark.parametrize("coeffs", CURVES, ids=[str(len(c) - 1) + ":" + str(c[0]) for c in CURVES])
def test_points_pass_and_non_points_fail(rpg, coeffs):
    text = " ".join(map(str, coeffs))
    points = passed = sites = 0
    for b in range(1, 41):
        for a in range(-120, 121):
            keep = rpg.preverify(text, a, b)
            point = is_point(coeffs, a, b)
            assert keep or not point, (a, b)
            sites += 1
            points += point
            passed += keep
    # residue tests at 2^64 and 28 primes leave essentially nothing but points
    assert passed - points <= sites // 100000 + 1, (passed, points)


def test_square_denominators_and_large_values(rpg):
    # d = k^2 and numerators near 10^9: F far beyond 64 bits
    coeffs = [1, -1, 0, 1]
    text = "1 -1 0 1"
    rng = random.Random(7)
    for k in range(1, 60):
        d = k * k
        for a in [rng.randint(-10 ** 9, 10 ** 9) for _ in range(40)] + [-d, 0, d, 2 * d]:
            assert rpg.preverify(text, a, d) or not is_point(coeffs, a, d)
    # planted points: a = x d with F(x, 1) a square: (x, y) = (0, 1), (1, 1), (-1, 1), (3, 5) on y^2 = x^3 - x + 1
    for x in (0, 1, -1, 3):
        assert is_point(coeffs, x, 1) and rpg.preverify(text, x, 1)


def test_big_coefficients(rpg):
    rng = random.Random(11)
    for trial in range(6):
        coeffs = [rng.randint(-(2 ** 200), 2 ** 200) for _ in range(rng.randint(3, 9))]
        # make (a0, b0) a point: choose c0 so that F(a0, b0) = y0^2 with b0 = 1
        a0, y0 = rng.randint(-1000, 1000), rng.randint(0, 2 ** 120)
        coeffs[0] = 0
        coeffs[0] = y0 * y0 - F(coeffs, a0, 1)
        text = " ".join(map(str, coeffs))
        assert is_point(coeffs, a0, 1)
        assert rpg.preverify(text, a0, 1)
        rejected = 0
        for _ in range(200):
            a, b = rng.randint(-10 ** 6, 10 ** 6), rng.randint(1, 10 ** 6)
            keep = rpg.preverify(text, a, b)
            assert keep or not is_point(coeffs, a, b)
            rejected += not keep
        assert rejected >= 195


def test_two_adic_edge_cases(rpg):
    # F(a, b) = a^2 + b^2 ... values with high 2-adic valuation: (2^31 + k)^2 wraps mod 2^64
    text = "0 0 1"  # y^2 = x^2: F(a, b) = a^2 is a square for every a
    for a in [1, 2 ** 31, 2 ** 31 + 1, 2 ** 32, 3 * 2 ** 30, 2 ** 40 + 7, -(2 ** 33)]:
        assert rpg.preverify(text, a, 1)
    # y^2 = 2 x^2 has no points with a != 0 (odd valuation)
    assert not rpg.preverify("0 0 2", 2 ** 31, 1)
    assert not rpg.preverify("0 0 2", 5, 1)


def test_argument_errors(rpg):
    with pytest.raises(rpg.RpgError):
        rpg.preverify("1 0 1", 1, 0)
    with pytest.raises(rpg.RpgError):
        rpg.preverify("x", 1, 1)
