"""The fast plan's extra filters hold for every point (host only, exact
integers): a site they drop can never be a point, so the fast plan finds the
reference plan's points.

- Denominator primes: for even degree, p | d, p odd and c_n a nonzero
  non-square mod p give F(a, d) = c_n a^n (mod p) with gcd(a, d) = 1, a
  non-square mod p: no site of such a denominator is a point.
- Class prime residues: for q | d the class layout keeps a numerator only
  when c_n is a square mod q (even degree).
"""

import math
import random


def homogeneous(coeffs, a, d):
    n = len(coeffs) - 1
    value = sum(c * a ** i * d ** (n - i) for i, c in enumerate(coeffs))
    return value * d if n % 2 else value


def is_square(v):
    return v >= 0 and math.isqrt(v) ** 2 == v


def odd_primes(limit):
    return [p for p in range(3, limit, 2) if all(p % f for f in range(3, math.isqrt(p) + 1, 2))]


def denominator_primes(coeffs):
    lead = coeffs[-1]
    if (len(coeffs) - 1) % 2:
        return []
    return [p for p in odd_primes(512) if lead % p and pow(lead % p, (p - 1) // 2, p) == p - 1]


def test_denominator_primes_leave_no_square():
    rng = random.Random(20261204)
    checked = 0
    for _ in range(60):
        degree = rng.choice([2, 4, 6, 8])
        coeffs = [rng.randint(-10 ** 6, 10 ** 6) for _ in range(degree + 1)]
        if coeffs[-1] == 0:
            coeffs[-1] = 3
        bad = denominator_primes(coeffs)
        for p in bad[:6]:
            for _ in range(40):
                d = p * rng.randint(1, 2000)
                a = rng.randint(-10 ** 7, 10 ** 7)
                if math.gcd(a, d) != 1:
                    continue
                v = homogeneous(coeffs, a, d)
                assert v % p and not is_square(v), (coeffs, a, d, p)
                checked += 1
    assert checked > 1000


def test_points_of_a_curve_avoid_its_denominator_primes():
    # y^2 = 2 x^4 - 1 (c_4 = 2: a non-square mod 3, 5, 11, 13, 19, ...) has
    # the points x = +-1 and x = +-13 (2 13^4 - 1 = 239^2); every denominator
    # of a point found by brute force is free of those primes
    coeffs = [-1, 0, 0, 0, 2]
    bad = denominator_primes(coeffs)
    assert 3 in bad and 5 in bad and 7 not in bad
    found = []
    for d in range(1, 400):
        for a in range(-2000, 2001):
            if math.gcd(a, d) == 1 and is_square(homogeneous(coeffs, a, d)):
                found.append((a, d))
    assert (1, 1) in found and len(found) >= 4
    assert all(d % p for _, d in found for p in bad)


def test_class_prime_rule_for_divisible_denominators():
    # q | d: F(a, d) = c_n a^n (mod q), a square mod q exactly when c_n is
    # (even degree, q !| a): the class layout's residue rule for q | d
    rng = random.Random(7)
    for _ in range(200):
        q = rng.choice([3, 5, 7, 11, 13])
        coeffs = [rng.randint(-500, 500) for _ in range(rng.choice([2, 4, 6]) + 1)]
        if coeffs[-1] % q == 0:
            coeffs[-1] += 1
        d = q * rng.randint(1, 50)
        a = rng.randint(1, 10 ** 5)
        if math.gcd(a, d) != 1:
            continue
        residue = homogeneous(coeffs, a, d) % q
        lead_square = pow(coeffs[-1] % q, (q - 1) // 2, q) == 1
        assert (pow(residue, (q - 1) // 2, q) == 1) == lead_square
