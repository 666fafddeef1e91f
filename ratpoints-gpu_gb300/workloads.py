"""Seeded synthetic workloads of the search's benchmark configurations.

All curves are squarefree integer polynomials written as decimal coefficient
lists c0 .. cn; sizes and distributions follow the benchmark definitions:

  single_curve   degree 6, coefficients uniform in [-2^32, 2^32), one box
  mixed_batch    many curves: degree uniform in {3, 4, 5, 6, 8, 10}, each
                 coefficient a random sign times a random integer of bit length
                 uniform in [8, 64]; numerator bound A and denominator bound B
                 independent, each log-uniform in [10^3, 10^6]
  wide_degree    degree uniform in 12..40, coefficients of bit length uniform
                 in [100, 256] with a random sign, box A = B = 10^5, x in a
                 union of 3 random closed intervals (lower bound uniform in
                 [-4, 4], length uniform in [0.05, 1], four decimals)
  square_cubics  x^3 + alpha x + beta with alpha, beta uniform in [-10^12, 10^12],
                 square denominators k^2 for k in [1, 46340], |a| <= 10^9
  serving_stream Poisson arrivals (200 per second): degree uniform in 2..12,
                 coefficient bit length uniform in [16, 128] with a random sign,
                 box a in [-H, H], b in [1, H] with H log-uniform in [10^2, 10^6],
                 30 % asking for the first point only
  RECORD_CURVE   the genus-2 curve with the most known rational points (its
                 points are the reference's known-answer test,
                 tests/verify_record_curve.py): a dense curve, square modulo
                 most small primes
"""

from __future__ import annotations

import math
import random

import numpy as np


RECORD_CURVE = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800"


def _squarefree(coeffs):
    import ratpoints_gb300 as rpg

    return rpg.is_squarefree(coeffs)


def single_curve(seed=5_000_000):
    """Degree-6 curve, coefficients uniform in [-2^32, 2^32)."""
    rng = random.Random(seed)
    while True:
        coeffs = [str(rng.randrange(-(2**32), 2**32)) for _ in range(7)]
        if coeffs[-1] != "0" and _squarefree(coeffs):
            return coeffs


def _log_uniform(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def mixed_batch(count=4096, seed=3, degrees=(3, 4, 5, 6, 8, 10), bits=(8, 64),
                heights=(10**3, 10**6), denominators=(10**3, 10**6)):
    """[{coefficients, bound, first, last}] for the mixed many-curve batch."""
    rng = random.Random(seed)
    curves = []
    while len(curves) < count:
        coeffs = _random_coefficients(rng, rng.choice(degrees), bits)
        if not _squarefree(coeffs):
            continue
        curves.append({"coefficients": coeffs, "bound": _log_uniform(rng, *heights),
                       "first": 1, "last": _log_uniform(rng, *denominators)})
    return curves


def _random_coefficients(rng, degree, bits):
    coeffs = []
    for _ in range(degree + 1):
        b = rng.randint(*bits)
        value = rng.getrandbits(b) | (1 << (b - 1))
        coeffs.append(str(rng.choice((-1, 1)) * value))
    return coeffs


def wide_degree(count=256, seed=11, bound=10**5):
    """[{coefficients, bound, first, last, intervals}] of high degree with big coefficients."""
    rng = random.Random(seed)
    curves = []
    while len(curves) < count:
        coeffs = _random_coefficients(rng, rng.randint(12, 40), (100, 256))
        if not _squarefree(coeffs):
            continue
        intervals = []
        for _ in range(3):
            lo = rng.uniform(-4, 4)
            intervals.append((f"{lo:.4f}", f"{lo + rng.uniform(0.05, 1):.4f}"))
        curves.append({"coefficients": coeffs, "bound": bound, "first": 1, "last": bound,
                       "intervals": intervals})
    return curves


def square_cubics(count=256, seed=13, bound=10**9, last=46340):
    """[{coefficients, bound, first, last, square}]: x^3 + alpha x + beta, square denominators."""
    rng = random.Random(seed)
    curves = []
    while len(curves) < count:
        alpha, beta = rng.randint(-10**12, 10**12), rng.randint(-10**12, 10**12)
        coeffs = [str(beta), str(alpha), "0", "1"]
        if not _squarefree(coeffs):
            continue
        curves.append({"coefficients": coeffs, "bound": bound, "first": 1, "last": last,
                       "square": True})
    return curves


def serving_stream(count=1000, rate=200.0, seed=5, first_fraction=0.3):
    """[(arrival seconds, request dict, first_point_only)] of a Poisson stream."""
    rng = random.Random(seed)
    t = 0.0
    stream = []
    while len(stream) < count:
        coeffs = _random_coefficients(rng, rng.randint(2, 12), (16, 128))
        if not _squarefree(coeffs):
            continue
        t += rng.expovariate(rate)
        h = _log_uniform(rng, 10**2, 10**6)
        stream.append((t, {"coefficients": coeffs, "bound": h, "first": 1, "last": h},
                       rng.random() < first_fraction))
    return stream


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


def reduced_sites(height, first, last, mu):
    """#{(a, b): |a| <= height, first <= b <= last, gcd(a, b) = 1}: the
    difference of sum_d mu(d) floor(N/d) (2 floor(height/d) + 1) at N = last
    and N = first - 1."""
    def upto(n):
        if n <= 0:
            return 0
        d = np.arange(1, n + 1, dtype=np.int64)
        return int((mu[1:n + 1].astype(np.int64) * (n // d) * (2 * (height // d) + 1)).sum())

    return upto(last) - upto(first - 1)
