"""Seeded synthetic workloads of the search's benchmark configurations.

All curves are squarefree integer polynomials written as decimal coefficient
lists c0 .. cn; sizes and distributions follow the benchmark definitions:

  single_curve   degree 6, coefficients uniform in [-2^32, 2^32), one box
  mixed_batch    many curves: degree uniform in {3, 4, 5, 6, 8, 10}, each
                 coefficient a random sign times a random integer of bit length
                 uniform in [8, 64]; numerator bound A and denominator bound B
                 independent, each log-uniform in [10^3, 10^6]
"""

from __future__ import annotations

import math
import random

import numpy as np


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
        degree = rng.choice(degrees)
        coeffs = []
        for i in range(degree + 1):
            b = rng.randint(*bits)
            value = rng.getrandbits(b) | (1 << (b - 1))  # bit length exactly b
            coeffs.append(str(rng.choice((-1, 1)) * value))
        if not _squarefree(coeffs):
            continue
        curves.append({"coefficients": coeffs, "bound": _log_uniform(rng, *heights),
                       "first": 1, "last": _log_uniform(rng, *denominators)})
    return curves


def mobius(limit):
    mu = np.ones(limit + 1, dtype=np.int8)
    is_composite = np.zeros(limit + 1, dtype=bool)
    for p in range(2, limit + 1):
        if is_composite[p]:
            continue
        is_composite[p * p::p] = True
        mu[p::p] *= -1
        mu[p * p::p * p] = 0
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
