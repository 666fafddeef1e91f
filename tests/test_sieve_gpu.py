"""Device sieve parity through the C ABI (rpg_sieve_run) against the oracle.

Reference plan: the delivered survivor set must equal the oracle's restatement
of the reference sieve exactly (same pairs, unreduced included, no duplicates).
"""

import math
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INT_MAX = 2**31 - 1


def pairs(a, d):
    """(a, d) pairs in the oracle's order: d ascending, then a."""
    return sorted(zip(a.tolist(), d.tolist()), key=lambda t: (t[1], t[0]))


def assert_same_set(rpg, oracle, coeffs, bound, first, last, square=False, plan="reference"):
    a, d, stats = rpg.sieve(coeffs, bound, first, last, square=square, plan=plan)
    got = pairs(a, d)
    assert len(got) == len(set(got)), "duplicate survivors"
    sieve = oracle.ModularSieve(coeffs, bound)
    expected = sieve.survivors(first, last, square)
    sieve.close()
    assert got == expected, (coeffs, bound, first, last, square)
    assert stats["survivor_count"] == len(expected)
    return got


def test_golden_boxes(rpg, oracle, golden):
    for case in golden["oracle_cases"]:
        coeffs = case["coefficients"].split()
        assert_same_set(rpg, oracle, coeffs, case["height"], case["first"],
                        min(case["last"], case["height"]))


def test_dense_stream_is_complete(rpg, golden):
    # tests/test_sieve_streaming.cpp:45-81: every site once, nothing outside the box.
    dense = golden["dense"]
    a, d, stats = rpg.sieve(dense["coefficients"].split(), 5000, 1, 2)
    assert len(a) == 20002 == stats["survivor_count"]
    assert a.min() >= -5000 and a.max() <= 5000 and set(d.tolist()) == {1, 2}
    keys = (d.astype(np.int64) - 1) * 10001 + (a + 5000)
    assert len(np.unique(keys)) == 20002


def test_dense_stream_through_small_buffers(rpg, golden, monkeypatch):
    # Overflowing launches are split (by denominator, then by word range) and re-run.
    dense = golden["dense"]
    monkeypatch.setenv("RPG_SURVIVOR_CAPACITY", "1000")
    a, d, stats = rpg.sieve(dense["coefficients"].split(), 5000, 1, 2)
    keys = (d.astype(np.int64) - 1) * 10001 + (a + 5000)
    assert len(a) == 20002 and len(np.unique(keys)) == 20002


@pytest.mark.parametrize("bound", [1, 2, 31, 32, 63, 64, 65, 95, 96, 97, 127, 128, 1000, 4096])
def test_last_word_clipping(rpg, oracle, bound):
    # sites end exactly at +H for every H mod 64 (src/sieve.cu:324-330)
    assert_same_set(rpg, oracle, ["1", "3", "0", "-7", "2"], bound, 1, 40)


def test_random_curves(rpg, oracle):
    rng = random.Random(23)
    for _ in range(12):
        degree = rng.choice([1, 2, 3, 4, 5, 6, 8, 10])
        bits = rng.choice([4, 16, 40, 120])
        coeffs = [str(rng.randint(-(2**bits), 2**bits)) for _ in range(degree + 1)]
        if coeffs[-1] == "0":
            coeffs[-1] = "5"
        bound = rng.choice([50, 700, 3000, 20000])
        first = rng.randint(1, 500)
        assert_same_set(rpg, oracle, coeffs, bound, first, first + rng.randint(0, 60))


def test_denominators_with_candidate_factors(rpg, oracle):
    # d divisible by up to three candidate primes: the selection skips them
    coeffs = ["2", "1", "0", "-3", "0", "1", "1"]
    for d in (509, 503 * 509, 499 * 503 * 509, 293 * 307):
        assert_same_set(rpg, oracle, coeffs, 400, d, d + 2)


def test_int_max_endpoint(rpg, oracle):
    assert_same_set(rpg, oracle, ["1", "0", "1"], 3000, INT_MAX - 40, INT_MAX)


def test_square_denominators(rpg, oracle, golden):
    assert_same_set(rpg, oracle, ["1", "-1", "0", "1"], 10, 1, 3, square=True)
    assert_same_set(rpg, oracle, ["5", "-3", "0", "1"], 5000, 1, 300, square=True)
    assert_same_set(rpg, oracle, ["1", "0", "1"], 100, 46300, 46340, square=True)


def test_large_bound_few_denominators(rpg, oracle):
    # long rows: many CTA steps per denominator
    assert_same_set(rpg, oracle, ["3", "-1", "4", "1", "-5", "9", "2"], 3_000_000, 1, 3)


def test_large_coefficients(rpg, oracle):
    rng = random.Random(29)
    coeffs = [str(rng.randint(-(2**256), 2**256)) for _ in range(41)]
    assert_same_set(rpg, oracle, coeffs, 5000, 1, 30)


def test_survivor_count_matches_oracle_at_scale(rpg, oracle):
    """Size-independent property: count and order-free digest over a larger box."""
    coeffs = ["247747600", "-985905640", "567207969", "2396040466", "52485681", "-470135160",
              "82342800"]
    a, d, _ = rpg.sieve(coeffs, 200_000, 1, 2000)
    sieve = oracle.ModularSieve(coeffs, 200_000)
    n, digest = sieve.count(1, 2000, threads=8)
    sieve.close()
    assert len(a) == n
    got = sum(oracle.mix_pair(x, y) for x, y in zip(a.tolist(), d.tolist())) % 2**64
    assert got == digest


def test_errors_are_reported(rpg):
    with pytest.raises(rpg.RpgError) as info:
        rpg.sieve(["1", "0", "1"], 10, 5, 4)
    assert info.value.status == 1
    with pytest.raises(rpg.RpgError):
        rpg.sieve(["1", "0", "1"], 10, 1, 50000, square=True)
