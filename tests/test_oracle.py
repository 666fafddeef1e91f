"""The oracle is pinned to the reference before anything is checked against it.

CPU only: the C restatement of the sieve plan and word sieve, the Python
restatement of exact verification, CLI parsing and formatting, against the
reference's own oracle outputs, known answers and boundary tests.
"""

import math
import random

import pytest

INT_MAX = 2**31 - 1


def test_candidate_primes_are_the_36_largest_below_512(oracle):
    # src/sieve_plan.cpp:83-100, 115-116
    primes = [p for p in range(2, 512) if all(p % q for q in range(2, math.isqrt(p) + 1))]
    assert oracle.candidate_primes() == primes[-36:]
    assert oracle.candidate_primes()[0] == 293 and oracle.candidate_primes()[-1] == 509


@pytest.mark.parametrize("first,last", [(1, 1), (65535, 65538), (INT_MAX - 2, INT_MAX)])
def test_selection_boundaries(oracle, first, last):
    # tests/test_sieve_plan.cpp:7-28: 32 primes per denominator, none divides it.
    for b in range(first, last + 1):
        chosen = oracle.selected_primes(b)
        assert len(chosen) == 32 and len(set(chosen)) == 32
        assert all(b % p for p in chosen)
        # largest-first among candidates that do not divide b
        expect = [p for p in reversed(oracle.candidate_primes()) if b % p][:32]
        assert chosen == expect


def test_selection_skips_divisors(oracle):
    d = 509 * 503 * 499  # three candidates divide d
    chosen = oracle.selected_primes(d)
    assert 509 not in chosen and 503 not in chosen and 499 not in chosen
    assert chosen[0] == 491


def test_mask_words_match_definition(oracle):
    # src/sieve.cu:141-172: bit j of word w (row r) = affine[((-H + 32w + j) r^-1) mod p]
    rng = random.Random(7)
    coeffs = ["3", "-5", "0", "7", "11", "-2", "9"]
    for bound in (1, 77, 10**6, 10**12 + 3):
        sieve = oracle.ModularSieve(coeffs, bound)
        primes = oracle.candidate_primes()
        for _ in range(40):
            i = rng.randrange(36)
            p = primes[i]
            r = rng.randrange(p)
            w = rng.randrange(10**6)
            word = sieve.mask_word(i, r, w)
            if r == 0:
                assert word == 0
                continue
            squares = {v * v % p for v in range(p)}
            inv = pow(r, -1, p)
            expect = 0
            for j in range(32):
                a = -bound + 32 * w + j
                x = a * inv % p
                fx = sum(int(c) * x**k for k, c in enumerate(coeffs)) % p
                if fx in squares:
                    expect |= 1 << j
            assert word == expect, (p, r, w)
        sieve.close()


def test_oracle_pipeline_matches_reference_oracle(oracle, golden):
    # tests/test_multi_gpu.py:17-40 evaluated by the reference itself.
    for case in golden["oracle_cases"]:
        argv = ["ratpoints_gpu", case["coefficients"], str(case["height"]),
                "-dl", str(case["first"]), "-du", str(case["last"])]
        code, out, err, _ = oracle.run(argv)
        assert code == 0, err
        assert out.decode() == case["stdout"], case["coefficients"]


def test_oracle_pipeline_with_small_batches(oracle, golden):
    case = golden["oracle_cases"][0]
    argv = ["ratpoints_gpu", case["coefficients"], str(case["height"]), "-dl",
            str(case["first"]), "-du", str(case["last"]), "--batch-size", "3"]
    assert oracle.run(argv)[1].decode() == case["stdout"]


def test_dense_known_answer(oracle, golden):
    # tests/test_multi_gpu.py:122-130: survivors=20002 exact_survivors=1
    dense = golden["dense"]
    argv = ["ratpoints_gpu", dense["coefficients"], "5000", "-du", "2", "-v"]
    code, out, _, metrics = oracle.run(argv)
    assert code == 0
    assert out.decode() == dense["stdout"]
    assert metrics["survivors"] == 20002 and metrics["exact_survivors"] == 1


def test_square_denominator_known_answer(oracle, golden):
    kat = golden["square_kat"]
    code, out, _, _ = oracle.run(["ratpoints_gpu", *kat["args"]])
    assert code == 0
    assert kat["contains"] in out.decode().splitlines()


def test_non_squarefree_rejected(oracle):
    assert not oracle.is_squarefree(["1", "-2", "1"])
    code, out, err, _ = oracle.run(["ratpoints_gpu", "1 -2 1", "10", "-q"])
    assert code == 1 and out == b"" and "not squarefree" in err


def test_c1_fixture(oracle, golden):
    c1 = golden["c1"]
    argv = ["ratpoints_gpu", c1["coefficients"], str(c1["height"]), "-dl", "1", "-du",
            str(c1["last"])]
    assert oracle.run(argv)[1].decode() == c1["stdout"]
    # pinned against the exhaustive reference oracle on a sub-box
    sub = ["ratpoints_gpu", c1["coefficients"], "2000", "-du", "12"]
    assert oracle.run(sub)[1] == oracle.exhaustive_output(c1["coefficients"], 2000, 1, 12)


def test_sieve_plus_verification_is_exhaustive(oracle):
    rng = random.Random(11)
    for _ in range(12):
        degree = rng.choice([2, 3, 4, 5, 6])
        while True:
            coeffs = [rng.randint(-9, 9) for _ in range(degree + 1)]
            if coeffs[-1] and oracle.is_squarefree(coeffs):
                break
        text = " ".join(map(str, coeffs))
        height, last = rng.randint(5, 40), rng.randint(1, 15)
        argv = ["ratpoints_gpu", text, str(height), "-du", str(last)]
        # -du is capped at the height (src/command_line.cpp:351-353)
        expected = oracle.exhaustive_output(text, height, 1, min(last, height))
        assert oracle.run(argv)[1] == expected, text


def test_survivor_digest_matches_python(oracle):
    sieve = oracle.ModularSieve(["1", "3", "0", "-7", "2"], 3000)
    survivors = sieve.survivors(1, 50)
    n, digest = sieve.count(1, 50)
    assert n == len(survivors)
    assert digest == sum(oracle.mix_pair(a, d) for a, d in survivors) % 2**64
    n_mt, digest_mt = sieve.count(1, 50, threads=4)
    assert (n_mt, digest_mt) == (n, digest)


@pytest.mark.parametrize("text,name,value", [
    ("1.5", "x", "3/2"), ("-2e-3", "x", "-1/500"), ("+.5E1", "x", "5"), ("7.", "x", "7")])
def test_parse_real(oracle, text, name, value):
    from fractions import Fraction
    assert oracle.parse_real(text, name) == Fraction(value)


@pytest.mark.parametrize("text,message", [
    ("", "must be real"), ("e5", "must be real"), ("1e", "must be real"), ("1x", "must be real"),
    ("1e10001", "exponent is too large")])
def test_parse_real_errors(oracle, text, message):
    with pytest.raises(oracle.UsageError, match=message):
        oracle.parse_real(text, "bound")
